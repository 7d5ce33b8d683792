// Peak FMA throughput of the device's CUDA cores, measured: the denominator
// of the compute roofline of the FP64 form (bound by the FP64 pipe) and the
// FP32 figure beside it.  Every thread runs independent FMA chains long
// enough that the launch is seconds of pipe time at most; the rate is the
// best of a few event-timed launches.
#include "sks_internal.h"

namespace {

constexpr int CHAINS = 8;            // independent chains per thread (covers the pipe latency)
constexpr int ITERS = 2048;          // FMAs per chain

template <typename T>
__global__ void __launch_bounds__(256) k_fma_probe(T* out, T b, T c)
{
    T a[CHAINS];
#pragma unroll
    for (int i = 0; i < CHAINS; i++) a[i] = (T)(threadIdx.x + i);
    for (int k = 0; k < ITERS; k++) {
#pragma unroll
        for (int i = 0; i < CHAINS; i++) a[i] = fma(a[i], b, c);
    }
    T s = 0;
#pragma unroll
    for (int i = 0; i < CHAINS; i++) s += a[i];
    if (s == (T)-1.2345e-30) out[0] = s;     // never true for these inputs; keeps the chains live
}

template <typename T>
int probe(int device, double* tflops)
{
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return set_err(SKS_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
    int sms = 0, per_sm = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fma_probe<T>, 256, 0));
    const int blocks = sms * std::max(1, per_sm) * 4;
    T* out = nullptr;
    CK(cudaMalloc(&out, sizeof(T)));
    cudaEvent_t ev[2];
    CK(cudaEventCreate(&ev[0]));
    CK(cudaEventCreate(&ev[1]));
    double best = 0.0;
    const T b = (T)0.999999, c = (T)1e-7;
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
        cudaEventRecord(ev[0]);
        k_fma_probe<T><<<blocks, 256>>>(out, b, c);
        cudaEventRecord(ev[1]);
        e = cudaEventSynchronize(ev[1]);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
        const double flops = 2.0 * CHAINS * ITERS * 256.0 * blocks;
        if (e == cudaSuccess && rep > 0 && ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    cudaFree(out);
    if (e != cudaSuccess) return set_err(SKS_ERR_CUDA, "FMA probe: %s", cudaGetErrorString(e));
    *tflops = best;
    return SKS_OK;
}

}  // namespace

extern "C" int sks_probe_fma_peak(int device, int precision, double* tflops)
{
    if (!tflops) return set_err(SKS_ERR_ARG, "tflops is NULL");
    if (precision == SKS_FP64) return probe<double>(device, tflops);
    if (precision == SKS_FP32C) return probe<float>(device, tflops);
    return set_err(SKS_ERR_ARG, "unknown precision %d", precision);
}
