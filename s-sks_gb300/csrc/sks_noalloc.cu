// Boundary increments without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need this
// computation: a serving process that has already divided the GPU's memory
// among its solve slots and hands each plugin only the buffers it owns, a
// host program that embeds the solver through a plugin interface whose rules
// forbid the plugin from allocating, or a latency-sensitive path where the
// implicit device synchronization of cudaMalloc/cudaFree is not acceptable.
// For them, sks_line_increments_noalloc() computes the same increments as
// sks_line_increments() from buffers the caller already has on the device,
// and keeps its FP64 interpolation rows in a fixed scratch array that is
// part of the library image instead of calling cudaMalloc.
#include "sks.h"
#include "sks_kernels.cuh"
#include "sks_aux_kernels.cuh"

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdio>
#include <mutex>

// Scratch for the FP64 interpolated traces: 1 Mi doubles (8 MiB).  Every GPU
// that loads the library holds it until the process exits.
static constexpr size_t kScratchDoubles = (size_t)1 << 20;
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

extern "C" int sks_internal_set_error(int code, const char* msg, cudaError_t e);

namespace {

// Device address of the scratch.  In host code the array's name is only a
// stand-in for the device symbol, never a usable address; the address itself
// belongs to a CUDA context (normally the device's primary context, which
// the runtime uses).  It is looked up with the device current on the first
// call, and again whenever the calling thread's current context is another
// one than the address was taken in (a context created after
// cudaDeviceReset, or a driver-API context the caller made current): contexts
// are told apart by their process-unique id (cuCtxGetId), reached through the
// runtime's driver entry points so the library needs no link to libcuda.
std::mutex g_mu;
struct Cached {
    unsigned long long ctx;   // id of the context the address is valid in (0: none yet)
    double* addr;
};
Cached g_addr[128] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;

int fail(int code, const char* msg, cudaError_t e = cudaSuccess) { return sks_internal_set_error(code, msg, e); }

// id of the calling thread's current context, 0 when none is current yet
// (called with g_mu held)
int current_context(unsigned long long* id)
{
    *id = 0;
    if (!g_ctx_current || !g_ctx_id) {
        void* p1 = nullptr;
        void* p2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p1, 12000, cudaEnableDefault, &q1);
        if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &p2, 12000, cudaEnableDefault, &q2);
        if (e != cudaSuccess || q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess)
            return fail(SKS_ERR_CUDA, "driver entry points cuCtxGetCurrent / cuCtxGetId", e);
        g_ctx_current = (CtxGetCurrentFn)p1;
        g_ctx_id = (CtxGetIdFn)p2;
    }
    CUcontext c = nullptr;
    if (g_ctx_current(&c) != CUDA_SUCCESS) return fail(SKS_ERR_CUDA, "cuCtxGetCurrent");
    if (c && g_ctx_id(c, id) != CUDA_SUCCESS) return fail(SKS_ERR_CUDA, "cuCtxGetId");
    return SKS_OK;
}

}  // namespace

extern "C" int sks_line_increments_noalloc(const float* rec_psv, const float* rec_sh, int32_t nx, int32_t nz,
                                           int32_t nbl, const int32_t* tap_psv, const double* w_psv,
                                           const int32_t* tap_sh, const double* w_sh, int32_t nsteps,
                                           double* out, void* stream)
{
    if (!rec_psv || !rec_sh || !tap_psv || !w_psv || !tap_sh || !w_sh || !out)
        return fail(SKS_ERR_ARG, "a device pointer is NULL");
    if (nx < 2 || nz < 2 || nbl < 0 || nbl >= nx - 1 || nbl >= nz - 1 || nsteps < 0)
        return fail(SKS_ERR_ARG, "bad sizes (nx, nz, nbl, nsteps)");
    if (nsteps == 0) return SKS_OK;
    // sizes in 64 bits, checked against the scratch before any narrowing
    const int64_t L64 = 3 * ((int64_t)nx + nz);
    const int64_t need = ((int64_t)nsteps + 2) * L64;
    if (need > (int64_t)kScratchDoubles)
        return fail(SKS_ERR_ARG, "nsteps too large for the fixed scratch: (nsteps+2)*(3*(nx+nz)) must be "
                                 "at most 1048576");
    const int mtotal = (int)(2 * ((int64_t)nx + nz)), shtotal = nx + nz, L = (int)L64;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SKS_ERR_CUDA, "cudaGetDevice", e);
    if (dev < 0 || dev >= 128) return fail(SKS_ERR_CUDA, "device index out of range");
    double* scratch;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        unsigned long long ctx = 0;
        int rc = current_context(&ctx);
        if (rc) return rc;
        if (!ctx || g_addr[dev].ctx != ctx) {
            // the lookup makes the runtime's context current when none is
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return fail(SKS_ERR_CUDA, "cudaGetSymbolAddress of the scratch", e);
            if ((rc = current_context(&ctx))) return rc;
            if (!ctx) return fail(SKS_ERR_CUDA, "no CUDA context is current after the scratch lookup");
            g_addr[dev] = Cached{ctx, (double*)p};
        }
        scratch = g_addr[dev].addr;
    }
    cudaStream_t st = (cudaStream_t)stream;
    // rows 1..nsteps+1 of the scratch hold g(step) for the nsteps+1 steps the
    // taps and weights describe; every row read below is written first, so
    // nothing needs clearing between calls
    sks::RecSource tables{};
    tables.kind = sks::REC_TABLE;
    sks::k_interp<<<nsteps + 1, 256, 0, st>>>(scratch, L, 0, nsteps + 1, tables, rec_psv, mtotal, rec_sh, shtotal,
                                              tap_psv, w_psv, tap_sh, w_sh);
    const int nline = (nx - nbl) + (nz - nbl - 1);
    const int64_t tot = (int64_t)nsteps * nline;
    sks::k_line_delta<double><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(out, scratch + L, L, nsteps, nx, nz, nbl,
                                                                             mtotal);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SKS_ERR_CUDA, "kernel launch", e);
    return SKS_OK;
}
