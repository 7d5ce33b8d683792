// Seismogram post-processing on the device: the band-pass the reference's
// scripts apply with SAC (`bp bu co 0.02 0.5 n 2 p 2`,
// applications/test/prem_epi83.pl:96-99) and the Silver & Chan (1991) shear-wave
// splitting measurement its cal_split.pl drives (applications/test/cal_split.pl:
// 7-56: the SKS window from 10 s before to 30 s after the arrival), for every
// receiver of a solve in one launch each.
//
// Band-pass: a Butterworth low-pass prototype of `poles` poles, transformed to
// a band-pass between the prewarped corners and to the z-plane by the bilinear
// transform: `poles` second-order sections, run in FP64 forward and, for two
// passes, backward (zero phase), one thread per trace.
// Splitting: one block per trace; the analysis window is placed around the
// largest radial amplitude (the arrival); the covariance of the fast and the
// advanced slow component of every trial (phi, delay) follows from windowed
// lagged sums of the two horizontal components; the smallest eigenvalue
// lambda2 is minimised on the grid (FP64).
#include "sks.h"

#include <cuda_runtime.h>
#include <cmath>
#include <complex>
#include <vector>

extern "C" int sks_internal_set_error(int code, const char* msg, cudaError_t e);

namespace {

int fail(int code, const char* msg, cudaError_t e = cudaSuccess) { return sks_internal_set_error(code, msg, e); }

constexpr int MAX_POLES = 8;

struct Sections {
    int n;
    double s[MAX_POLES][6];   // b0 b1 b2 a0 a1 a2 (a0 = 1)
};

// direct form II transposed, FP64 state; in place on x[0..nt) with stride 1
__device__ void run_sections(const Sections& S, float* x, int nt, bool backward)
{
    for (int k = 0; k < S.n; k++) {
        const double b0 = S.s[k][0], b1 = S.s[k][1], b2 = S.s[k][2], a1 = S.s[k][4], a2 = S.s[k][5];
        double z1 = 0.0, z2 = 0.0;
        for (int i = 0; i < nt; i++) {
            const int t = backward ? nt - 1 - i : i;
            const double v = x[t];
            const double y = b0 * v + z1;
            z1 = b1 * v - a1 * y + z2;
            z2 = b2 * v - a2 * y;
            x[t] = (float)y;
        }
    }
}

// one thread per trace and component: copy the strided trace into work and filter it
__global__ void k_bandpass(const float* __restrict__ rad, const float* __restrict__ trn, int ntrace, int nt, long long ld,
                           float* __restrict__ work, Sections S, int passes)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * ntrace) return;
    const int r = i % ntrace, comp = i / ntrace;
    const float* src = comp ? trn : rad;
    float* x = work + (size_t)comp * ntrace * nt + (size_t)r * nt;
    for (int t = 0; t < nt; t++) x[t] = src[(size_t)t * ld + r];
    if (S.n > 0) {
        run_sections(S, x, nt, false);
        if (passes == 2) run_sections(S, x, nt, true);
    }
}

struct SplitGrid {
    int kmax;          // delays 0..kmax samples
    int nphi;          // fast axes -90 + j*dphi
    double dphi_rad, dphi_deg;
    int before, after; // window samples around the radial peak
};

constexpr int SPLIT_THREADS = 256;

// one block per trace: window, lagged sums, grid search; out[r] = {phi deg,
// delay samples, lambda2/lambda1, window start sample}
__global__ void __launch_bounds__(SPLIT_THREADS) k_split(const float* __restrict__ work, int ntrace, int nt, SplitGrid g,
                                                         double* __restrict__ sums, float* __restrict__ out)
{
    const int r = blockIdx.x;
    const float* x = work + (size_t)r * nt;
    const float* y = work + (size_t)ntrace * nt + (size_t)r * nt;
    __shared__ float s_max[SPLIT_THREADS];
    __shared__ int s_arg[SPLIT_THREADS];
    __shared__ double s_l2[SPLIT_THREADS], s_l1[SPLIT_THREADS];
    __shared__ int s_j[SPLIT_THREADS];
    // 1. the arrival: the largest |radial| (first index on ties)
    float m = -1.f;
    int a = 0;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        const float v = fabsf(x[t]);
        if (v > m) { m = v; a = t; }
    }
    s_max[threadIdx.x] = m;
    s_arg[threadIdx.x] = a;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const float m2 = s_max[threadIdx.x + w];
            const int a2 = s_arg[threadIdx.x + w];
            if (m2 > s_max[threadIdx.x] || (m2 == s_max[threadIdx.x] && a2 < s_arg[threadIdx.x])) {
                s_max[threadIdx.x] = m2;
                s_arg[threadIdx.x] = a2;
            }
        }
        __syncthreads();
    }
    const int peak = s_arg[0];
    const int i0 = max(0, peak - g.before), i1 = min(nt, peak + g.after);
    // 2. S_ab(k) = sum_t a(t) b(t+k), T_ab(k) = sum_t a(t+k) b(t+k) over t in [i0, i1)
    double* S = sums + (size_t)r * 7 * (g.kmax + 1);
    for (int k = threadIdx.x; k <= g.kmax; k += blockDim.x) {
        double sxx = 0, sxy = 0, syx = 0, syy = 0, txx = 0, txy = 0, tyy = 0;
        for (int t = i0; t < i1; t++) {
            const double xw = x[t], yw = y[t];
            const double xs = t + k < nt ? (double)x[t + k] : 0.0, ys = t + k < nt ? (double)y[t + k] : 0.0;
            sxx += xw * xs; sxy += xw * ys; syx += yw * xs; syy += yw * ys;
            txx += xs * xs; txy += xs * ys; tyy += ys * ys;
        }
        double* o = S + k;
        o[0 * (g.kmax + 1)] = sxx; o[1 * (g.kmax + 1)] = sxy; o[2 * (g.kmax + 1)] = syx; o[3 * (g.kmax + 1)] = syy;
        o[4 * (g.kmax + 1)] = txx; o[5 * (g.kmax + 1)] = txy; o[6 * (g.kmax + 1)] = tyy;
    }
    __syncthreads();
    // 3. the (phi, delay) grid: smallest lambda2 (lowest phi, then lowest delay, on ties)
    const int K = g.kmax + 1;
    const double sxx0 = S[0], sxy0 = S[K], syy0 = S[3 * K];
    double best = INFINITY, best1 = 0.0;
    int bj = 0x7fffffff;
    for (int jp = threadIdx.x; jp < g.nphi; jp += blockDim.x) {
        const double phi = -0.5 * M_PI + jp * g.dphi_rad, c = cos(phi), s = sin(phi);
        const double c11 = c * c * sxx0 + 2 * c * s * sxy0 + s * s * syy0;
        for (int k = 0; k < K; k++) {
            const double c22 = s * s * S[4 * K + k] - 2 * c * s * S[5 * K + k] + c * c * S[6 * K + k];
            const double c12 = -c * s * S[k] + c * c * S[K + k] - s * s * S[2 * K + k] + c * s * S[3 * K + k];
            const double half = 0.5 * (c11 + c22);
            const double rad = sqrt(fmax(0.25 * (c11 - c22) * (c11 - c22) + c12 * c12, 0.0));
            const double l2 = half - rad;
            if (l2 < best) { best = l2; best1 = half + rad; bj = jp * K + k; }
        }
    }
    s_l2[threadIdx.x] = best;
    s_l1[threadIdx.x] = best1;
    s_j[threadIdx.x] = bj;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const double o2 = s_l2[threadIdx.x + w];
            const int oj = s_j[threadIdx.x + w];
            if (o2 < s_l2[threadIdx.x] || (o2 == s_l2[threadIdx.x] && oj < s_j[threadIdx.x])) {
                s_l2[threadIdx.x] = o2;
                s_l1[threadIdx.x] = s_l1[threadIdx.x + w];
                s_j[threadIdx.x] = oj;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int j = s_j[0];
        const int jp = j / K, k = j - jp * K;
        out[4 * r + 0] = (float)(-90.0 + jp * g.dphi_deg);
        out[4 * r + 1] = (float)k;
        out[4 * r + 2] = s_l1[0] > 0 ? (float)(s_l2[0] / s_l1[0]) : NAN;
        out[4 * r + 3] = (float)i0;
    }
}

}  // namespace

// Butterworth band-pass as second-order sections (see the file comment)
extern "C" int sks_bandpass_design(double f_lo, double f_hi, int32_t poles, double dt, double* sos)
{
    using cd = std::complex<double>;
    if (!sos || poles < 1 || poles > MAX_POLES) return fail(SKS_ERR_ARG, "band-pass: 1..8 poles");
    if (!(dt > 0) || !(f_lo > 0) || !(f_hi > f_lo) || !(f_hi < 0.5 / dt))
        return fail(SKS_ERR_ARG, "band-pass: need 0 < f_lo < f_hi < Nyquist");
    const double fs2 = 2.0 / dt;
    const double w1 = fs2 * std::tan(M_PI * f_lo * dt), w2 = fs2 * std::tan(M_PI * f_hi * dt);
    const double bw = w2 - w1, w0 = std::sqrt(w1 * w2);
    // analog prototype poles (unit cutoff), upper half plane first of each conjugate pair
    std::vector<cd> bp;
    for (int k = 0; k < poles; k++) {
        const cd p = std::exp(cd(0.0, M_PI * (2.0 * k + poles + 1) / (2.0 * poles)));
        // low-pass to band-pass: s^2 - p*bw*s + w0^2 = 0
        const cd pb = p * bw, disc = std::sqrt(pb * pb - 4.0 * w0 * w0);
        bp.push_back(0.5 * (pb + disc));
        bp.push_back(0.5 * (pb - disc));
    }
    // bilinear: z = (fs2 + s) / (fs2 - s); band-pass gain bw^poles, zeros at s = 0 (poles times) and infinity
    std::vector<cd> zp;
    cd gain = std::pow(cd(bw, 0.0), poles);
    for (const cd& s : bp) {
        zp.push_back((fs2 + s) / (fs2 - s));
        gain /= (fs2 - s);
    }
    gain *= std::pow(cd(fs2, 0.0), poles);      // the zeros at s = 0 map to z = 1 with factor fs2 each
    // pair the poles into sections: each complex pole with its conjugate, real
    // poles two by two (a real pair appears for odd prototypes and wide bands)
    std::vector<std::pair<cd, cd>> pairs;
    std::vector<cd> reals;
    for (const cd& z : zp) {
        if (std::fabs(z.imag()) <= 1e-14 * std::abs(z)) reals.push_back(cd(z.real(), 0.0));
        else if (z.imag() > 0) pairs.push_back({z, std::conj(z)});
    }
    for (size_t i = 0; i + 1 < reals.size(); i += 2) pairs.push_back({reals[i], reals[i + 1]});
    if ((int)pairs.size() != poles || reals.size() % 2) return fail(SKS_ERR_ARG, "band-pass: pole pairing failed");
    for (int k = 0; k < poles; k++) {
        const cd pa = pairs[k].first, pb = pairs[k].second;
        double* o = sos + 6 * k;
        // zeros {1, -1}: (1 - z^-1)(1 + z^-1) = 1 - z^-2; the whole gain in the first section
        const double g = k == 0 ? gain.real() : 1.0;
        o[0] = g; o[1] = 0.0; o[2] = -g;
        o[3] = 1.0; o[4] = -(pa + pb).real(); o[5] = (pa * pb).real();
    }
    return poles;
}

extern "C" int sks_split_scratch(int32_t ntrace, int32_t nt, double dt, const sks_split_opts_t* o, int64_t* work_floats,
                                 int64_t* sum_doubles)
{
    if (!o || !work_floats || !sum_doubles || ntrace < 1 || nt < 1 || !(dt > 0)) return fail(SKS_ERR_ARG, "bad arguments");
    *work_floats = 2 * (int64_t)ntrace * nt;
    *sum_doubles = 7 * (int64_t)ntrace * ((int64_t)std::lround(o->max_delay / dt) + 1);
    return SKS_OK;
}

extern "C" int sks_split_traces(const float* radial, const float* transverse, int32_t ntrace, int32_t nt, int64_t ld,
                                double dt, const sks_split_opts_t* o, float* work, double* sums, float* out,
                                void* stream)
{
    if (!radial || !transverse || !o || !work || !sums || !out) return fail(SKS_ERR_ARG, "NULL argument");
    if (ntrace < 1 || nt < 2 || ld < ntrace || !(dt > 0)) return fail(SKS_ERR_ARG, "bad trace dimensions");
    if (!(o->max_delay >= 0) || !(o->dphi > 0) || o->dphi > 90 || !(o->before >= 0) || !(o->after > 0))
        return fail(SKS_ERR_ARG, "bad splitting grid or window");
    if (o->passes != 1 && o->passes != 2) return fail(SKS_ERR_ARG, "passes: 1 or 2");
    Sections S;
    S.n = 0;
    if (o->f_lo > 0 && o->f_hi > 0) {
        double sos[MAX_POLES * 6];
        const int n = sks_bandpass_design(o->f_lo, o->f_hi, o->poles, dt, sos);
        if (n < 0) return n;
        S.n = n;
        for (int k = 0; k < n; k++)
            for (int i = 0; i < 6; i++) S.s[k][i] = sos[6 * k + i];
    }
    cudaStream_t st = (cudaStream_t)stream;
    k_bandpass<<<(2 * ntrace + 127) / 128, 128, 0, st>>>(radial, transverse, ntrace, nt, ld, work, S, o->passes);
    SplitGrid g;
    g.kmax = (int)std::lround(o->max_delay / dt);
    g.nphi = (int)std::floor(180.0 / o->dphi + 0.5);
    g.dphi_rad = o->dphi * M_PI / 180.0;
    g.dphi_deg = o->dphi;
    g.before = (int)std::lround(o->before / dt);
    g.after = (int)std::lround(o->after / dt);
    k_split<<<ntrace, SPLIT_THREADS, 0, st>>>(work, ntrace, nt, g, sums, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SKS_ERR_CUDA, "post-processing launch", e);
    return SKS_OK;
}
