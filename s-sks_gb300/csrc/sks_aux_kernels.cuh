// Kernels of the SEM time loop other than the step kernel: boundary-trace
// interpolation, the step-0 line set-up and injection, step-0 receiver
// sampling.  Included by the solver's translation unit only.
#pragma once
#include "sks_kernels.cuh"

namespace sks {

// coordinate of grid point j along a row or column of degree-deg elements
// of size eh (deg 3..6): element j/deg, GLL node j%deg at
// e*eh + (xi + 1)*eh/2 -- the node positions of the reference's
// boundary-trace generator (semsyn/src/aserpsv_sem.c:887-920), in the host
// generator's operation order.  Nodes: +-1 and the roots of P'_deg
// (3: +-1/sqrt(5); 4: 0, +-sqrt(3/7); 6: 0, +-sqrt((15 -+ 2 sqrt(15))/33)).
__device__ __forceinline__ double gll_pos(int j, double eh, int deg)
{
    const double xi3[3] = {-1.0, -0.4472135954999579, 0.4472135954999579};
    const double xi4[4] = {-1.0, -0.6546536707079771, 0.0, 0.6546536707079771};
    const double xi5[5] = {-1.0, -0.7650553239294647, -0.2852315164806451, 0.2852315164806451, 0.7650553239294647};
    const double xi6[6] = {-1.0, -0.8302238962785669, -0.46884879347071423, 0.0, 0.46884879347071423,
                           0.8302238962785669};
    const int e = j / deg, a = j - deg * e;
    const double xi = deg == 3 ? xi3[a] : deg == 5 ? xi5[a] : deg == 6 ? xi6[a] : xi4[a];
    return __dadd_rn(__dmul_rn((double)e, eh), __ddiv_rn(__dmul_rn(__dadd_rn(xi, 1.0), eh), 2.0));
}

// position of value c of a record on the interface line: family 0 (P-SV:
// u_bot(nx), w_bot(nx), u_left(nz), w_left(nz)) or 1 (SH: v_bot(nx),
// v_left(nz)); `vert` marks the w values
__device__ __forceinline__ void line_point(const RecSource& g, int fam, int c, double& x, double& z, bool& vert)
{
    const double line = gll_pos(g.nbl, g.eh, g.deg);               // height of row nbl = x of column nbl
    int part, j;
    if (!fam) {
        part = (c >= 2 * g.nx) ? 1 : 0;
        j = part ? (c - 2 * g.nx) % g.nz : c % g.nx;
        vert = part ? (c - 2 * g.nx) >= g.nz : c >= g.nx;
    } else {
        part = c >= g.nx ? 1 : 0;
        j = part ? c - g.nx : c;
        vert = false;
    }
    x = part ? line : gll_pos(j, g.eh, g.deg);
    z = part ? gll_pos(j, g.eh, g.deg) : line;
}

// Ricker pulse of the plane-wave generator, explicitly rounded FP64
// operations (only exp may round differently from a host evaluation)
__device__ __forceinline__ double ricker_at(double t, double pf)
{
    const double x = __dmul_rn(pf, t);
    const double a = __dmul_rn(x, x);
    return __dmul_rn(__dsub_rn(1.0, __dmul_rn(2.0, a)), exp(-a));
}

// An upgoing plane P-SV / SH wave with a Ricker pulse in the bottom layer
// (velocity vs, ray parameter p, dominant frequency f0), sampled every dp at
// the line's GLL node positions: value c of record r is amp_c R(r dp - 1.5/f0
// - tau_c), tau = p*x + eta*z, eta = sqrt(1/vs^2 - p^2); SV polarisation
// (eta*vs, -p*vs), z up; the w values hold -u_z, as the boundary files do.
// The per-value delay and amplitude are tabulated once (k_plane_line).
__device__ __forceinline__ double plane_eta(const RecSource& g)
{
    return sqrt(fmax(__dsub_rn(__ddiv_rn(1.0, __dmul_rn(g.vs, g.vs)), __dmul_rn(g.p, g.p)), 0.0));
}

static __global__ void __launch_bounds__(256) k_plane_line(RecSource g, double* __restrict__ lt)
{
    const int mtotal = 2 * (g.nx + g.nz), L = mtotal + g.nx + g.nz;
    const double eta = plane_eta(g);
    const double ux = __dmul_rn(__dmul_rn(g.sv_amp, eta), g.vs), uz = __dmul_rn(__dmul_rn(-g.sv_amp, g.p), g.vs);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) {
        const int fam = i >= mtotal ? 1 : 0, c = fam ? i - mtotal : i;
        double x, z;
        bool vert;
        line_point(g, fam, c, x, z, vert);
        lt[i] = __dadd_rn(__dmul_rn(g.p, x), __dmul_rn(eta, z));
        lt[L + i] = fam ? g.sh_amp : (vert ? -uz : ux);
    }
}

__device__ __forceinline__ float plane_record(const RecSource& g, int fam, int r, int c)
{
    const int mtotal = 2 * (g.nx + g.nz), L = mtotal + g.nx + g.nz, i = fam ? mtotal + c : c;
    const double delay = __ddiv_rn(1.5, g.f0);
    const double pf = __dmul_rn(3.141592653589793, g.f0);
    const double rk = ricker_at(__dsub_rn(__dsub_rn(__dmul_rn((double)r, g.dp), delay), g.lt[i]), pf);
    return (float)__dmul_rn(g.lt[L + i], rk);
}

// a series sampled every dt, periodic in nt samples, at time t: cubic
// Lagrange through the four samples around t
__device__ __forceinline__ double series_at(const double* __restrict__ f, int64_t nt, double t_over_dt)
{
    const double fl = floor(t_over_dt);
    const double d = t_over_dt - fl;
    int64_t i0 = (int64_t)fl % nt;
    if (i0 < 0) i0 += nt;
    const int64_t im = i0 == 0 ? nt - 1 : i0 - 1, i1 = i0 + 1 < nt ? i0 + 1 : i0 + 1 - nt,
                  i2 = i0 + 2 < nt ? i0 + 2 : i0 + 2 - nt;
    const double wm = -d * (d - 1.0) * (d - 2.0) / 6.0;
    const double w0 = (d + 1.0) * (d - 1.0) * (d - 2.0) / 2.0;
    const double w1 = -(d + 1.0) * d * (d - 2.0) / 2.0;
    const double w2 = (d + 1.0) * d * (d - 1.0) / 6.0;
    return wm * f[im] + w0 * f[i0] + w1 * f[i1] + w2 * f[i2];
}

// The upgoing P, SV and SH series a layered stack leaves in the bottom medium
// (vp0, vs0), each at t - p x - eta_m z: displacement P (p vp0, eta_p vp0),
// SV (eta_s vs0, -p vs0), SH u_y; the w values hold -u_z.  Per line value the
// two delays and the P and S coefficients are tabulated once (k_layered_line).
static __global__ void __launch_bounds__(256) k_layered_line(RecSource g, double* __restrict__ lt)
{
    const int mtotal = 2 * (g.nx + g.nz), L = mtotal + g.nx + g.nz;
    const double ep = sqrt(fmax(1.0 / (g.vp0 * g.vp0) - g.p * g.p, 0.0));
    const double es = sqrt(fmax(1.0 / (g.vs0 * g.vs0) - g.p * g.p, 0.0));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) {
        const int fam = i >= mtotal ? 1 : 0, c = fam ? i - mtotal : i;
        double x, z;
        bool vert;
        line_point(g, fam, c, x, z, vert);
        lt[i] = g.p * x + ep * z;
        lt[L + i] = g.p * x + es * z;
        lt[2 * L + i] = fam ? 0.0 : (vert ? -ep * g.vp0 : g.p * g.vp0);
        lt[3 * L + i] = fam ? 1.0 : (vert ? g.p * g.vs0 : es * g.vs0);
    }
}

__device__ __forceinline__ float layered_record(const RecSource& g, int fam, int r, int c)
{
    const int mtotal = 2 * (g.nx + g.nz), L = mtotal + g.nx + g.nz, i = fam ? mtotal + c : c;
    const double t = (double)r * g.dp;
    if (fam) return (float)series_at(g.ser + 2 * g.nt, g.nt, (t - g.lt[L + i]) / g.dts);
    const double fp = series_at(g.ser, g.nt, (t - g.lt[i]) / g.dts);
    const double fs = series_at(g.ser + g.nt, g.nt, (t - g.lt[L + i]) / g.dts);
    return (float)(fp * g.lt[2 * L + i] + fs * g.lt[3 * L + i]);
}

// record r, value c of family fam as the interpolation reads it
__device__ __forceinline__ double record_at(const RecSource& g, const float* __restrict__ rec, int fam, int n, int r,
                                            int c)
{
    if (g.kind == REC_PLANE) return (double)plane_record(g, fam, r, c);
    if (g.kind == REC_LAYERED) return (double)layered_record(g, fam, r, c);
    return (double)rec[(int64_t)r * n + c];
}

// Boundary-trace interpolation of one step (interpl.c:16-54) into one row of
// L = mtotal + shtotal values: four taps of FP32 records with FP64 weights,
// then the |g| >= 10 guard of sem2d_psvsh.c:432-444 (sequential, ends read 0).
// Called by a whole block.
__device__ __forceinline__ void interp_row(double* __restrict__ out, int it, const RecSource& g,
                                           const float* __restrict__ rpsv, int mtotal,
                                           const float* __restrict__ rsh, int shtotal,
                                           const int32_t* __restrict__ tap_psv, const double* __restrict__ w_psv,
                                           const int32_t* __restrict__ tap_sh, const double* __restrict__ w_sh,
                                           int* bad)
{
    if (threadIdx.x < 2) bad[threadIdx.x] = 0;
    __syncthreads();
    for (int fam = 0; fam < 2; fam++) {
        const int n = fam ? shtotal : mtotal;
        const float* rec = fam ? rsh : rpsv;
        const int32_t* tp = (fam ? tap_sh : tap_psv) + 4 * it;
        const double* wp = (fam ? w_sh : w_psv) + 4 * it;
        double* o = out + (fam ? mtotal : 0);
        int t[4]; double w[4];
#pragma unroll
        for (int j = 0; j < 4; j++) { t[j] = tp[j]; w[j] = wp[j]; }
        int anybad = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < 4; j++)
                // a zero weight adds exactly nothing to a generated (finite)
                // record: skip its evaluation (with dp = sdt the weights are
                // (0, 1, 0, 0)); table records keep every tap, as a non-finite
                // value in a file must reach the guard below
                if (t[j] >= 0 && (w[j] != 0.0 || g.kind == REC_TABLE))
                    s = fma(w[j], record_at(g, rec, fam, n, t[j], i), s);
            o[i] = s;
            if (!(s < 10.0 && s > -10.0)) anybad = 1;
        }
        if (anybad) bad[fam] = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int fam = 0; fam < 2; fam++) {
            if (!bad[fam]) continue;
            const int n = fam ? shtotal : mtotal;
            double* o = out + (fam ? mtotal : 0);
            for (int i = 0; i < n; i++)
                if (!(o[i] < 10.0 && o[i] > -10.0)) {
                    const double l = i > 0 ? o[i - 1] : 0.0, rr = i + 1 < n ? o[i + 1] : 0.0;
                    o[i] = (l + rr) / 2;
                }
        }
    }
}

// Interpolation for a chunk of steps: row r of Gout (r = 1..nsteps) is step s0+r-1.
static __global__ void __launch_bounds__(256) k_interp(double* __restrict__ Gout, int L, int s0, int nsteps,
                                                const RecSource g, const float* __restrict__ rpsv, int mtotal,
                                                const float* __restrict__ rsh, int shtotal,
                                                const int32_t* __restrict__ tap_psv, const double* __restrict__ w_psv,
                                                const int32_t* __restrict__ tap_sh, const double* __restrict__ w_sh)
{
    const int r = blockIdx.x;
    if (r >= nsteps) return;
    __shared__ int bad[2];
    interp_row(Gout + (int64_t)(r + 1) * L, s0 + r, g, rpsv, mtotal, rsh, shtotal, tap_psv, w_psv, tap_sh, w_sh, bad);
}

// One value triple of the interface-line increments: g(step of G row r+1) -
// g(step of G row r) at line point li, with the FP64 expressions of
// GRT_Interface4 (sem2d_psvsh.c:2076-2111), converted once to the form's type.
// Line points: row nbl (ix >= nbl), then column nbl (iz > nbl).
template <typename T>
__device__ __forceinline__ void line_delta_one(T* __restrict__ o, const double* __restrict__ G, int L, int r, int li,
                                               int nx, int nz, int nbl, int mtotal)
{
    const int nrow = nx - nbl;
    const double* g1 = G + (int64_t)(r + 1) * L;
    const double* g0 = G + (int64_t)r * L;
    const double *v1 = g1 + mtotal, *v0 = g0 + mtotal;
    double d3[3];
    if (li < nrow) {
        const int ix = nbl + li;
        d3[0] = -g0[ix] + g1[ix];
        d3[1] = -v0[ix] + v1[ix];
        d3[2] = g0[nx + ix] - g1[nx + ix];
    } else {
        const int iz = nbl + 1 + (li - nrow);
        d3[0] = -g0[2 * nx + iz] + g1[2 * nx + iz];
        d3[1] = -v0[nx + iz] + v1[nx + iz];
        d3[2] = g0[2 * nx + nz + iz] - g1[2 * nx + nz + iz];
    }
    o[0] = (T)d3[0]; o[1] = (T)d3[1]; o[2] = (T)d3[2];
}

// Increments of the interface line for the steps of a chunk: row r of Dl is
// step it0+r's injection g(it0+r) - g(it0+r-1) taken from G rows r+1 and r.
template <typename T>
__global__ void __launch_bounds__(256) k_line_delta(T* __restrict__ Dl, const double* __restrict__ G, int L,
                                                    int nsteps, int nx, int nz, int nbl, int mtotal)
{
    const int nline = (nx - nbl) + (nz - nbl - 1);
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)nsteps * nline) return;
    const int r = (int)(i / nline), li = (int)(i - (int64_t)r * nline);
    line_delta_one<T>(Dl + ((int64_t)r * nline + li) * 3, G, L, r, li, nx, nz, nbl, mtotal);
}

// Boundary inputs of one batch member, for the batched interpolation.
struct BatchAux {
    double* G;                     // interpolation rows [(chunk+2)][L]
    void* dl;                      // line increments [chunk+1][nline][3] in the form's type
    RecSource rs;                  // the records' source (tables below, or a generator)
    const float* rec_psv;
    const float* rec_sh;
    const int32_t* tap_psv;
    const int32_t* tap_sh;
    const double* w_psv;
    const double* w_sh;
    int mtotal, shtotal, nt_sem, nx, nz, nbl, L, nline;
};

// Batched interpolation: block (r, m) computes member m's G row r+1, the step
// it0+r, for the rows its chunk injects from (as run by one mesh's chunk).
static __global__ void __launch_bounds__(256) k_interp_batch(const BatchAux* __restrict__ aux,
                                                      const BatchState* __restrict__ state,
                                                      const BatchHeader* __restrict__ hdr)
{
    const int m = blockIdx.y, r = blockIdx.x;
    if (m >= hdr->nmem) return;
    const BatchState st = state[m];
    const BatchAux a = aux[m];
    if (st.n <= 0) return;
    const int ni = min(st.it0 + st.n + 1, a.nt_sem) - st.it0;
    if (r >= ni) return;
    __shared__ int bad[2];
    interp_row(a.G + (int64_t)(r + 1) * a.L, st.it0 + r, a.rs, a.rec_psv, a.mtotal, a.rec_sh, a.shtotal, a.tap_psv,
               a.w_psv, a.tap_sh, a.w_sh, bad);
}

// Batched line increments: blocks (x, m) stride over member m's rows.
template <typename T>
__global__ void __launch_bounds__(256) k_line_delta_batch(const BatchAux* __restrict__ aux,
                                                          const BatchState* __restrict__ state,
                                                          const BatchHeader* __restrict__ hdr)
{
    const int m = blockIdx.y;
    if (m >= hdr->nmem) return;
    const BatchState st = state[m];
    const BatchAux a = aux[m];
    if (st.n <= 0) return;
    const int nd = max(0, min(st.it0 + st.n + 1, a.nt_sem) - st.it0 - 1);
    const int64_t tot = (int64_t)nd * a.nline;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / a.nline), li = (int)(i - (int64_t)r * a.nline);
        line_delta_one<T>((T*)a.dl + ((int64_t)r * a.nline + li) * 3, a.G + a.L, a.L, r, li, a.nx, a.nz, a.nbl,
                          a.mtotal);
    }
}

// End of a chunk: every member's step moves on by the steps it took, and the
// next chunk takes up to `chunk` more, stopping at the member's target.
static __global__ void k_batch_advance(BatchState* __restrict__ state, const BatchHeader* __restrict__ hdr)
{
    for (int m = threadIdx.x; m < hdr->nmem; m += blockDim.x) {
        BatchState st = state[m];
        st.it0 += st.n;
        st.n = max(0, min(hdr->chunk, st.target - st.it0));
        state[m] = st;
    }
}

// GRT_Interface4 (sem2d_psvsh.c:2076-2111): u^n += g(it) - g(it-1) on row nbl
// (ix >= nbl) and column nbl (iz > nbl); the vertical component changes sign.
template <typename T, bool LF>
__global__ void __launch_bounds__(256) k_inject(T* __restrict__ u, T* __restrict__ dv, T* __restrict__ cc, int64_t np,
                                                int nx, int nz, int nbl, const double* __restrict__ Gcur,
                                                const double* __restrict__ Gprev, int mtotal)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nrow = nx - nbl, ncol = nz - nbl - 1;
    if (i >= nrow + ncol) return;
    const double *V = Gcur + mtotal, *V0 = Gprev + mtotal;
    int64_t g;
    double du, dvv, dw;
    if (i < nrow) {
        const int ix = nbl + i;
        g = (int64_t)nbl * nx + ix;
        du = -Gprev[ix] + Gcur[ix];
        dvv = -V0[ix] + V[ix];
        dw = Gprev[nx + ix] - Gcur[nx + ix];
    } else {
        const int iz = nbl + 1 + (i - nrow);
        g = (int64_t)iz * nx + nbl;
        du = -Gprev[2 * nx + iz] + Gcur[2 * nx + iz];
        dvv = -V0[nx + iz] + V[nx + iz];
        dw = Gprev[2 * nx + nz + iz] - Gcur[2 * nx + nz + iz];
    }
    const double dd[3] = {du, dvv, dw};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if constexpr (!LF) {
            u[ucomp(c, g, np)] += (T)dd[c];
        } else {
            float2* dc = reinterpret_cast<float2*>(dv);
            const T add = (T)dd[c];
            float2 p = dc[c * np + g];
            const T uu = u[ucomp(c, g, np)];
            const T y = add - p.y;
            const T t = uu + y;
            p.y = (t - uu) - y;
            p.x += add;
            u[ucomp(c, g, np)] = t;
            dc[c * np + g] = p;
        }
    }
}

// GRT_Interface (sem2d_psvsh.c:1953-2005) at step 0: set the line to g(0);
// the column pass wins at the corner (nbl, nbl).  u^{-1} = 0, so d = u.
template <typename T, bool LF>
__global__ void __launch_bounds__(256) k_init_line(T* __restrict__ u, T* __restrict__ dv, int64_t np,
                                                   int nx, int nz, int nbl, const double* __restrict__ G0, int mtotal)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nrow = nx - nbl - 1, ncol = nz - nbl;
    if (i >= nrow + ncol) return;
    const double* V = G0 + mtotal;
    int64_t g;
    double v3[3];
    if (i < nrow) {
        const int ix = nbl + 1 + i;
        g = (int64_t)nbl * nx + ix;
        v3[0] = G0[ix]; v3[1] = V[ix]; v3[2] = -G0[nx + ix];
    } else {
        const int iz = nbl + (i - nrow);
        g = (int64_t)iz * nx + nbl;
        v3[0] = G0[2 * nx + iz]; v3[1] = V[nx + iz]; v3[2] = -G0[2 * nx + nz + iz];
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
        u[ucomp(c, g, np)] = (T)v3[c];
        if constexpr (LF) reinterpret_cast<float2*>(dv)[c * np + g] = make_float2((T)v3[c], 0.f);
    }
}

// snapshot (sem2d.c:1667-1683) of the field in u: (u_x, u_y) of every second
// point, [ix/2][iz/2][2]
template <typename T>
__global__ void __launch_bounds__(256) k_snap(const T* __restrict__ u, int64_t np, int nx, int nz,
                                              float* __restrict__ out, int nzs)
{
    const int nxs = (nx + 1) / 2;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)nxs * nzs) return;
    const int ix = 2 * (int)(i / nzs), iz = 2 * (int)(i - (i / nzs) * nzs);
    const int64_t g = (int64_t)iz * nx + ix;
    out[2 * i] = (float)u[2 * g];
    out[2 * i + 1] = (float)u[2 * np + g];
}

// kirrecord_zhl (sem2d_psvsh.c:2116-2160): u_x, u_y, -u_z at the receivers;
// offset np addresses the reference's never-written extra point (reads 0)
template <typename T>
__global__ void __launch_bounds__(128) k_record(const T* __restrict__ u, int64_t np, const int64_t* __restrict__ off,
                                                int ntrace, float* __restrict__ out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= ntrace) return;
    const int64_t g = off[r];
    float vx = 0.f, vy = 0.f, vz = 0.f;
    if (g < np) { vx = (float)u[2 * g]; vy = (float)u[2 * np + g]; vz = (float)(-u[2 * g + 1]); }
    out[r] = vx;
    out[ntrace + r] = vy;
    out[2 * ntrace + r] = vz;
}

}  // namespace sks

