// Device kernels of the SEM time step (sm_103a, CUDA cores).
//
// One time step of semsyn's solver (semsyn/src/sem2d_psvsh.c:418-513) is
//   GRT_Interface4   u^n += incident-trace increment on the interface line
//   Stiff_Matrix     K = sum over elements of the element internal force
//   Time_diff_hybrid u^{n+1} = 2u^n - u^{n-1} - dt^2 M^-1 K
//   Absorbs          centred Stacey form on the left/bottom/right edges
//   kirrecord_zhl    sample the surface receivers.
// Here the element force, the assembly and the update are one kernel.
//
// Tiling.  A warp covers TEX=6 consecutive elements in x: lane l = 5e + a
// (e = element 0..5, a = GLL column 0..4) holds the 5 points of column a of
// its element for the current element row in registers.  d/dz contractions
// run inside a lane (its own column), d/dx and the x part of the divergence
// read the other 4 columns of the element with warp shuffles.  A CTA puts NW
// warps side by side and walks a band of HZ element rows bottom-up; the top
// row of one element row is the bottom row of the next, so its displacement
// and its partial force are carried in registers.  Each CTA recomputes one
// element column to its left and one element row below its band (halos), so
// every point it owns receives all of its element contributions inside the
// CTA: the force of a point is gathered in a fixed order (left element
// first, lower element first; in-warp by shuffle, warp to warp through shared
// memory), with no atomics, no global force array and no second pass.  The
// update, the receiver sampling and the next step's boundary injection are
// applied where the point's force is complete.
//
// Forms.  LF=false: FP64, the reference's 3-level update (two displacement
// buffers; u^{n+1} overwrites u^{n-1}).  LF=true: FP32 leapfrog on
// (u, d = u^n - u^{n-1}) with Kahan compensation of u += d; it is the same
// recurrence as the 3-level form (d^{n+1} = d^n - dt^2 M^-1 K inside,
// ((M-A) d^n - dt^2 K)/(M+A) on the Stacey edges, injection adds the
// increment to both u and d).  The FP64 kernels are bound by the FP64 pipe
// and spend registers to save its operations: z contractions in even-odd
// form (mirror_sum) and the x-divergence weights times the row weight from a
// shared table; the FP32 kernels are bound by issue and registers and keep
// row-by-row sums.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sks {

constexpr int N = 4;          // GLL degree of the default instantiation
constexpr int NP = N + 1;     // points per element edge
constexpr int TEX = 6;        // elements per warp tile in x
constexpr int TW = TEX * N;   // grid columns per warp tile

// The kernels are templates on the degree DEG (default 4; 3, 5 and 6 are
// instantiated too): DEG+1 lanes per element and 30 / (DEG+1) elements per
// warp, so degrees 4 and 5 fill lanes 0..29 and leave 30, 31 idle, degrees 3
// (7 elements of 4 lanes) and 6 (4 elements of 7 lanes) fill lanes 0..27.
__host__ __device__ constexpr int tex_of(int deg) { return 30 / (deg + 1); }
constexpr int MAT_STRIDE = 16;

// GLL tables of degree N, the same for every mesh.  The element size drops out
// of the internal force: d/dx = (2/eh) d/dxi and the quadrature carries
// (eh/2)^2, so K = sum C (l' u) l' w w with unscaled derivatives.  The tables
// hold l'_i(xi_j) and l'_i(xi_j) w_j without the 2/eh and eh/2 factors, and
// one kernel argument serves every instance of a batch.
template <typename T, int DEG = N>
struct Coef {
    static constexpr int NP = DEG + 1, H = NP / 2;
    T D[NP * NP];    // D[j*NP+i]  = l'_i(xi_j)
    T DWs[NP * NP];  // DWs[j*NP+i] = l'_i(xi_j) * w_j
    T w[NP];         // GLL weights
    T winv[NP];      // 1/w_a: inverse lumped-mass weight of a point inside an element edge
    T winv2;         // 1/(2 w_0): a point shared by two elements along x (or z)
    // The FP64 kernels' in-lane z contractions in even-odd form (mirror_sum):
    // [0] the gradient, A[a][t] = D[a][t]; [1] the divergence, A[a][t] = DWs[t][a]
    T P[2][H * H];   // (A[a][t] - A[a][N-t]) / 2, a, t < H
    T Q[2][H * H];   // (A[a][t] + A[a][N-t]) / 2
    T R[2][H];       // A[a][H]   (odd NP: the middle column)
    T Mid[2][H];     // A[H][t]   (odd NP: the middle row)
};

// y_a = sum_t A[a][t] v_t (a, t = 0..DEG) for a matrix with A[N-a][N-t] =
// -A[a][t], as l'_t(xi_a) and l'_a(xi_t) w_t are on the mirror-symmetric GLL
// points: from the mirrored sums e_t = v_t + v_{N-t} and differences
// o_t = v_t - v_{N-t}, y_a + y_{N-a} = 2 sum_t P[a][t] o_t and
// y_a - y_{N-a} = 2 (sum_t Q[a][t] e_t + R[a] v_H), and y_H = sum_t Mid[t] o_t.
// Degree 4: 20 operations instead of 25 (a sum of the same terms in another
// order, within FP64 rounding of the direct sum).  The sums and differences
// are rounded adds that the compiler never fuses with a product (v may be a
// product, e.g. an isotropic stress mu e): fused or not could then depend on
// the kernel the code is inlined into, and every kernel must give the same bits.
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }

template <typename T, int DEG>
__device__ __forceinline__ void mirror_sum(const T v[DEG + 1], const T* P, const T* Q, const T* R, const T* Mid,
                                           T y[DEG + 1])
{
    constexpr int N = DEG, NP = DEG + 1, H = NP / 2;
    T e[H], o[H];
#pragma unroll
    for (int t = 0; t < H; t++) { e[t] = add_rn(v[t], v[N - t]); o[t] = sub_rn(v[t], v[N - t]); }
#pragma unroll
    for (int a = 0; a < H; a++) {
        T sp = P[a * H] * o[0], sm = Q[a * H] * e[0];
#pragma unroll
        for (int t = 1; t < H; t++) { sp = fma(P[a * H + t], o[t], sp); sm = fma(Q[a * H + t], e[t], sm); }
        if constexpr (NP & 1) sm = fma(R[a], v[H], sm);
        y[a] = add_rn(sp, sm);
        y[N - a] = sub_rn(sp, sm);
    }
    if constexpr (NP & 1) {
        T m = Mid[0] * o[0];
#pragma unroll
        for (int t = 1; t < H; t++) m = fma(Mid[t], o[t], m);
        y[H] = m;
    }
}

template <typename T>
struct Geo {
    int nex, nez, nx, nz;
    int ncx, ncz, HZ, nblocks;    // CTA grid: ncx columns x ncz row bands of HZ element rows
    const int4* items;            // or per CTA (column, band, first row, end row): balanced bands
    int nbl;                      // GRT interface line: row nbl (ix >= nbl), column nbl (iz > nbl)
    int64_t np;                   // nx*nz
    T dt2_Je;                     // sdt^2 / Je   (M^-1 dt^2 = dt2_Je / (rho Wx Wz))
};

// Where the boundary records the interpolation reads come from: the record
// tables (files or caller memory), or a device generator evaluated at each
// record the interpolation reads, so generated runs hold no record table.
enum { REC_TABLE = 0, REC_PLANE = 1, REC_LAYERED = 2 };
struct RecSource {
    int kind;
    int nx, nz, nbl, deg;              // the grid, the interface line, the GLL degree (4 or 5)
    double eh, dp, p;                  // element size, record step, ray parameter
    double vs, f0, sv_amp, sh_amp;     // REC_PLANE: the half-space wave
    const double* lt;                  //   per line value (P-SV then SH): delay p x + eta z [L], amplitude [L]
    const double* ser;                 // REC_LAYERED: mode series [3][nt], samples dts apart; lt: per line
                                       //   value tau_p, tau_s [L] each, then the P and S coefficients [L] each
    int64_t nt;
    double dts, vp0, vs0;              //   the top medium of the stack
};

template <typename T>
struct Field {
    const T* __restrict__ uc;     // u^n: (u_x, u_z) pairs [np], then u_y [np]
    T* __restrict__ un;           // FP64: u^{n-1} in, u^{n+1} out; FP32: u^{n+1} out
    T* __restrict__ dv;           // FP32 form: per component a float2 (d, c): the increment
                                  // d = u^n - u^{n-1} and the Kahan compensation of u, [3][np]
    // boundary taper (atten > 0): factors taper[0..nh-1], 1 at the zone's
    // inner edge; the zones and nh are in taper_zones at the end
    const T* __restrict__ taper;
    const uint16_t* __restrict__ mid;   // material index per point
    const T* __restrict__ mat;          // [nmat][16]: 15 stiffness entries, 1/rho
    const T* __restrict__ stc;          // Stacey coefficients [nbnd][3][3]: dt^2/(M+A), 2M/(M+A), (M-A)/(M+A)
    // next step's boundary injection, fused into this step's write: the
    // increments g(it+1) - g(it) of the interface line, [line point][3]
    // (row points ix >= nbl first, then column points iz > nbl)
    const T* __restrict__ dline;
    int inject_next;                    // it+1 < number of injecting steps
    // receivers, fused: a bitmap over points, then the sorted offsets
    const uint32_t* __restrict__ recbits;
    const int64_t* __restrict__ rec_off;     // sorted
    const int32_t* __restrict__ rec_idx;     // trace index of each sorted offset
    int nrec, ntrace;
    int rec_iz0, rec_iz1;                    // rows holding receivers
    float* __restrict__ seis_row;            // [3][ntrace] of this step
    // band seams (ZS variants): the force a band-boundary row gets from the
    // band below (lo) and the band above (hi), [segment][nx][6] = the left
    // element's part (3) and the own element's part (3), and one arrival
    // counter per (segment, CTA column)
    T* __restrict__ seam_lo;
    T* __restrict__ seam_hi;
    int* __restrict__ seam_cnt;
    // snapshot of this step (plot_snap), or null: (u_x, u_y) of every second
    // point, [ix/2][iz/2][2] with snap_nzs = (nz+1)/2 rows of iz per ix
    float* __restrict__ snap;
    int snap_nzs;
    // the taper's zones in the struct's tail padding: atten (0: none; 1..4:
    // bottom, + left, + right, + top) in bits 0-2, nh = neh*hpn above them
    int taper_zones;
    // set to 1 by any point whose new displacement is not finite (sticky;
    // the host reads and clears it)
    int* nonfinite;
    // per element row: 1 when every point of its grid rows has an isotropic
    // material (the anisotropic kernels take the isotropic stress there)
    const uint8_t* __restrict__ row_iso;
    // per element row: the material of all its points when they share one
    // (layered models: nearly every row), else -1 (read per point from mid)
    const int16_t* __restrict__ row_mat;
};

// Displacement layout: the P-SV pair (u_x, u_z) of every point as one 2-vector
// ([np] pairs), then u_y ([np]); 3*np values in all.
template <typename T> struct Pair;
template <> struct Pair<float> { using type = float2; };
template <> struct Pair<double> { using type = double2; };

__device__ __forceinline__ int64_t ucomp(int c, int64_t g, int64_t np)
{
    return c == 1 ? 2 * np + g : 2 * g + (c == 2 ? 1 : 0);
}

// loads of values other CTAs of the same launch may have written (CG: through
// L2 only, never a stale L1 line) or that no one writes during the launch
template <bool CG, typename X>
__device__ __forceinline__ X ldv(const X* p)
{
    if constexpr (CG) return __ldcg(p);
    else return *p;
}

template <typename T, bool CG = false>
__device__ __forceinline__ void load_u(const T* __restrict__ U, int np, int g, T out[3])
{
    using V = typename Pair<T>::type;
    const V p = ldv<CG>(reinterpret_cast<const V*>(U) + g);
    out[0] = p.x;
    out[2] = p.y;
    out[1] = ldv<CG>(U + 2 * np + g);
}

template <typename T>
__device__ __forceinline__ void store_u(T* __restrict__ U, int np, int g, const T v[3])
{
    using V = typename Pair<T>::type;
    V p;
    p.x = v[0];
    p.y = v[2];
    reinterpret_cast<V*>(U)[g] = p;
    U[2 * np + g] = v[1];
}

template <int DEG = N>
__device__ __forceinline__ int64_t stacey_index(int ix, int iz, int nx, int nz)
{
    constexpr int N = DEG;
    if (ix == 0) return iz;
    if (iz == 0) return (int64_t)nz + ix;
    if (ix == nx - 1) return (int64_t)nz + nx + iz;
    if (iz == nz - 1 && ix >= 1 && ix <= 3 * N) return 2 * (int64_t)nz + nx + ix;
    return -1;
}

// material row -> registers
template <typename T, bool ANISO>
struct MatRow;

template <>
struct MatRow<double, true> {
    double s[MAT_STRIDE];
    __device__ __forceinline__ void load(const double* __restrict__ m) {
        const double2* p = reinterpret_cast<const double2*>(m);
#pragma unroll
        for (int i = 0; i < 8; i++) { double2 v = __ldg(p + i); s[2 * i] = v.x; s[2 * i + 1] = v.y; }
    }
};
template <>
struct MatRow<float, true> {
    float s[MAT_STRIDE];
    __device__ __forceinline__ void load(const float* __restrict__ m) {
        const float4* p = reinterpret_cast<const float4*>(m);
#pragma unroll
        for (int i = 0; i < 4; i++) { float4 v = __ldg(p + i); s[4 * i] = v.x; s[4 * i + 1] = v.y; s[4 * i + 2] = v.z; s[4 * i + 3] = v.w; }
    }
};
template <typename T>
struct MatRow<T, false> {
    T s[MAT_STRIDE];   // only s[0] (C11=C33), s[4] (C13), s[5] (C66=C55=C44), s[15] (1/rho) used
    __device__ __forceinline__ void load(const T* __restrict__ m) {
        s[0] = __ldg(m); s[4] = __ldg(m + 4); s[5] = __ldg(m + 5); s[15] = __ldg(m + 15);
    }
};

// stress on the strain list (e11, e12=u_y,x, e13=u_z,x+u_x,z, e23=u_y,z, e33):
// sigma_a = sum_b C[a][b] e_b in b order, as Stress_ij (sem2d_psvsh.c:1345-1380).
// iso (anisotropic FP64 kernels, an element row of isotropic materials only):
// the isotropic form, which gives the anisotropic sums' values for an
// isotropic material (the zero entries' products add nothing but the sign of
// an exact zero; C33 = C11, C55 = C44 = C66), with 7 operations instead of 25
template <typename T, bool ANISO>
__device__ __forceinline__ void stress(const MatRow<T, ANISO>& M, const T e[5], T s[5], bool iso = false)
{
    if (ANISO && !iso) {
        const T* c = M.s;   // upper triangle: 0..4 row0, 5..8 row1, 9..11 row2, 12..13 row3, 14 row4
        s[0] = c[0] * e[0];  s[0] = fma(c[1], e[1], s[0]);  s[0] = fma(c[2], e[2], s[0]);  s[0] = fma(c[3], e[3], s[0]);  s[0] = fma(c[4], e[4], s[0]);
        s[1] = c[1] * e[0];  s[1] = fma(c[5], e[1], s[1]);  s[1] = fma(c[6], e[2], s[1]);  s[1] = fma(c[7], e[3], s[1]);  s[1] = fma(c[8], e[4], s[1]);
        s[2] = c[2] * e[0];  s[2] = fma(c[6], e[1], s[2]);  s[2] = fma(c[9], e[2], s[2]);  s[2] = fma(c[10], e[3], s[2]); s[2] = fma(c[11], e[4], s[2]);
        s[3] = c[3] * e[0];  s[3] = fma(c[7], e[1], s[3]);  s[3] = fma(c[10], e[2], s[3]); s[3] = fma(c[12], e[3], s[3]); s[3] = fma(c[13], e[4], s[3]);
        s[4] = c[4] * e[0];  s[4] = fma(c[8], e[1], s[4]);  s[4] = fma(c[11], e[2], s[4]); s[4] = fma(c[13], e[3], s[4]); s[4] = fma(c[14], e[4], s[4]);
    } else {
        const T l2m = M.s[0], lam = M.s[4], mu = M.s[5];
        s[0] = fma(lam, e[4], l2m * e[0]);
        s[1] = mu * e[1];
        s[2] = mu * e[2];
        s[3] = mu * e[3];
        s[4] = fma(l2m, e[4], lam * e[0]);
    }
}

// The state a lane needs to update one owned point, loaded at the start of
// the element row so its latency overlaps the element force.
template <typename T, bool LF>
struct Aux {
    T a[3];            // FP64: u^{n-1};  FP32: d
    T b[LF ? 3 : 1];   // FP32: Kahan compensation
};

template <typename T, bool LF, bool CG = false>
__device__ __forceinline__ void load_aux(const Field<T>& F, int np, int g, Aux<T, LF>& x)
{
    // 32-bit offsets: 3*np < 2^31 (checked on the host)
    if constexpr (!LF) {
        load_u<T, CG>(F.un, np, g, x.a);
    } else {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float2 v = ldv<CG>(reinterpret_cast<const float2*>(F.dv) + c * np + g);
            x.a[c] = v.x;
            x.b[c] = v.y;
        }
    }
}

// Where a lane's point sits, as far as the update cares: the lane-constant
// part of the absorbing-edge, interface-line and receiver tests.
struct PointFlags {
    bool edge_x;     // left or right column of the box
    bool top_ok;     // column 1..3N (the top-row Stacey points)
    bool on_col;     // the interface column ix == nbl
    bool row_ok;     // ix >= nbl (the interface row's extent)
};

// atten_wave2 (sem2d_psvsh.c:1780-1822) at one point: u^{n+1} times the
// factor of each zone holding the point, in the reference's zone order.  The
// FP32 form keeps its state consistent with the scaled value: the Kahan term
// scales with u (the product's rounding error folded in), and the increment d
// = u^{n+1} - u^n takes the change of u (exact while the factors are at
// least 1/2, as with the default ass = 0.93).
template <typename T, bool LF>
__device__ __forceinline__ void taper_point(const Field<T>& F, const Geo<T>& G, int ix, int iz, T un[3], T dn[3],
                                            T cn[3])
{
    const int atten = F.taper_zones & 7, nh = F.taper_zones >> 3, nx = G.nx, nz = G.nz;
    auto scale = [&](T f) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            if constexpr (!LF) {
                un[c] *= f;
            } else {
                const T u0 = un[c], u1 = u0 * f;
                const T e = fma(f, u0, -u1);
                cn[c] = fma(f, cn[c], -e);
                dn[c] += u1 - u0;
                un[c] = u1;
            }
        }
    };
    if (iz < nh) scale(F.taper[nh - iz - 1]);
    if (atten > 1 && ix < nh && iz >= nh) scale(F.taper[nh - ix - 1]);
    if (atten > 2 && ix >= nx - nh && iz >= nh) scale(F.taper[ix - nx + nh]);
    if (atten > 3 && iz >= nz - nh && ix < nx - nh && ix >= nh) scale(F.taper[iz - nz + nh]);
}

// A point's new displacement is bad when a component is NaN or infinite.
// FP32: the magnitudes' sum is not below the largest finite float (also true
// when finite components sum past it: a blown-up field).  FP64: an exponent
// field of all ones, tested on the high words with integer instructions, so
// the check takes nothing from the FP64 pipe the form is bound by.
__device__ __forceinline__ bool not_finite3(const float v[3])
{
    return !(fabsf(v[0]) + fabsf(v[1]) + fabsf(v[2]) <= 3.402823466e38f);
}
__device__ __forceinline__ bool not_finite3(const double v[3])
{
    const unsigned e0 = (unsigned)__double2hiint(v[0]) & 0x7ff00000u;
    const unsigned e1 = (unsigned)__double2hiint(v[1]) & 0x7ff00000u;
    const unsigned e2 = (unsigned)__double2hiint(v[2]) & 0x7ff00000u;
    return max(max(e0, e1), e2) == 0x7ff00000u;
}

// update one owned point, sample it if it is a receiver, then add the next
// step's boundary increment if it lies on the interface line.
// M^-1 dt^2 = wxi * wzi * rinv: wxi is the column's inverse lumped-mass
// weight times dt^2/Je, wzi the row's, rinv 1/rho.
// plain: the CTA's tile holds no Stacey edge point, receiver, snapshot point,
// interface-line point or taper zone (tile-uniform), so none of their tests runs
template <typename T, bool LF, bool TP = false, int DEG = N>
__device__ __forceinline__ void finish_point(const Field<T>& F, const Geo<T>& G, const Coef<T, DEG>& k,
                                             int ix, int iz, const T u[3], const T K[3], T rinv,
                                             T wxi, T wzi, const Aux<T, LF>& x, const PointFlags& pf, bool plain)
{
    const int g = iz * G.nx + ix;
    const bool edge = !plain && (pf.edge_x || iz == 0 || (iz == G.nz - 1 && pf.top_ok));
    T un[3], dn[3], cn[3];
    if (!LF) {
        if (!edge) {
            const T mdt2 = (wxi * wzi) * rinv;   // wxi carries dt^2/Je
            // two FMAs a component (2u - u_prev is one rounding)
#pragma unroll
            for (int c = 0; c < 3; c++) un[c] = fma(-mdt2, K[c], fma((T)2, u[c], -x.a[c]));
        } else {
            const T* p = F.stc + stacey_index<DEG>(ix, iz, G.nx, G.nz) * 9;
#pragma unroll
            for (int c = 0; c < 3; c++) un[c] = (-p[3 * c] * K[c] + p[3 * c + 1] * u[c]) - p[3 * c + 2] * x.a[c];
        }
    } else {
        if (!edge) {
            const T mdt2 = (wxi * wzi) * rinv;   // wxi carries dt^2/Je
#pragma unroll
            for (int c = 0; c < 3; c++) dn[c] = fma(-mdt2, K[c], x.a[c]);
        } else {
            const T* p = F.stc + stacey_index<DEG>(ix, iz, G.nx, G.nz) * 9;
#pragma unroll
            for (int c = 0; c < 3; c++) dn[c] = p[3 * c + 2] * x.a[c] - p[3 * c] * K[c];
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const T y = dn[c] - x.b[c];
            const T t = u[c] + y;
            cn[c] = (t - u[c]) - y;
            un[c] = t;
        }
    }
    if constexpr (TP) {
        if (F.taper_zones) taper_point<T, LF>(F, G, ix, iz, un, dn, cn);
    }
    if (!plain) {
    // kirrecord_zhl: the field after the update, before the next injection
    if (iz >= F.rec_iz0 && iz <= F.rec_iz1 && ((__ldg(F.recbits + (g >> 5)) >> (g & 31)) & 1u)) {
        int lo = 0, hi = F.nrec;
        while (lo < hi) { const int mdl = (lo + hi) >> 1; if (F.rec_off[mdl] < g) lo = mdl + 1; else hi = mdl; }
        for (int r = lo; r < F.nrec && F.rec_off[r] == g; r++) {
            const int t = F.rec_idx[r];
            F.seis_row[t] = (float)un[0];
            F.seis_row[F.ntrace + t] = (float)un[1];
            F.seis_row[2 * F.ntrace + t] = (float)(-un[2]);
        }
    }
    // snapshot (sem2d.c:1667-1683): the same field as the receivers see
    if (F.snap && !((ix | iz) & 1)) {
        float* q = F.snap + ((size_t)(ix >> 1) * F.snap_nzs + (iz >> 1)) * 2;
        q[0] = (float)un[0];
        q[1] = (float)un[1];
    }
    // GRT_Interface4 of the next step (sem2d_psvsh.c:2076-2111)
    if (F.inject_next && ((iz == G.nbl && pf.row_ok) || (pf.on_col && iz > G.nbl))) {
        const int li = iz == G.nbl ? ix - G.nbl : (G.nx - G.nbl) + (iz - G.nbl - 1);
        const T* d3 = F.dline + 3 * li;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            if (!LF) {
                un[c] += d3[c];
            } else {
                const T add = d3[c];
                const T y = add - cn[c];
                const T t = un[c] + y;
                cn[c] = (t - un[c]) - y;
                un[c] = t;
                dn[c] += add;
            }
        }
    }
    }
    if (not_finite3(un)) *F.nonfinite = 1;
    const int np = (int)G.np;
    store_u<T>(F.un, np, g, un);
    if constexpr (LF) {
#pragma unroll
        for (int c = 0; c < 3; c++) reinterpret_cast<float2*>(F.dv)[c * np + g] = make_float2(dn[c], cn[c]);
    }
}

// The SEM step.  CTA = NW warps side by side in x: 6*NW elements, the first
// one a halo (recomputed, owned by the CTA to the left), so every owned point
// receives all its x contributions inside the CTA; a band of HZ element rows.
// Warps hand the force of their last column to the next warp through shared
// memory, once per element row.  The row between two bands takes force from
// both: with ZS=false each band recomputes the element row below it (halo);
// with ZS=true each band writes its partial force of the boundary row to
// global memory and bumps the segment's arrival counter, and the band that
// arrives second adds the two partials (lower band first) and updates the
// row -- nothing waits and nothing is computed twice.
//
// Per element row a lane keeps its 5 displacements (3 components) and 5
// force accumulators: row b's stress adds its x-divergence to accumulator b
// and its z-divergence to all five, so no per-point stress is stored.
//
// CAP: 0 = the compiler's register choice; 1 / 2 = ask for 16 / 20 (FP32)
// or 8 / 12 (FP64) resident warps per SM (at most 128 / 102 or 255 / 170
// registers a thread).
template <typename T>
constexpr int cap_warps(int cap) { return cap == 0 ? 0 : (sizeof(T) == 4 ? (cap == 1 ? 16 : 20) : (cap == 1 ? 8 : 12)); }

// shared memory of one CTA tile
template <typename T, int NW, int DEG = N>
struct TileShared {
    static constexpr int NP = DEG + 1, XW = sizeof(T) == 8 ? NP * (NP * NP + 1) : 1;
    T xch[2][NW][DEG][3];   // force of a warp's last column, for the next warp
    T xtop[NW][3];          // the same for the band's top row
    // FP64: the x-divergence weights of each GLL column a and row b, in the
    // rotated order the lanes read them, times the row weight:
    // xw[a][b][r] = l'_a(xi_t) w_t w_b, t = (a + r) mod NP (a's stride
    // NP*NP+1 keeps the 5-7 columns a warp reads in distinct banks)
    T xw[XW];
    int second_arrival;
};

// a kernel's first act: the CTA's constant shared tables (FP64 forms), then a
// barrier; nothing for the FP32 forms
template <typename T, int NW, int DEG>
__device__ __forceinline__ void init_tile_shared(TileShared<T, NW, DEG>& sh, const Coef<T, DEG>& k)
{
    if constexpr (sizeof(T) == 8) {
        constexpr int NP = DEG + 1, SA = NP * NP + 1;
        for (int i = threadIdx.x; i < NP * SA; i += blockDim.x) {
            const int a = i / SA, q = i - a * SA, b = q / NP, r = q - b * NP;
            const int t = a + r < NP ? a + r : a + r - NP;
            sh.xw[i] = q < NP * NP ? k.DWs[t * NP + a] * k.w[b] : (T)0;
        }
        __syncthreads();
    }
}

// One CTA tile: element column cx (S = 6*NW-1 owned elements), band cz of
// element rows [ez0, ez1).
template <typename T, bool ANISO, bool LF, int NW, bool ZS, bool CG = false, bool TP = false, int DEG = N>
__device__ __forceinline__ void step_tile(const Field<T>& F, const Geo<T>& G, const Coef<T, DEG>& k, int cx, int cz,
                                          int ez0, int ez1, TileShared<T, NW, DEG>& sh)
{
    constexpr int N = DEG, NP = DEG + 1, TEX = tex_of(DEG);
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    constexpr int S = TEX * NW - 1;                // owned elements per CTA
    constexpr int LANES = TEX * NP;                // lanes holding element columns (28 or 30)
    const int e = lane / NP, al = lane - e * NP;   // lanes >= LANES: e = TEX
    const int q = TEX * w + e;                     // element within the CTA
    const int ex = cx * S - 1 + q;
    const bool live = lane < LANES && ex >= 0 && ex < G.nex;
    const int nx = G.nx;
    // lanes off the mesh read a valid column; their force never reaches a
    // live lane (shuffles stay inside an element, the left neighbour is masked)
    const int ix = live ? ex * N + al : min(max(ex * N + al, 0), nx - 1);
    const bool own_x = live && q >= 1 && (al < N || ex == G.nex - 1);
    const int ezs = (!ZS && ez0 > 0) ? ez0 - 1 : ez0;
    const int base = e * NP;
    const bool add_left = al == 0 && (e > 0 || w > 0) && ex > 0;
    const int np = (int)G.np;                      // 3*np < 2^31 (checked on the host)
    PointFlags pfl;
    pfl.edge_x = ix == 0 || ix == nx - 1;
    pfl.top_ok = ix >= 1 && ix <= 3 * N;
    pfl.on_col = ix == G.nbl;
    pfl.row_ok = ix >= G.nbl;
    // the tile's owned columns [ix0, ix1] and rows [iz0, iz1] miss every
    // special point: no box edge (left, right, bottom, top), no receiver row,
    // no snapshot this step, no interface line, no taper
    bool plain;
    {
        const int ix0 = cx * S * N, ix1 = min((cx + 1) * S * N, nx - 1);
        const int iz0 = ez0 * N, iz1 = ez1 * N;
        plain = ix0 > 0 && ix1 < nx - 1 && iz0 > 0 && iz1 < G.nz - 1 && !F.snap &&
                (F.rec_iz1 < iz0 || F.rec_iz0 > iz1) && !(TP && F.taper_zones) &&
                !(F.inject_next && ((G.nbl >= iz0 && G.nbl <= iz1) || (G.nbl >= ix0 && G.nbl <= ix1)));
    }

    // x contractions: the lane's own column term first, then the element's
    // other 4 columns in rotation (al+1, al+2, ... mod 5) by shuffle
    int src[N];
    T Dx[NP], DWc[NP];
    Dx[0] = k.D[al * NP + al];
    DWc[0] = k.DWs[al * NP + al];
#pragma unroll
    for (int r = 1; r < NP; r++) {
        const int t = al + r < NP ? al + r : al + r - NP;
        src[r - 1] = base + t;
        Dx[r] = k.D[al * NP + t];
        DWc[r] = k.DWs[t * NP + al];
    }
    const T wal = k.w[al];
    // lumped-mass weight of this lane's column: inside an element, on an
    // element edge shared by two elements, or on the box's left/right edge
    // times dt^2/Je: the lane's factor of the update's M^-1 dt^2
    const T wxi = G.dt2_Je * ((al > 0 && al < N) ? k.winv[al] : (pfl.edge_x ? k.winv[0] : k.winv2));

    T u[NP][3];
    uint16_t m[NP];
    T kc[3] = {0, 0, 0};
    T rinvN = 0;
    MatRow<T, ANISO> M;
    int mcur = -1;

    {
        const int o = ezs * N * nx + ix;
        const int rm = F.row_mat[ezs];
#pragma unroll
        for (int b = 0; b < NP; b++) load_u<T, CG>(F.uc, np, o + b * nx, u[b]);
        if (rm < 0) {
#pragma unroll
            for (int b = 0; b < NP; b++) m[b] = F.mid[o + b * nx];
        } else {
#pragma unroll
            for (int b = 0; b < NP; b++) m[b] = (uint16_t)rm;
        }
    }
    int par = 0;
    for (int ez = ezs; ez < ez1; ++ez) {
        const bool halo = !ZS && ez < ez0;
        // the element row's material when all its points share one: no
        // per-point material index to read or compare
        const int rm = F.row_mat[ez];
        if (ez > ezs) {
#pragma unroll
            for (int c = 0; c < 3; c++) u[0][c] = u[N][c];
            m[0] = m[N];
            const int o = ez * N * nx + ix;
#pragma unroll
            for (int b = 1; b < NP; b++) load_u<T, CG>(F.uc, np, o + b * nx, u[b]);
            if (rm < 0) {
#pragma unroll
                for (int b = 1; b < NP; b++) m[b] = F.mid[o + b * nx];
            } else {
#pragma unroll
                for (int b = 1; b < NP; b++) m[b] = (uint16_t)rm;
            }
        }
        if (rm >= 0 && rm != mcur) {
            M.load(F.mat + (size_t)rm * MAT_STRIDE);
            mcur = rm;
        }
        // FP64 only: there it saves 36 of the ~276 flops of a point on the
        // FP64 pipe the form is bound by (8 % of the step on the 3.8 M-point
        // mesh); the FP32 form is issue-bound and measured 1 % slower with it
        const bool iso_row = ANISO && sizeof(T) == 8 && F.row_iso[ez];
        Aux<T, LF> aux[N];
        if (!halo && own_x) {
#pragma unroll
            for (int b = 0; b < N; b++) load_aux<T, LF, CG>(F, np, (ez * N + b) * nx + ix, aux[b]);
        }
        T kk[NP][3];
#pragma unroll
        for (int b = 0; b < NP; b++)
#pragma unroll
            for (int c = 0; c < 3; c++) kk[b][c] = (T)0;
        // FP64 (bound by its FP64 operations): the z gradients of the element
        // row's NP point rows at once and, after the rows, their z divergence
        // in even-odd form; each row's z flux (sigma_13, sigma_23, sigma_33)
        // waits in fz.  FP32 (bound by issue and registers): row by row.
        constexpr bool EO = sizeof(T) == 8;
        T dzr[EO ? NP : 1][3], fz[EO ? NP : 1][3];
        if constexpr (EO) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                T v[NP], y[NP];
#pragma unroll
                for (int t = 0; t < NP; t++) v[t] = u[t][c];
                mirror_sum<T, DEG>(v, k.P[0], k.Q[0], k.R[0], k.Mid[0], y);
#pragma unroll
                for (int t = 0; t < NP; t++) dzr[t][c] = y[t];
            }
        }
        T rinv[NP];
#pragma unroll
        for (int bb = 0; bb < NP; bb++) {
            // dx[2] is the strain u_z,x + u_x,z: its x sum starts from u_x,z
            T dx[3], dz[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                if constexpr (EO) {
                    dz[c] = dzr[bb][c];
                } else {
                    T z = 0;
#pragma unroll
                    for (int t = 0; t < NP; t++) z = fma(u[t][c], k.D[bb * NP + t], z);
                    dz[c] = z;
                }
                T s = c == 2 ? fma(u[bb][c], Dx[0], dz[0]) : u[bb][c] * Dx[0];
#pragma unroll
                for (int r = 1; r < NP; r++) s = fma(__shfl_sync(FULL, u[bb][c], src[r - 1]), Dx[r], s);
                dx[c] = s;
            }
            const T ee[5] = {dx[0], dx[1], dx[2], dz[1], dz[2]};
            if (rm < 0 && (int)m[bb] != mcur) {      // rows across a material boundary
                M.load(F.mat + (size_t)m[bb] * MAT_STRIDE);
                mcur = m[bb];
            }
            rinv[bb] = M.s[15];
            T sg[5];
            stress<T, ANISO>(M, ee, sg, iso_row);
            // x-divergence of row bb (a halo element row only needs its top row)
            if (!halo || bb == N) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    if constexpr (EO) {
                        // the row weight w_bb is in the table (one product fewer)
                        const T* xw = sh.xw + al * (NP * NP + 1) + bb * NP;
                        T s = sg[c] * xw[0];
#pragma unroll
                        for (int r = 1; r < NP; r++) s = fma(__shfl_sync(FULL, sg[c], src[r - 1]), xw[r], s);
                        kk[bb][c] = s;
                    } else {
                        T s = sg[c] * DWc[0];
#pragma unroll
                        for (int r = 1; r < NP; r++) s = fma(__shfl_sync(FULL, sg[c], src[r - 1]), DWc[r], s);
                        kk[bb][c] = fma(s, k.w[bb], kk[bb][c]);
                    }
                }
            }
            if constexpr (EO) {
#pragma unroll
                for (int c = 0; c < 3; c++) fz[bb][c] = sg[2 + c];
            } else {
                // z-divergence: row bb's stress feeds every row of the element
                const T f2[3] = {sg[2] * wal, sg[3] * wal, sg[4] * wal};
#pragma unroll
                for (int b = 0; b < NP; b++) {
                    if (halo && b < N) continue;
#pragma unroll
                    for (int c = 0; c < 3; c++) kk[b][c] = fma(f2[c], k.DWs[bb * NP + b], kk[b][c]);
                }
            }
        }
        if constexpr (EO) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                T v[NP], y[NP];
#pragma unroll
                for (int t = 0; t < NP; t++) v[t] = fz[t][c];
                mirror_sum<T, DEG>(v, k.P[1], k.Q[1], k.R[1], k.Mid[1], y);
#pragma unroll
                for (int b = 0; b < NP; b++)
                    if (!halo || b == N) kk[b][c] = fma(wal, y[b], kk[b][c]);
            }
        }
        // the element row below contributed to row 0 first (the reference's order)
        if (ez > ezs) {
#pragma unroll
            for (int c = 0; c < 3; c++) kk[0][c] = kc[c] + kk[0][c];
        }
#pragma unroll
        for (int c = 0; c < 3; c++) kc[c] = kk[N][c];
        rinvN = rinv[N];
        if (!halo) {
            // the last column of each warp goes to the next warp
            if (lane == LANES - 1) {
#pragma unroll
                for (int b = 0; b < N; b++)
#pragma unroll
                    for (int c = 0; c < 3; c++) sh.xch[par][w][b][c] = kk[b][c];
            }
            __syncthreads();
            const bool seam_row0 = ZS && ez == ez0 && ez0 > 0;
#pragma unroll
            for (int b = 0; b < N; b++) {
                T kt[3], lft[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    T left = __shfl_up_sync(FULL, kk[b][c], 1);
                    if (e == 0) left = sh.xch[par][w > 0 ? w - 1 : 0][b][c];
                    lft[c] = add_left ? left : (T)0;
                    kt[c] = add_left ? left + kk[b][c] : kk[b][c];
                }
                if (b == 0 && seam_row0) {
                    // the band's bottom row: publish this band's parts of its force
                    if (own_x) {
                        T* p = F.seam_hi + ((size_t)cz * nx + ix) * 6;
#pragma unroll
                        for (int c = 0; c < 3; c++) { p[c] = lft[c]; p[3 + c] = kk[0][c]; }
                    }
                    continue;
                }
                if (own_x) {
                    const T wzi = b > 0 ? k.winv[b] : (ez == 0 ? k.winv[0] : k.winv2);
                    finish_point<T, LF, TP, DEG>(F, G, k, ix, ez * N + b, u[b], kt, rinv[b], wxi, wzi, aux[b], pfl, plain);
                }
            }
            if (seam_row0) {
                __threadfence();
                __syncthreads();
                if (threadIdx.x == 0) sh.second_arrival = atomicAdd(F.seam_cnt + cz * G.ncx + cx, 1) & 1;
                __syncthreads();
                if (sh.second_arrival) {
                    __threadfence();
                    if (own_x) {
                        // (left carry + left row) + (own carry + own row), as inside a band
                        const T* lo = F.seam_lo + ((size_t)cz * nx + ix) * 6;
                        const T* hi = F.seam_hi + ((size_t)cz * nx + ix) * 6;
                        T K[3];
#pragma unroll
                        for (int c = 0; c < 3; c++)
                            K[c] = (__ldcg(lo + c) + __ldcg(hi + c)) + (__ldcg(lo + 3 + c) + __ldcg(hi + 3 + c));
                        finish_point<T, LF, TP, DEG>(F, G, k, ix, ez0 * N, u[0], K, rinv[0], wxi, k.winv2, aux[0], pfl, plain);
                    }
                }
            }
            par ^= 1;
        }
    }
    // the band's top row: the box's top (complete now) or a seam with the band above
    if (ez1 == G.nez || ZS) {
        if (lane == LANES - 1) {
#pragma unroll
            for (int c = 0; c < 3; c++) sh.xtop[w][c] = kc[c];
        }
        __syncthreads();
        T kt[3], lft[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            T left = __shfl_up_sync(FULL, kc[c], 1);
            if (e == 0) left = sh.xtop[w > 0 ? w - 1 : 0][c];
            lft[c] = add_left ? left : (T)0;
            kt[c] = add_left ? left + kc[c] : kc[c];
        }
        const int iz = ez1 * N;
        if (ez1 == G.nez) {
            if (own_x) {
                Aux<T, LF> x;
                load_aux<T, LF, CG>(F, np, iz * nx + ix, x);
                finish_point<T, LF, TP, DEG>(F, G, k, ix, iz, u[N], kt, rinvN, wxi, k.winv[0], x, pfl, plain);
            }
        } else {
            if (own_x) {
                T* p = F.seam_lo + ((size_t)(cz + 1) * nx + ix) * 6;
#pragma unroll
                for (int c = 0; c < 3; c++) { p[c] = lft[c]; p[3 + c] = kc[c]; }
            }
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) sh.second_arrival = atomicAdd(F.seam_cnt + (cz + 1) * G.ncx + cx, 1) & 1;
            __syncthreads();
            if (sh.second_arrival) {
                __threadfence();
                if (own_x) {
                    const T* hi = F.seam_hi + ((size_t)(cz + 1) * nx + ix) * 6;
                    T K[3];
#pragma unroll
                    for (int c = 0; c < 3; c++)
                        K[c] = (lft[c] + __ldcg(hi + c)) + (kc[c] + __ldcg(hi + 3 + c));
                    Aux<T, LF> x;
                    load_aux<T, LF, CG>(F, np, iz * nx + ix, x);
                    finish_point<T, LF, TP, DEG>(F, G, k, ix, iz, u[N], K, rinvN, wxi, k.winv2, x, pfl, plain);
                }
            }
        }
    }
}

// The step of one mesh: CTA b takes tile b of the band table, or of the
// regular ncx x ncz grid.  The arguments are plain by-value kernel
// parameters: marking them __grid_constant__ measured 4 % slower.
template <typename T, bool ANISO, bool LF, int NW, bool ZS, int CAP, bool TP = false, int DEG = N>
__global__ void __launch_bounds__(NW * 32, CAP ? cap_warps<T>(CAP) / NW : 1)
k_step(Field<T> F, Geo<T> G, Coef<T, DEG> k)
{
    __shared__ TileShared<T, NW, DEG> sh;
    init_tile_shared<T, NW, DEG>(sh, k);
    int cx, cz, ez0, ez1;
    if (G.items) {
        const int4 it = G.items[blockIdx.x];
        cx = it.x; cz = it.y; ez0 = it.z; ez1 = it.w;
    } else {
        cx = blockIdx.x % G.ncx; cz = blockIdx.x / G.ncx;
        ez0 = cz * G.HZ; ez1 = min(ez0 + G.HZ, G.nez);
    }
    step_tile<T, ANISO, LF, NW, ZS, false, TP, DEG>(F, G, k, cx, cz, ez0, ez1, sh);
}

// ---------------------------------------------------------------------------
// Batches: many meshes (sizes, materials, time steps of their own) advance one
// step each in one launch.  Per member, a device descriptor holds its Field
// and Geo; the per-launch parts of the Field (which buffer holds u^n, the
// seismogram row, the injection row) follow from the member's step, which the
// device keeps in BatchState and advances after each chunk of steps, so one
// captured graph runs every chunk and survives members joining and leaving.
template <typename T>
struct BatchMember {
    Field<T> F;            // uc, un, dline, inject_next, seis_row are set per launch
    Geo<T> G;
    T* U[2];               // displacement buffers; step it reads U[(it-1)&1], writes U[it&1]
    const T* dl;           // line increments of the chunk, [chunk+1][nline][3]
    float* seis;           // whole-run seismograms, [nst][3][ntrace]
    int nt_sem;            // steps that inject
    int nline;
    int item0;             // the member's first tile in the batch's tile table
};

// per member: step at the chunk's start, steps in this chunk, step to stop at
struct BatchState {
    int it0, n, target, pad;
};

// header of a batch's device tables
struct BatchHeader {
    int nitems;            // tiles in the item table
    int nmem;              // members
    int chunk;             // steps per chunk
    int pad;
};

// Persistent CTAs stride over the batch's tiles (item = member, cx | cz<<16,
// ez0, ez1); launch j of a chunk advances each member with j < n by one step.
template <typename T, bool ANISO, bool LF, int NW, bool ZS, int CAP, bool TP = false, int DEG = N>
__global__ void __launch_bounds__(NW * 32, CAP ? cap_warps<T>(CAP) / NW : 1)
k_step_batch(const BatchMember<T>* __restrict__ mem, const BatchState* __restrict__ state,
             const int4* __restrict__ items, const BatchHeader* __restrict__ hdr, int j, Coef<T, DEG> k)
{
    __shared__ TileShared<T, NW, DEG> sh;
    init_tile_shared<T, NW, DEG>(sh, k);
    __shared__ __align__(16) Field<T> sF;
    __shared__ __align__(16) Geo<T> sG;
    __shared__ int s_go;
    const int nitems = hdr->nitems;
    int cur = -1;
    for (int i = blockIdx.x; i < nitems; i += gridDim.x) {
        const int4 it = items[i];
        if (it.x != cur) {
            // descriptor of a new member: copy it, then set the per-launch fields
            cur = it.x;
            const BatchMember<T>* M = mem + cur;
            constexpr int FW = (int)(sizeof(Field<T>) / 4), GW = (int)(sizeof(Geo<T>) / 4);
            for (int q = threadIdx.x; q < FW + GW; q += blockDim.x) {
                if (q < FW) reinterpret_cast<int*>(&sF)[q] = __ldg(reinterpret_cast<const int*>(&M->F) + q);
                else reinterpret_cast<int*>(&sG)[q - FW] = __ldg(reinterpret_cast<const int*>(&M->G) + q - FW);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                const BatchState st = state[cur];
                const int step = st.it0 + j;
                const int go = j < st.n && step >= 1;
                s_go = go;
                if (go) {
                    sF.uc = M->U[(step - 1) & 1];
                    sF.un = M->U[step & 1];
                    sF.dline = M->dl + (size_t)j * M->nline * 3;
                    sF.inject_next = step + 1 < M->nt_sem ? 1 : 0;
                    sF.seis_row = M->seis + (size_t)step * 3 * sF.ntrace;
                }
            }
            __syncthreads();
        }
        if (s_go)
            step_tile<T, ANISO, LF, NW, ZS, false, TP, DEG>(sF, sG, k, it.y & 0xffff, it.y >> 16, it.z, it.w, sh);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Pipelined chunk: the steps of a chunk of one mesh in one launch.  Persistent
// CTAs claim (step, tile) pairs in step-major order from a counter; tile t of
// step s waits until the tiles around it (its 3 x 3 neighbourhood of the band
// grid, all the tiles whose points it reads or whose reads of its points it
// would overwrite) have finished step s-1, then runs the same step_tile as a
// single-step launch, loading the wavefield through L2.  A CTA only waits on
// tiles claimed before its own, by CTAs that were running then, so the waits
// end; each wait is still bounded, and a wait that runs out sets the error
// flag, which stops every CTA.  One launch replaces a chunk of step launches:
// the per-launch ramp and tail of a small mesh are paid once per chunk.
// With band seams (ZS) the boundary row between bands cz and cz+1 of step s
// is finished by the later of the two; neither waits, and both have finished
// step s -- read the partial forces, bumped the arrival counter -- before
// either neighbour starts step s+1 (the 3 x 3 wait), so the seam buffers and
// the counter's parity carry over from step to step.
struct PipeCtl {
    int* claim;            // next (step, tile) index
    int* done;             // per tile: steps of the chunk it has finished
    int* error;            // set when a wait ran out
    int spin_limit;        // polls before a wait gives up
    int stall_tile;        // -1; for tests of the failure path, a tile that never marks a step finished
};

struct PipeChunk {
    const void* U[2];      // displacement buffers; step it reads U[(it-1)&1]
    int it0, n;            // the chunk's first step (>= 1) and its length
    int nt_sem;            // steps that inject
    int nline;
    const void* dl;        // [n+1][nline][3] increments of the chunk (row s: step it0+s)
    float* seis;           // [n][3][ntrace] seismogram rows of the chunk
    float* snaps;          // snapshot k of step snap_start + k*snap_incre (k < nsnap), or null
    int snap_start, snap_incre, nsnap;
    size_t snap_size;      // floats per snapshot
};

// which snapshot step it takes: the k < n with it == start + k*incre (the
// reference tests the 26 candidates in turn; with incre == 0 they all name
// the step `start`, whose snapshot is k = 0), or -1
__host__ __device__ __forceinline__ int snap_index(int it, int start, int incre, int n)
{
    const int d = it - start;
    if (incre == 0) return d == 0 && n > 0 ? 0 : -1;
    if (d % incre) return -1;
    const int k = d / incre;
    return k >= 0 && k < n ? k : -1;
}

// the snapshot buffer of step it, or null
__device__ __forceinline__ float* snap_of(float* snaps, int it, int start, int incre, int n, size_t size)
{
    const int k = snaps ? snap_index(it, start, incre, n) : -1;
    return k >= 0 ? snaps + (size_t)k * size : nullptr;
}

__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int* p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr int PIPE_SPIN_LIMIT = 1 << 22;   // polls of one wait (with 128 ns sleeps: about a second)
constexpr int PIPE_TEST_SPIN_LIMIT = 1 << 14;   // the failure-path tests' limit (a few ms)

template <typename T, bool ANISO, bool LF, int NW, bool ZS, int CAP, bool TP = false, int DEG = N>
__global__ void __launch_bounds__(NW * 32, CAP ? cap_warps<T>(CAP) / NW : 1)
k_step_pipe(Field<T> F, Geo<T> G, Coef<T, DEG> k, PipeChunk C, PipeCtl ctl)
{
    __shared__ TileShared<T, NW, DEG> sh;
    init_tile_shared<T, NW, DEG>(sh, k);
    __shared__ __align__(16) Field<T> sF;
    __shared__ int s_claim, s_step, s_next, s_fail;
    const int ntiles = G.ncx * G.ncz;
    const int total = C.n * ntiles;
    if (threadIdx.x == 0) { sF = F; s_step = -1; s_claim = atomicAdd(ctl.claim, 1); }
    __syncthreads();
    for (;;) {
        const int c = s_claim;
        if (c >= total) break;
        const int st = c / ntiles, t = c - st * ntiles;
        const int cz = t / G.ncx, cx = t - cz * G.ncx;
        if (threadIdx.x < 32) {
            // lanes 0..8 wait, each for one tile of the 3 x 3 neighbourhood to
            // finish step st-1; lane 0 claims the next pair meanwhile (this CTA
            // takes it up after the current one)
            int next = 0;
            if (threadIdx.x == 0) { next = atomicAdd(ctl.claim, 1); s_fail = 0; }
            int fail = 0;
            if (st > 0 && threadIdx.x < 9) {
                const int z = cz + (int)threadIdx.x / 3 - 1, x = cx + (int)threadIdx.x % 3 - 1;
                if (z >= 0 && z < G.ncz && x >= 0 && x < G.ncx) {
                    const int* f = ctl.done + z * G.ncx + x;
                    int spins = 0;
                    while (ld_acquire(f) < st) {
                        if (++spins > ctl.spin_limit || ld_acquire(ctl.error)) { fail = 1; break; }
                        __nanosleep(128);
                    }
                }
            }
            fail = __any_sync(0xffffffffu, fail);
            if (threadIdx.x == 0) {
                s_next = next;
                if (fail) { atomicExch(ctl.error, 1); s_fail = 1; }
                else if (st != s_step) {
                    const int it = C.it0 + st;
                    sF.uc = (const T*)C.U[(it - 1) & 1];
                    sF.un = (T*)C.U[it & 1];
                    sF.dline = (const T*)C.dl + (size_t)st * C.nline * 3;
                    sF.inject_next = it + 1 < C.nt_sem ? 1 : 0;
                    sF.seis_row = C.seis + (size_t)st * 3 * F.ntrace;
                    sF.snap = snap_of(C.snaps, it, C.snap_start, C.snap_incre, C.nsnap, C.snap_size);
                    s_step = st;
                }
            }
        }
        __syncthreads();
        if (s_fail) break;
        step_tile<T, ANISO, LF, NW, ZS, true, TP, DEG>(sF, G, k, cx, cz, cz * G.HZ, min(cz * G.HZ + G.HZ, G.nez), sh);
        // the CTA's stores are ordered before thread 0's fence by the barrier
        // (fences are cumulative), so one fence publishes the whole tile
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            if (t != ctl.stall_tile) st_release(ctl.done + t, st + 1);
            s_claim = ld_acquire(ctl.error) ? total : s_next;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Pipelined batch chunk: the steps of a chunk of every member of a batch in
// one launch.  Persistent CTAs claim (step j, tile i) pairs in step-major
// order over the batch's tile table (members one after another, each
// member's tiles row by row); tile i of step j starts once the 3 x 3
// neighbourhood of its member's own tiles has finished step j-1, exactly as
// in the single-mesh pipelined chunk, and a member whose chunk has fewer
// steps has no tile at step j.  The steps' own fields (displacement buffers,
// injection row, seismogram row) follow from the member's step as in
// k_step_batch.  One launch replaces the chunk's per-step launches and their
// partly idle tails.
struct BatchPipeCtl {
    int* claim;            // next (step, tile) index
    int* error;            // set when a wait ran out
    int* done;             // per tile: steps of the chunk it has finished
    int spin_limit;        // polls before a wait gives up
    int stall_item;        // -1; for tests of the failure path, a tile that never marks a step finished
};

template <typename T, bool ANISO, bool LF, int NW, bool ZS, int CAP, bool TP = false, int DEG = N>
__global__ void __launch_bounds__(NW * 32, CAP ? cap_warps<T>(CAP) / NW : 1)
k_step_batch_pipe(const BatchMember<T>* __restrict__ mem, const BatchState* __restrict__ state,
                  const int4* __restrict__ items, const BatchHeader* __restrict__ hdr, int nsteps, BatchPipeCtl ctl,
                  Coef<T, DEG> k)
{
    __shared__ TileShared<T, NW, DEG> sh;
    init_tile_shared<T, NW, DEG>(sh, k);
    __shared__ __align__(16) Field<T> sF;
    __shared__ __align__(16) Geo<T> sG;
    __shared__ int s_claim, s_next, s_fail, s_go, s_m, s_j;
    const int nitems = hdr->nitems;
    const int total = nsteps * nitems;
    if (threadIdx.x == 0) { s_m = -1; s_j = -1; s_claim = atomicAdd(ctl.claim, 1); }
    __syncthreads();
    for (;;) {
        const int c = s_claim;
        if (c >= total) break;
        const int j = c / nitems, i = c - j * nitems;
        const int4 it = items[i];
        const int m = it.x, cx = it.y & 0xffff, cz = it.y >> 16;
        const BatchMember<T>* M = mem + m;
        if (m != s_m) {
            // descriptor of a new member
            constexpr int FW = (int)(sizeof(Field<T>) / 4), GW = (int)(sizeof(Geo<T>) / 4);
            for (int q = threadIdx.x; q < FW + GW; q += blockDim.x) {
                if (q < FW) reinterpret_cast<int*>(&sF)[q] = __ldg(reinterpret_cast<const int*>(&M->F) + q);
                else reinterpret_cast<int*>(&sG)[q - FW] = __ldg(reinterpret_cast<const int*>(&M->G) + q - FW);
            }
            __syncthreads();
            if (threadIdx.x == 0) { s_m = m; s_j = -1; }
            __syncthreads();
        }
        if (threadIdx.x < 32) {
            // lanes 0..8 wait, each for one tile of the member's 3 x 3
            // neighbourhood to finish step j-1; lane 0 claims the next pair
            const BatchState st = state[m];
            const int step = st.it0 + j;
            const bool go = j < st.n && step >= 1;
            int next = 0;
            if (threadIdx.x == 0) { next = atomicAdd(ctl.claim, 1); s_fail = 0; }
            int fail = 0;
            if (go && j > 0 && threadIdx.x < 9) {
                const int z = cz + (int)threadIdx.x / 3 - 1, x = cx + (int)threadIdx.x % 3 - 1;
                if (z >= 0 && z < sG.ncz && x >= 0 && x < sG.ncx) {
                    const int* f = ctl.done + M->item0 + z * sG.ncx + x;
                    int spins = 0;
                    while (ld_acquire(f) < j) {
                        if (++spins > ctl.spin_limit || ld_acquire(ctl.error)) { fail = 1; break; }
                        __nanosleep(128);
                    }
                }
            }
            fail = __any_sync(0xffffffffu, fail);
            if (threadIdx.x == 0) {
                s_next = next;
                s_go = go;
                if (fail) { atomicExch(ctl.error, 1); s_fail = 1; }
                else if (go && j != s_j) {
                    sF.uc = M->U[(step - 1) & 1];
                    sF.un = M->U[step & 1];
                    sF.dline = M->dl + (size_t)j * M->nline * 3;
                    sF.inject_next = step + 1 < M->nt_sem ? 1 : 0;
                    sF.seis_row = M->seis + (size_t)step * 3 * sF.ntrace;
                    s_j = j;
                }
            }
        }
        __syncthreads();
        if (s_fail) break;
        if (s_go) step_tile<T, ANISO, LF, NW, ZS, true, TP, DEG>(sF, sG, k, cx, cz, it.z, it.w, sh);
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();                // publishes the whole tile (see k_step_pipe)
            if (s_go && i != ctl.stall_item) st_release(ctl.done + i, j + 1);
            s_claim = ld_acquire(ctl.error) ? total : s_next;
        }
        __syncthreads();
    }
}

}  // namespace sks

namespace sks {
// taper: the variant with the boundary taper (atten > 0) compiled in; the
// others carry no code for it
struct StepVariant { int nw; int zseam; int cap; int taper = 0; };
cudaError_t launch_step_f32(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                            const Field<float>& F, const Geo<float>& G, const Coef<float>& k);
cudaError_t launch_step_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                            const Field<double>& F, const Geo<double>& G, const Coef<double>& k);
cudaError_t launch_batch_f32(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const BatchMember<float>* mem,
                             const BatchState* state, const int4* items, const BatchHeader* hdr, int j,
                             const Coef<float>& k);
cudaError_t launch_batch_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const BatchMember<double>* mem,
                             const BatchState* state, const int4* items, const BatchHeader* hdr, int j,
                             const Coef<double>& k);
int batch_occupancy_f32(const StepVariant& v, bool aniso);
cudaError_t launch_batch_pipe_f32(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                  const BatchMember<float>* mem, const BatchState* state, const int4* items,
                                  const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl, const Coef<float>& k);
cudaError_t launch_batch_pipe_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                  const BatchMember<double>* mem, const BatchState* state, const int4* items,
                                  const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl, const Coef<double>& k);
int batch_pipe_occupancy_f32(const StepVariant& v, bool aniso);
int batch_pipe_occupancy_f64(const StepVariant& v, bool aniso);
cudaError_t launch_pipe_f32(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<float>& F,
                            const Geo<float>& G, const Coef<float>& k, const PipeChunk& C, const PipeCtl& ctl);
cudaError_t launch_pipe_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<double>& F,
                            const Geo<double>& G, const Coef<double>& k, const PipeChunk& C, const PipeCtl& ctl);
int pipe_occupancy_f32(const StepVariant& v, bool aniso);
int pipe_occupancy_f64(const StepVariant& v, bool aniso);
int batch_occupancy_f64(const StepVariant& v, bool aniso);
// resident CTAs per SM of a variant (cudaOccupancyMaxActiveBlocksPerMultiprocessor)
int step_occupancy_f32(const StepVariant& v, bool aniso);
int step_occupancy_f64(const StepVariant& v, bool aniso);
// GLL degree 5 (4 warps, register cap 0 or 1)
int batch_occupancy_f32_d5(const StepVariant& v, bool aniso);
cudaError_t launch_batch_f32_d5(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                const BatchMember<float>* mem, const BatchState* state, const int4* items,
                                const BatchHeader* hdr, int j, const Coef<float, 5>& k);
int batch_pipe_occupancy_f32_d5(const StepVariant& v, bool aniso);
cudaError_t launch_batch_pipe_f32_d5(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                     const BatchMember<float>* mem, const BatchState* state, const int4* items,
                                     const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl,
                                     const Coef<float, 5>& k);
int batch_occupancy_f64_d5(const StepVariant& v, bool aniso);
cudaError_t launch_batch_f64_d5(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                const BatchMember<double>* mem, const BatchState* state, const int4* items,
                                const BatchHeader* hdr, int j, const Coef<double, 5>& k);
int batch_pipe_occupancy_f64_d5(const StepVariant& v, bool aniso);
cudaError_t launch_batch_pipe_f64_d5(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                     const BatchMember<double>* mem, const BatchState* state, const int4* items,
                                     const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl,
                                     const Coef<double, 5>& k);
int step_occupancy_f32_d5(const StepVariant& v, bool aniso);
cudaError_t launch_step_f32_d5(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                               const Field<float>& F, const Geo<float>& G, const Coef<float, 5>& k);
int pipe_occupancy_f32_d5(const StepVariant& v, bool aniso);
cudaError_t launch_pipe_f32_d5(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<float>& F,
                               const Geo<float>& G, const Coef<float, 5>& k, const PipeChunk& C, const PipeCtl& ctl);
int step_occupancy_f64_d5(const StepVariant& v, bool aniso);
cudaError_t launch_step_f64_d5(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                               const Field<double>& F, const Geo<double>& G, const Coef<double, 5>& k);
int pipe_occupancy_f64_d5(const StepVariant& v, bool aniso);
cudaError_t launch_pipe_f64_d5(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<double>& F,
                               const Geo<double>& G, const Coef<double, 5>& k, const PipeChunk& C, const PipeCtl& ctl);
// GLL degrees 3 and 6 (4 warps, register cap 0 or 1; single solves)
#define SKS_DEG_DECL(F, T, D)                                                                                   \
    int step_occupancy_##F##_d##D(const StepVariant& v, bool aniso);                                          \
    cudaError_t launch_step_##F##_d##D(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,         \
                                       const Field<T>& F_, const Geo<T>& G, const Coef<T, D>& k);             \
    int pipe_occupancy_##F##_d##D(const StepVariant& v, bool aniso);                                          \
    cudaError_t launch_pipe_##F##_d##D(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,         \
                                       const Field<T>& F_, const Geo<T>& G, const Coef<T, D>& k,              \
                                       const PipeChunk& C, const PipeCtl& ctl);
SKS_DEG_DECL(f32, float, 3)
SKS_DEG_DECL(f64, double, 3)
SKS_DEG_DECL(f32, float, 6)
SKS_DEG_DECL(f64, double, 6)
#undef SKS_DEG_DECL
// batches of GLL degrees 3 and 6 (4 warps, register cap 0 or 1)
#define SKS_BATCH_DEG_DECL(F, T, D)                                                                             \
    int batch_occupancy_##F##_d##D(const StepVariant& v, bool aniso);                                         \
    cudaError_t launch_batch_##F##_d##D(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,        \
                                        const BatchMember<T>* mem, const BatchState* state, const int4* items, \
                                        const BatchHeader* hdr, int j, const Coef<T, D>& k);                  \
    int batch_pipe_occupancy_##F##_d##D(const StepVariant& v, bool aniso);                                    \
    cudaError_t launch_batch_pipe_##F##_d##D(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,   \
                                             const BatchMember<T>* mem, const BatchState* state,              \
                                             const int4* items, const BatchHeader* hdr, int nsteps,           \
                                             const BatchPipeCtl& ctl, const Coef<T, D>& k);
SKS_BATCH_DEG_DECL(f32, float, 3)
SKS_BATCH_DEG_DECL(f64, double, 3)
SKS_BATCH_DEG_DECL(f32, float, 6)
SKS_BATCH_DEG_DECL(f64, double, 6)
#undef SKS_BATCH_DEG_DECL
// the same with the boundary taper compiled in (the entry points above call
// these for a variant with taper set)
int step_occupancy_f32_tp(const StepVariant& v, bool aniso);
cudaError_t launch_step_f32_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                               const Field<float>& F, const Geo<float>& G, const Coef<float>& k);
int pipe_occupancy_f32_tp(const StepVariant& v, bool aniso);
cudaError_t launch_pipe_f32_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<float>& F,
                               const Geo<float>& G, const Coef<float>& k, const PipeChunk& C, const PipeCtl& ctl);
int batch_occupancy_f32_tp(const StepVariant& v, bool aniso);
cudaError_t launch_batch_f32_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                const BatchMember<float>* mem, const BatchState* state, const int4* items,
                                const BatchHeader* hdr, int j, const Coef<float>& k);
int batch_pipe_occupancy_f32_tp(const StepVariant& v, bool aniso);
cudaError_t launch_batch_pipe_f32_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                     const BatchMember<float>* mem, const BatchState* state, const int4* items,
                                     const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl,
                                     const Coef<float>& k);
int step_occupancy_f64_tp(const StepVariant& v, bool aniso);
cudaError_t launch_step_f64_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                               const Field<double>& F, const Geo<double>& G, const Coef<double>& k);
int pipe_occupancy_f64_tp(const StepVariant& v, bool aniso);
cudaError_t launch_pipe_f64_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<double>& F,
                               const Geo<double>& G, const Coef<double>& k, const PipeChunk& C, const PipeCtl& ctl);
int batch_occupancy_f64_tp(const StepVariant& v, bool aniso);
cudaError_t launch_batch_f64_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                const BatchMember<double>* mem, const BatchState* state, const int4* items,
                                const BatchHeader* hdr, int j, const Coef<double>& k);
int batch_pipe_occupancy_f64_tp(const StepVariant& v, bool aniso);
cudaError_t launch_batch_pipe_f64_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                     const BatchMember<double>* mem, const BatchState* state, const int4* items,
                                     const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl,
                                     const Coef<double>& k);
}  // namespace sks
