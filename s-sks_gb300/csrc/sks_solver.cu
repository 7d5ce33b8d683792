// C ABI of the GB300 SEM time-stepping library (include/sks.h): device state,
// step scheduling, and the entry points that replace main() and the time loop
// of semsyn/src/sem2d_psvsh.c.
#include "sks_internal.h"
#include "sks_aux_kernels.cuh"

#include <cuda_runtime.h>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>

using namespace sks;
using namespace sksi;

static thread_local char g_err[1024];

int sks_err(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

extern "C" const char* sks_last_error(void) { return g_err; }

// error reporting for the library's C translation units
extern "C" __attribute__((visibility("hidden"))) int sks_internal_error_c(int code, const char* msg)
{
    return set_err(code, "%s", msg);
}

// error reporting for the library's other translation units
extern "C" __attribute__((visibility("hidden"))) int sks_internal_set_error(int code, const char* msg, cudaError_t e)
{
    if (e != cudaSuccess) return set_err(code, "%s: %s", msg, cudaGetErrorString(e));
    return set_err(code, "%s", msg);
}


// per element row: 1 when every point of its grid rows has an isotropic material
static std::vector<uint8_t> isotropic_rows(const sks_model& m)
{
    std::vector<uint8_t> iso((size_t)m.nez, 1);
    std::vector<uint8_t> mat_iso((size_t)m.nmat);
    for (int i = 0; i < m.nmat; i++) mat_iso[i] = (uint8_t)sks_material_is_isotropic(m.mat + (size_t)i * SKS_MAT_STRIDE);
    for (int ez = 0; ez < m.nez; ez++)
        for (int iz = ez * m.hpn; iz <= ez * m.hpn + m.hpn && iso[ez]; iz++)
            for (int ix = 0; ix < m.nx; ix++)
                if (!mat_iso[m.mat_id[(size_t)iz * m.nx + ix]]) { iso[ez] = 0; break; }
    return iso;
}

static void fill_info(const sks_model& m, sks_info_t* info)
{
    memset(info, 0, sizeof *info);
    {
        const std::vector<uint8_t> iso = isotropic_rows(m);
        for (uint8_t v : iso) info->iso_rows += v;
    }
    info->nex = m.nex; info->nez = m.nez; info->hpn = m.hpn;
    info->nx = m.nx; info->nz = m.nz; info->nst = m.nst; info->nt_inject = m.nt_sem;
    info->ntrace = m.ntrace; info->mtotal = m.mtotal; info->shtotal = m.shtotal;
    info->nrec_psv = m.nrec_psv; info->nrec_sh = m.nrec_sh; info->nmat = m.nmat;
    info->anisotropic = m.anisotropic;
    info->eh = m.eh; info->h = m.h; info->sdt = m.sdt;
    info->neh = m.neh;
}

extern "C" int sks_setup_open(int argc, const char* const* argv, sks_setup** out)
{
    if (!out) return set_err(SKS_ERR_ARG, "out is NULL");
    *out = nullptr;
    sks_setup* su = new (std::nothrow) sks_setup();
    if (!su) return set_err(SKS_ERR_NOMEM, "cannot allocate the set-up");
    char err[512] = {0};
    int rc = sks_model_from_par(&su->m, argc, argv, err, sizeof err);
    if (rc) { delete su; return set_err(rc, "%s", err); }
    *out = su;
    return SKS_OK;
}

extern "C" int sks_setup_info(const sks_setup* su, sks_info_t* info)
{
    if (!su || !info) return set_err(SKS_ERR_ARG, "NULL argument");
    fill_info(su->m, info);
    return SKS_OK;
}

extern "C" int sks_setup_material(const sks_setup* su, double* out16)
{
    if (!su || !out16) return set_err(SKS_ERR_ARG, "NULL argument");
    const sks_model& m = su->m;
    const size_t np = (size_t)m.nx * m.nz;
    for (size_t g = 0; g < np; g++)
        memcpy(out16 + g * 16, m.mat + (size_t)m.mat_id[g] * SKS_MAT_STRIDE, 16 * sizeof(double));
    return SKS_OK;
}

extern "C" int sks_setup_mass(const sks_setup* su, double* mass, double* ab3)
{
    if (!su) return set_err(SKS_ERR_ARG, "NULL argument");
    const sks_model& m = su->m;
    const size_t np = (size_t)m.nx * m.nz;
    if (mass) memcpy(mass, m.mass, np * sizeof(double));
    if (ab3) memcpy(ab3, m.ab, 3 * np * sizeof(double));
    return SKS_OK;
}

extern "C" int sks_setup_receivers(const sks_setup* su, int64_t* off)
{
    if (!su || (!off && su->m.ntrace > 0)) return set_err(SKS_ERR_ARG, "NULL argument");
    if (su->m.ntrace > 0) memcpy(off, su->m.rec_off, sizeof(int64_t) * su->m.ntrace);
    return SKS_OK;
}

extern "C" int sks_setup_schedule(const sks_setup* su, int32_t* tap_psv, double* w_psv, int32_t* tap_sh, double* w_sh)
{
    if (!su) return set_err(SKS_ERR_ARG, "NULL argument");
    const sks_model& m = su->m;
    const size_t n = 4 * (size_t)m.nt_sem;
    if (n == 0) return SKS_OK;
    if (tap_psv) memcpy(tap_psv, m.tap_psv, n * sizeof(int32_t));
    if (w_psv) memcpy(w_psv, m.w_psv, n * sizeof(double));
    if (tap_sh) memcpy(tap_sh, m.tap_sh, n * sizeof(int32_t));
    if (w_sh) memcpy(w_sh, m.w_sh, n * sizeof(double));
    return SKS_OK;
}

extern "C" void sks_setup_close(sks_setup* su)
{
    if (!su) return;
    sks_model_free(&su->m);
    delete su;
}

namespace sksi {

template <typename T>
int dmalloc(sks_solver* s, T** p, size_t n)
{
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) return set_err(SKS_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
    s->device_bytes += (int64_t)(n * sizeof(T));
    return SKS_OK;
}

void free_device(sks_solver* s)
{
    void* ps[] = {s->U[0], s->U[1], s->Dv, s->Cc, s->mid, s->mat, s->stc, s->taper,
                  s->rec_off, s->recbits, s->rec_sorted, s->rec_idx, s->seisbuf[0], s->seisbuf[1], s->G, s->Dl, s->rec_psv, s->rec_sh,
                  s->tap_psv, s->tap_sh, s->w_psv, s->w_sh, s->seam_lo, s->seam_hi, s->seam_cnt, s->items, s->seis_full,
                  s->pipe_ctl, s->snaps, s->ser, s->nonfinite, s->row_iso, s->row_mat};
    for (void* p : ps)
        if (p) cudaFree(p);
    s->U[0] = s->U[1] = s->Dv = s->Cc = s->mat = s->stc = s->taper = nullptr;
    s->mid = nullptr; s->rec_off = nullptr; s->recbits = nullptr; s->rec_sorted = nullptr; s->rec_idx = nullptr;
    s->seis = nullptr; s->seisbuf[0] = s->seisbuf[1] = nullptr; s->G = nullptr; s->Dl = nullptr;
    s->rec_psv = s->rec_sh = nullptr; s->tap_psv = s->tap_sh = nullptr; s->w_psv = s->w_sh = nullptr;
    s->ser = nullptr; s->ser_n = 0; s->rs.kind = REC_TABLE;
    s->seam_lo = s->seam_hi = nullptr; s->seam_cnt = nullptr; s->seam_bytes = 0; s->seam_cnt_n = 0;
    s->items = nullptr; s->items_n = 0;
    s->seis_full = nullptr;
    s->pipe_ctl = nullptr;
    s->pipe_ctl_n = 0;
    s->snaps = nullptr;
    s->nonfinite = nullptr;
    s->row_iso = nullptr;
    s->row_mat = nullptr;
}

// per-kernel-class timing: an event pair around each launch when enabled
struct KTimer {
    sks_solver* s;
    int cls;
    int idx;
    KTimer(sks_solver* sv, int c) : s(sv), cls(c), idx(-1) {
        if (!s->timing) return;
        if ((size_t)(2 * s->kused + 2) > s->kev.size()) {
            const size_t old = s->kev.size();
            s->kev.resize(old + 64);
            for (size_t i = old; i < s->kev.size(); i++) cudaEventCreate(&s->kev[i]);
            s->kcls.resize(s->kev.size() / 2);
        }
        idx = s->kused++;
        s->kcls[idx] = cls;
        cudaEventRecord(s->kev[2 * idx], s->stream);
    }
    ~KTimer() {
        if (idx >= 0) cudaEventRecord(s->kev[2 * idx + 1], s->stream);
        s->launches++;
    }
};

int collect_timing(sks_solver* s)
{
    if (!s->timing || s->kused == 0) return SKS_OK;
    CK(cudaEventSynchronize(s->kev[2 * s->kused - 1]));
    for (int i = 0; i < s->kused; i++) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, s->kev[2 * i], s->kev[2 * i + 1]));
        s->kms[s->kcls[i]] += ms;
        s->kcount[s->kcls[i]]++;
    }
    s->kused = 0;
    return SKS_OK;
}

// CTA band height: at least `per_sm` CTAs per SM in the grid, and bands as
// tall as that allows (each band recomputes one element row below it)
int pick_band(const sks_model& m, int ncx, int sm_count, int per_sm)
{
    const int64_t target = (int64_t)sm_count * per_sm;
    const int cands[] = {32, 24, 16, 12, 10, 8, 6, 4, 3, 2};
    for (int hz : cands) {
        if (hz > m.nez) continue;
        const int ncz = (m.nez + hz - 1) / hz;
        if ((int64_t)ncx * ncz >= target) return hz;
    }
    return std::max(1, std::min(2, m.nez));
}

template <typename T>
int upload_tables(sks_solver* s)
{
    const sks_model& m = s->m;
    const int N1 = m.hpn + 1;
    // material table: 15 stiffness entries + 1/rho
    std::vector<T> mat((size_t)m.nmat * MAT_STRIDE);
    for (int i = 0; i < m.nmat; i++) {
        for (int k = 0; k < 15; k++) mat[(size_t)i * MAT_STRIDE + k] = (T)m.mat[(size_t)i * SKS_MAT_STRIDE + k];
        mat[(size_t)i * MAT_STRIDE + 15] = (T)(1.0 / m.mat[(size_t)i * SKS_MAT_STRIDE + 15]);
    }
    // Stacey coefficients per boundary point and component
    const int64_t nb = sks_stacey_count(m.nx, m.nz, m.hpn);
    std::vector<T> stc((size_t)nb * 9, (T)0);
    const double dt2 = m.sdt * m.sdt;
    for (int iz = 0; iz < m.nz; iz++)
        for (int ix = 0; ix < m.nx; ix++) {
            const int64_t bi = sks_stacey_index(ix, iz, m.nx, m.nz, m.hpn);
            if (bi < 0) continue;
            const size_t g = (size_t)iz * m.nx + ix;
            const double M = m.mass[g];
            for (int c = 0; c < 3; c++) {
                const double A = m.ab[3 * g + c];
                stc[(size_t)bi * 9 + 3 * c + 0] = (T)(dt2 / (M + A));
                stc[(size_t)bi * 9 + 3 * c + 1] = (T)(2.0 * M / (M + A));
                stc[(size_t)bi * 9 + 3 * c + 2] = (T)((M - A) / (M + A));
            }
        }
    (void)N1;
    T *dmat, *dstc;
    int rc;
    if ((rc = dmalloc(s, &dmat, mat.size()))) return rc;
    s->mat = dmat;
    if ((rc = dmalloc(s, &dstc, stc.size()))) return rc;
    s->stc = dstc;
    CK(cudaMemcpy(dmat, mat.data(), mat.size() * sizeof(T), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dstc, stc.data(), stc.size() * sizeof(T), cudaMemcpyHostToDevice));
    if (m.nh_att > 0) {
        // the FP32 form multiplies by the reference's float factors, the FP64 form by FP64 ones
        std::vector<T> taper((size_t)m.nh_att);
        for (int n = 0; n < m.nh_att; n++) taper[n] = sizeof(T) == 4 ? (T)m.taper_f[n] : (T)m.taper_d[n];
        T* dtap;
        if ((rc = dmalloc(s, &dtap, taper.size()))) return rc;
        s->taper = dtap;
        CK(cudaMemcpy(dtap, taper.data(), taper.size() * sizeof(T), cudaMemcpyHostToDevice));
    }
    // wavefield
    const size_t np = (size_t)m.nx * m.nz;
    T* u0; T* u1;
    if ((rc = dmalloc(s, &u0, 3 * np))) return rc;
    s->U[0] = u0;
    if ((rc = dmalloc(s, &u1, 3 * np))) return rc;
    s->U[1] = u1;
    if (s->precision == SKS_FP32C) {
        T* dv;                      // (d, Kahan c) pairs, [3][np] float2
        if ((rc = dmalloc(s, &dv, 6 * np))) return rc;
        s->Dv = dv;
        s->Cc = nullptr;
    }
    return SKS_OK;
}

// CTA grid for a tuning: NW warps (6*NW-1 owned elements) by bands of rows.
// waves == 0: bands of HZ rows.  waves > 0: exactly SMs x resident-CTAs x
// waves CTAs, each column split into bands of near-equal height, so every
// SM carries the same work (no partly filled last wave).  The band-seam
// buffers grow to fit and their counters restart at 0.
// The compiled kernels of one GLL degree D (3..6) and form T: occupancy and
// launch of the per-step and the pipelined step kernel.
template <typename T, int D>
struct DegKernels {
    static constexpr bool F32 = sizeof(T) == 4;
    static int step_occ(const StepVariant& v, bool a)
    {
        if constexpr (D == 3) return F32 ? step_occupancy_f32_d3(v, a) : step_occupancy_f64_d3(v, a);
        else if constexpr (D == 5) return F32 ? step_occupancy_f32_d5(v, a) : step_occupancy_f64_d5(v, a);
        else if constexpr (D == 6) return F32 ? step_occupancy_f32_d6(v, a) : step_occupancy_f64_d6(v, a);
        else return F32 ? step_occupancy_f32(v, a) : step_occupancy_f64(v, a);
    }
    static int pipe_occ(const StepVariant& v, bool a)
    {
        if constexpr (D == 3) return F32 ? pipe_occupancy_f32_d3(v, a) : pipe_occupancy_f64_d3(v, a);
        else if constexpr (D == 5) return F32 ? pipe_occupancy_f32_d5(v, a) : pipe_occupancy_f64_d5(v, a);
        else if constexpr (D == 6) return F32 ? pipe_occupancy_f32_d6(v, a) : pipe_occupancy_f64_d6(v, a);
        else return F32 ? pipe_occupancy_f32(v, a) : pipe_occupancy_f64(v, a);
    }
    static cudaError_t step(const StepVariant& v, bool a, int blocks, cudaStream_t st, const Field<T>& F,
                            const Geo<T>& G, const Coef<T, D>& k)
    {
        if constexpr (F32) {
            if constexpr (D == 3) return launch_step_f32_d3(v, a, blocks, st, F, G, k);
            else if constexpr (D == 5) return launch_step_f32_d5(v, a, blocks, st, F, G, k);
            else if constexpr (D == 6) return launch_step_f32_d6(v, a, blocks, st, F, G, k);
            else return launch_step_f32(v, a, blocks, st, F, G, k);
        } else {
            if constexpr (D == 3) return launch_step_f64_d3(v, a, blocks, st, F, G, k);
            else if constexpr (D == 5) return launch_step_f64_d5(v, a, blocks, st, F, G, k);
            else if constexpr (D == 6) return launch_step_f64_d6(v, a, blocks, st, F, G, k);
            else return launch_step_f64(v, a, blocks, st, F, G, k);
        }
    }
    static cudaError_t pipe(const StepVariant& v, bool a, int blocks, cudaStream_t st, const Field<T>& F,
                            const Geo<T>& G, const Coef<T, D>& k, const PipeChunk& C, const PipeCtl& ctl)
    {
        if constexpr (F32) {
            if constexpr (D == 3) return launch_pipe_f32_d3(v, a, blocks, st, F, G, k, C, ctl);
            else if constexpr (D == 5) return launch_pipe_f32_d5(v, a, blocks, st, F, G, k, C, ctl);
            else if constexpr (D == 6) return launch_pipe_f32_d6(v, a, blocks, st, F, G, k, C, ctl);
            else return launch_pipe_f32(v, a, blocks, st, F, G, k, C, ctl);
        } else {
            if constexpr (D == 3) return launch_pipe_f64_d3(v, a, blocks, st, F, G, k, C, ctl);
            else if constexpr (D == 5) return launch_pipe_f64_d5(v, a, blocks, st, F, G, k, C, ctl);
            else if constexpr (D == 6) return launch_pipe_f64_d6(v, a, blocks, st, F, G, k, C, ctl);
            else return launch_pipe_f64(v, a, blocks, st, F, G, k, C, ctl);
        }
    }
};

// calls f.template run<D>() for the solver's degree D (3..6)
template <typename Fn>
auto with_degree(int hpn, Fn& f)
{
    switch (hpn) {
    case 3: return f.template run<3>();
    case 5: return f.template run<5>();
    case 6: return f.template run<6>();
    default: return f.template run<4>();
    }
}

struct OccOf {
    const sks_solver* s;
    const StepVariant& v;
    bool pipe;
    template <int D>
    int run()
    {
        const bool a = s->m.anisotropic != 0;
        if (s->precision == SKS_FP64)
            return pipe ? DegKernels<double, D>::pipe_occ(v, a) : DegKernels<double, D>::step_occ(v, a);
        return pipe ? DegKernels<float, D>::pipe_occ(v, a) : DegKernels<float, D>::step_occ(v, a);
    }
};

// resident CTAs per SM of the solver's step / pipelined variant (form and degree)
int step_occ(const sks_solver* s, const StepVariant& v)
{
    OccOf o{s, v, false};
    return with_degree(s->m.hpn, o);
}

int pipe_occ(const sks_solver* s, const StepVariant& v)
{
    OccOf o{s, v, true};
    return with_degree(s->m.hpn, o);
}

// one step launch (C == nullptr) or one pipelined chunk of the solver's form T
// and degree
template <typename T>
struct StepOf {
    const sks_solver* s;
    const StepVariant& v;
    const Field<T>& F;
    const Geo<T>& G;
    const PipeChunk* C;
    const PipeCtl* ctl;
    template <int D>
    cudaError_t run()
    {
        static thread_local Coef<T, D> k;
        k = make_coef<T, D>(s->m);
        const bool a = s->m.anisotropic != 0;
        if (C) return DegKernels<T, D>::pipe(v, a, s->pipe_blocks, s->stream, F, G, k, *C, *ctl);
        return DegKernels<T, D>::step(v, a, s->nblocks, s->stream, F, G, k);
    }
};

// the tunings compiled for a degree: every one for 4; for 3, 5 and 6, 4
// warps per CTA and register cap 0 or 1
bool tuning_compiled(int hpn, int NW, int CAP) { return hpn == 4 || (NW == 4 && CAP <= 1); }

int set_grid(sks_solver* s, int NW, int HZ, int ZS, int CAP, int WAVES, int PIPE)
{
    if (PIPE && WAVES) return set_err(SKS_ERR_ARG, "pipeline=1 needs waves=0");
    if (!tuning_compiled(s->m.hpn, NW, CAP))
        return set_err(SKS_ERR_UNSUPPORTED, "GLL degree %d runs with 4 warps per CTA and register cap 0 or 1", s->m.hpn);
    s->NW = NW;
    s->ZS = ZS;
    s->CAP = CAP;
    s->WAVES = WAVES;
    s->PIPE = PIPE;
    const int owned = tex_of(s->m.hpn) * NW - 1;
    s->ncx = (s->m.nex + owned - 1) / owned;
    const int nez = s->m.nez;
    if (WAVES <= 0) {
        s->HZ = std::max(1, std::min(HZ, nez));
        s->ncz = (nez + s->HZ - 1) / s->HZ;
        s->nblocks = s->ncx * s->ncz;
    } else {
        const StepVariant v{NW, ZS, CAP, s->m.nh_att > 0};
        const int occ = step_occ(s, v);
        int64_t target = (int64_t)s->sms * occ * WAVES;
        target = std::max<int64_t>(s->ncx, std::min<int64_t>(target, (int64_t)s->ncx * nez));
        std::vector<int4> it;
        it.reserve((size_t)target);
        int maxb = 1;
        for (int cx = 0; cx < s->ncx; cx++) {
            const int nb = (int)(target / s->ncx + (cx < target % s->ncx ? 1 : 0));
            maxb = std::max(maxb, nb);
            for (int b = 0; b < nb; b++) {
                const int e0 = (int)((int64_t)nez * b / nb), e1 = (int)((int64_t)nez * (b + 1) / nb);
                it.push_back(make_int4(cx, b, e0, e1));
            }
        }
        // lower bands first, columns side by side
        std::stable_sort(it.begin(), it.end(), [](const int4& a, const int4& b) { return a.z < b.z; });
        if (it.size() > s->items_n) {
            if (s->items) { cudaFree(s->items); s->device_bytes -= (int64_t)(s->items_n * sizeof(int4)); }
            s->items = nullptr;
            s->items_n = 0;
            CK(cudaMalloc(&s->items, it.size() * sizeof(int4)));
            s->items_n = it.size();
            s->device_bytes += (int64_t)(it.size() * sizeof(int4));
        }
        CK(cudaMemcpy(s->items, it.data(), it.size() * sizeof(int4), cudaMemcpyHostToDevice));
        s->ncz = maxb;
        s->HZ = (nez + maxb - 1) / maxb;
        s->nblocks = (int)it.size();
    }
    if (PIPE) {
        const StepVariant pv{NW, ZS, CAP, s->m.nh_att > 0};
        const int occ = pipe_occ(s, pv);
        s->pipe_blocks = std::max(1, std::min(s->sms * occ, s->ncx * s->ncz));
        const size_t need = 2 + (size_t)s->ncx * s->ncz;
        if (need > s->pipe_ctl_n) {
            if (s->pipe_ctl) { cudaFree(s->pipe_ctl); s->device_bytes -= 4 * (int64_t)s->pipe_ctl_n; }
            s->pipe_ctl = nullptr;
            s->pipe_ctl_n = 0;
            CK(cudaMalloc(&s->pipe_ctl, need * sizeof(int)));
            s->pipe_ctl_n = need;
            s->device_bytes += 4 * (int64_t)need;
        }
        CK(cudaMemsetAsync(s->pipe_ctl, 0, need * sizeof(int), s->stream));
    }
    if (!ZS) return SKS_OK;
    const size_t el = s->precision == SKS_FP64 ? sizeof(double) : sizeof(float);
    const size_t need = (size_t)s->ncz * s->m.nx * 6 * el;
    const size_t ncnt = (size_t)s->ncz * s->ncx;
    if (need > s->seam_bytes) {
        if (s->seam_lo) { cudaFree(s->seam_lo); cudaFree(s->seam_hi); s->device_bytes -= 2 * (int64_t)s->seam_bytes; }
        s->seam_lo = s->seam_hi = nullptr;
        s->seam_bytes = 0;
        CK(cudaMalloc(&s->seam_lo, need));
        CK(cudaMalloc(&s->seam_hi, need));
        s->seam_bytes = need;
        s->device_bytes += 2 * (int64_t)need;
    }
    if (ncnt > s->seam_cnt_n) {
        if (s->seam_cnt) { cudaFree(s->seam_cnt); s->device_bytes -= 4 * (int64_t)s->seam_cnt_n; }
        s->seam_cnt = nullptr;
        s->seam_cnt_n = 0;
        CK(cudaMalloc(&s->seam_cnt, ncnt * sizeof(int)));
        s->seam_cnt_n = ncnt;
        s->device_bytes += 4 * (int64_t)ncnt;
    }
    CK(cudaMemsetAsync(s->seam_cnt, 0, ncnt * sizeof(int), s->stream));
    return SKS_OK;
}

// one time step it >= 1: a single fused kernel (force, assembly, update,
// receivers, and the boundary increment of step it+1)
template <typename T, bool LF>
int step_impl(sks_solver* s, int it, const T* dline, float* seis_row)
{
    const sks_model& m = s->m;
    Field<T> F = make_field<T>(s);
    F.dline = dline;
    F.inject_next = (it + 1 < m.nt_sem) ? 1 : 0;
    F.seis_row = seis_row;
    {
        const int k = s->snaps ? snap_index(it, m.snap_start, m.snap_incre, s->nsnap) : -1;
        F.snap = k >= 0 ? s->snaps + (size_t)k * s->snap_size : nullptr;
    }
    Geo<T> G = make_geo<T>(s);
    {
        KTimer t(s, SKS_KC_ELEMENT);
        const StepVariant v{s->NW, s->ZS, s->CAP, s->m.nh_att > 0};
        StepOf<T> f{s, v, F, G, nullptr, nullptr};
        with_degree(m.hpn, f);
    }
    s->cur = 1 - s->cur;
    return SKS_OK;
}

template <typename T, bool LF>
int step0_impl(sks_solver* s, const double* G0, const double* G1, float* seis_row)
{
    const sks_model& m = s->m;
    const int64_t np = (int64_t)m.nx * m.nz;
    cudaStream_t st = s->stream;
    s->cur = 0;
    CK(cudaMemsetAsync(s->U[0], 0, 3 * np * sizeof(T), st));
    CK(cudaMemsetAsync(s->U[1], 0, 3 * np * sizeof(T), st));
    if (LF) {
        CK(cudaMemsetAsync(s->Dv, 0, 6 * np * sizeof(T), st));
    }
    if (m.nt_sem > 0) {
        const int n = (m.nx - s->nbl - 1) + (m.nz - s->nbl);
        KTimer t(s, SKS_KC_INJECT);
        k_init_line<T, LF><<<(n + 255) / 256, 256, 0, st>>>((T*)s->U[0], (T*)s->Dv, np, m.nx, m.nz, s->nbl, G0, m.mtotal);
    }
    if (m.ntrace > 0) {
        KTimer t(s, SKS_KC_RECORD);
        k_record<T><<<(m.ntrace + 127) / 128, 128, 0, st>>>((const T*)s->U[0], np, s->rec_off, m.ntrace, seis_row);
    }
    if (s->snaps) {
        const int k = snap_index(0, m.snap_start, m.snap_incre, s->nsnap);
        if (k >= 0) {
            const int64_t n = (int64_t)((m.nx + 1) / 2) * ((m.nz + 1) / 2);
            k_snap<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const T*)s->U[0], np, m.nx, m.nz,
                                                                 s->snaps + (size_t)k * s->snap_size, (m.nz + 1) / 2);
        }
    }
    if (m.nt_sem > 1) {   // step 1's GRT_Interface4, applied to the step-0 field
        const int n = (m.nx - s->nbl) + (m.nz - s->nbl - 1);
        KTimer t(s, SKS_KC_INJECT);
        k_inject<T, LF><<<(n + 255) / 256, 256, 0, st>>>((T*)s->U[0], (T*)s->Dv, (T*)s->Cc, np, m.nx, m.nz,
                                                         s->nbl, G1, G0, m.mtotal);
    }
    return SKS_OK;
}

// steps it1 .. it1+cnt-1 (it1 >= 1) of the chunk in one pipelined launch;
// i0 = the first of them within the chunk (its row of Dl and of the seismograms)
template <typename T, bool LF>
int pipe_impl(sks_solver* s, int it1, int cnt, int i0)
{
    const sks_model& m = s->m;
    const size_t nline = (size_t)(m.nx - s->nbl) + (m.nz - s->nbl - 1);
    Field<T> F = make_field<T>(s);
    Geo<T> G = make_geo<T>(s);
    PipeChunk C;
    C.U[0] = s->U[0];
    C.U[1] = s->U[1];
    C.it0 = it1;
    C.n = cnt;
    C.nt_sem = m.nt_sem;
    C.nline = (int)nline;
    C.dl = (const T*)s->Dl + (size_t)i0 * nline * 3;
    C.seis = s->seis + (size_t)i0 * 3 * m.ntrace;
    C.snaps = s->snaps;
    C.snap_start = m.snap_start;
    C.snap_incre = m.snap_incre;
    C.nsnap = s->nsnap;
    C.snap_size = s->snap_size;
    const PipeCtl ctl{s->pipe_ctl, s->pipe_ctl + 2, s->pipe_ctl + 1, s->test_stall ? s->test_spins : PIPE_SPIN_LIMIT,
                      s->test_stall - 1};
    const int ntiles = s->ncx * s->ncz;
    CK(cudaMemsetAsync(ctl.claim, 0, sizeof(int), s->stream));
    CK(cudaMemsetAsync(ctl.done, 0, sizeof(int) * (size_t)ntiles, s->stream));
    {
        KTimer t(s, SKS_KC_ELEMENT);
        const StepVariant v{s->NW, s->ZS, s->CAP, s->m.nh_att > 0};
        StepOf<T> f{s, v, F, G, &C, &ctl};
        CK(with_degree(m.hpn, f));
    }
    s->cur = (it1 + cnt - 1) & 1;
    return SKS_OK;
}

int run_chunk(sks_solver* s, int it0, int n)
{
    const sks_model& m = s->m;
    const int L = m.mtotal + m.shtotal;
    cudaStream_t st = s->stream;
    // G row r holds the interpolated traces of step it0-1+r; a step it needs
    // rows of it and it+1, so the chunk interpolates steps [it0, it0+n]
    const int ni = std::max(0, std::min(it0 + n + 1, m.nt_sem) - it0);
    if (ni > 0) {
        if (it0 > 0 && s->g_last > 0)
            CK(cudaMemcpyAsync(s->G, s->G + (size_t)s->g_last * L, sizeof(double) * L, cudaMemcpyDeviceToDevice, st));
        {
            KTimer t(s, SKS_KC_INTERP);
            k_interp<<<ni, 256, 0, st>>>(s->G, L, it0, ni, s->rs, s->rec_psv, m.mtotal, s->rec_sh, m.shtotal,
                                         s->tap_psv, s->w_psv, s->tap_sh, s->w_sh);
        }
        s->g_last = n;     // row of step it0+n-1: the previous step of the next chunk
        // increments g(it+1) - g(it) for the steps it0..it0+n-1 that inject next
        const int nd = std::max(0, std::min(it0 + n + 1, m.nt_sem) - it0 - 1);
        if (nd > 0) {
            const int nline = (m.nx - s->nbl) + (m.nz - s->nbl - 1);
            const int64_t tot = (int64_t)nd * nline;
            KTimer t(s, SKS_KC_INTERP);
            if (s->precision == SKS_FP64)
                k_line_delta<double><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>((double*)s->Dl, s->G + L, L, nd, m.nx, m.nz,
                                                                                  s->nbl, m.mtotal);
            else
                k_line_delta<float><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>((float*)s->Dl, s->G + L, L, nd, m.nx, m.nz,
                                                                                 s->nbl, m.mtotal);
        }
    }
    if (m.ntrace > 0) CK(cudaMemsetAsync(s->seis, 0, sizeof(float) * (size_t)n * 3 * m.ntrace, st));
    for (int i = 0; i < n; i++) {
        const int it = it0 + i;
        if (s->PIPE && it > 0) {        // the rest of the chunk as one pipelined launch
            const int rc = s->precision == SKS_FP64 ? pipe_impl<double, false>(s, it, n - i, i)
                                                    : pipe_impl<float, true>(s, it, n - i, i);
            if (rc) return rc;
            break;
        }
        const double* Gcur = s->G + (size_t)(i + 1) * L;
        const double* Gnext = s->G + (size_t)(i + 2) * L;
        const size_t nline = (size_t)(m.nx - s->nbl) + (m.nz - s->nbl - 1);
        float* row = s->seis + (size_t)i * 3 * m.ntrace;
        int rc;
        if (s->precision == SKS_FP64) {
            rc = it == 0 ? step0_impl<double, false>(s, Gcur, Gnext, row)
                         : step_impl<double, false>(s, it, (const double*)s->Dl + (size_t)i * nline * 3, row);
        } else {
            rc = it == 0 ? step0_impl<float, true>(s, Gcur, Gnext, row)
                         : step_impl<float, true>(s, it, (const float*)s->Dl + (size_t)i * nline * 3, row);
        }
        if (rc) return rc;
    }
    CK(cudaGetLastError());
    return SKS_OK;
}

}  // namespace sksi

extern "C" int sks_open_setup(sks_setup* su, int precision, int device, sks_solver** out)
{
    if (!su) return set_err(SKS_ERR_ARG, "set-up is NULL");
    if (!out) { sks_setup_close(su); return set_err(SKS_ERR_ARG, "out is NULL"); }
    *out = nullptr;
    if (precision != SKS_FP64 && precision != SKS_FP32C) { sks_setup_close(su); return set_err(SKS_ERR_ARG, "unknown precision %d", precision); }
    sks_solver* s = new (std::nothrow) sks_solver();
    if (!s) { sks_setup_close(su); return set_err(SKS_ERR_NOMEM, "cannot allocate the solver"); }
    s->m = su->m;                 // take ownership of the host model
    memset(&su->m, 0, sizeof su->m);
    delete su;
    int rc = SKS_OK;
    const sks_model& m = s->m;
    if (m.hpn < 3 || m.hpn > 6) { sks_model_free(&s->m); delete s; return set_err(SKS_ERR_UNSUPPORTED, "hpn=%d: the kernels are built for GLL degrees 3 to 6", m.hpn); }
    s->precision = precision;
    s->device = device;
    s->nbl = m.neh * m.hpn;
    cudaError_t ce = cudaSetDevice(device);
    if (ce != cudaSuccess) { sks_model_free(&s->m); delete s; return set_err(SKS_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(ce)); }
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    ce = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) { sks_model_free(&s->m); delete s; return set_err(SKS_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(ce)); }
    s->sms = sms;
    if ((int64_t)m.nx * m.nz * 3 >= ((int64_t)1 << 31)) {
        free_device(s); cudaStreamDestroy(s->stream); sks_model_free(&s->m); delete s;
        return set_err(SKS_ERR_UNSUPPORTED, "mesh of %d x %d points: 3*nx*nz must stay below 2^31", m.nx, m.nz);
    }
    {
        // defaults from sweeps on a GB300 (what sks_autotune would pick, without
        // its cost).  Up to 2 M points: one balanced wave of CTAs (the 0.32 M-
        // point mesh: 0.018 ms per FP32C step against 0.024 for the next best).
        // Above: pipelined chunks -- FP32C with halo rows in bands of 8
        // (3.8 M points: 0.091 ms against 0.102 per-step), FP64 with band
        // seams in bands of 6 (1.28 ms against 1.43) -- except FP32C above
        // 16 M points, where per-step launches of 12-row bands win (64 M
        // points: 1.26 ms against 1.43 pipelined).  One wave of tall bands is
        // not used on large meshes: with fewer CTA slots than twice the
        // element columns its bands differ in height by up to 2x (FP64, 64 M
        // points: 30.5 ms against 21.1).  Other GLL degrees, FP32C, pipelined
        // on the 800 x 300 km box (3.84 M points): degree 5 with band seams
        // (0.103 ms against 0.116 with halo rows), degree 3 in bands of 12
        // (0.090 against 0.094), degree 6 without the register cap, which
        // spills it (0.124 against 0.153).
        const int ncx4 = (m.nex + (tex_of(m.hpn) * 4 - 1) - 1) / (tex_of(m.hpn) * 4 - 1);
        const int64_t pts = (int64_t)m.nx * m.nz;
        const int cap32 = m.hpn == 6 ? 0 : 1;
        int rcg;
        if (pts <= ((int64_t)2 << 20))
            rcg = precision == SKS_FP32C ? set_grid(s, 4, pick_band(m, ncx4, sms, 10), 0, cap32, 1)
                                         : set_grid(s, 4, pick_band(m, ncx4, sms, 5), 1, 0, 1);
        else if (precision == SKS_FP64)
            rcg = set_grid(s, 4, 6, 1, 1, 0, 1);
        else if (pts <= ((int64_t)16 << 20))
            rcg = set_grid(s, 4, m.hpn == 3 ? 12 : 8, m.hpn == 5 ? 1 : 0, cap32, 0, 1);
        else
            rcg = set_grid(s, 4, 12, 0, cap32, 0, 0);
        if (rcg) { free_device(s); cudaStreamDestroy(s->stream); sks_model_free(&s->m); delete s; return rcg; }
    }
    s->chunk = 64;
    const size_t np = (size_t)m.nx * m.nz;
    rc = precision == SKS_FP64 ? upload_tables<double>(s) : upload_tables<float>(s);
    if (!rc) rc = dmalloc(s, &s->mid, np);
    if (!rc) {
        ce = cudaMemcpy(s->mid, m.mat_id, np * sizeof(uint16_t), cudaMemcpyHostToDevice);
        if (ce != cudaSuccess) rc = set_err(SKS_ERR_CUDA, "upload of material indices: %s", cudaGetErrorString(ce));
    }
    s->rec_iz0 = 1 << 30;
    s->rec_iz1 = -1;
    if (!rc && m.ntrace > 0) {
        // receivers inside the mesh, sorted by point, and a bitmap of their points
        std::vector<std::pair<int64_t, int32_t>> rs;
        for (int i = 0; i < m.ntrace; i++)
            if (m.rec_off[i] < (int64_t)np) rs.push_back({m.rec_off[i], i});
        std::sort(rs.begin(), rs.end());
        s->nrec_in = (int)rs.size();
        s->rec_iz0 = 1 << 30;
        s->rec_iz1 = -1;
        for (auto& r : rs) {
            const int iz = (int)(r.first / m.nx);
            s->rec_iz0 = std::min(s->rec_iz0, iz);
            s->rec_iz1 = std::max(s->rec_iz1, iz);
        }
        std::vector<int64_t> off(rs.size());
        std::vector<int32_t> idx(rs.size());
        std::vector<uint32_t> bits((np + 31) / 32, 0u);
        for (size_t i = 0; i < rs.size(); i++) {
            off[i] = rs[i].first; idx[i] = rs[i].second;
            bits[rs[i].first >> 5] |= 1u << (rs[i].first & 31);
        }
        rc = dmalloc(s, &s->recbits, bits.size());
        if (!rc) rc = dmalloc(s, &s->rec_sorted, std::max<size_t>(1, off.size()));
        if (!rc) rc = dmalloc(s, &s->rec_idx, std::max<size_t>(1, idx.size()));
        if (!rc) {
            cudaMemcpy(s->recbits, bits.data(), bits.size() * 4, cudaMemcpyHostToDevice);
            if (!off.empty()) cudaMemcpy(s->rec_sorted, off.data(), off.size() * 8, cudaMemcpyHostToDevice);
            if (!idx.empty()) ce = cudaMemcpy(s->rec_idx, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice);
            else ce = cudaSuccess;
            if (ce != cudaSuccess) rc = set_err(SKS_ERR_CUDA, "upload of receivers: %s", cudaGetErrorString(ce));
        }
    }
    if (!rc) rc = dmalloc(s, &s->rec_off, std::max(1, m.ntrace));
    if (!rc && m.ntrace > 0) {
        ce = cudaMemcpy(s->rec_off, m.rec_off, sizeof(int64_t) * m.ntrace, cudaMemcpyHostToDevice);
        if (ce != cudaSuccess) rc = set_err(SKS_ERR_CUDA, "upload of receivers: %s", cudaGetErrorString(ce));
    }
    if (!rc) rc = dmalloc(s, &s->seisbuf[0], (size_t)s->chunk * 3 * std::max(1, m.ntrace));
    if (!rc) rc = dmalloc(s, &s->seisbuf[1], (size_t)s->chunk * 3 * std::max(1, m.ntrace));
    if (!rc) {
        s->seis = s->seisbuf[0];
        ce = cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking);
        for (int i = 0; i < 2 && ce == cudaSuccess; i++) {
            ce = cudaEventCreateWithFlags(&s->chunk_done[i], cudaEventDisableTiming);
            if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&s->copy_done[i], cudaEventDisableTiming);
        }
        if (ce != cudaSuccess) rc = set_err(SKS_ERR_CUDA, "copy stream/events: %s", cudaGetErrorString(ce));
    }
    if (!rc) {
        // element rows whose points are all of isotropic materials (the
        // anisotropic FP64 step kernels take the isotropic stress there)
        const std::vector<uint8_t> iso = isotropic_rows(m);
        rc = dmalloc(s, &s->row_iso, iso.size());
        if (!rc && cudaMemcpy(s->row_iso, iso.data(), iso.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            rc = set_err(SKS_ERR_CUDA, "upload of the isotropic element rows");
        // element rows whose points share one material (-1: they do not)
        std::vector<int16_t> rmat((size_t)m.nez);
        for (int ez = 0; ez < m.nez; ez++) {
            const uint16_t first = m.mat_id[(size_t)ez * m.hpn * m.nx];
            int v = first < 32768 ? first : -1;
            for (int iz = ez * m.hpn; iz <= ez * m.hpn + m.hpn && v >= 0; iz++)
                for (int ix = 0; ix < m.nx; ix++)
                    if (m.mat_id[(size_t)iz * m.nx + ix] != first) { v = -1; break; }
            rmat[ez] = (int16_t)v;
        }
        if (!rc) rc = dmalloc(s, &s->row_mat, rmat.size());
        if (!rc && cudaMemcpy(s->row_mat, rmat.data(), rmat.size() * sizeof(int16_t), cudaMemcpyHostToDevice) !=
                       cudaSuccess)
            rc = set_err(SKS_ERR_CUDA, "upload of the element rows' materials");
    }
    if (!rc) rc = dmalloc(s, &s->nonfinite, 1);
    if (!rc && cudaMemset(s->nonfinite, 0, sizeof(int)) != cudaSuccess) rc = set_err(SKS_ERR_CUDA, "wavefield flag");
    if (!rc && cudaMallocHost((void**)&s->hflags, 2 * sizeof(int)) != cudaSuccess) {
        s->hflags = nullptr;
        rc = set_err(SKS_ERR_NOMEM, "pinned host flags");
    }
    if (!rc) s->hflags[0] = s->hflags[1] = 0;
    if (!rc) rc = dmalloc(s, &s->G, (size_t)(s->chunk + 2) * (m.mtotal + m.shtotal));
    if (!rc) {
        const size_t nline = (size_t)(m.nx - s->nbl) + (m.nz - s->nbl - 1);
        double* dl = nullptr;
        const size_t el = precision == SKS_FP64 ? 1 : 2;   // doubles, or floats packed two per double
        rc = dmalloc(s, &dl, ((size_t)s->chunk + 1) * nline * 3 / el + 1);
        s->Dl = dl;
    }
    if (!rc && m.nt_sem > 0) {
        rc = dmalloc(s, &s->tap_psv, 4 * (size_t)m.nt_sem);
        if (!rc) rc = dmalloc(s, &s->tap_sh, 4 * (size_t)m.nt_sem);
        if (!rc) rc = dmalloc(s, &s->w_psv, 4 * (size_t)m.nt_sem);
        if (!rc) rc = dmalloc(s, &s->w_sh, 4 * (size_t)m.nt_sem);
        if (!rc) {
            cudaMemcpy(s->tap_psv, m.tap_psv, 16 * (size_t)m.nt_sem, cudaMemcpyHostToDevice);
            cudaMemcpy(s->tap_sh, m.tap_sh, 16 * (size_t)m.nt_sem, cudaMemcpyHostToDevice);
            cudaMemcpy(s->w_psv, m.w_psv, 32 * (size_t)m.nt_sem, cudaMemcpyHostToDevice);
            ce = cudaMemcpy(s->w_sh, m.w_sh, 32 * (size_t)m.nt_sem, cudaMemcpyHostToDevice);
            if (ce != cudaSuccess) rc = set_err(SKS_ERR_CUDA, "upload of the boundary schedule: %s", cudaGetErrorString(ce));
        }
    }
    if (!rc && m.plot_snap) {
        // as many of the 26 candidate steps start + k*incre as fall in the run
        s->nsnap = 0;
        for (int k = 0; k < SKS_NSNAP; k++) {
            const int64_t it = (int64_t)m.snap_start + (int64_t)k * m.snap_incre;
            if (it >= 0 && it < m.nst) s->nsnap = k + 1;
        }
        if (m.snap_incre == 0) s->nsnap = (m.snap_start >= 0 && m.snap_start < m.nst) ? 1 : 0;
        s->snap_size = (size_t)((m.nx + 1) / 2) * ((m.nz + 1) / 2) * 2;
        if (s->nsnap > 0) {
            rc = dmalloc(s, &s->snaps, (size_t)s->nsnap * s->snap_size);
            if (!rc && cudaMemset(s->snaps, 0, sizeof(float) * (size_t)s->nsnap * s->snap_size) != cudaSuccess)
                rc = set_err(SKS_ERR_CUDA, "snapshot buffers");
        }
    }
    if (rc) {
        free_device(s);
        if (s->hflags) cudaFreeHost(s->hflags);
        cudaStreamDestroy(s->stream);
        sks_model_free(&s->m);
        delete s;
        return rc;
    }
    s->boundary_ready = (m.nt_sem == 0);
    *out = s;
    return SKS_OK;
}

extern "C" int sks_open_par(int argc, const char* const* argv, int precision, int device, sks_solver** out)
{
    sks_setup* su = nullptr;
    int rc = sks_setup_open(argc, argv, &su);
    if (rc) return rc;
    return sks_open_setup(su, precision, device, out);
}

namespace {

// device buffers for the records the run reads
int alloc_records(sks_solver* s)
{
    const sks_model& m = s->m;
    const size_t npsv = (size_t)m.nrec_psv * m.mtotal, nsh = (size_t)m.nrec_sh * m.shtotal;
    if (s->nrec_psv_loaded < m.nrec_psv || !s->rec_psv) {
        if (s->rec_psv) { cudaFree(s->rec_psv); s->device_bytes -= (int64_t)(sizeof(float) * (size_t)s->nrec_psv_loaded * m.mtotal); s->rec_psv = nullptr; }
        int rc = dmalloc(s, &s->rec_psv, npsv);
        if (rc) return rc;
        s->nrec_psv_loaded = m.nrec_psv;
    }
    if (s->nrec_sh_loaded < m.nrec_sh || !s->rec_sh) {
        if (s->rec_sh) { cudaFree(s->rec_sh); s->device_bytes -= (int64_t)(sizeof(float) * (size_t)s->nrec_sh_loaded * m.shtotal); s->rec_sh = nullptr; }
        int rc = dmalloc(s, &s->rec_sh, nsh);
        if (rc) return rc;
        s->nrec_sh_loaded = m.nrec_sh;
    }
    return SKS_OK;
}

}  // namespace

namespace {

// release the record tables and the mode series (a generator replaces them)
void free_records(sks_solver* s)
{
    const sks_model& m = s->m;
    if (s->rec_psv) { cudaFree(s->rec_psv); s->device_bytes -= (int64_t)(sizeof(float) * (size_t)s->nrec_psv_loaded * m.mtotal); }
    if (s->rec_sh) { cudaFree(s->rec_sh); s->device_bytes -= (int64_t)(sizeof(float) * (size_t)s->nrec_sh_loaded * m.shtotal); }
    s->rec_psv = s->rec_sh = nullptr;
    s->nrec_psv_loaded = s->nrec_sh_loaded = 0;
}

void free_series(sks_solver* s)
{
    if (s->ser) { cudaFree(s->ser); s->device_bytes -= (int64_t)(sizeof(double) * s->ser_n); }
    s->ser = nullptr;
    s->ser_n = 0;
}

// the generator's part of a record source that the grid fixes
RecSource grid_source(const sks_solver* s, int kind)
{
    const sks_model& m = s->m;
    RecSource g;
    memset(&g, 0, sizeof g);
    g.kind = kind;
    g.nx = m.nx;
    g.nz = m.nz;
    g.nbl = s->nbl;
    g.deg = m.hpn;
    g.eh = m.eh;
    g.dp = m.dp;
    return g;
}

}  // namespace

extern "C" int sks_set_boundary_plane_wave(sks_solver* s, const sks_plane_wave_t* pw)
{
    if (!s || !pw) return set_err(SKS_ERR_ARG, "NULL argument");
    if (!(pw->vs > 0.0) || !(pw->f0 > 0.0) || !(pw->p >= 0.0)) return set_err(SKS_ERR_ARG, "plane wave needs vs > 0, f0 > 0, p >= 0");
    if (s->batch) return set_err(SKS_ERR_STATE, "the solver is a member of a batch: set its boundary before adding it");
    cudaSetDevice(s->device);
    CK(cudaStreamSynchronize(s->stream));
    free_records(s);
    free_series(s);
    RecSource g = grid_source(s, REC_PLANE);
    g.p = pw->p;
    g.vs = pw->vs;
    g.f0 = pw->f0;
    g.sv_amp = pw->sv_amp;
    g.sh_amp = s->m.psv_only ? 0.0 : pw->sh_amp;
    // the line's delays and amplitudes, once: [2][L] doubles in the series buffer
    const size_t L = (size_t)s->m.mtotal + s->m.shtotal;
    int rc;
    if ((rc = dmalloc(s, &s->ser, 2 * L))) return rc;
    s->ser_n = 2 * L;
    k_plane_line<<<(unsigned)((L + 255) / 256), 256, 0, s->stream>>>(g, s->ser);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->stream));
    g.lt = s->ser;
    s->rs = g;
    s->boundary_ready = true;
    return SKS_OK;
}

extern "C" int sks_set_boundary_layered_wave(sks_solver* s, const sks_stack_layer_t* layers, int32_t n,
                                             const sks_layered_wave_t* w)
{
    if (!s || !layers || !w) return set_err(SKS_ERR_ARG, "NULL argument");
    if (n < 2) return set_err(SKS_ERR_ARG, "layered wave: at least 2 media (top, half-space)");
    if (s->batch) return set_err(SKS_ERR_STATE, "the solver is a member of a batch: set its boundary before adding it");
    const sks_model& m = s->m;
    // the series: samples dp/4 apart over the records' span plus the largest
    // delay along the line (p x + eta z at the far corner, slowest mode)
    const double dts = m.dp / 4.0;
    const double xmax = (double)(m.nx - 1) * m.h + m.eh, zmax = (double)(m.nz - 1) * m.h + m.eh;
    const double smax = 1.0 / layers[0].vs;
    const double span = (double)std::max(m.nrec_psv, m.nrec_sh) * m.dp + w->p * xmax + smax * zmax;
    const int64_t nt = sks_layered_series_length(layers, n, w->p, w->f0, dts, span);
    if (nt < 0) return (int)nt;
    std::vector<double> ser;
    try {
        ser.resize((size_t)nt * 3);
    } catch (...) {
        return set_err(SKS_ERR_NOMEM, "layered wave: out of host memory");
    }
    sks_layered_wave_t ww = *w;
    if (m.psv_only) ww.sh_amp = 0.0;
    int rc = sks_layered_series(layers, n, &ww, dts, nt, ser.data());
    if (rc) return rc;
    cudaSetDevice(s->device);
    CK(cudaStreamSynchronize(s->stream));
    free_records(s);
    // the mode series [3][nt], then the line's delays and coefficients [4][L]
    const size_t L = (size_t)m.mtotal + m.shtotal, need = 3 * (size_t)nt + 4 * L;
    if (s->ser_n != need) {
        free_series(s);
        if ((rc = dmalloc(s, &s->ser, need))) return rc;
        s->ser_n = need;
    }
    CK(cudaMemcpy(s->ser, ser.data(), sizeof(double) * 3 * (size_t)nt, cudaMemcpyHostToDevice));
    RecSource g = grid_source(s, REC_LAYERED);
    g.p = w->p;
    g.ser = s->ser;
    g.nt = nt;
    g.dts = dts;
    g.vp0 = layers[0].vp;
    g.vs0 = layers[0].vs;
    k_layered_line<<<(unsigned)((L + 255) / 256), 256, 0, s->stream>>>(g, s->ser + 3 * (size_t)nt);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->stream));
    g.lt = s->ser + 3 * (size_t)nt;
    s->rs = g;
    s->boundary_ready = true;
    return SKS_OK;
}

extern "C" int sks_set_boundary(sks_solver* s, const float* psv, int32_t nrec_psv, const float* sh, int32_t nrec_sh)
{
    if (!s) return set_err(SKS_ERR_ARG, "solver is NULL");
    if (s->batch) return set_err(SKS_ERR_STATE, "the solver is a member of a batch: set its boundary before adding it");
    const sks_model& m = s->m;
    if (nrec_psv < m.nrec_psv) return set_err(SKS_ERR_BOUNDARY, "the run reads %d P-SV records, %d given", m.nrec_psv, nrec_psv);
    if (!m.psv_only && nrec_sh < m.nrec_sh) return set_err(SKS_ERR_BOUNDARY, "the run reads %d SH records, %d given", m.nrec_sh, nrec_sh);
    if (m.nrec_psv > 0 && !psv) return set_err(SKS_ERR_ARG, "psv records are NULL");
    if (!m.psv_only && m.nrec_sh > 0 && !sh) return set_err(SKS_ERR_ARG, "sh records are NULL");
    cudaSetDevice(s->device);
    const size_t npsv = (size_t)m.nrec_psv * m.mtotal, nsh = (size_t)m.nrec_sh * m.shtotal;
    {
        int rc = alloc_records(s);
        if (rc) return rc;
    }
    if (npsv) CK(cudaMemcpyAsync(s->rec_psv, psv, npsv * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    if (nsh) {
        if (m.psv_only || !sh) CK(cudaMemsetAsync(s->rec_sh, 0, nsh * sizeof(float), s->stream));
        else CK(cudaMemcpyAsync(s->rec_sh, sh, nsh * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    free_series(s);
    s->rs = RecSource{};
    s->rs.kind = REC_TABLE;
    s->boundary_ready = true;
    return SKS_OK;
}

extern "C" int sks_load_boundary_files(sks_solver* s)
{
    if (!s) return set_err(SKS_ERR_ARG, "solver is NULL");
    const sks_model& m = s->m;
    std::vector<float> psv((size_t)m.nrec_psv * m.mtotal), sh;
    FILE* f = fopen(m.greenfile, "rb");
    if (!f) return set_err(SKS_ERR_IO, "cannot open P-SV boundary file %s", m.greenfile);
    size_t got = psv.empty() ? 0 : fread(psv.data(), sizeof(float), psv.size(), f);
    fclose(f);
    if (got != psv.size())
        return set_err(SKS_ERR_BOUNDARY, "%s holds %zu of the %d records of %d values the run reads", m.greenfile,
                       got / (size_t)m.mtotal, m.nrec_psv, m.mtotal);
    if (!m.psv_only) {
        sh.resize((size_t)m.nrec_sh * m.shtotal);
        f = fopen(m.shgreenfile, "rb");
        if (!f) return set_err(SKS_ERR_IO, "cannot open SH boundary file %s", m.shgreenfile);
        got = sh.empty() ? 0 : fread(sh.data(), sizeof(float), sh.size(), f);
        fclose(f);
        if (got != sh.size())
            return set_err(SKS_ERR_BOUNDARY, "%s holds %zu of the %d records of %d values the run reads", m.shgreenfile,
                           got / (size_t)m.shtotal, m.nrec_sh, m.shtotal);
    }
    return sks_set_boundary(s, psv.data(), m.nrec_psv, m.psv_only ? nullptr : sh.data(), m.nrec_sh);
}

extern "C" int sks_run(sks_solver* s, int32_t nsteps, float* su, float* sv, float* sw)
{
    if (!s) return set_err(SKS_ERR_ARG, "solver is NULL");
    if (nsteps < 0) return set_err(SKS_ERR_ARG, "nsteps=%d", nsteps);
    if (s->batch && batch_running(s->batch)) return set_err(SKS_ERR_STATE, "the solver's batch is running");
    const sks_model& m = s->m;
    if (s->step < m.nt_sem && !s->boundary_ready)
        return set_err(SKS_ERR_STATE, "boundary records not set: call sks_load_boundary_files or sks_set_boundary");
    cudaSetDevice(s->device);
    const int end = std::min(m.nst, s->step + nsteps);
    const int total = end - s->step;
    const bool want = m.ntrace > 0 && (su || sv || sw);
    int done = 0, chunk_i = 0;
    // a chunk's seismograms are copied out on the copy stream while the next
    // chunk computes; strided copies put each component straight into the
    // caller's arrays
    struct Pending { int slot, n, done; } pend = {-1, 0, 0};
    auto issue_copy = [&](const Pending& p) -> int {
        const size_t w = sizeof(float) * (size_t)m.ntrace, sp = 3 * w;
        float* dst[3] = {su, sv, sw};
        CK(cudaStreamWaitEvent(s->copy_stream, s->chunk_done[p.slot], 0));
        for (int c = 0; c < 3; c++)
            if (dst[c])
                CK(cudaMemcpy2DAsync(dst[c] + (size_t)p.done * m.ntrace, w, s->seisbuf[p.slot] + (size_t)c * m.ntrace, sp,
                                     w, (size_t)p.n, cudaMemcpyDeviceToHost, s->copy_stream));
        CK(cudaEventRecord(s->copy_done[p.slot], s->copy_stream));
        s->slot_busy[p.slot] = true;
        return SKS_OK;
    };
    if (!s->run_ev[0]) {
        CK(cudaEventCreate(&s->run_ev[0]));
        CK(cudaEventCreate(&s->run_ev[1]));
    }
    if (s->PIPE) CK(cudaMemsetAsync(s->pipe_ctl + 1, 0, sizeof(int), s->stream));
    CK(cudaEventRecord(s->run_ev[0], s->stream));
    while (s->step < end) {
        const int n = std::min(s->chunk, end - s->step);
        const int slot = chunk_i & 1;
        if (s->slot_busy[slot]) {            // its previous contents are still being copied out
            CK(cudaStreamWaitEvent(s->stream, s->copy_done[slot], 0));
            s->slot_busy[slot] = false;
        }
        s->seis = s->seisbuf[slot];
        // a failed chunk returns only once the copies already queued into the
        // caller's arrays have landed, so the caller may free them at once
        auto bail = [&](int code) {
            cudaStreamSynchronize(s->copy_stream);
            s->slot_busy[0] = s->slot_busy[1] = false;
            return code;
        };
        int rc = run_chunk(s, s->step, n);
        if (rc) return bail(rc);
        if (want) CK(cudaEventRecord(s->chunk_done[slot], s->stream));
        rc = collect_timing(s);
        if (rc) return bail(rc);
        if (want && pend.slot >= 0 && (rc = issue_copy(pend))) return bail(rc);
        pend = want ? Pending{slot, n, done} : Pending{-1, 0, 0};
        if (s->snaps)
            for (int it = s->step; it < s->step + n; it++) {
                const int k = snap_index(it, m.snap_start, m.snap_incre, s->nsnap);
                if (k >= 0) s->snap_taken[k] = true;
            }
        s->step += n;
        done += n;
        chunk_i++;
    }
    if (want && pend.slot >= 0) {
        int rc = issue_copy(pend);
        if (rc) return rc;
    }
    CK(cudaEventRecord(s->run_ev[1], s->stream));
    // the run's flags, read with the final synchronisation
    s->hflags[0] = s->hflags[1] = 0;
    CK(cudaMemcpyAsync(s->hflags, s->nonfinite, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    if (s->PIPE) CK(cudaMemcpyAsync(s->hflags + 1, s->pipe_ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaStreamSynchronize(s->copy_stream));
    s->slot_busy[0] = s->slot_busy[1] = false;
    s->test_stall = 0;
    {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, s->run_ev[0], s->run_ev[1]));
        s->last_run_ms = ms;
    }
    if (s->hflags[1]) return set_err(SKS_ERR_CUDA, "pipelined step: a wait for neighbouring tiles ran out");
    if (s->hflags[0])
        return set_err(SKS_ERR_NONFINITE, "the wavefield holds a non-finite displacement (steps up to %d)", s->step - 1);
    return total;
}

extern "C" int sks_wavefield_finite(const sks_solver* s)
{
    if (!s) return set_err(SKS_ERR_ARG, "solver is NULL");
    return s->hflags[0] ? 0 : 1;
}

extern "C" int sks_test_stall_pipeline(sks_solver* s, int32_t tile, int32_t spin_limit)
{
    if (!s) return set_err(SKS_ERR_ARG, "solver is NULL");
    if (!s->PIPE) return set_err(SKS_ERR_STATE, "the solver does not run pipelined chunks (tuning pipeline=0)");
    if (tile < 0 || tile >= s->ncx * s->ncz) return set_err(SKS_ERR_ARG, "tile %d: 0..%d", tile, s->ncx * s->ncz - 1);
    if (spin_limit < 1 || spin_limit > PIPE_SPIN_LIMIT) return set_err(SKS_ERR_ARG, "spin_limit=%d: 1..%d", spin_limit, PIPE_SPIN_LIMIT);
    s->test_stall = tile + 1;
    s->test_spins = spin_limit;
    return SKS_OK;
}

extern "C" int sks_reset(sks_solver* s)
{
    if (!s) return set_err(SKS_ERR_ARG, "solver is NULL");
    if (s->batch && batch_running(s->batch)) return set_err(SKS_ERR_STATE, "the solver's batch is running");
    s->step = 0;
    s->cur = 0;
    s->g_last = 0;
    for (bool& t : s->snap_taken) t = false;
    cudaSetDevice(s->device);
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemset(s->nonfinite, 0, sizeof(int)));
    s->hflags[0] = 0;
    return SKS_OK;
}

// ---- state save / load -----------------------------------------------------
namespace {

struct StateHeader {
    char magic[8];            // "SKSSTATE"
    int32_t version, precision, nx, nz, nst, step, cur, nsnap;
    int64_t field_bytes;      // bytes of the wavefield arrays that follow
    int64_t snap_bytes;       // bytes of the snapshot buffers that follow
    uint8_t snap_taken[SKS_NSNAP];
    uint8_t pad[6];
};

// the device arrays of a solve's state, in save order
int state_arrays(const sks_solver* s, void* const* ptrs[3], size_t sizes[3])
{
    const size_t np = (size_t)s->m.nx * s->m.nz;
    const size_t el = s->precision == SKS_FP64 ? sizeof(double) : sizeof(float);
    ptrs[0] = (void* const*)&s->U[0];
    ptrs[1] = (void* const*)&s->U[1];
    ptrs[2] = (void* const*)&s->Dv;
    sizes[0] = sizes[1] = 3 * np * el;
    sizes[2] = s->precision == SKS_FP32C ? 6 * np * el : 0;
    return 3;
}

}  // namespace

extern "C" int64_t sks_state_bytes(const sks_solver* s)
{
    if (!s) return set_err(SKS_ERR_ARG, "solver is NULL");
    void* const* p[3];
    size_t sz[3];
    state_arrays(s, p, sz);
    return (int64_t)(sizeof(StateHeader) + sz[0] + sz[1] + sz[2] + (s->snaps ? s->nsnap * s->snap_size * sizeof(float) : 0));
}

extern "C" int sks_state_save(sks_solver* s, void* host, int64_t bytes)
{
    if (!s || !host) return set_err(SKS_ERR_ARG, "NULL argument");
    if (bytes < sks_state_bytes(s)) return set_err(SKS_ERR_ARG, "state buffer of %lld bytes, %lld needed", (long long)bytes, (long long)sks_state_bytes(s));
    if (s->batch && batch_running(s->batch)) return set_err(SKS_ERR_STATE, "the solver's batch is running");
    cudaSetDevice(s->device);
    void* const* p[3];
    size_t sz[3];
    state_arrays(s, p, sz);
    StateHeader h;
    memset(&h, 0, sizeof h);
    memcpy(h.magic, "SKSSTATE", 8);
    h.version = 1;
    h.precision = s->precision;
    h.nx = s->m.nx; h.nz = s->m.nz; h.nst = s->m.nst;
    h.step = s->step; h.cur = s->cur;
    h.nsnap = s->snaps ? s->nsnap : 0;
    h.field_bytes = (int64_t)(sz[0] + sz[1] + sz[2]);
    h.snap_bytes = (int64_t)(h.nsnap * s->snap_size * sizeof(float));
    for (int k = 0; k < SKS_NSNAP; k++) h.snap_taken[k] = s->snap_taken[k] ? 1 : 0;
    char* o = (char*)host;
    memcpy(o, &h, sizeof h);
    o += sizeof h;
    CK(cudaStreamSynchronize(s->stream));
    for (int i = 0; i < 3; i++) {
        if (!sz[i]) continue;
        CK(cudaMemcpy(o, *p[i], sz[i], cudaMemcpyDeviceToHost));
        o += sz[i];
    }
    if (h.snap_bytes) CK(cudaMemcpy(o, s->snaps, (size_t)h.snap_bytes, cudaMemcpyDeviceToHost));
    return SKS_OK;
}

extern "C" int sks_state_load(sks_solver* s, const void* host, int64_t bytes)
{
    if (!s || !host) return set_err(SKS_ERR_ARG, "NULL argument");
    if (bytes < (int64_t)sizeof(StateHeader)) return set_err(SKS_ERR_ARG, "state buffer too short");
    StateHeader h;
    memcpy(&h, host, sizeof h);
    if (memcmp(h.magic, "SKSSTATE", 8) || h.version != 1) return set_err(SKS_ERR_ARG, "not a saved solver state");
    if (h.precision != s->precision || h.nx != s->m.nx || h.nz != s->m.nz || h.nst != s->m.nst)
        return set_err(SKS_ERR_ARG, "the state belongs to another solve (form %d, %d x %d points, %d steps)",
                       h.precision, h.nx, h.nz, h.nst);
    if (h.nsnap != (s->snaps ? s->nsnap : 0)) return set_err(SKS_ERR_ARG, "the state's snapshot set differs");
    if (bytes < sks_state_bytes(s)) return set_err(SKS_ERR_ARG, "state buffer too short");
    void* const* p[3];
    size_t sz[3];
    state_arrays(s, p, sz);
    // the header's step and buffer index pick the device buffers the next run
    // reads, so a damaged header is refused before anything is copied
    if (h.step < 0 || h.step > h.nst || (h.cur != 0 && h.cur != 1))
        return set_err(SKS_ERR_ARG, "the state's step %d or buffer index %d is out of range", h.step, h.cur);
    if (h.field_bytes != (int64_t)(sz[0] + sz[1] + sz[2]) ||
        h.snap_bytes != (int64_t)((size_t)h.nsnap * s->snap_size * sizeof(float)))
        return set_err(SKS_ERR_ARG, "the state's array sizes differ from the solve's");
    if (s->batch && batch_running(s->batch)) return set_err(SKS_ERR_STATE, "the solver's batch is running");
    cudaSetDevice(s->device);
    const char* in = (const char*)host + sizeof h;
    CK(cudaStreamSynchronize(s->stream));
    for (int i = 0; i < 3; i++) {
        if (!sz[i]) continue;
        CK(cudaMemcpy(*p[i], in, sz[i], cudaMemcpyHostToDevice));
        in += sz[i];
    }
    if (h.snap_bytes) CK(cudaMemcpy(s->snaps, in, (size_t)h.snap_bytes, cudaMemcpyHostToDevice));
    s->step = h.step;
    s->cur = h.cur;
    s->g_last = 0;
    for (int k = 0; k < SKS_NSNAP; k++) s->snap_taken[k] = h.snap_taken[k] != 0;
    CK(cudaMemset(s->nonfinite, 0, sizeof(int)));
    s->hflags[0] = 0;
    return SKS_OK;
}

extern "C" int sks_snapshot(const sks_solver* s, int32_t k, float* out, int32_t* dims)
{
    if (!s) return set_err(SKS_ERR_ARG, "solver is NULL");
    const sks_model& m = s->m;
    if (dims) { dims[0] = (m.nx + 1) / 2; dims[1] = (m.nz + 1) / 2; }
    if (!m.plot_snap) return set_err(SKS_ERR_STATE, "snapshots need plot_snap=1");
    if (k < 0 || k >= SKS_NSNAP) return set_err(SKS_ERR_ARG, "snapshot %d: 0..%d", k, SKS_NSNAP - 1);
    const int kk = m.snap_incre == 0 ? 0 : k;         // every candidate names the same step
    if (kk >= s->nsnap || !s->snap_taken[kk]) return set_err(SKS_ERR_STATE, "snapshot %d has not been taken", k);
    if (out) {
        cudaSetDevice(s->device);
        CK(cudaStreamSynchronize(s->stream));
        CK(cudaMemcpy(out, s->snaps + (size_t)kk * s->snap_size, sizeof(float) * s->snap_size, cudaMemcpyDeviceToHost));
    }
    return m.snap_start + kk * m.snap_incre;
}

extern "C" int sks_get_info(const sks_solver* s, sks_info_t* info)
{
    if (!s || !info) return set_err(SKS_ERR_ARG, "NULL argument");
    fill_info(s->m, info);
    info->precision = s->precision;
    info->step = s->step;
    info->device_bytes = s->device_bytes;
    info->seam_points = 0;
    info->tile_rows = s->HZ;
    return SKS_OK;
}

extern "C" int64_t sks_kernel_launches(const sks_solver* s) { return s ? s->launches : -1; }

extern "C" void sks_destroy(sks_solver* s)
{
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->batch) batch_detach(s);
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_device(s);
    for (cudaEvent_t e : s->kev) cudaEventDestroy(e);
    for (int i = 0; i < 2; i++) {
        if (s->chunk_done[i]) cudaEventDestroy(s->chunk_done[i]);
        if (s->copy_done[i]) cudaEventDestroy(s->copy_done[i]);
    }
    if (s->copy_stream) { cudaStreamSynchronize(s->copy_stream); cudaStreamDestroy(s->copy_stream); }
    if (s->run_ev[0]) { cudaEventDestroy(s->run_ev[0]); cudaEventDestroy(s->run_ev[1]); }
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->hflags) cudaFreeHost(s->hflags);
    sks_model_free(&s->m);
    delete s;
}

extern "C" double sks_last_run_ms(const sks_solver* s) { return s ? s->last_run_ms : -1.0; }

extern "C" int sks_enable_kernel_timing(sks_solver* s, int on)
{
    if (!s) return set_err(SKS_ERR_ARG, "solver is NULL");
    s->timing = on ? 1 : 0;
    for (int i = 0; i < SKS_KERNEL_CLASSES; i++) { s->kms[i] = 0; s->kcount[i] = 0; }
    s->kused = 0;
    return SKS_OK;
}

extern "C" int sks_kernel_timing(const sks_solver* s, double* ms, int64_t* count)
{
    if (!s) return set_err(SKS_ERR_ARG, "solver is NULL");
    for (int i = 0; i < SKS_KERNEL_CLASSES; i++) {
        if (ms) ms[i] = s->kms[i];
        if (count) count[i] = s->kcount[i];
    }
    return SKS_OK;
}

extern "C" int sks_set_tuning(sks_solver* s, const sks_tuning_t* t)
{
    if (!s || !t) return set_err(SKS_ERR_ARG, "NULL argument");
    if (t->warps_per_block != 2 && t->warps_per_block != 4)
        return set_err(SKS_ERR_ARG, "warps_per_block=%d: 2 or 4", t->warps_per_block);
    if (t->register_cap < 0 || t->register_cap > 2)
        return set_err(SKS_ERR_ARG, "register_cap=%d: 0, 1 or 2", t->register_cap);
    if (t->waves == 0 && t->band_rows < 1) return set_err(SKS_ERR_ARG, "band_rows=%d must be positive", t->band_rows);
    if (t->waves < 0 || t->waves > 64) return set_err(SKS_ERR_ARG, "waves=%d: 0..64", t->waves);
    if (s->batch) return set_err(SKS_ERR_STATE, "the solver is a member of a batch: tune the batch");
    if (t->pipeline != 0 && t->pipeline != 1) return set_err(SKS_ERR_ARG, "pipeline=%d: 0 or 1", t->pipeline);
    return set_grid(s, t->warps_per_block, t->band_rows, t->zseam ? 1 : 0, t->register_cap, t->waves, t->pipeline);
}

extern "C" int sks_get_tuning(const sks_solver* s, sks_tuning_t* t)
{
    if (!s || !t) return set_err(SKS_ERR_ARG, "NULL argument");
    t->warps_per_block = s->NW;
    t->band_rows = s->HZ;
    t->zseam = s->ZS;
    t->waves = s->WAVES;
    t->register_cap = s->CAP;
    t->blocks = s->PIPE ? s->pipe_blocks : s->nblocks;
    t->ms_per_step = 0.f;
    t->pipeline = s->PIPE;
    return SKS_OK;
}

namespace sksi {

int snap_take(sks_solver* s, Snapshot& S)
{
    const size_t np = (size_t)s->m.nx * s->m.nz;
    const size_t el = s->precision == SKS_FP64 ? sizeof(double) : sizeof(float);
    void* bufs[] = {s->U[0], s->U[1], s->Dv, s->Cc, s->G};
    const size_t sz[] = {3 * np * el, 3 * np * el, 6 * np * el, 3 * np * el,
                         sizeof(double) * (size_t)(s->chunk + 2) * (s->m.mtotal + s->m.shtotal)};
    for (int i = 0; i < 5; i++) {
        if (!bufs[i]) continue;
        void* d = nullptr;
        cudaError_t e = cudaMalloc(&d, sz[i]);
        if (e != cudaSuccess) {
            for (void* p : S.dev) cudaFree(p);
            S.dev.clear();
            return set_err(SKS_ERR_NOMEM, "autotune snapshot: %s", cudaGetErrorString(e));
        }
        CK(cudaMemcpyAsync(d, bufs[i], sz[i], cudaMemcpyDeviceToDevice, s->stream));
        S.dev.push_back(d); S.bytes.push_back(sz[i]); S.src.push_back(bufs[i]);
    }
    S.step = s->step; S.cur = s->cur; S.g_last = s->g_last;
    return SKS_OK;
}

int snap_restore(sks_solver* s, const Snapshot& S)
{
    for (size_t i = 0; i < S.dev.size(); i++)
        CK(cudaMemcpyAsync(S.src[i], S.dev[i], S.bytes[i], cudaMemcpyDeviceToDevice, s->stream));
    s->step = S.step; s->cur = S.cur; s->g_last = S.g_last;
    return SKS_OK;
}

void snap_free(Snapshot& S)
{
    for (void* p : S.dev) cudaFree(p);
    S.dev.clear();
    S.bytes.clear();
    S.src.clear();
}

}  // namespace sksi

extern "C" int sks_autotune(sks_solver* s, int32_t steps, sks_tuning_t* best)
{
    if (!s) return set_err(SKS_ERR_ARG, "solver is NULL");
    const sks_model& m = s->m;
    if (steps < 1) steps = 8;
    if (s->batch) return set_err(SKS_ERR_STATE, "the solver is a member of a batch: tune the batch");
    if (s->step < m.nt_sem && !s->boundary_ready) return set_err(SKS_ERR_STATE, "boundary records not set");
    if (s->step + 1 + steps > m.nst) return set_err(SKS_ERR_STATE, "autotune needs %d more steps than the run has left", steps + 1);
    cudaSetDevice(s->device);
    Snapshot snap;
    int rc = snap_take(s, snap);
    if (rc) return rc;
    const int old_timing = s->timing;
    s->timing = 0;
    const int nws[] = {2, 4};
    // short bands for small meshes (the 321,201-point isotropic case: FP64
    // pipelined with 2-row bands 0.096 ms per step against 0.107 for one
    // balanced wave), tall ones for large
    const int hzs[] = {2, 3, 4, 6, 8, 9, 12};
    sks_tuning_t b = {s->NW, s->HZ, s->ZS, s->CAP, s->WAVES, s->nblocks, 1e30f, s->PIPE};
    // fixed band heights, then balanced partitions of 1..3 waves; pipelined
    // chunks with fixed band heights
    const int nhz = (int)(sizeof hzs / sizeof hzs[0]);
    for (int pipe = 0; pipe < 2; pipe++)
    for (int nw : nws)
        for (int zs = 0; zs < 2; zs++)
          for (int cap = 0; cap < 3; cap++)
            for (int cand = 0; cand < nhz + 3; cand++) {
                const int hz = cand < nhz ? hzs[cand] : 0, wv = cand < nhz ? 0 : cand - nhz + 1;
                if (wv == 0 && hz > m.nez && hz != hzs[0]) continue;
                if (pipe && wv) continue;
                if (!tuning_compiled(m.hpn, nw, cap)) continue;
                if ((rc = snap_restore(s, snap))) break;
                if ((rc = set_grid(s, nw, hz, zs, cap, wv, pipe))) break;
                // one untimed step, then the timed ones
                rc = sks_run(s, 1, nullptr, nullptr, nullptr);
                if (rc < 0) break;
                rc = sks_run(s, steps, nullptr, nullptr, nullptr);
                if (rc < 0) break;
                const float ms = (float)(s->last_run_ms / rc);
                if (ms < b.ms_per_step) b = {nw, s->HZ, zs, cap, wv, pipe ? s->pipe_blocks : s->nblocks, ms, pipe};
                rc = SKS_OK;
            }
    const int rc2 = snap_restore(s, snap);
    cudaStreamSynchronize(s->stream);
    for (void* p : snap.dev) cudaFree(p);
    s->timing = old_timing;
    const int rc3 = set_grid(s, b.warps_per_block, b.band_rows, b.zseam, b.register_cap, b.waves, b.pipeline);
    if (rc < 0) return rc;
    if (rc3) return rc3;
    if (rc2) return rc2;
    if (best) *best = b;
    return SKS_OK;
}

extern "C" int sks_line_increments(sks_solver* s, int32_t it0, int32_t nsteps, double* out)
{
    if (!s || !out) return set_err(SKS_ERR_ARG, "NULL argument");
    const sks_model& m = s->m;
    const int nline = (m.nx - s->nbl) + (m.nz - s->nbl - 1);
    if (it0 < 0 || nsteps < 0) return set_err(SKS_ERR_ARG, "it0=%d nsteps=%d", it0, nsteps);
    memset(out, 0, sizeof(double) * (size_t)nsteps * nline * 3);
    // step it injects into its output g(it+1) - g(it) while it+1 < nt_inject
    const int nd = std::max(0, std::min(it0 + nsteps, m.nt_sem - 1) - it0);
    if (nd == 0) return SKS_OK;
    if (!s->boundary_ready) return set_err(SKS_ERR_STATE, "boundary records not set");
    cudaSetDevice(s->device);
    const int L = m.mtotal + m.shtotal;
    double *G = nullptr, *D = nullptr;
    cudaError_t e = cudaMalloc((void**)&G, sizeof(double) * (size_t)(nd + 2) * L);
    if (e == cudaSuccess) e = cudaMalloc((void**)&D, sizeof(double) * (size_t)nd * nline * 3);
    if (e != cudaSuccess) {
        cudaFree(G);
        return set_err(SKS_ERR_NOMEM, "cudaMalloc for the boundary increments: %s", cudaGetErrorString(e));
    }
    // rows 1..nd+1 of G: steps it0..it0+nd (k_interp writes row r+1 for step it0+r)
    k_interp<<<nd + 1, 256, 0, s->stream>>>(G, L, it0, nd + 1, s->rs, s->rec_psv, m.mtotal, s->rec_sh, m.shtotal,
                                             s->tap_psv, s->w_psv, s->tap_sh, s->w_sh);
    const int64_t tot = (int64_t)nd * nline;
    k_line_delta<double><<<(unsigned)((tot + 255) / 256), 256, 0, s->stream>>>(D, G + L, L, nd, m.nx, m.nz, s->nbl, m.mtotal);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, D, sizeof(double) * (size_t)tot * 3, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(G);
    cudaFree(D);
    if (e != cudaSuccess) return set_err(SKS_ERR_CUDA, "boundary increments: %s", cudaGetErrorString(e));
    return SKS_OK;
}
