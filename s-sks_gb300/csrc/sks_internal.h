// Internal to the library: the solver's state and the host helpers shared by
// the single-mesh path (sks_solver.cu) and the batch path (sks_batch.cu).
#pragma once
#include "sks.h"
#include "sks_model.h"
#include "sks_kernels.cuh"

#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include <vector>

#define SKS_HIDDEN __attribute__((visibility("hidden")))

// sets the thread's error message and returns code
SKS_HIDDEN int sks_err(int code, const char* fmt, ...);
#define set_err sks_err

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return set_err(SKS_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                           __FILE__, __LINE__);                                               \
    } while (0)

struct sks_batch;

// a host set-up (sks_setup_open): the model, before any device state
struct sks_setup {
    sks_model m;
};

struct sks_solver {
    sks_model m;
    int precision, device;
    int step;                  // next step to take
    int64_t launches;
    cudaStream_t stream;
    // geometry: CTA grid of the step kernel (tunable)
    int NW, ncx, ncz, HZ, nblocks, ZS, CAP, WAVES, PIPE;
    int* pipe_ctl;             // pipelined chunks: [claim, error, done[ncx*ncz]] (grow-only)
    size_t pipe_ctl_n;
    int pipe_blocks;           // persistent CTAs of a pipelined launch
    int4* items;               // balanced band table (grow-only)
    size_t items_n;
    void* seam_lo;             // band-seam partial forces (grow-only)
    void* seam_hi;
    int* seam_cnt;
    size_t seam_bytes, seam_cnt_n;
    int sms;
    int nbl;
    // device buffers
    void* U[2];                // displacement buffers, [3][np] each
    void* Dv;                  // FP32 form: increment d
    void* Cc;                  // FP32 form: Kahan compensation
    uint16_t* mid;
    void* mat;                 // [nmat][16] in the form's type
    void* stc;                 // Stacey coefficients
    void* taper;               // boundary taper factors (atten > 0), nh_att of the form's type
    int64_t* rec_off;          // per trace (step-0 recording)
    uint32_t* recbits;         // receiver bitmap over points
    int64_t* rec_sorted;       // receiver offsets, sorted
    int32_t* rec_idx;          // trace index of each sorted offset
    int nrec_in;               // receivers inside the mesh (offset < np)
    int rec_iz0, rec_iz1;      // rows holding them (empty range when none)
    float* seis;               // [chunk][3][ntrace], the slot in use
    float* seisbuf[2];         // two slots: one filled by kernels while the other is copied out
    cudaStream_t copy_stream;
    cudaEvent_t chunk_done[2], copy_done[2];
    bool slot_busy[2];
    double* G;                 // [(chunk+2)][mtotal+shtotal]
    void* Dl;                  // [chunk+1][nline][3] line increments in the form's type
    float* rec_psv;            // boundary records (tables: files or caller memory)
    float* rec_sh;
    sks::RecSource rs;         // where the interpolation takes record values from
    double* ser;               // generator tables: the plane wave's line delays and amplitudes
    size_t ser_n;              //   [2][L], or the layered stack's mode series [3][nt]; doubles held
    int32_t* tap_psv;
    int32_t* tap_sh;
    double* w_psv;
    double* w_sh;
    int nrec_psv_loaded, nrec_sh_loaded;
    int cur;                   // index of the buffer holding u^n
    int g_last;                // row of G holding the last interpolated step
    int chunk;
    int64_t device_bytes;
    bool boundary_ready;
    // instrumentation: whole-run events, per-kernel-class event pairs
    cudaEvent_t run_ev[2];
    double last_run_ms;
    int timing;
    std::vector<cudaEvent_t> kev;     // pool of event pairs for one chunk
    std::vector<int> kcls;            // class of each recorded pair
    int kused;
    double kms[SKS_KERNEL_CLASSES];
    int64_t kcount[SKS_KERNEL_CLASSES];
    // batch membership: the batch that owns this solver's tuning, and the
    // whole-run seismograms its launches write ([nst][3][ntrace])
    sks_batch* batch;
    float* seis_full;
    // snapshots (plot_snap): SKS_NSNAP buffers of snap_size floats, and which
    // of them the run has taken
    float* snaps;
    size_t snap_size;
    int nsnap;
    bool snap_taken[SKS_NSNAP];
    // wavefield health: a device flag the step kernels set when a point's new
    // displacement is not finite (cleared by sks_reset / sks_state_load), and
    // pinned host words the end of a run copies the flags into: [0] that
    // flag, [1] the pipelined chunks' wait-ran-out flag
    int* nonfinite;
    int* hflags;
    // per element row: 1 when all its points are of isotropic materials; the
    // material all its points share, or -1
    uint8_t* row_iso;
    int16_t* row_mat;
    // failure-path tests (sks_test_stall_pipeline): for the next run, tile
    // test_stall-1 of the pipelined chunks never marks a step finished and a
    // wait gives up after test_spins polls; 0 = off
    int test_stall, test_spins;
};

namespace sksi {

using namespace sks;

struct Snapshot {
    std::vector<void*> dev;
    std::vector<size_t> bytes;
    std::vector<void*> src;
    int step, cur, g_last;
};

SKS_HIDDEN int set_grid(sks_solver* s, int NW, int HZ, int ZS, int CAP, int WAVES, int PIPE = 0);
SKS_HIDDEN int run_chunk(sks_solver* s, int it0, int n);
SKS_HIDDEN int snap_take(sks_solver* s, Snapshot& S);
SKS_HIDDEN int snap_restore(sks_solver* s, const Snapshot& S);
SKS_HIDDEN void snap_free(Snapshot& S);
SKS_HIDDEN void batch_detach(sks_solver* s);   // sks_batch.cu: leave the batch (on destroy)
// a batch run in two halves (sks_batch.cu), for the serving loop
SKS_HIDDEN int batch_launch(sks_batch* b, int32_t nsteps, float* const* su, float* const* sv, float* const* sw);
SKS_HIDDEN int batch_finish(sks_batch* b);
SKS_HIDDEN bool batch_done(const sks_batch* b);
SKS_HIDDEN bool batch_running(const sks_batch* b);
SKS_HIDDEN std::vector<sks_solver*>& batch_members(sks_batch* b);
SKS_HIDDEN int batch_set_priority(sks_batch* b, bool high);

template <typename T, int DEG = N>
Coef<T, DEG> make_coef(const sks_model& m)
{
    constexpr int NP = DEG + 1;
    Coef<T, DEG> k;
    for (int j = 0; j < NP; j++)
        for (int i = 0; i < NP; i++) {
            k.D[j * NP + i] = (T)m.dlagP[j * NP + i];
            k.DWs[j * NP + i] = (T)(m.dlagP[j * NP + i] * m.gllw[j]);
        }
    for (int i = 0; i < NP; i++) { k.w[i] = (T)m.gllw[i]; k.winv[i] = (T)(1.0 / m.gllw[i]); }
    k.winv2 = (T)(1.0 / (2.0 * m.gllw[0]));
    // even-odd tables of the two in-lane z contractions: the gradient's
    // A[a][t] = l'_t(xi_a), the divergence's A[a][t] = l'_a(xi_t) w_t
    constexpr int H = NP / 2, NN = DEG;
    for (int f = 0; f < 2; f++) {
        auto A = [&](int a, int t) { return f == 0 ? m.dlagP[a * NP + t] : m.dlagP[t * NP + a] * m.gllw[t]; };
        for (int a = 0; a < H; a++) {
            for (int t = 0; t < H; t++) {
                k.P[f][a * H + t] = (T)((A(a, t) - A(a, NN - t)) * 0.5);
                k.Q[f][a * H + t] = (T)((A(a, t) + A(a, NN - t)) * 0.5);
            }
            k.R[f][a] = (T)((NP & 1) ? A(a, H) : 0.0);
            k.Mid[f][a] = (T)((NP & 1) ? A(H, a) : 0.0);
        }
    }
    return k;
}

template <typename T>
Field<T> make_field(sks_solver* s)
{
    Field<T> F;
    memset(&F, 0, sizeof F);
    F.uc = (const T*)s->U[s->cur];
    F.un = (T*)s->U[1 - s->cur];
    F.dv = (T*)s->Dv;
    F.mid = s->mid;
    F.mat = (const T*)s->mat;
    F.stc = (const T*)s->stc;
    F.taper = (const T*)s->taper;
    F.taper_zones = s->m.nh_att > 0 ? (std::min(s->m.atten, 4) | (s->m.nh_att << 3)) : 0;
    F.recbits = s->recbits;
    F.rec_off = s->rec_sorted;
    F.rec_idx = s->rec_idx;
    F.nrec = s->nrec_in;
    F.ntrace = s->m.ntrace;
    F.rec_iz0 = s->rec_iz0;
    F.rec_iz1 = s->rec_iz1;
    F.seam_lo = (T*)s->seam_lo;
    F.seam_hi = (T*)s->seam_hi;
    F.seam_cnt = s->seam_cnt;
    F.snap = nullptr;
    F.snap_nzs = (s->m.nz + 1) / 2;
    F.nonfinite = s->nonfinite;
    F.row_iso = s->row_iso;
    F.row_mat = s->row_mat;
    return F;
}

template <typename T>
Geo<T> make_geo(const sks_solver* s)
{
    Geo<T> G;
    G.nex = s->m.nex; G.nez = s->m.nez; G.nx = s->m.nx; G.nz = s->m.nz;
    G.ncx = s->ncx; G.ncz = s->ncz; G.HZ = s->HZ; G.nblocks = s->nblocks;
    G.items = s->WAVES > 0 ? s->items : nullptr;
    G.nbl = s->nbl;
    G.np = (int64_t)s->m.nx * s->m.nz;
    G.dt2_Je = (T)(s->m.sdt * s->m.sdt / s->m.Je);
    return G;
}

}  // namespace sksi
