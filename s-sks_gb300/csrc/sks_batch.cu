// Batches: many meshes advanced together, one step of every member per launch
// of a persistent kernel, a chunk of 64 steps per launch of one captured CUDA
// graph.
//
// A member is an ordinary solver (sks_open_par / sks_open_setup) with its own
// mesh size, materials, time step, boundary records and step count.  While in
// a batch it runs with the batch's tuning (warps per CTA, band rows, band
// seams, register cap), so the tiles and the summation order are those of a
// solver with that tuning alone: a member's seismograms are bit-identical to
// the same solver run by itself with the same tuning.
//
// The device keeps every member's step (BatchState) and advances it at the end
// of each chunk, so the graph -- batched boundary interpolation, batched
// interface increments, 64 step launches, the advance -- is the same for every
// chunk and every call; joining and leaving members only rewrite the tables
// the graph reads.  Step 0 (zero the field, set the interface line, record,
// inject step 1) runs once per member through the single-mesh path before its
// first batched chunk.
#include "sks_internal.h"
#include "sks_aux_kernels.cuh"

#include <algorithm>
#include <cstdio>
#include <string>

using namespace sks;
using namespace sksi;

struct sks_batch {
    int precision = SKS_FP32C, device = 0, sms = 152;
    std::vector<sks_solver*> mem;
    cudaStream_t stream = nullptr;
    int NW = 4, HZ = 6, ZS = 0, CAP = 1;  // tuning shared by the members
    int PIPE = 0;                         // 1: a chunk is one pipelined launch (k_step_batch_pipe)
    int chunk = 64;
    bool aniso = false;                   // the step variant: any member anisotropic
    bool taper = false;                   // ... any member with the boundary taper (atten > 0)
    int deg = 0;                          // ... the members' GLL degree (the captured graph's)
    int grid = 0;                         // persistent CTAs of a step launch
    // device tables (capacity `cap` members, `items_cap` tiles)
    void* dmem = nullptr;                 // BatchMember<T>[cap]
    BatchAux* daux = nullptr;
    BatchState* dstate = nullptr;
    BatchHeader* dhdr = nullptr;
    int4* ditems = nullptr;
    int* dpipe = nullptr;                 // pipelined chunks: [claim, error, done[items_cap]]
    int cap = 0;
    size_t items_cap = 0;
    int nitems = 0;
    BatchState* hstate = nullptr;         // pinned staging of the members' steps
    int* herr = nullptr;                  // pinned: the pipelined chunks' wait-ran-out flag of the last run
    // failure-path tests (sks_batch_test_stall_pipeline): for the next run,
    // tile test_stall-1 never marks a step finished and a wait gives up after
    // test_spins polls; 0 = off
    int test_stall = 0, test_spins = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_kernels = 0;                // kernels one graph launch runs
    bool tables_dirty = true;
    bool graph_dirty = true;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    double last_ms = 0.0;
    int64_t launches = 0;
    int64_t device_bytes = 0;
    // the run in flight (batch_launch .. batch_finish)
    bool running = false;
    std::vector<int> start, target;
};

namespace {

bool member_aniso(const sks_solver* s) { return s->m.anisotropic != 0; }

// the members' GLL degree (they share one; 4 while the batch is empty)
int batch_deg(const sks_batch* b) { return b->mem.empty() ? N : b->mem[0]->m.hpn; }

// the tunings compiled for a degree: every one for 4; for 3, 5 and 6, 4 warps
// per CTA and register cap 0 or 1
bool batch_tuning_compiled(int deg, int NW, int CAP) { return deg == N || (NW == 4 && CAP <= 1); }

int nline_of(const sks_solver* s) { return (s->m.nx - s->nbl) + (s->m.nz - s->nbl - 1); }

void free_tables(sks_batch* b)
{
    void* ps[] = {b->dmem, b->daux, b->dstate, b->dhdr, b->ditems, b->dpipe};
    for (void* p : ps)
        if (p) cudaFree(p);
    if (b->hstate) cudaFreeHost(b->hstate);
    b->dmem = nullptr; b->daux = nullptr; b->dstate = nullptr; b->dhdr = nullptr; b->ditems = nullptr;
    b->dpipe = nullptr;
    b->hstate = nullptr;
    b->cap = 0;
    b->items_cap = 0;
    b->device_bytes = 0;
}

void free_graph(sks_batch* b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_dirty = true;
}

// a member's grid follows the batch's tuning (plain bands of HZ rows)
int apply_tuning(sks_batch* b, sks_solver* s)
{
    int rc = set_grid(s, b->NW, b->HZ, b->ZS, b->CAP, 0);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream));
    return SKS_OK;
}

template <typename T>
BatchMember<T> member_desc(sks_solver* s)
{
    BatchMember<T> d;
    memset(&d, 0, sizeof d);
    d.F = make_field<T>(s);
    d.G = make_geo<T>(s);
    d.G.items = nullptr;
    d.U[0] = (T*)s->U[0];
    d.U[1] = (T*)s->U[1];
    d.dl = (const T*)s->Dl;
    d.seis = s->seis_full;
    d.nt_sem = s->m.nt_sem;
    d.nline = nline_of(s);
    return d;
}

BatchAux aux_desc(sks_solver* s)
{
    BatchAux a;
    memset(&a, 0, sizeof a);
    a.G = s->G;
    a.dl = s->Dl;
    a.rs = s->rs;
    a.rec_psv = s->rec_psv;
    a.rec_sh = s->rec_sh;
    a.tap_psv = s->tap_psv;
    a.tap_sh = s->tap_sh;
    a.w_psv = s->w_psv;
    a.w_sh = s->w_sh;
    a.mtotal = s->m.mtotal;
    a.shtotal = s->m.shtotal;
    a.nt_sem = s->m.nt_sem;
    a.nx = s->m.nx;
    a.nz = s->m.nz;
    a.nbl = s->nbl;
    a.L = s->m.mtotal + s->m.shtotal;
    a.nline = nline_of(s);
    return a;
}

// Rebuild and upload the member descriptors and the tile table; the tables
// grow (and the graph is captured again) when they are too small.
template <typename T>
int build_tables(sks_batch* b)
{
    const int n = (int)b->mem.size();
    std::vector<BatchMember<T>> md;
    std::vector<BatchAux> ad;
    std::vector<int4> items;
    bool aniso = false, taper = false;
    for (int i = 0; i < n; i++) {
        sks_solver* s = b->mem[i];
        aniso = aniso || member_aniso(s);
        taper = taper || s->m.nh_att > 0;
        md.push_back(member_desc<T>(s));
        md.back().item0 = (int)items.size();
        ad.push_back(aux_desc(s));
        if (s->ncx >= (1 << 16) || s->ncz >= (1 << 15))
            return set_err(SKS_ERR_UNSUPPORTED, "member %d: %d x %d tiles exceed the batch's tile index", i, s->ncx, s->ncz);
        for (int cz = 0; cz < s->ncz; cz++)
            for (int cx = 0; cx < s->ncx; cx++)
                items.push_back(make_int4(i, cx | (cz << 16), cz * s->HZ, std::min((cz + 1) * s->HZ, s->m.nez)));
    }
    const int deg = batch_deg(b);
    if (aniso != b->aniso || taper != b->taper || deg != b->deg) {
        b->aniso = aniso;
        b->taper = taper;
        b->deg = deg;
        b->graph_dirty = true;
    }
    if (n > b->cap) {
        const int cap = std::max(n, std::max(8, 2 * b->cap));
        void* ps[] = {b->dmem, b->daux, b->dstate};
        for (void* p : ps)
            if (p) cudaFree(p);
        if (b->hstate) cudaFreeHost(b->hstate);
        b->dmem = nullptr; b->daux = nullptr; b->dstate = nullptr; b->hstate = nullptr;
        b->cap = 0;
        CK(cudaMalloc(&b->dmem, sizeof(BatchMember<T>) * cap));
        CK(cudaMalloc((void**)&b->daux, sizeof(BatchAux) * cap));
        CK(cudaMalloc((void**)&b->dstate, sizeof(BatchState) * cap));
        CK(cudaMallocHost((void**)&b->hstate, sizeof(BatchState) * cap));
        CK(cudaMemset(b->dstate, 0, sizeof(BatchState) * cap));
        b->cap = cap;
        b->graph_dirty = true;
    }
    if (!b->dhdr) {
        CK(cudaMalloc((void**)&b->dhdr, sizeof(BatchHeader)));
        b->graph_dirty = true;
    }
    if (items.size() > b->items_cap) {
        const size_t ic = std::max(items.size(), 2 * b->items_cap);
        if (b->ditems) cudaFree(b->ditems);
        if (b->dpipe) cudaFree(b->dpipe);
        b->ditems = nullptr;
        b->dpipe = nullptr;
        b->items_cap = 0;
        CK(cudaMalloc((void**)&b->ditems, sizeof(int4) * ic));
        CK(cudaMalloc((void**)&b->dpipe, sizeof(int) * (2 + ic)));
        b->items_cap = ic;
        b->graph_dirty = true;
    }
    b->device_bytes = (int64_t)(sizeof(BatchMember<T>) + sizeof(BatchAux) + sizeof(BatchState)) * b->cap +
                      (int64_t)(sizeof(int4) + sizeof(int)) * (int64_t)b->items_cap + 8 + (int64_t)sizeof(BatchHeader);
    if (n) {
        CK(cudaMemcpyAsync(b->dmem, md.data(), sizeof(BatchMember<T>) * n, cudaMemcpyHostToDevice, b->stream));
        CK(cudaMemcpyAsync(b->daux, ad.data(), sizeof(BatchAux) * n, cudaMemcpyHostToDevice, b->stream));
    }
    if (!items.empty())
        CK(cudaMemcpyAsync(b->ditems, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, b->stream));
    BatchHeader h = {(int)items.size(), n, b->chunk, 0};
    CK(cudaMemcpyAsync(b->dhdr, &h, sizeof h, cudaMemcpyHostToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    b->nitems = (int)items.size();
    b->tables_dirty = false;
    return SKS_OK;
}

// The compiled batch kernels of one GLL degree D (3..6) and form T
template <typename T, int D>
struct DegBatch {
    static constexpr bool F32 = sizeof(T) == 4;
    using M = BatchMember<T>;
    static int occ(const StepVariant& v, bool a, bool pipe)
    {
        if constexpr (D == 3) {
            if (pipe) return F32 ? batch_pipe_occupancy_f32_d3(v, a) : batch_pipe_occupancy_f64_d3(v, a);
            return F32 ? batch_occupancy_f32_d3(v, a) : batch_occupancy_f64_d3(v, a);
        } else if constexpr (D == 5) {
            if (pipe) return F32 ? batch_pipe_occupancy_f32_d5(v, a) : batch_pipe_occupancy_f64_d5(v, a);
            return F32 ? batch_occupancy_f32_d5(v, a) : batch_occupancy_f64_d5(v, a);
        } else if constexpr (D == 6) {
            if (pipe) return F32 ? batch_pipe_occupancy_f32_d6(v, a) : batch_pipe_occupancy_f64_d6(v, a);
            return F32 ? batch_occupancy_f32_d6(v, a) : batch_occupancy_f64_d6(v, a);
        } else {
            if (pipe) return F32 ? batch_pipe_occupancy_f32(v, a) : batch_pipe_occupancy_f64(v, a);
            return F32 ? batch_occupancy_f32(v, a) : batch_occupancy_f64(v, a);
        }
    }
    static cudaError_t step(const StepVariant& v, bool a, int grid, cudaStream_t st, const M* mem,
                            const BatchState* state, const int4* items, const BatchHeader* hdr, int j,
                            const Coef<T, D>& k)
    {
        if constexpr (F32) {
            if constexpr (D == 3) return launch_batch_f32_d3(v, a, grid, st, mem, state, items, hdr, j, k);
            else if constexpr (D == 5) return launch_batch_f32_d5(v, a, grid, st, mem, state, items, hdr, j, k);
            else if constexpr (D == 6) return launch_batch_f32_d6(v, a, grid, st, mem, state, items, hdr, j, k);
            else return launch_batch_f32(v, a, grid, st, mem, state, items, hdr, j, k);
        } else {
            if constexpr (D == 3) return launch_batch_f64_d3(v, a, grid, st, mem, state, items, hdr, j, k);
            else if constexpr (D == 5) return launch_batch_f64_d5(v, a, grid, st, mem, state, items, hdr, j, k);
            else if constexpr (D == 6) return launch_batch_f64_d6(v, a, grid, st, mem, state, items, hdr, j, k);
            else return launch_batch_f64(v, a, grid, st, mem, state, items, hdr, j, k);
        }
    }
    static cudaError_t pipe(const StepVariant& v, bool a, int grid, cudaStream_t st, const M* mem,
                            const BatchState* state, const int4* items, const BatchHeader* hdr, int nsteps,
                            const BatchPipeCtl& ctl, const Coef<T, D>& k)
    {
        if constexpr (F32) {
            if constexpr (D == 3) return launch_batch_pipe_f32_d3(v, a, grid, st, mem, state, items, hdr, nsteps, ctl, k);
            else if constexpr (D == 5) return launch_batch_pipe_f32_d5(v, a, grid, st, mem, state, items, hdr, nsteps, ctl, k);
            else if constexpr (D == 6) return launch_batch_pipe_f32_d6(v, a, grid, st, mem, state, items, hdr, nsteps, ctl, k);
            else return launch_batch_pipe_f32(v, a, grid, st, mem, state, items, hdr, nsteps, ctl, k);
        } else {
            if constexpr (D == 3) return launch_batch_pipe_f64_d3(v, a, grid, st, mem, state, items, hdr, nsteps, ctl, k);
            else if constexpr (D == 5) return launch_batch_pipe_f64_d5(v, a, grid, st, mem, state, items, hdr, nsteps, ctl, k);
            else if constexpr (D == 6) return launch_batch_pipe_f64_d6(v, a, grid, st, mem, state, items, hdr, nsteps, ctl, k);
            else return launch_batch_pipe_f64(v, a, grid, st, mem, state, items, hdr, nsteps, ctl, k);
        }
    }
};

// calls f.template run<D>() for the batch's degree D (3..6)
template <typename Fn>
auto with_batch_degree(int deg, Fn& f)
{
    switch (deg) {
    case 3: return f.template run<3>();
    case 5: return f.template run<5>();
    case 6: return f.template run<6>();
    default: return f.template run<4>();
    }
}

// one step launch of every member (j = the launch within the chunk), or, with
// nsteps > 0, one pipelined chunk of nsteps steps
template <typename T>
struct BatchLaunch {
    sks_batch* b;
    int j, nsteps;
    const BatchPipeCtl* ctl;
    template <int D>
    cudaError_t run()
    {
        const StepVariant v{b->NW, b->ZS, b->CAP, b->taper};
        static thread_local Coef<T, D> k;
        k = make_coef<T, D>(b->mem[0]->m);     // GLL tables: the same for every member
        const BatchMember<T>* mem = (const BatchMember<T>*)b->dmem;
        if (ctl)
            return DegBatch<T, D>::pipe(v, b->aniso, b->grid, b->stream, mem, b->dstate, b->ditems, b->dhdr, nsteps,
                                        *ctl, k);
        return DegBatch<T, D>::step(v, b->aniso, b->grid, b->stream, mem, b->dstate, b->ditems, b->dhdr, j, k);
    }
};

template <typename T>
cudaError_t launch_steps(sks_batch* b, int j)
{
    BatchLaunch<T> l{b, j, 0, nullptr};
    return with_batch_degree(batch_deg(b), l);
}

// a pipelined chunk of nsteps steps: the counters back to zero, then one launch
template <typename T>
cudaError_t launch_pipe_chunk(sks_batch* b, int nsteps)
{
    // the claim counter and the done counters; the error flag stays set for
    // the rest of a run once a wait ran out (batch_launch clears it)
    cudaError_t e = cudaMemsetAsync(b->dpipe, 0, sizeof(int), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->dpipe + 2, 0, sizeof(int) * b->items_cap, b->stream);
    if (e != cudaSuccess) return e;
    const BatchPipeCtl ctl{b->dpipe, b->dpipe + 1, b->dpipe + 2, b->test_stall ? b->test_spins : PIPE_SPIN_LIMIT,
                           b->test_stall - 1};
    BatchLaunch<T> l{b, 0, nsteps, &ctl};
    return with_batch_degree(batch_deg(b), l);
}

struct BatchOcc {
    const sks_batch* b;
    template <int D>
    int run()
    {
        const StepVariant v{b->NW, b->ZS, b->CAP, b->taper};
        return b->precision == SKS_FP64 ? DegBatch<double, D>::occ(v, b->aniso, b->PIPE != 0)
                                        : DegBatch<float, D>::occ(v, b->aniso, b->PIPE != 0);
    }
};

// persistent grid: every SM full of resident CTAs of the step variant
void set_persistent_grid(sks_batch* b)
{
    BatchOcc o{b};
    b->grid = b->sms * with_batch_degree(batch_deg(b), o);
}

template <typename T>
int capture_graph(sks_batch* b)
{
    free_graph(b);
    set_persistent_grid(b);
    cudaStream_t st = b->stream;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    k_interp_batch<<<dim3(b->chunk + 1, b->cap), 256, 0, st>>>(b->daux, b->dstate, b->dhdr);
    k_line_delta_batch<T><<<dim3(32, b->cap), 256, 0, st>>>(b->daux, b->dstate, b->dhdr);
    cudaError_t e = cudaSuccess;
    if (b->PIPE)
        e = launch_pipe_chunk<T>(b, b->chunk);
    else
        for (int j = 0; j < b->chunk && e == cudaSuccess; j++) e = launch_steps<T>(b, j);
    k_batch_advance<<<1, 256, 0, st>>>(b->dstate, b->dhdr);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(st, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return set_err(SKS_ERR_CUDA, "capture of the batch graph: %s",
                       cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    b->graph = g;
    CK(cudaGraphInstantiate(&b->exec, g, 0));
    b->graph_kernels = (b->PIPE ? 1 : b->chunk) + 3;
    b->graph_dirty = false;
    return SKS_OK;
}

int prepare(sks_batch* b)
{
    int rc = SKS_OK;
    if (b->tables_dirty)
        rc = b->precision == SKS_FP64 ? build_tables<double>(b) : build_tables<float>(b);
    if (!rc && b->graph_dirty)
        rc = b->precision == SKS_FP64 ? capture_graph<double>(b) : capture_graph<float>(b);
    return rc;
}

// step 0 of a member through the single-mesh path, its seismogram row into
// the member's whole-run buffer
int first_step(sks_solver* s)
{
    s->seis = s->seis_full;
    int rc = run_chunk(s, 0, 1);
    s->seis = s->seisbuf[0];
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream));
    s->step = 1;
    return SKS_OK;
}

int check_member(const sks_batch* b, const sks_solver* s, int i)
{
    if (s->step < s->m.nt_sem && !s->boundary_ready)
        return set_err(SKS_ERR_STATE, "member %d: boundary records not set", i);
    (void)b;
    return SKS_OK;
}

}  // namespace

namespace sksi {

void batch_detach(sks_solver* s)
{
    sks_batch* b = s->batch;
    if (!b) return;
    if (b->running) batch_finish(b);
    cudaStreamSynchronize(b->stream);
    b->mem.erase(std::remove(b->mem.begin(), b->mem.end(), s), b->mem.end());
    b->tables_dirty = true;
    s->batch = nullptr;
}

}  // namespace sksi

extern "C" int sks_batch_create(int precision, int device, sks_batch** out)
{
    if (!out) return set_err(SKS_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (precision != SKS_FP64 && precision != SKS_FP32C) return set_err(SKS_ERR_ARG, "unknown precision %d", precision);
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return set_err(SKS_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
    sks_batch* b = new (std::nothrow) sks_batch();
    if (!b) return set_err(SKS_ERR_NOMEM, "cannot allocate the batch");
    b->precision = precision;
    b->device = device;
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device);
    if (precision == SKS_FP64) { b->NW = 4; b->HZ = 8; b->ZS = 1; b->CAP = 0; }
    e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev[1]);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->herr, sizeof(int));
    if (e == cudaSuccess) *b->herr = 0;
    if (e != cudaSuccess) {
        if (b->stream) cudaStreamDestroy(b->stream);
        if (b->herr) cudaFreeHost(b->herr);
        delete b;
        return set_err(SKS_ERR_CUDA, "batch stream/events: %s", cudaGetErrorString(e));
    }
    *out = b;
    return SKS_OK;
}

extern "C" int sks_batch_add(sks_batch* b, sks_solver* s)
{
    if (!b || !s) return set_err(SKS_ERR_ARG, "NULL argument");
    if (s->batch) return set_err(SKS_ERR_STATE, "the solver is already a member of a batch");
    if (b->running) return set_err(SKS_ERR_STATE, "the batch is running");
    if (s->precision != b->precision) return set_err(SKS_ERR_ARG, "the solver's form differs from the batch's");
    if (s->device != b->device) return set_err(SKS_ERR_ARG, "the solver is on device %d, the batch on %d", s->device, b->device);
    if (s->snaps) return set_err(SKS_ERR_UNSUPPORTED, "snapshots (plot_snap=1) are taken by sks_run, not in batches");
    if (s->m.hpn < 3 || s->m.hpn > 6) return set_err(SKS_ERR_UNSUPPORTED, "hpn=%d: batches run GLL degrees 3 to 6", s->m.hpn);
    if (!b->mem.empty() && s->m.hpn != batch_deg(b))
        return set_err(SKS_ERR_ARG, "hpn=%d: the batch's members are of GLL degree %d", s->m.hpn, batch_deg(b));
    if (!batch_tuning_compiled(s->m.hpn, b->NW, b->CAP))
        return set_err(SKS_ERR_UNSUPPORTED, "GLL degree %d needs a batch tuning of 4 warps and register cap 0 or 1", s->m.hpn);
    cudaSetDevice(b->device);
    const sks_model& m = s->m;
    if (!s->seis_full) {
        const size_t n = (size_t)std::max(1, m.nst) * 3 * std::max(1, m.ntrace);
        cudaError_t e = cudaMalloc((void**)&s->seis_full, n * sizeof(float));
        if (e != cudaSuccess) {
            s->seis_full = nullptr;
            return set_err(SKS_ERR_NOMEM, "whole-run seismograms (%zu bytes): %s", n * sizeof(float), cudaGetErrorString(e));
        }
        s->device_bytes += (int64_t)(n * sizeof(float));
        CK(cudaMemsetAsync(s->seis_full, 0, n * sizeof(float), s->stream));
    }
    int rc = apply_tuning(b, s);
    if (rc) return rc;
    s->batch = b;
    b->mem.push_back(s);
    b->tables_dirty = true;
    return SKS_OK;
}

extern "C" int sks_batch_remove(sks_batch* b, sks_solver* s)
{
    if (!b || !s) return set_err(SKS_ERR_ARG, "NULL argument");
    if (s->batch != b) return set_err(SKS_ERR_STATE, "the solver is not a member of this batch");
    batch_detach(s);
    return SKS_OK;
}

extern "C" int sks_batch_size(const sks_batch* b) { return b ? (int)b->mem.size() : -1; }

namespace sksi {

// First half of a batch run: step 0 of new members, then every member's
// chunks and (for non-NULL arrays) the copies of its new seismogram rows, all
// enqueued on the batch's stream.  Copies to pageable host memory make the
// call wait for the stream; the serving loop passes no arrays.
int batch_launch(sks_batch* b, int32_t nsteps, float* const* su, float* const* sv, float* const* sw)
{
    if (!b) return set_err(SKS_ERR_ARG, "batch is NULL");
    if (nsteps < 0) return set_err(SKS_ERR_ARG, "nsteps=%d", nsteps);
    if (b->running) return set_err(SKS_ERR_STATE, "the batch's previous run has not finished");
    cudaSetDevice(b->device);
    const int n = (int)b->mem.size();
    b->start.assign(n, 0);
    b->target.assign(n, 0);
    if (n == 0) return SKS_OK;
    int rc = SKS_OK;
    for (int i = 0; i < n; i++) {
        sks_solver* s = b->mem[i];
        if ((rc = check_member(b, s, i))) return rc;
        b->start[i] = s->step;
        b->target[i] = std::min(s->m.nst, s->step + nsteps);
    }
    CK(cudaEventRecord(b->ev[0], b->stream));
    for (int i = 0; i < n; i++) {
        sks_solver* s = b->mem[i];
        if (s->step == 0 && b->target[i] > 0 && (rc = first_step(s))) return rc;
    }
    if ((rc = prepare(b))) return rc;
    int most = 0;
    for (int i = 0; i < n; i++) {
        sks_solver* s = b->mem[i];
        const int left = std::max(0, b->target[i] - s->step);
        b->hstate[i] = BatchState{s->step, std::min(b->chunk, left), b->target[i], 0};
        most = std::max(most, left);
    }
    CK(cudaMemcpyAsync(b->dstate, b->hstate, sizeof(BatchState) * n, cudaMemcpyHostToDevice, b->stream));
    if (b->PIPE) CK(cudaMemsetAsync(b->dpipe + 1, 0, sizeof(int), b->stream));
    const int nchunks = (most + b->chunk - 1) / b->chunk;
    for (int c = 0; c < nchunks; c++) {
        CK(cudaGraphLaunch(b->exec, b->stream));
        b->launches += b->graph_kernels;
    }
    CK(cudaEventRecord(b->ev[1], b->stream));
    // the run's flags: the pipelined chunks' and every member's wavefield flag
    *b->herr = 0;
    if (b->PIPE) CK(cudaMemcpyAsync(b->herr, b->dpipe + 1, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    for (int i = 0; i < n; i++) {
        sks_solver* s = b->mem[i];
        s->hflags[0] = 0;
        CK(cudaMemcpyAsync(s->hflags, s->nonfinite, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    }
    b->running = true;
    // the new seismogram rows of each member into the caller's arrays
    for (int i = 0; i < n; i++) {
        sks_solver* s = b->mem[i];
        const int nt = s->m.ntrace, rows = b->target[i] - b->start[i];
        if (nt <= 0 || rows <= 0) continue;
        float* dst[3] = {su ? su[i] : nullptr, sv ? sv[i] : nullptr, sw ? sw[i] : nullptr};
        const size_t w = sizeof(float) * (size_t)nt;
        for (int c = 0; c < 3; c++)
            if (dst[c])
                CK(cudaMemcpy2DAsync(dst[c], w, s->seis_full + (size_t)b->start[i] * 3 * nt + (size_t)c * nt, 3 * w, w,
                                     (size_t)rows, cudaMemcpyDeviceToHost, b->stream));
    }
    return SKS_OK;
}

bool batch_done(const sks_batch* b)
{
    return !b->running || cudaEventQuery(b->ev[1]) != cudaErrorNotReady;
}

bool batch_running(const sks_batch* b) { return b->running; }

// Second half: wait for the stream, then move every member's step on.
// Returns the most steps any member took.
int batch_finish(sks_batch* b)
{
    if (!b->running) return 0;
    cudaSetDevice(b->device);
    b->running = false;
    CK(cudaStreamSynchronize(b->stream));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
    b->last_ms = ms;
    const int err = b->PIPE ? *b->herr : 0;
    if (b->test_stall) {
        b->test_stall = 0;
        b->graph_dirty = true;
    }
    int adv = 0, bad = -1;
    for (size_t i = 0; i < b->mem.size() && i < b->target.size(); i++) {
        sks_solver* s = b->mem[i];
        if (b->target[i] > s->step) {
            s->step = b->target[i];
            s->cur = (b->target[i] - 1) & 1;
            s->g_last = 0;
        }
        adv = std::max(adv, b->target[i] - b->start[i]);
        if (bad < 0 && s->hflags[0]) bad = (int)i;
    }
    if (err) return set_err(SKS_ERR_CUDA, "pipelined batch chunk: a wait for neighbouring tiles ran out");
    if (bad >= 0)
        return set_err(SKS_ERR_NONFINITE, "member %d: the wavefield holds a non-finite displacement (sks_wavefield_finite "
                       "names every such member)", bad);
    return adv;
}

std::vector<sks_solver*>& batch_members(sks_batch* b) { return b->mem; }

// the batch's stream at the device's highest (high = true) or lowest stream
// priority: where two batches share the GPU, the scheduler starts the
// high-priority batch's CTAs first.  Only between runs.
int batch_set_priority(sks_batch* b, bool high)
{
    if (b->running) return set_err(SKS_ERR_STATE, "the batch is running");
    cudaSetDevice(b->device);
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    cudaStream_t st = nullptr;
    CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, high ? greatest : least));
    CK(cudaStreamSynchronize(b->stream));
    cudaStreamDestroy(b->stream);
    b->stream = st;
    return SKS_OK;
}

}  // namespace sksi

extern "C" int sks_batch_run(sks_batch* b, int32_t nsteps, float* const* su, float* const* sv, float* const* sw)
{
    int rc = batch_launch(b, nsteps, su, sv, sw);
    if (rc) {
        if (b && b->running) { cudaStreamSynchronize(b->stream); b->running = false; }
        return rc;
    }
    return batch_finish(b);
}

extern "C" int sks_batch_set_tuning(sks_batch* b, const sks_tuning_t* t)
{
    if (!b || !t) return set_err(SKS_ERR_ARG, "NULL argument");
    if (t->warps_per_block != 2 && t->warps_per_block != 4)
        return set_err(SKS_ERR_ARG, "warps_per_block=%d: 2 or 4", t->warps_per_block);
    if (t->register_cap < 0 || t->register_cap > 2) return set_err(SKS_ERR_ARG, "register_cap=%d: 0, 1 or 2", t->register_cap);
    if (t->band_rows < 1) return set_err(SKS_ERR_ARG, "band_rows=%d must be positive", t->band_rows);
    if (t->waves != 0) return set_err(SKS_ERR_ARG, "a batch uses plain bands (waves=0)");
    if (t->pipeline != 0 && t->pipeline != 1) return set_err(SKS_ERR_ARG, "pipeline=%d: 0 or 1", t->pipeline);
    if (!batch_tuning_compiled(batch_deg(b), t->warps_per_block, t->register_cap))
        return set_err(SKS_ERR_UNSUPPORTED, "GLL degree %d runs with 4 warps per CTA and register cap 0 or 1", batch_deg(b));
    if (b->running) return set_err(SKS_ERR_STATE, "the batch is running");
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    const int old[5] = {b->NW, b->HZ, b->ZS, b->CAP, b->PIPE};
    b->NW = t->warps_per_block;
    b->HZ = t->band_rows;
    b->ZS = t->zseam ? 1 : 0;
    b->CAP = t->register_cap;
    b->PIPE = t->pipeline;
    for (sks_solver* s : b->mem) {
        int rc = apply_tuning(b, s);
        if (rc) {
            // a member's grid could not follow (e.g. no memory for its seam
            // buffers): every member goes back to the previous tuning, so the
            // batch never runs with members on different grids
            const std::string msg = sks_last_error();
            b->NW = old[0]; b->HZ = old[1]; b->ZS = old[2]; b->CAP = old[3]; b->PIPE = old[4];
            for (sks_solver* r : b->mem) apply_tuning(b, r);
            set_persistent_grid(b);
            b->tables_dirty = true;
            b->graph_dirty = true;
            return set_err(rc, "%s", msg.c_str());
        }
    }
    set_persistent_grid(b);
    b->tables_dirty = true;
    b->graph_dirty = true;
    return SKS_OK;
}

extern "C" int sks_batch_get_tuning(const sks_batch* b, sks_tuning_t* t)
{
    if (!b || !t) return set_err(SKS_ERR_ARG, "NULL argument");
    t->warps_per_block = b->NW;
    t->band_rows = b->HZ;
    t->zseam = b->ZS;
    t->register_cap = b->CAP;
    t->waves = 0;
    t->blocks = b->grid;
    t->ms_per_step = 0.f;
    t->pipeline = b->PIPE;
    return SKS_OK;
}

// Time candidate tunings on the members' own next steps (state restored): each
// candidate runs `steps` batched step launches once untimed and once timed.
extern "C" int sks_batch_autotune(sks_batch* b, int32_t steps, sks_tuning_t* best)
{
    if (!b) return set_err(SKS_ERR_ARG, "batch is NULL");
    if (steps < 1) steps = 4;
    const int n = (int)b->mem.size();
    if (n == 0) return set_err(SKS_ERR_STATE, "the batch is empty");
    if (b->running) return set_err(SKS_ERR_STATE, "the batch is running");
    cudaSetDevice(b->device);
    for (int i = 0; i < n; i++) {
        sks_solver* s = b->mem[i];
        int rc = check_member(b, s, i);
        if (rc) return rc;
        if (s->step + 1 + steps > s->m.nst)
            return set_err(SKS_ERR_STATE, "member %d: autotune needs %d more steps than its run has left", i, steps + 1);
    }
    std::vector<Snapshot> snaps(n);
    int rc = SKS_OK;
    for (int i = 0; i < n && !rc; i++) rc = snap_take(b->mem[i], snaps[i]);
    for (int i = 0; i < n && !rc; i++) rc = cudaStreamSynchronize(b->mem[i]->stream) == cudaSuccess ? SKS_OK : SKS_ERR_CUDA;
    for (int i = 0; i < n && !rc; i++)
        if (b->mem[i]->step == 0) rc = first_step(b->mem[i]);
    const sks_tuning_t old = {b->NW, b->HZ, b->ZS, b->CAP, 0, b->grid, 0.f, b->PIPE};
    sks_tuning_t bt = old;
    bt.ms_per_step = 1e30f;
    const int hzs[] = {3, 4, 6, 8, 12};
    for (int pipe = 0; pipe < 2 && !rc; pipe++)
    for (int nw = 2; nw <= 4 && !rc; nw += 2)
        for (int zs = 0; zs < 2 && !rc; zs++)
            for (int cap = 0; cap < 3 && !rc; cap++)
                for (int hz : hzs) {
                    if (!batch_tuning_compiled(batch_deg(b), nw, cap)) continue;
                    sks_tuning_t t = {nw, hz, zs, cap, 0, 0, 0.f, pipe};
                    if ((rc = sks_batch_set_tuning(b, &t))) break;
                    rc = b->precision == SKS_FP64 ? build_tables<double>(b) : build_tables<float>(b);
                    if (rc) break;
                    set_persistent_grid(b);
                    for (int i = 0; i < n; i++) {
                        sks_solver* s = b->mem[i];
                        b->hstate[i] = BatchState{s->step, steps, s->step + steps, 0};
                    }
                    cudaMemcpyAsync(b->dstate, b->hstate, sizeof(BatchState) * n, cudaMemcpyHostToDevice, b->stream);
                    // the chunk's boundary increments, so every launch reads defined values
                    k_interp_batch<<<dim3(b->chunk + 1, n), 256, 0, b->stream>>>(b->daux, b->dstate, b->dhdr);
                    if (b->precision == SKS_FP64)
                        k_line_delta_batch<double><<<dim3(32, n), 256, 0, b->stream>>>(b->daux, b->dstate, b->dhdr);
                    else
                        k_line_delta_batch<float><<<dim3(32, n), 256, 0, b->stream>>>(b->daux, b->dstate, b->dhdr);
                    cudaError_t e = cudaSuccess;
                    for (int pass = 0; pass < 2 && e == cudaSuccess; pass++) {
                        if (pass) cudaEventRecord(b->ev[0], b->stream);
                        if (pipe)
                            e = b->precision == SKS_FP64 ? launch_pipe_chunk<double>(b, steps)
                                                         : launch_pipe_chunk<float>(b, steps);
                        else
                            for (int j = 0; j < steps && e == cudaSuccess; j++)
                                e = b->precision == SKS_FP64 ? launch_steps<double>(b, j) : launch_steps<float>(b, j);
                    }
                    cudaEventRecord(b->ev[1], b->stream);
                    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
                    if (e != cudaSuccess) { rc = set_err(SKS_ERR_CUDA, "batch autotune: %s", cudaGetErrorString(e)); break; }
                    if (pipe) {
                        int err = 0;
                        CK(cudaMemcpy(&err, b->dpipe + 1, sizeof(int), cudaMemcpyDeviceToHost));
                        if (err) { rc = set_err(SKS_ERR_CUDA, "batch autotune: a pipelined wait ran out"); break; }
                    }
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
                    b->launches += 2 + 2 * (pipe ? 1 : steps);
                    ms /= (float)steps;
                    if (ms < bt.ms_per_step) bt = {nw, hz, zs, cap, 0, b->grid, ms, pipe};
                }
    for (int i = 0; i < n; i++) {
        const int r2 = snap_restore(b->mem[i], snaps[i]);
        cudaStreamSynchronize(b->mem[i]->stream);
        snap_free(snaps[i]);
        if (!rc) rc = r2;
    }
    const sks_tuning_t use = rc ? old : bt;
    const int r3 = sks_batch_set_tuning(b, &use);
    if (rc) return rc;
    if (r3) return r3;
    if (best) *best = bt;
    return SKS_OK;
}

extern "C" double sks_batch_last_run_ms(const sks_batch* b) { return b ? b->last_ms : -1.0; }

extern "C" int64_t sks_batch_kernel_launches(const sks_batch* b) { return b ? b->launches : -1; }

extern "C" void sks_batch_destroy(sks_batch* b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->running) batch_finish(b);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (sks_solver* s : b->mem) s->batch = nullptr;
    b->mem.clear();
    free_graph(b);
    free_tables(b);
    if (b->ev[0]) cudaEventDestroy(b->ev[0]);
    if (b->ev[1]) cudaEventDestroy(b->ev[1]);
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->herr) cudaFreeHost(b->herr);
    delete b;
}

extern "C" int sks_batch_test_stall_pipeline(sks_batch* b, int32_t tile, int32_t spin_limit)
{
    if (!b) return set_err(SKS_ERR_ARG, "batch is NULL");
    if (b->running) return set_err(SKS_ERR_STATE, "the batch is running");
    if (!b->PIPE) return set_err(SKS_ERR_STATE, "the batch does not run pipelined chunks (tuning pipeline=0)");
    if (spin_limit < 1 || spin_limit > PIPE_SPIN_LIMIT) return set_err(SKS_ERR_ARG, "spin_limit=%d: 1..%d", spin_limit, PIPE_SPIN_LIMIT);
    if (b->tables_dirty) {
        const int rc = b->precision == SKS_FP64 ? build_tables<double>(b) : build_tables<float>(b);
        if (rc) return rc;
    }
    if (tile < 0 || tile >= b->nitems) return set_err(SKS_ERR_ARG, "tile %d: 0..%d", tile, b->nitems - 1);
    b->test_stall = tile + 1;
    b->test_spins = spin_limit;
    b->graph_dirty = true;
    return SKS_OK;
}
