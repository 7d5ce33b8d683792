// The serving loop: solve requests arrive at any time and are admitted by
// their device-memory footprint; admitted requests join the batch of their
// form (FP32C or FP64), keep their wavefields on the device and advance one
// quantum of steps per scheduling round together with every other admitted
// request of that form (continuous batching: requests join and leave between
// quanta, never waiting for a batch to drain).  The two forms' batches run on
// their own streams and overlap on the device.  A finished request's whole
// seismogram is copied once into the caller's arrays and its device memory
// is released.
//
// The reference has no serving path: one solve is one process
// (sem2d_psvsh.c:82), started per event by the driver scripts
// (applications/test/prem_epi83.pl:81-82).  A request here is that process's
// par words (as an sks_setup) plus its boundary records.
#include "sks_internal.h"

#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

using namespace sks;
using namespace sksi;

namespace {

struct Request {
    int64_t id = 0;
    sks_setup* su = nullptr;           // owned until admission
    int precision = SKS_FP32C;
    bool has_pw = false;
    sks_plane_wave_t pw{};
    std::vector<sks_stack_layer_t> stack;  // non-empty: records from the layered stack
    sks_layered_wave_t lw{};
    float* out[3] = {nullptr, nullptr, nullptr};
    // the serving thread owns the solver; what other threads read (state,
    // status, step, bytes, times) is written under the server's mutex
    sks_solver* s = nullptr;           // while running
    int64_t est_bytes = 0, bytes = 0;
    double t_submit = -1, t_admit = -1, t_done = -1;
    int state = SKS_REQ_QUEUED;
    int status = SKS_OK;
    int step = 0;                      // steps done, as of the last finished quantum
    int nst = 0, ntrace = 0;
    int64_t points = 0;                // grid points of the mesh
};

// device bytes a request will hold, from its model (an upper bound of what
// the solver, its boundary records and its whole-run seismograms allocate);
// rec_bytes: the record tables, or a generator's own (none for the plane
// wave, the mode series for a layered stack)
int64_t estimate_bytes(const sks_model& m, int precision, int64_t rec_bytes)
{
    const int64_t np = (int64_t)m.nx * m.nz;
    const int64_t el = precision == SKS_FP64 ? 8 : 4;
    const int64_t L = (int64_t)m.mtotal + m.shtotal;
    const int64_t nline = (int64_t)m.nx + m.nz;
    const int64_t nb = (int64_t)2 * m.nz + m.nx + 3 * m.hpn + 1;
    int64_t b = 0;
    b += 2 * 3 * np * el;                                   // two displacement buffers
    if (precision == SKS_FP32C) b += 6 * np * 4;            // (d, c) pairs
    b += 2 * np + np / 8 + 64;                              // material index, receiver bitmap
    b += nb * 9 * el + (int64_t)m.nmat * 16 * el;           // Stacey coefficients, material table
    b += rec_bytes;                                                              // boundary records
    b += (int64_t)std::max(1, m.nst) * 3 * std::max(1, m.ntrace) * 4;          // whole-run seismograms
    b += (int64_t)2 * 64 * 3 * std::max(1, m.ntrace) * 4;                        // chunk seismograms
    b += (int64_t)66 * L * 8 + (int64_t)65 * nline * 3 * el;                     // interpolation rows, increments
    b += (int64_t)m.nt_sem * 48 * 2;                                             // schedule
    b += (int64_t)m.ntrace * 20;                                                 // receiver tables
    b += 2 * ((int64_t)m.nez + 1) * m.nx * 6 * el + (int64_t)(m.nez + 1) * (m.nex + 1) * 4;  // band seams
    return b + b / 50 + ((int64_t)1 << 20);
}

// boundary files named relative to the submitter's working directory, made
// absolute at submission (they are read at admission, on the serving thread)
int absolute_path(char* path, size_t cap)
{
    if (!path[0] || path[0] == '/') return SKS_OK;
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return set_err(SKS_ERR_IO, "getcwd failed");
    char buf[4096 + 512 + 2];
    const int n = snprintf(buf, sizeof buf, "%s/%s", cwd, path);
    if (n < 0 || (size_t)n >= cap) return set_err(SKS_ERR_IO, "boundary file path too long: %s/%s", cwd, path);
    memcpy(path, buf, (size_t)n + 1);
    return SKS_OK;
}

}  // namespace

struct sks_server {
    int device = 0;
    int64_t budget = 0;
    int64_t in_use = 0;
    int quantum = 64;
    // active grid points per form (index = precision): a cap of about twice
    // what fills the GPU, so admitted requests finish in arrival order instead
    // of all sharing the device
    int64_t max_points[2] = {(int64_t)8 << 20, (int64_t)24 << 20};
    int64_t active_points[2] = {0, 0};
    // per form: the batch's tuning runs GLL degrees other than 4 (4 warps
    // per CTA, register cap 0 or 1); guarded by mu
    bool other_deg_ok[2] = {true, true};
    sks_batch* batch[2] = {nullptr, nullptr};      // by precision
    std::mutex mu;                                 // guards queue, reqs, next_id, in_use and the
                                                   // request fields other threads read
    std::deque<Request*> queue;
    std::unordered_map<int64_t, Request*> reqs;
    std::vector<Request*> active[2];
    int64_t next_id = 1;
    std::chrono::steady_clock::time_point t0;
    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

// A running request leaves: its solver leaves the batch and is destroyed,
// its memory and grid points are returned, and its end state is published.
void finish_request(sks_server* v, Request* r, int rc)
{
    sks_solver* s = r->s;
    {
        std::lock_guard<std::mutex> lk(v->mu);
        r->s = nullptr;
    }
    sks_batch_remove(v->batch[r->precision], s);
    sks_destroy(s);
    v->active_points[r->precision] -= r->points;
    std::lock_guard<std::mutex> lk(v->mu);
    v->in_use -= r->bytes;
    r->t_done = v->now();
    r->state = rc ? SKS_REQ_FAILED : SKS_REQ_DONE;
    r->status = rc;
    if (!rc) r->step = r->nst;
}

// every running request of form f failed with status rc (its quantum did)
void fail_form(sks_server* v, int f, int rc)
{
    for (Request* r : v->active[f]) finish_request(v, r, rc);
    v->active[f].clear();
}

// A finished request: its seismograms to the caller, its device memory freed.
void retire(sks_server* v, Request* r)
{
    sks_solver* s = r->s;
    int rc = SKS_OK;
    const int nt = s->m.ntrace;
    if (nt > 0 && s->seis_full) {
        const size_t w = sizeof(float) * (size_t)nt;
        for (int c = 0; c < 3 && !rc; c++)
            if (r->out[c] &&
                cudaMemcpy2DAsync(r->out[c], w, s->seis_full + (size_t)c * nt, 3 * w, w, (size_t)s->m.nst,
                                  cudaMemcpyDeviceToHost, s->stream) != cudaSuccess)
                rc = set_err(SKS_ERR_CUDA, "copy of the seismograms of request %lld", (long long)r->id);
        if (!rc && cudaStreamSynchronize(s->stream) != cudaSuccess)
            rc = set_err(SKS_ERR_CUDA, "copy of the seismograms of request %lld", (long long)r->id);
    }
    finish_request(v, r, rc);
}

// open the request's solver and make it a member of its form's batch
int admit_one(sks_server* v, Request* r)
{
    sks_solver* s = nullptr;
    sks_setup* su = r->su;
    r->su = nullptr;
    int rc = sks_open_setup(su, r->precision, v->device, &s);   // takes the set-up over
    if (!rc) {
        if (!r->stack.empty()) rc = sks_set_boundary_layered_wave(s, r->stack.data(), (int32_t)r->stack.size(), &r->lw);
        else if (r->has_pw) rc = sks_set_boundary_plane_wave(s, &r->pw);
        else rc = sks_load_boundary_files(s);
    }
    if (!rc) rc = sks_batch_add(v->batch[r->precision], s);
    if (rc) {
        if (s) sks_destroy(s);
        std::lock_guard<std::mutex> lk(v->mu);
        r->state = SKS_REQ_FAILED;
        r->status = rc;
        r->t_done = v->now();
        return rc;
    }
    v->active_points[r->precision] += r->points;
    v->active[r->precision].push_back(r);
    std::lock_guard<std::mutex> lk(v->mu);
    r->s = s;
    r->bytes = s->device_bytes;
    v->in_use += r->bytes;
    r->t_admit = v->now();
    r->step = s->step;
    r->state = SKS_REQ_RUNNING;
    return SKS_OK;
}

// Admission, first come first served within each form: the oldest queued
// request of a form is admitted when its footprint fits the device budget and
// the form's active grid points stay within its cap (a request larger than
// the cap is admitted when the form has nothing running); later requests of
// that form wait behind it.  Only forms whose batch is between quanta admit.
void admit(sks_server* v, const bool idle[2])
{
    std::vector<Request*> take;
    {
        std::lock_guard<std::mutex> lk(v->mu);
        int64_t room = v->budget - v->in_use;
        int64_t pts[2] = {v->active_points[0], v->active_points[1]};
        bool blocked[2] = {!idle[0], !idle[1]};
        // a form's batch runs one GLL degree: a request of another degree
        // waits (in order) until the form's running requests have left
        int deg[2] = {0, 0};
        for (int f = 0; f < 2; f++)
            if (!v->active[f].empty()) deg[f] = v->active[f][0]->s->m.hpn;
        for (auto it = v->queue.begin(); it != v->queue.end() && !(blocked[0] && blocked[1]);) {
            Request* r = *it;
            const int f = r->precision;
            if (blocked[f]) { ++it; continue; }
            const int rd = r->su ? r->su->m.hpn : 0;
            if (deg[f] && rd && rd != deg[f]) {
                blocked[f] = true;
                ++it;
                continue;
            }
            const bool fits_work = pts[f] == 0 || pts[f] + r->points <= v->max_points[f];
            if (r->est_bytes <= room && fits_work) {
                room -= r->est_bytes;
                pts[f] += r->points;
                if (rd) deg[f] = rd;
                take.push_back(r);
                it = v->queue.erase(it);
                continue;
            }
            blocked[f] = true;
            ++it;
        }
    }
    for (Request* r : take) admit_one(v, r);
}

}  // namespace

extern "C" int sks_server_create(int device, int64_t budget, int32_t quantum, sks_server** out)
{
    if (!out) return set_err(SKS_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (quantum < 1) return set_err(SKS_ERR_ARG, "quantum_steps=%d", quantum);
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return set_err(SKS_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
    if (budget <= 0) {
        size_t fr = 0, tot = 0;
        e = cudaMemGetInfo(&fr, &tot);
        if (e != cudaSuccess) return set_err(SKS_ERR_CUDA, "cudaMemGetInfo: %s", cudaGetErrorString(e));
        budget = (int64_t)(fr / 10 * 9);
    }
    sks_server* v = new (std::nothrow) sks_server();
    if (!v) return set_err(SKS_ERR_NOMEM, "cannot allocate the server");
    v->device = device;
    v->budget = budget;
    v->quantum = quantum;
    v->t0 = std::chrono::steady_clock::now();
    int rc = sks_batch_create(SKS_FP64, device, &v->batch[SKS_FP64]);
    if (!rc) rc = sks_batch_create(SKS_FP32C, device, &v->batch[SKS_FP32C]);
    // FP32C quanta are short and many; FP64 quanta long: FP32C first
    if (!rc) rc = batch_set_priority(v->batch[SKS_FP32C], true);
    if (!rc) rc = batch_set_priority(v->batch[SKS_FP64], false);
    // tunings measured on the served workload (FP32C requests at saturation:
    // pipelined chunks of 12-row bands, 14,437 solves/h against 14,044 with
    // per-step launches of 6-row bands); sks_server_set_tuning overrides them
    if (!rc) {
        sks_tuning_t t32 = {4, 12, 0, 1, 0, 0, 0.f, 1};
        sks_tuning_t t64 = {4, 8, 1, 0, 0, 0, 0.f, 0};
        rc = sks_batch_set_tuning(v->batch[SKS_FP32C], &t32);
        if (!rc) rc = sks_batch_set_tuning(v->batch[SKS_FP64], &t64);
    }
    if (rc) {
        sks_batch_destroy(v->batch[0]);
        sks_batch_destroy(v->batch[1]);
        delete v;
        return rc;
    }
    *out = v;
    return SKS_OK;
}

extern "C" int sks_server_set_tuning(sks_server* v, int precision, const sks_tuning_t* t)
{
    if (!v || !t) return set_err(SKS_ERR_ARG, "NULL argument");
    if (precision != SKS_FP64 && precision != SKS_FP32C) return set_err(SKS_ERR_ARG, "unknown precision %d", precision);
    const bool other_deg = t->warps_per_block == 4 && t->register_cap <= 1;
    {
        // a tuning that can run degree 4 only is refused while the form has
        // requests of another degree queued or running
        std::lock_guard<std::mutex> lk(v->mu);
        if (!other_deg) {
            for (const Request* r : v->queue)
                if (r->precision == precision && r->su && r->su->m.hpn != 4)
                    return set_err(SKS_ERR_STATE, "request %lld is of GLL degree %d, which runs with 4 warps per CTA "
                                                  "and register cap 0 or 1", (long long)r->id, r->su->m.hpn);
            for (const Request* r : v->active[precision])
                if (r->s && r->s->m.hpn != 4)
                    return set_err(SKS_ERR_STATE, "request %lld is of GLL degree %d, which runs with 4 warps per CTA "
                                                  "and register cap 0 or 1", (long long)r->id, r->s->m.hpn);
        }
    }
    if (batch_running(v->batch[precision])) batch_finish(v->batch[precision]);
    const int rc = sks_batch_set_tuning(v->batch[precision], t);
    if (!rc) {
        std::lock_guard<std::mutex> lk(v->mu);
        v->other_deg_ok[precision] = other_deg;
    }
    return rc;
}

extern "C" int sks_server_set_active_points(sks_server* v, int precision, int64_t max_points)
{
    if (!v) return set_err(SKS_ERR_ARG, "server is NULL");
    if (precision != SKS_FP64 && precision != SKS_FP32C) return set_err(SKS_ERR_ARG, "unknown precision %d", precision);
    if (max_points < 1) return set_err(SKS_ERR_ARG, "max_points=%lld", (long long)max_points);
    std::lock_guard<std::mutex> lk(v->mu);
    v->max_points[precision] = max_points;
    return SKS_OK;
}

namespace {

// queue a request; pw or (layers, n, lw) name a device generator, neither the files
int submit(sks_server* v, sks_setup* su, int precision, const sks_plane_wave_t* pw, const sks_stack_layer_t* layers,
           int32_t n, const sks_layered_wave_t* lw, float* su_out, float* sv_out, float* sw_out, int64_t* id)
{
    if (!v || !su || !id) {
        if (su) sks_setup_close(su);
        return set_err(SKS_ERR_ARG, "NULL argument");
    }
    if (precision != SKS_FP64 && precision != SKS_FP32C) {
        sks_setup_close(su);
        return set_err(SKS_ERR_ARG, "unknown precision %d", precision);
    }
    if (su->m.hpn != 4) {
        const int hpn = su->m.hpn;
        std::lock_guard<std::mutex> lk(v->mu);
        if (!v->other_deg_ok[precision]) {
            sks_setup_close(su);
            return set_err(SKS_ERR_UNSUPPORTED, "GLL degree %d requests need the form's tuning to be 4 warps per CTA "
                                                "and register cap 0 or 1 (sks_server_set_tuning)", hpn);
        }
    }
    if (!pw && !layers) {
        int rc = absolute_path(su->m.greenfile, sizeof su->m.greenfile);
        if (!rc && !su->m.psv_only) rc = absolute_path(su->m.shgreenfile, sizeof su->m.shgreenfile);
        if (rc) { sks_setup_close(su); return rc; }
    }
    Request* r = new (std::nothrow) Request();
    if (!r) { sks_setup_close(su); return set_err(SKS_ERR_NOMEM, "cannot allocate the request"); }
    r->su = su;
    r->precision = precision;
    if (pw) { r->has_pw = true; r->pw = *pw; }
    if (layers) {
        try {
            r->stack.assign(layers, layers + n);
        } catch (...) {
            delete r;
            sks_setup_close(su);
            return set_err(SKS_ERR_NOMEM, "cannot copy the layer stack");
        }
        r->lw = *lw;
    }
    r->out[0] = su_out; r->out[1] = sv_out; r->out[2] = sw_out;
    int64_t rec_bytes = ((int64_t)su->m.nrec_psv * su->m.mtotal + (int64_t)su->m.nrec_sh * su->m.shtotal) * 4;
    const int64_t Lline = (int64_t)su->m.mtotal + su->m.shtotal;
    if (pw) rec_bytes = 16 * Lline;                      // the line's delays and amplitudes
    if (layers) {
        const sks_model& m = su->m;
        const double xmax = (double)(m.nx - 1) * m.h + m.eh, zmax = (double)(m.nz - 1) * m.h + m.eh;
        const double span = (double)std::max(m.nrec_psv, m.nrec_sh) * m.dp + lw->p * xmax + zmax / layers[0].vs;
        const int64_t nt = sks_layered_series_length(layers, n, lw->p, lw->f0, m.dp / 4.0, span);
        if (nt < 0) {
            delete r;
            sks_setup_close(su);
            return (int)nt;
        }
        rec_bytes = 24 * nt + 32 * Lline;                 // mode series, line delays and coefficients
    }
    r->est_bytes = estimate_bytes(su->m, precision, rec_bytes);
    r->nst = su->m.nst;
    r->ntrace = su->m.ntrace;
    r->points = (int64_t)su->m.nx * su->m.nz;
    r->t_submit = v->now();
    std::lock_guard<std::mutex> lk(v->mu);
    r->id = v->next_id++;
    v->reqs[r->id] = r;
    if (r->est_bytes > v->budget) {
        r->state = SKS_REQ_FAILED;
        r->status = SKS_ERR_NOMEM;
        r->t_done = r->t_submit;
        sks_setup_close(r->su);
        r->su = nullptr;
    } else {
        v->queue.push_back(r);
    }
    *id = r->id;
    return SKS_OK;
}

}  // namespace

extern "C" int sks_server_submit(sks_server* v, sks_setup* su, int precision, const sks_plane_wave_t* pw, float* su_out,
                                 float* sv_out, float* sw_out, int64_t* id)
{
    return submit(v, su, precision, pw, nullptr, 0, nullptr, su_out, sv_out, sw_out, id);
}

extern "C" int sks_server_submit_layered(sks_server* v, sks_setup* su, int precision, const sks_stack_layer_t* layers,
                                         int32_t n, const sks_layered_wave_t* wave, float* su_out, float* sv_out,
                                         float* sw_out, int64_t* id)
{
    if (!layers || !wave || n < 2) {
        if (su) sks_setup_close(su);
        return set_err(SKS_ERR_ARG, "layered request: a stack of 2 media at least and a wave");
    }
    return submit(v, su, precision, nullptr, layers, n, wave, su_out, sv_out, sw_out, id);
}

extern "C" int sks_server_step(sks_server* v)
{
    if (!v) return set_err(SKS_ERR_ARG, "server is NULL");
    cudaSetDevice(v->device);
    bool progressed = false;
    // finished quanta: move steps on, retire the requests that reached their
    // end; a quantum that failed fails its form's running requests, except
    // that a request whose wavefield stopped being finite fails alone (its
    // batch mates' results do not depend on it)
    for (int f = 0; f < 2; f++) {
        sks_batch* b = v->batch[f];
        if (!batch_running(b) || !batch_done(b)) continue;
        const int rc = batch_finish(b);
        progressed = true;
        if (rc < 0 && rc != SKS_ERR_NONFINITE) {
            fail_form(v, f, rc);
            continue;
        }
        {
            std::lock_guard<std::mutex> lk(v->mu);
            for (Request* r : v->active[f]) r->step = r->s->step;
        }
        std::vector<Request*> keep;
        for (Request* r : v->active[f]) {
            if (!sks_wavefield_finite(r->s)) finish_request(v, r, SKS_ERR_NONFINITE);
            else if (r->s->step >= r->s->m.nst) retire(v, r);
            else keep.push_back(r);
        }
        v->active[f].swap(keep);
    }
    // admission into the idle forms, then their next quantum
    bool idle[2] = {!batch_running(v->batch[0]), !batch_running(v->batch[1])};
    admit(v, idle);
    for (int f = 0; f < 2; f++) {
        if (!idle[f] || v->active[f].empty()) continue;
        const int rc = batch_launch(v->batch[f], v->quantum, nullptr, nullptr, nullptr);
        if (rc < 0) {
            if (batch_running(v->batch[f])) batch_finish(v->batch[f]);
            fail_form(v, f, rc);
            continue;
        }
        progressed = true;
    }
    if (!progressed && (batch_running(v->batch[0]) || batch_running(v->batch[1])))
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    std::lock_guard<std::mutex> lk(v->mu);
    return (int)(v->queue.size() + v->active[0].size() + v->active[1].size());
}

extern "C" int sks_server_request_info(sks_server* v, int64_t id, sks_request_info_t* info)
{
    if (!v || !info) return set_err(SKS_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(v->mu);
    auto it = v->reqs.find(id);
    if (it == v->reqs.end()) return set_err(SKS_ERR_ARG, "no request %lld", (long long)id);
    const Request* r = it->second;
    info->state = r->state;
    info->status = r->status;
    info->precision = r->precision;
    info->step = r->step;
    info->nst = r->nst;
    info->ntrace = r->ntrace;
    info->submit_s = r->t_submit;
    info->admit_s = r->t_admit;
    info->done_s = r->t_done;
    info->device_bytes = r->s ? r->bytes : r->est_bytes;
    return SKS_OK;
}

extern "C" int sks_server_release(sks_server* v, int64_t id)
{
    if (!v) return set_err(SKS_ERR_ARG, "server is NULL");
    std::lock_guard<std::mutex> lk(v->mu);
    auto it = v->reqs.find(id);
    if (it == v->reqs.end()) return set_err(SKS_ERR_ARG, "no request %lld", (long long)id);
    if (it->second->state != SKS_REQ_DONE && it->second->state != SKS_REQ_FAILED)
        return set_err(SKS_ERR_STATE, "request %lld has not finished", (long long)id);
    delete it->second;
    v->reqs.erase(it);
    return SKS_OK;
}

extern "C" double sks_server_clock(const sks_server* v) { return v ? v->now() : -1.0; }

extern "C" int64_t sks_server_device_bytes(const sks_server* v)
{
    if (!v) return -1;
    std::lock_guard<std::mutex> lk(const_cast<sks_server*>(v)->mu);
    return v->in_use;
}

extern "C" void sks_server_destroy(sks_server* v)
{
    if (!v) return;
    cudaSetDevice(v->device);
    for (int f = 0; f < 2; f++)
        if (v->batch[f] && batch_running(v->batch[f])) batch_finish(v->batch[f]);
    for (int f = 0; f < 2; f++)
        for (Request* r : v->active[f])
            if (r->s) { sks_batch_remove(v->batch[f], r->s); sks_destroy(r->s); r->s = nullptr; }
    sks_batch_destroy(v->batch[0]);
    sks_batch_destroy(v->batch[1]);
    for (auto& kv : v->reqs) {
        if (kv.second->su) sks_setup_close(kv.second->su);
        delete kv.second;
    }
    delete v;
}
