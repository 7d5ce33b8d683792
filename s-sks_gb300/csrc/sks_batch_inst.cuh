// Launchers of the batch step kernel for one form (T, LF) and taper flag
// (TP); included by one translation unit per (form, TP).
#pragma once
#include "sks_variants.cuh"

namespace sks {
namespace {

template <typename T, bool LF, bool TP, int DEG = N>
struct BatchLaunch {
    int blocks;
    cudaStream_t st;
    const BatchMember<T>* mem;
    const BatchState* state;
    const int4* items;
    const BatchHeader* hdr;
    int j;
    const Coef<T, DEG>& k;
    template <bool A, int NW, bool ZS, int CAP>
    int run()
    {
        k_step_batch<T, A, LF, NW, ZS, CAP, TP, DEG><<<blocks, NW * 32, 0, st>>>(mem, state, items, hdr, j, k);
        return 0;
    }
};

template <typename T, bool LF, bool TP, int DEG = N>
struct BatchPipeLaunch {
    int blocks;
    cudaStream_t st;
    const BatchMember<T>* mem;
    const BatchState* state;
    const int4* items;
    const BatchHeader* hdr;
    int nsteps;
    const BatchPipeCtl& ctl;
    const Coef<T, DEG>& k;
    template <bool A, int NW, bool ZS, int CAP>
    int run()
    {
        k_step_batch_pipe<T, A, LF, NW, ZS, CAP, TP, DEG><<<blocks, NW * 32, 0, st>>>(mem, state, items, hdr, nsteps, ctl, k);
        return 0;
    }
};

template <typename T, bool LF, bool TP, int DEG = N>
struct BatchPipeOcc {
    template <bool A, int NW, bool ZS, int CAP>
    int run() { return occupancy_of(k_step_batch_pipe<T, A, LF, NW, ZS, CAP, TP, DEG>, NW * 32); }
};

template <typename T, bool LF, bool TP, int DEG = N>
struct BatchOcc {
    template <bool A, int NW, bool ZS, int CAP>
    int run() { return occupancy_of(k_step_batch<T, A, LF, NW, ZS, CAP, TP, DEG>, NW * 32); }
};

// the launchers of one form with (TP) or without the boundary taper
template <typename T, bool LF, bool TP, int DEG = N>
int batch_occupancy_t(const StepVariant& v, bool aniso)
{
    BatchOcc<T, LF, TP, DEG> o;
    return visit_deg<DEG>(v, aniso, o);
}

template <typename T, bool LF, bool TP, int DEG = N>
cudaError_t launch_batch_t(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const BatchMember<T>* mem,
                           const BatchState* state, const int4* items, const BatchHeader* hdr, int j,
                           const Coef<T, DEG>& k)
{
    BatchLaunch<T, LF, TP, DEG> l{blocks, st, mem, state, items, hdr, j, k};
    visit_deg<DEG>(v, aniso, l);
    return cudaGetLastError();
}

template <typename T, bool LF, bool TP, int DEG = N>
int batch_pipe_occupancy_t(const StepVariant& v, bool aniso)
{
    BatchPipeOcc<T, LF, TP, DEG> o;
    return visit_deg<DEG>(v, aniso, o);
}

template <typename T, bool LF, bool TP, int DEG = N>
cudaError_t launch_batch_pipe_t(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                const BatchMember<T>* mem, const BatchState* state, const int4* items,
                                const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl, const Coef<T, DEG>& k)
{
    BatchPipeLaunch<T, LF, TP, DEG> l{blocks, st, mem, state, items, hdr, nsteps, ctl, k};
    visit_deg<DEG>(v, aniso, l);
    return cudaGetLastError();
}

}  // namespace
}  // namespace sks
