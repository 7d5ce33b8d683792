// Launchers of the batch step kernel for one form (T, LF); included by one
// translation unit per form.
#pragma once
#include "sks_variants.cuh"

namespace sks {
namespace {

template <typename T, bool LF>
struct BatchLaunch {
    int blocks;
    cudaStream_t st;
    const BatchMember<T>* mem;
    const BatchState* state;
    const int4* items;
    const BatchHeader* hdr;
    int j;
    const Coef<T>& k;
    template <bool A, int NW, bool ZS, int CAP>
    int run()
    {
        k_step_batch<T, A, LF, NW, ZS, CAP><<<blocks, NW * 32, 0, st>>>(mem, state, items, hdr, j, k);
        return 0;
    }
};

template <typename T, bool LF>
struct BatchPipeLaunch {
    int blocks;
    cudaStream_t st;
    const BatchMember<T>* mem;
    const BatchState* state;
    const int4* items;
    const BatchHeader* hdr;
    int nsteps;
    const BatchPipeCtl& ctl;
    const Coef<T>& k;
    template <bool A, int NW, bool ZS, int CAP>
    int run()
    {
        k_step_batch_pipe<T, A, LF, NW, ZS, CAP><<<blocks, NW * 32, 0, st>>>(mem, state, items, hdr, nsteps, ctl, k);
        return 0;
    }
};

template <typename T, bool LF>
struct BatchPipeOcc {
    template <bool A, int NW, bool ZS, int CAP>
    int run() { return occupancy_of(k_step_batch_pipe<T, A, LF, NW, ZS, CAP>, NW * 32); }
};

template <typename T, bool LF>
struct BatchOcc {
    template <bool A, int NW, bool ZS, int CAP>
    int run() { return occupancy_of(k_step_batch<T, A, LF, NW, ZS, CAP>, NW * 32); }
};

}  // namespace
}  // namespace sks
