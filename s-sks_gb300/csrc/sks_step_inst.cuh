// Launchers of the single-mesh step kernel for one form (T, LF); included by
// one translation unit per form so the variants compile in parallel.
#pragma once
#include "sks_variants.cuh"

namespace sks {
namespace {

template <typename T, bool LF>
struct StepLaunch {
    int blocks;
    cudaStream_t st;
    const Field<T>& F;
    const Geo<T>& G;
    const Coef<T>& k;
    template <bool A, int NW, bool ZS, int CAP>
    int run()
    {
        k_step<T, A, LF, NW, ZS, CAP><<<blocks, NW * 32, 0, st>>>(F, G, k);
        return 0;
    }
};

template <typename T, bool LF>
struct PipeLaunch {
    int blocks;
    cudaStream_t st;
    const Field<T>& F;
    const Geo<T>& G;
    const Coef<T>& k;
    const PipeChunk& C;
    const PipeCtl& ctl;
    template <bool A, int NW, bool ZS, int CAP>
    int run()
    {
        k_step_pipe<T, A, LF, NW, ZS, CAP><<<blocks, NW * 32, 0, st>>>(F, G, k, C, ctl);
        return 0;
    }
};

template <typename T, bool LF>
struct PipeOcc {
    template <bool A, int NW, bool ZS, int CAP>
    int run() { return occupancy_of(k_step_pipe<T, A, LF, NW, ZS, CAP>, NW * 32); }
};

template <typename T, bool LF>
struct StepOcc {
    template <bool A, int NW, bool ZS, int CAP>
    int run() { return occupancy_of(k_step<T, A, LF, NW, ZS, CAP>, NW * 32); }
};

}  // namespace
}  // namespace sks
