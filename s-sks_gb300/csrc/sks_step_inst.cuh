// Launchers of the single-mesh step kernel for one form (T, LF) and taper
// flag (TP); included by one translation unit per (form, TP) so the variants
// compile in parallel.
#pragma once
#include "sks_variants.cuh"

namespace sks {
namespace {

template <typename T, bool LF, bool TP, int DEG = N>
struct StepLaunch {
    int blocks;
    cudaStream_t st;
    const Field<T>& F;
    const Geo<T>& G;
    const Coef<T, DEG>& k;
    template <bool A, int NW, bool ZS, int CAP>
    int run()
    {
        k_step<T, A, LF, NW, ZS, CAP, TP, DEG><<<blocks, NW * 32, 0, st>>>(F, G, k);
        return 0;
    }
};

template <typename T, bool LF, bool TP, int DEG = N>
struct PipeLaunch {
    int blocks;
    cudaStream_t st;
    const Field<T>& F;
    const Geo<T>& G;
    const Coef<T, DEG>& k;
    const PipeChunk& C;
    const PipeCtl& ctl;
    template <bool A, int NW, bool ZS, int CAP>
    int run()
    {
        k_step_pipe<T, A, LF, NW, ZS, CAP, TP, DEG><<<blocks, NW * 32, 0, st>>>(F, G, k, C, ctl);
        return 0;
    }
};

template <typename T, bool LF, bool TP, int DEG = N>
struct PipeOcc {
    template <bool A, int NW, bool ZS, int CAP>
    int run() { return occupancy_of(k_step_pipe<T, A, LF, NW, ZS, CAP, TP, DEG>, NW * 32); }
};

template <typename T, bool LF, bool TP, int DEG = N>
struct StepOcc {
    template <bool A, int NW, bool ZS, int CAP>
    int run() { return occupancy_of(k_step<T, A, LF, NW, ZS, CAP, TP, DEG>, NW * 32); }
};

// the launchers of one form with (TP) or without the boundary taper
template <typename T, bool LF, bool TP, int DEG = N>
int step_occupancy_t(const StepVariant& v, bool aniso)
{
    StepOcc<T, LF, TP, DEG> o;
    return visit_deg<DEG>(v, aniso, o);
}

template <typename T, bool LF, bool TP, int DEG = N>
cudaError_t launch_step_t(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<T>& F,
                          const Geo<T>& G, const Coef<T, DEG>& k)
{
    StepLaunch<T, LF, TP, DEG> l{blocks, st, F, G, k};
    visit_deg<DEG>(v, aniso, l);
    return cudaGetLastError();
}

template <typename T, bool LF, bool TP, int DEG = N>
int pipe_occupancy_t(const StepVariant& v, bool aniso)
{
    PipeOcc<T, LF, TP, DEG> o;
    return visit_deg<DEG>(v, aniso, o);
}

template <typename T, bool LF, bool TP, int DEG = N>
cudaError_t launch_pipe_t(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<T>& F,
                          const Geo<T>& G, const Coef<T, DEG>& k, const PipeChunk& C, const PipeCtl& ctl)
{
    PipeLaunch<T, LF, TP, DEG> l{blocks, st, F, G, k, C, ctl};
    visit_deg<DEG>(v, aniso, l);
    return cudaGetLastError();
}

}  // namespace
}  // namespace sks
