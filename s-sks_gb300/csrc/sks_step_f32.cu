// Step kernel variants of the FP32-compensated form.
#include "sks_step_inst.cuh"

namespace sks {

int step_occupancy_f32(const StepVariant& v, bool aniso)
{
    StepOcc<float, true> o;
    return visit_variant(v, aniso, o);
}

cudaError_t launch_step_f32(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                            const Field<float>& F, const Geo<float>& G, const Coef<float>& k)
{
    StepLaunch<float, true> l{blocks, st, F, G, k};
    visit_variant(v, aniso, l);
    return cudaGetLastError();
}

int pipe_occupancy_f32(const StepVariant& v, bool aniso)
{
    const StepVariant p{v.nw, v.zseam, v.cap};
    PipeOcc<float, true> o;
    return visit_variant(p, aniso, o);
}

cudaError_t launch_pipe_f32(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<float>& F,
                            const Geo<float>& G, const Coef<float>& k, const PipeChunk& C, const PipeCtl& ctl)
{
    const StepVariant p{v.nw, v.zseam, v.cap};
    PipeLaunch<float, true> l{blocks, st, F, G, k, C, ctl};
    visit_variant(p, aniso, l);
    return cudaGetLastError();
}

}  // namespace sks
