// Step kernel variants of the FP32-compensated form with the boundary taper (atten > 0).
#include "sks_step_inst.cuh"

namespace sks {

int step_occupancy_f32_tp(const StepVariant& v, bool aniso) { return step_occupancy_t<float, true, true>(v, aniso); }

cudaError_t launch_step_f32_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                               const Field<float>& F, const Geo<float>& G, const Coef<float>& k)
{
    return launch_step_t<float, true, true>(v, aniso, blocks, st, F, G, k);
}

int pipe_occupancy_f32_tp(const StepVariant& v, bool aniso) { return pipe_occupancy_t<float, true, true>(v, aniso); }

cudaError_t launch_pipe_f32_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<float>& F,
                               const Geo<float>& G, const Coef<float>& k, const PipeChunk& C, const PipeCtl& ctl)
{
    return launch_pipe_t<float, true, true>(v, aniso, blocks, st, F, G, k, C, ctl);
}

}  // namespace sks
