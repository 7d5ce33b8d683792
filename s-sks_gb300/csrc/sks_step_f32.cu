// Step kernel variants of the FP32-compensated form without the boundary taper; the
// tapered ones (atten > 0) compile in sks_step_f32_tp.cu.
#include "sks_step_inst.cuh"

namespace sks {

int step_occupancy_f32(const StepVariant& v, bool aniso)
{
    return v.taper ? step_occupancy_f32_tp(v, aniso) : step_occupancy_t<float, true, false>(v, aniso);
}

cudaError_t launch_step_f32(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                            const Field<float>& F, const Geo<float>& G, const Coef<float>& k)
{
    return v.taper ? launch_step_f32_tp(v, aniso, blocks, st, F, G, k)
                   : launch_step_t<float, true, false>(v, aniso, blocks, st, F, G, k);
}

int pipe_occupancy_f32(const StepVariant& v, bool aniso)
{
    return v.taper ? pipe_occupancy_f32_tp(v, aniso) : pipe_occupancy_t<float, true, false>(v, aniso);
}

cudaError_t launch_pipe_f32(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<float>& F,
                            const Geo<float>& G, const Coef<float>& k, const PipeChunk& C, const PipeCtl& ctl)
{
    return v.taper ? launch_pipe_f32_tp(v, aniso, blocks, st, F, G, k, C, ctl)
                   : launch_pipe_t<float, true, false>(v, aniso, blocks, st, F, G, k, C, ctl);
}

}  // namespace sks
