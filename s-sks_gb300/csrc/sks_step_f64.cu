// Step kernel variants of the FP64 form without the boundary taper; the
// tapered ones (atten > 0) compile in sks_step_f64_tp.cu.
#include "sks_step_inst.cuh"

namespace sks {

int step_occupancy_f64(const StepVariant& v, bool aniso)
{
    return v.taper ? step_occupancy_f64_tp(v, aniso) : step_occupancy_t<double, false, false>(v, aniso);
}

cudaError_t launch_step_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                            const Field<double>& F, const Geo<double>& G, const Coef<double>& k)
{
    return v.taper ? launch_step_f64_tp(v, aniso, blocks, st, F, G, k)
                   : launch_step_t<double, false, false>(v, aniso, blocks, st, F, G, k);
}

int pipe_occupancy_f64(const StepVariant& v, bool aniso)
{
    return v.taper ? pipe_occupancy_f64_tp(v, aniso) : pipe_occupancy_t<double, false, false>(v, aniso);
}

cudaError_t launch_pipe_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<double>& F,
                            const Geo<double>& G, const Coef<double>& k, const PipeChunk& C, const PipeCtl& ctl)
{
    return v.taper ? launch_pipe_f64_tp(v, aniso, blocks, st, F, G, k, C, ctl)
                   : launch_pipe_t<double, false, false>(v, aniso, blocks, st, F, G, k, C, ctl);
}

}  // namespace sks
