// Step kernel variants of the FP64 form with the boundary taper (atten > 0).
#include "sks_step_inst.cuh"

namespace sks {

int step_occupancy_f64_tp(const StepVariant& v, bool aniso) { return step_occupancy_t<double, false, true>(v, aniso); }

cudaError_t launch_step_f64_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                               const Field<double>& F, const Geo<double>& G, const Coef<double>& k)
{
    return launch_step_t<double, false, true>(v, aniso, blocks, st, F, G, k);
}

int pipe_occupancy_f64_tp(const StepVariant& v, bool aniso) { return pipe_occupancy_t<double, false, true>(v, aniso); }

cudaError_t launch_pipe_f64_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<double>& F,
                               const Geo<double>& G, const Coef<double>& k, const PipeChunk& C, const PipeCtl& ctl)
{
    return launch_pipe_t<double, false, true>(v, aniso, blocks, st, F, G, k, C, ctl);
}

}  // namespace sks
