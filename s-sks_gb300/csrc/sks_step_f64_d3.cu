// Step kernel variants of the FP64 form for GLL degree 3 (the reference
// accepts hpn = 3..6), with and without the boundary taper: 4 warps per
// CTA, register cap 0 or 1, halo rows or band seams.
#include "sks_step_inst.cuh"

namespace sks {

int step_occupancy_f64_d3(const StepVariant& v, bool aniso)
{
    return v.taper ? step_occupancy_t<double, false, true, 3>(v, aniso) : step_occupancy_t<double, false, false, 3>(v, aniso);
}

cudaError_t launch_step_f64_d3(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                               const Field<double>& F, const Geo<double>& G, const Coef<double, 3>& k)
{
    return v.taper ? launch_step_t<double, false, true, 3>(v, aniso, blocks, st, F, G, k)
                   : launch_step_t<double, false, false, 3>(v, aniso, blocks, st, F, G, k);
}

int pipe_occupancy_f64_d3(const StepVariant& v, bool aniso)
{
    return v.taper ? pipe_occupancy_t<double, false, true, 3>(v, aniso) : pipe_occupancy_t<double, false, false, 3>(v, aniso);
}

cudaError_t launch_pipe_f64_d3(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<double>& F,
                               const Geo<double>& G, const Coef<double, 3>& k, const PipeChunk& C, const PipeCtl& ctl)
{
    return v.taper ? launch_pipe_t<double, false, true, 3>(v, aniso, blocks, st, F, G, k, C, ctl)
                   : launch_pipe_t<double, false, false, 3>(v, aniso, blocks, st, F, G, k, C, ctl);
}

}  // namespace sks
