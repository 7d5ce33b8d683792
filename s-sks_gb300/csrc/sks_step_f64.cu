// Step kernel variants of the FP64 form.
#include "sks_step_inst.cuh"

namespace sks {

int step_occupancy_f64(const StepVariant& v, bool aniso)
{
    StepOcc<double, false> o;
    return visit_variant(v, aniso, o);
}

cudaError_t launch_step_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                            const Field<double>& F, const Geo<double>& G, const Coef<double>& k)
{
    StepLaunch<double, false> l{blocks, st, F, G, k};
    visit_variant(v, aniso, l);
    return cudaGetLastError();
}

int pipe_occupancy_f64(const StepVariant& v, bool aniso)
{
    const StepVariant p{v.nw, v.zseam, v.cap};
    PipeOcc<double, false> o;
    return visit_variant(p, aniso, o);
}

cudaError_t launch_pipe_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const Field<double>& F,
                            const Geo<double>& G, const Coef<double>& k, const PipeChunk& C, const PipeCtl& ctl)
{
    const StepVariant p{v.nw, v.zseam, v.cap};
    PipeLaunch<double, false> l{blocks, st, F, G, k, C, ctl};
    visit_variant(p, aniso, l);
    return cudaGetLastError();
}

}  // namespace sks
