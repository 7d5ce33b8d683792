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

}  // namespace sks
