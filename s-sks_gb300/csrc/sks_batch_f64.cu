// Batch step kernel variants of the FP64 form.
#include "sks_batch_inst.cuh"

namespace sks {

int batch_occupancy_f64(const StepVariant& v, bool aniso)
{
    BatchOcc<double, false> o;
    return visit_variant(v, aniso, o);
}

cudaError_t launch_batch_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const BatchMember<double>* mem,
                             const BatchState* state, const int4* items, const BatchHeader* hdr, int j,
                             const Coef<double>& k)
{
    BatchLaunch<double, false> l{blocks, st, mem, state, items, hdr, j, k};
    visit_variant(v, aniso, l);
    return cudaGetLastError();
}

int batch_pipe_occupancy_f64(const StepVariant& v, bool aniso)
{
    BatchPipeOcc<double, false> o;
    return visit_variant(v, aniso, o);
}

cudaError_t launch_batch_pipe_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                  const BatchMember<double>* mem, const BatchState* state, const int4* items,
                                  const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl, const Coef<double>& k)
{
    BatchPipeLaunch<double, false> l{blocks, st, mem, state, items, hdr, nsteps, ctl, k};
    visit_variant(v, aniso, l);
    return cudaGetLastError();
}

}  // namespace sks
