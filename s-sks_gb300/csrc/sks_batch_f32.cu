// Batch step kernel variants of the FP32-compensated form.
#include "sks_batch_inst.cuh"

namespace sks {

int batch_occupancy_f32(const StepVariant& v, bool aniso)
{
    BatchOcc<float, true> o;
    return visit_variant(v, aniso, o);
}

cudaError_t launch_batch_f32(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const BatchMember<float>* mem,
                             const BatchState* state, const int4* items, const BatchHeader* hdr, int j,
                             const Coef<float>& k)
{
    BatchLaunch<float, true> l{blocks, st, mem, state, items, hdr, j, k};
    visit_variant(v, aniso, l);
    return cudaGetLastError();
}

int batch_pipe_occupancy_f32(const StepVariant& v, bool aniso)
{
    BatchPipeOcc<float, true> o;
    return visit_variant(v, aniso, o);
}

cudaError_t launch_batch_pipe_f32(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                  const BatchMember<float>* mem, const BatchState* state, const int4* items,
                                  const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl, const Coef<float>& k)
{
    BatchPipeLaunch<float, true> l{blocks, st, mem, state, items, hdr, nsteps, ctl, k};
    visit_variant(v, aniso, l);
    return cudaGetLastError();
}

}  // namespace sks
