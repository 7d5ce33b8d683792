// Batch step kernel variants of the FP64 form without the boundary taper;
// the tapered ones (a member with atten > 0) compile in sks_batch_f64_tp.cu.
#include "sks_batch_inst.cuh"

namespace sks {

int batch_occupancy_f64(const StepVariant& v, bool aniso)
{
    return v.taper ? batch_occupancy_f64_tp(v, aniso) : batch_occupancy_t<double, false, false>(v, aniso);
}

cudaError_t launch_batch_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st, const BatchMember<double>* mem,
                             const BatchState* state, const int4* items, const BatchHeader* hdr, int j,
                             const Coef<double>& k)
{
    return v.taper ? launch_batch_f64_tp(v, aniso, blocks, st, mem, state, items, hdr, j, k)
                   : launch_batch_t<double, false, false>(v, aniso, blocks, st, mem, state, items, hdr, j, k);
}

int batch_pipe_occupancy_f64(const StepVariant& v, bool aniso)
{
    return v.taper ? batch_pipe_occupancy_f64_tp(v, aniso) : batch_pipe_occupancy_t<double, false, false>(v, aniso);
}

cudaError_t launch_batch_pipe_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                  const BatchMember<double>* mem, const BatchState* state, const int4* items,
                                  const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl, const Coef<double>& k)
{
    return v.taper ? launch_batch_pipe_f64_tp(v, aniso, blocks, st, mem, state, items, hdr, nsteps, ctl, k)
                   : launch_batch_pipe_t<double, false, false>(v, aniso, blocks, st, mem, state, items, hdr, nsteps, ctl, k);
}

}  // namespace sks
