// Batch step kernel variants of the FP64 form for GLL degree 3, with and
// without the boundary taper: 4 warps per CTA, register cap 0 or 1.
#include "sks_batch_inst.cuh"

namespace sks {

int batch_occupancy_f64_d3(const StepVariant& v, bool aniso)
{
    return v.taper ? batch_occupancy_t<double, false, true, 3>(v, aniso) : batch_occupancy_t<double, false, false, 3>(v, aniso);
}

cudaError_t launch_batch_f64_d3(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                const BatchMember<double>* mem, const BatchState* state, const int4* items,
                                const BatchHeader* hdr, int j, const Coef<double, 3>& k)
{
    return v.taper ? launch_batch_t<double, false, true, 3>(v, aniso, blocks, st, mem, state, items, hdr, j, k)
                   : launch_batch_t<double, false, false, 3>(v, aniso, blocks, st, mem, state, items, hdr, j, k);
}

int batch_pipe_occupancy_f64_d3(const StepVariant& v, bool aniso)
{
    return v.taper ? batch_pipe_occupancy_t<double, false, true, 3>(v, aniso)
                   : batch_pipe_occupancy_t<double, false, false, 3>(v, aniso);
}

cudaError_t launch_batch_pipe_f64_d3(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                     const BatchMember<double>* mem, const BatchState* state, const int4* items,
                                     const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl,
                                     const Coef<double, 3>& k)
{
    return v.taper ? launch_batch_pipe_t<double, false, true, 3>(v, aniso, blocks, st, mem, state, items, hdr, nsteps, ctl, k)
                   : launch_batch_pipe_t<double, false, false, 3>(v, aniso, blocks, st, mem, state, items, hdr, nsteps, ctl,
                                                             k);
}

}  // namespace sks
