// Batch step kernel variants of the FP64 form with the boundary taper
// (some member has atten > 0; members without it skip the taper).
#include "sks_batch_inst.cuh"

namespace sks {

int batch_occupancy_f64_tp(const StepVariant& v, bool aniso) { return batch_occupancy_t<double, false, true>(v, aniso); }

cudaError_t launch_batch_f64_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                const BatchMember<double>* mem, const BatchState* state, const int4* items,
                                const BatchHeader* hdr, int j, const Coef<double>& k)
{
    return launch_batch_t<double, false, true>(v, aniso, blocks, st, mem, state, items, hdr, j, k);
}

int batch_pipe_occupancy_f64_tp(const StepVariant& v, bool aniso)
{
    return batch_pipe_occupancy_t<double, false, true>(v, aniso);
}

cudaError_t launch_batch_pipe_f64_tp(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                                     const BatchMember<double>* mem, const BatchState* state, const int4* items,
                                     const BatchHeader* hdr, int nsteps, const BatchPipeCtl& ctl,
                                     const Coef<double>& k)
{
    return launch_batch_pipe_t<double, false, true>(v, aniso, blocks, st, mem, state, items, hdr, nsteps, ctl, k);
}

}  // namespace sks
