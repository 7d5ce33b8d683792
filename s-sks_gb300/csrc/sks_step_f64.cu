// Instantiations of the step kernel for the FP64 form, one translation unit
// per precision so the variants compile in parallel.
#include "sks_kernels.cuh"

namespace sks {
namespace {

template <bool ANISO, int NW, bool ZS, int CAP>
void go(int blocks, cudaStream_t st, const Field<double>& F, const Geo<double>& G, const Coef<double>& k)
{
    k_step<double, ANISO, false, NW, ZS, CAP><<<blocks, NW * 32, 0, st>>>(F, G, k);
}

template <bool ANISO, int NW>
void go_nw(const StepVariant& v, int blocks, cudaStream_t st, const Field<double>& F, const Geo<double>& G,
           const Coef<double>& k)
{
    if (v.zseam) {
        if (v.cap == 2) go<ANISO, NW, true, 2>(blocks, st, F, G, k);
        else if (v.cap == 1) go<ANISO, NW, true, 1>(blocks, st, F, G, k);
        else go<ANISO, NW, true, 0>(blocks, st, F, G, k);
    } else {
        if (v.cap == 2) go<ANISO, NW, false, 2>(blocks, st, F, G, k);
        else if (v.cap == 1) go<ANISO, NW, false, 1>(blocks, st, F, G, k);
        else go<ANISO, NW, false, 0>(blocks, st, F, G, k);
    }
}

template <bool ANISO>
void go_aniso(const StepVariant& v, int blocks, cudaStream_t st, const Field<double>& F, const Geo<double>& G,
              const Coef<double>& k)
{
    if (v.nw == 2) go_nw<ANISO, 2>(v, blocks, st, F, G, k);
    else go_nw<ANISO, 4>(v, blocks, st, F, G, k);
}

template <bool ANISO, int NW, bool ZS, int CAP>
int occ()
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step<double, ANISO, false, NW, ZS, CAP>, NW * 32, 0) != cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}

template <bool ANISO, int NW>
int occ_nw(const StepVariant& v)
{
    if (v.zseam) return v.cap == 2 ? occ<ANISO, NW, true, 2>() : v.cap == 1 ? occ<ANISO, NW, true, 1>() : occ<ANISO, NW, true, 0>();
    return v.cap == 2 ? occ<ANISO, NW, false, 2>() : v.cap == 1 ? occ<ANISO, NW, false, 1>() : occ<ANISO, NW, false, 0>();
}

}  // namespace

int step_occupancy_f64(const StepVariant& v, bool aniso)
{
    if (aniso) return v.nw == 2 ? occ_nw<true, 2>(v) : occ_nw<true, 4>(v);
    return v.nw == 2 ? occ_nw<false, 2>(v) : occ_nw<false, 4>(v);
}

cudaError_t launch_step_f64(const StepVariant& v, bool aniso, int blocks, cudaStream_t st,
                            const Field<double>& F, const Geo<double>& G, const Coef<double>& k)
{
    if (aniso) go_aniso<true>(v, blocks, st, F, G, k);
    else go_aniso<false>(v, blocks, st, F, G, k);
    return cudaGetLastError();
}

}  // namespace sks
