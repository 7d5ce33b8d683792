// Compile-time variants of the step kernels (anisotropy, warps per CTA, band
// seams, register cap) reached from a run-time StepVariant.  A visitor is a
// struct with `template <bool ANISO, int NW, bool ZS, int CAP> R run()`.
#pragma once
#include "sks_kernels.cuh"

namespace sks {

template <bool A, int NW, bool ZS, typename V>
auto visit_cap(const StepVariant& v, V& vis)
{
    if (v.cap == 2) return vis.template run<A, NW, ZS, 2>();
    if (v.cap == 1) return vis.template run<A, NW, ZS, 1>();
    return vis.template run<A, NW, ZS, 0>();
}

template <bool A, int NW, typename V>
auto visit_zs(const StepVariant& v, V& vis)
{
    return v.zseam ? visit_cap<A, NW, true>(v, vis) : visit_cap<A, NW, false>(v, vis);
}

template <bool A, typename V>
auto visit_nw(const StepVariant& v, V& vis)
{
    return v.nw == 2 ? visit_zs<A, 2>(v, vis) : visit_zs<A, 4>(v, vis);
}

template <typename V>
auto visit_variant(const StepVariant& v, bool aniso, V& vis)
{
    return aniso ? visit_nw<true>(v, vis) : visit_nw<false>(v, vis);
}

// resident CTAs per SM of a kernel (at least 1)
template <typename K>
int occupancy_of(K kernel, int threads)
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, 0) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

}  // namespace sks
