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

// Degrees other than 4 (3, 5, 6) compile the 4-warp variants with register
// cap 0 or 1 only (the tunings the solver allows for them).
template <bool A, bool ZS, typename V>
auto visit_deg_cap(const StepVariant& v, V& vis)
{
    return v.cap ? vis.template run<A, 4, ZS, 1>() : vis.template run<A, 4, ZS, 0>();
}

template <int DEG, typename V>
auto visit_deg(const StepVariant& v, bool aniso, V& vis)
{
    if constexpr (DEG != N) {
        if (aniso) return v.zseam ? visit_deg_cap<true, true>(v, vis) : visit_deg_cap<true, false>(v, vis);
        return v.zseam ? visit_deg_cap<false, true>(v, vis) : visit_deg_cap<false, false>(v, vis);
    } else {
        return visit_variant(v, aniso, vis);
    }
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
