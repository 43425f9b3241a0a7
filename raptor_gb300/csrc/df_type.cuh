// The double-float value type (arithmetic in df64.cuh) and the per-image
// constants the mixed-DF geodesic reads, kept apart from the arithmetic so
// that DevImage can hold them.
#pragma once
#include <cuda_runtime.h>

namespace raptor {

// hi + lo, two FP32 numbers with |lo| <= ulp(hi)/2
struct DF {
    float hi, lo;
};

// From a double: hi = the double rounded to FP32, lo = the remainder rounded
// to FP32.  With a literal argument the whole expression folds at compile
// time; at run time it costs FP64 instructions, so kernels take DF copies of
// their constants from the host.
__host__ __device__ __forceinline__ DF df_const(double c) {
    const float h = (float)c;
    return DF{h, (float)(c - (double)h)};
}

// A plain double constant as scalar type T (dual.cuh): a cast, or the DF
// split for DF.
template <class T>
__host__ __device__ inline T scalar_cast(double x) {
    return (T)x;
}
template <>
__host__ __device__ inline DF scalar_cast<DF>(double x) {
    return df_const(x);
}

// The photon state after an RK step (ray_kernel.cuh): the value itself for
// FP64; the DF overload (df64.cuh) renormalises it, the dual-number one
// (dual.cuh) its value.
template <class R>
__device__ __forceinline__ R renorm(const R& x) {
    return x;
}

// Geo (kerr_mks.cuh) with DF fields
struct GeoDF {
    DF a, a2, hslope, R0;
    DF one_m_h, th_coef;
};

// Type of the RK stage weights for a state type: FP64 constants for double
// and dual numbers, FP32 for DF (df64.cuh).
template <class R>
struct StageWeight {
    using type = double;
};

}  // namespace raptor
