// FP32 quotient and square root for the FP32 transfer samples (the mixed
// and mixed-DF forms and their adjoints), and the double -> float rounding
// those samples and the mixed adjoint's tangents use (f32_of, below).
//
// CUDA's IEEE-rounded FP32 division and square root carry a branch to an
// out-of-line slow path at every use.  The samples run between geodesic
// steps whose loop already fills the instruction cache; with some twenty
// such operations the mixed-DF kernel's sample was 6 % of its instructions
// and 30 % of its time.  The PTX instructions div.full.f32 and
// sqrt.approx.f32 have no slow path: with them the 1024x1024 mixed-DF render
// went from 79.5 to 69 ms.  On the GPU they are within 2 ulp of the IEEE
// quotient (subnormal results included) and 1 ulp of the IEEE square root,
// with IEEE's special values (tests/test_gpu_math.py): a few ulp in a
// transfer whose tolerance is 1e-4 in flux.
//
// Templated code (the sample's fluid, shared with FP32 duals) calls fdiv and
// fsqrt; for other types they are the type's own division and sqrt.
#pragma once
#include <cuda_runtime.h>

namespace raptor {

__device__ __forceinline__ float fdiv(float a, float b) {
    float q;
    asm("div.full.f32 %0, %1, %2;" : "=f"(q) : "f"(a), "f"(b));
    return q;
}
__device__ __forceinline__ float fsqrt(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// double -> float on the integer pipes, for the FP32 tangents of FP64 values
// (the mixed adjoint's dual products convert both factors' values).  The
// hardware conversion issues to the FP64 pipe, one warp instruction per 16
// SM cycles on this part: there the conversions were 8.7e9 of the mixed
// adjoint's 23e9 FP64-pipe thread instructions.  This one rebiases the
// exponent and rounds the significand to nearest, ties away from zero.  It
// equals the IEEE conversion for magnitudes from 2^-126 up, except at exact
// ties (one ulp apart there); it gives a signed zero below 2^-126, where
// the IEEE conversion gives subnormals, and a signed infinity for NaN.
__device__ __forceinline__ float f32_of(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    // exponent and 23 significand bits, the exponent's low 9 bits at 31:23;
    // rebiased 1023 -> 127 (-0x380 = +0x80 in 9 bits), rounded on the 24th
    unsigned f = __funnelshift_l(lo, hi, 3) + 0x40000000u + ((lo >> 28) & 1u);
    // outside [2^-126, 2^128): zero below, infinity above (NaN included)
    const unsigned e2 = hi << 1;
    if (e2 - 0x70200000u >= 0x1fc00000u) f = e2 < 0x70200000u ? 0u : 0x7f800000u;
    return __uint_as_float(f | (hi & 0x80000000u));
}

// a double in the working type T: f32_of for FP32, else the type's own
// conversion
template <class T>
__device__ __forceinline__ T narrow(double x) {
    return (T)x;
}
template <>
__device__ __forceinline__ float narrow<float>(double x) {
    return f32_of(x);
}

template <class T>
__device__ __forceinline__ T fdiv(const T& a, const T& b) {
    return a / b;
}
template <class T>
__device__ __forceinline__ T fsqrt(const T& x) {
    return sqrt(x);
}

}  // namespace raptor
