// Table-driven FP64 exp and sincospi for the geodesic's point evaluation.
//
// On GB300 the FP64 pipe issues 2 lanes per clock per SM, so every FP64
// instruction in the per-point transcendentals costs the whole kernel.
// These follow Tang's table-driven method (P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989): reduce the argument against a table
// of correctly rounded values so that a short polynomial suffices, trading
// FP64 instructions for one L1-resident table load.  Measured on GB300
// (FP64-pipe slots per call, including ~5 of loop overhead, with tables of
// 64 and 256 entries): exp 21.5 -> 16.6; sincos + sincospi 66.8 -> 46.3.
// The tables now have 128 and 1024 entries (1 KB and 16 KB, L1-resident):
// one polynomial term fewer for exp and for each of sin and cos.  Accuracy
// against CUDA's own functions: <= 1 ulp (exp) and <= 2 ulp (sincospi),
// tested on the GPU by tests/test_gpu_math.py.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>

#include "fp32_math.cuh"

namespace raptor {

#include "math_tables.inc"

// 1/x: the hardware's approximate FP64 reciprocal (rcp.approx.ftz.f64,
// about 20 correct bits from the high word) refined by two Newton-Raphson
// steps y <- y + y (1 - x y), each of which squares the relative error;
// within an ulp of the correctly rounded quotient for normal x (tested on
// the GPU by tests/test_gpu_math.py).  Zero, infinity and NaN take the
// approximation itself (infinity, zero, NaN, as IEEE division gives them;
// subnormal x gives infinity).  Five FP64-pipe instructions and an integer
// test where an IEEE division takes about twice as many.
__device__ __forceinline__ double fast_rcp(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    const double y1 = fma(y, e, y);
    e = fma(-x, y1, 1.0);
    const double y2 = fma(y1, e, y1);
    const unsigned ex = (unsigned)__double2hiint(x) & 0x7ff00000u;
    return (ex == 0u || ex == 0x7ff00000u) ? y : y2;
}

// 1/x in the templated geodesic and dual code: fast_rcp for FP64, the
// full-range approximate division of fp32_math.cuh for FP32, the type's own
// division for the dual and double-float types.
template <class R>
__device__ __forceinline__ R recip(const R& x) {
    return 1.0 / x;
}
__device__ __forceinline__ double recip(double x) { return fast_rcp(x); }
__device__ __forceinline__ float recip(float x) { return fdiv(1.0f, x); }

// e^x for |x| < 512 (exp(x) outside).  x = (128 m + j) ln2/128 + r with
// |r| <= ln2/256: e^x = 2^m 2^(j/128) e^r, e^r - 1 by a degree-5 polynomial
// (truncation below 6e-19 relative).
__device__ __forceinline__ double fast_exp(double x) {
    const long long xb = __double_as_longlong(x);
    if (((xb >> 52) & 0x7ff) >= 0x408) return exp(x);  // |x| >= 512, inf, nan
    const double k128_ln2 = 184.6649652337873;         // 128 / ln 2
    const double ln2_128_hi = 0.0054152123481245725;   // ln 2 / 128, rounded
    const double ln2_128_lo = 1.8117553233174215e-19;  // ln 2 / 128 - hi
    const double shifter = 6755399441055744.0;         // 1.5 * 2^52: rounds to an integer in the low bits
    const double t = fma(x, k128_ln2, shifter);
    const int m = (int)(__double_as_longlong(t) & 0xffffffffll);
    const double md = t - shifter;
    double r = fma(-md, ln2_128_hi, x);
    r = fma(-md, ln2_128_lo, r);
    double p = 1.0 / 120.0;
    p = fma(p, r, 1.0 / 24.0);
    p = fma(p, r, 1.0 / 6.0);
    p = fma(p, r, 0.5);
    p = fma(p, r, 1.0);
    p = p * r;  // e^r - 1
    const double T = __ldg(&kExp2Table[m & 127]);
    const double v = fma(T, p, T);
    return __longlong_as_double(__double_as_longlong(v) + ((long long)(m >> 7) << 52));
}

// sin(pi x), cos(pi x) for |x| < 2^20.  x = n/512 + r with |r| <= 1/1024
// (r exact by Sterbenz); sin and cos of a = pi r by degree-5 / degree-4
// polynomials (truncation below 2e-19 and 1.2e-18), recombined with the
// table entry for n mod 1024 by the angle-addition formulas.
__device__ __forceinline__ void fast_sincospi(double x, double* s, double* c) {
    const double shifter = 6755399441055744.0;
    const double t = fma(x, 512.0, shifter);
    const int n = (int)(__double_as_longlong(t) & 0xffffffffll);
    const double nd = t - shifter;
    const double r = fma(nd, -0.001953125, x);  // x - n/512, exact
    const double a = r * CUDART_PI;
    const double a2 = a * a;
    const double ps = fma(a2, 1.0 / 120.0, -1.0 / 6.0) * a2;
    const double sa = fma(ps, a, a);                    // sin a
    const double cm1 = fma(a2, 1.0 / 24.0, -0.5) * a2;  // cos a - 1
    const double2 SC = __ldg(&kSinCosPiTable[n & 1023]);
    *s = fma(SC.x, cm1, fma(SC.y, sa, SC.x));
    *c = fma(SC.y, cm1, fma(-SC.x, sa, SC.y));
}

}  // namespace raptor
