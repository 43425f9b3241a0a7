// Double-float arithmetic ("DF") for the geodesic of the mixed-DF form.
//
// A DF value is the unevaluated sum hi + lo of two FP32 numbers with
// |lo| a few ulp(hi) or less: a 48-bit significand (relative rounding
// ~3.6e-15, against 1.1e-16 for FP64) with FP32's exponent range.  Neither
// products nor sums are renormalised: a product's lo stays below ~4 ulp(hi),
// a sum's is the exact error of its leading parts plus the operands' lo
// parts, which every operation here accepts as input.  Leaving products
// unnormalised saves 3 of a product's 7 instructions, sums 3 of 11.  A sum
// whose leading parts cancel keeps a lo larger than ulp(hi); its rounding
// then adds an error of the order of the one the cancellation already
// carries.  Renormalised values (df_norm, add_norm) are kept where a value
// accumulates over many steps (the photon state) or where its leading part
// is read alone (sin and cos of a point, the cell coordinate); comparisons
// and signs read hi + lo rounded to FP32, which has the sign of the exact
// value.  GB300 runs FP64 at
// 2 operations per clock per SM and FP32 at 128, so a DF operation built
// from 6-11 FP32 instructions costs the SM far less than one FP64
// instruction.  The algorithms are the classical error-free
// transformations: Knuth's two-sum, Dekker's fast two-sum, the FMA form of
// the exact product, and the double-length add / multiply / divide of
// Dekker (1971) in the variants of Hida, Li and Bailey's QD library (2001)
// paper; exp follows Tang's table method and sincospi the same 256-entry
// angle-addition table as fp64_math.cuh, both with DF tables from
// gen_math_tables.py.  Every FP32 operation is an explicitly rounded
// intrinsic, so the compiler can neither contract nor reorder them.
//
// Used only by ray_kernel_df.cuh.  The FP64 and mixed forms never see it.
#pragma once
#include <cuda_runtime.h>

#include "df_type.cuh"

namespace raptor {

// the DF overloads below must not hide the FP64 ones inside this namespace
using ::fabs;
using ::fma;
using ::fmax;
using ::fmin;

#include "df_tables.inc"

// ------------------------------------------------------------ conversions
__device__ __forceinline__ double df_to_double(DF a) { return (double)a.hi + (double)a.lo; }

// ------------------------------------------------- error-free transforms
__device__ __forceinline__ DF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ DF quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}

// ------------------------------------------------------------ arithmetic
__device__ __forceinline__ DF operator-(DF a) { return DF{-a.hi, -a.lo}; }

// sums: the exact sum of the leading parts, the lo parts added to its error
__device__ __forceinline__ DF operator+(DF a, DF b) {
    const DF s = two_sum(a.hi, b.hi);
    return DF{s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo))};
}
__device__ __forceinline__ DF add_f(DF a, float b) {
    const DF s = two_sum(a.hi, b);
    return DF{s.hi, __fadd_rn(s.lo, a.lo)};
}
__device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }

// |lo| <= ulp(hi)/2 again
__device__ __forceinline__ DF df_norm(DF a) { return quick_two_sum(a.hi, a.lo); }
// a renormalised sum (the photon state's updates)
__device__ __forceinline__ DF add_norm(DF a, DF b) { return df_norm(a + b); }
// the value rounded to FP32
__device__ __forceinline__ float df_value(DF a) { return __fadd_rn(a.hi, a.lo); }

// products: the exact product of the leading parts plus the cross terms,
// left unnormalised
__device__ __forceinline__ DF operator*(DF a, DF b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return DF{p, e};
}
__device__ __forceinline__ DF mul_f(DF a, float b) {
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return DF{p, e};
}

// 1/b by the hardware approximation refined once in FP32 (~2^-23).
__device__ __forceinline__ float rcp_refined(float b) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(b));
    return __fmul_rn(r, __fmaf_rn(-b, r, 2.0f));
}

// a / b: q1 = a / b in FP32, one DF correction (relative error ~2^-46).
__device__ __forceinline__ DF operator/(DF a, DF b) {
    const float rb = rcp_refined(df_value(b));
    const float q1 = __fmul_rn(df_value(a), rb);
    const float q2 = __fmul_rn(df_value(a - mul_f(b, q1)), rb);
    return quick_two_sum(q1, q2);
}

// ----------------------------------------------------- mixed with double
// These take compile-time constants (literals of the templated geodesic
// code).  Constants exact in FP32 take the cheaper FP32 path, powers of two
// an exact scaling; the tests on the constant fold away.
__device__ __forceinline__ bool df_pow2(float f) { return (__float_as_uint(f) & 0x007fffffu) == 0u && f != 0.0f; }

__device__ __forceinline__ DF operator*(double c, DF a) {
    const DF k = df_const(c);
    if (k.lo == 0.0f) {
        if (df_pow2(k.hi)) return DF{__fmul_rn(a.hi, k.hi), __fmul_rn(a.lo, k.hi)};
        return mul_f(a, k.hi);
    }
    return a * k;
}
__device__ __forceinline__ DF operator*(DF a, double c) { return c * a; }
__device__ __forceinline__ DF operator*(float c, DF a) { return mul_f(a, c); }
__device__ __forceinline__ DF operator*(DF a, float c) { return mul_f(a, c); }
__device__ __forceinline__ DF operator+(DF a, double c) {
    const DF k = df_const(c);
    return k.lo == 0.0f ? add_f(a, k.hi) : a + k;
}
__device__ __forceinline__ DF operator+(double c, DF a) { return a + c; }
__device__ __forceinline__ DF operator-(DF a, double c) { return a + (-c); }
__device__ __forceinline__ DF operator-(double c, DF a) { return (-a) + c; }
__device__ __forceinline__ DF operator/(double c, DF a) { return df_const(c) / a; }
__device__ __forceinline__ DF operator/(DF a, double c) { return a / df_const(c); }

__device__ __forceinline__ DF fma(DF a, DF b, DF c) { return a * b + c; }
__device__ __forceinline__ DF fma(DF a, DF b, double c) { return a * b + c; }

// ----------------------------------------------------------- comparisons
// by the sign of the difference rounded to FP32
__device__ __forceinline__ bool operator<(DF a, DF b) { return df_value(a - b) < 0.0f; }
__device__ __forceinline__ bool operator>(DF a, DF b) { return b < a; }
__device__ __forceinline__ bool operator<=(DF a, DF b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(DF a, DF b) { return !(a < b); }
__device__ __forceinline__ bool operator==(DF a, DF b) { return df_value(a - b) == 0.0f; }
__device__ __forceinline__ bool operator!=(DF a, DF b) { return !(a == b); }
__device__ __forceinline__ bool operator==(DF a, double c) { return a == df_const(c); }
__device__ __forceinline__ DF fabs(DF a) { return df_value(a) < 0.0f ? -a : a; }
__device__ __forceinline__ DF fmin(DF a, DF b) { return (b < a) ? b : a; }
__device__ __forceinline__ DF fmax(DF a, DF b) { return (a < b) ? b : a; }

// ------------------------------------------------------- transcendentals
// e^x for |x| < 40 (the MKS x1 = ln r of a ray).  x = (64 m + j) ln2/64 + r,
// |r| <= ln2/128, r reduced against a three-part ln2/64 whose first part has
// 12 significant bits (m ln2/64 exact for |m| < 2^12).  e^r - 1 =
// r + r^2/2 (DF) + r^3 (1/6 + r/24 + r^2/120 + r^3/720) (FP32, below 3e-8).
__device__ __forceinline__ DF fast_exp(DF x) {
    const float nf = rintf(__fmul_rn(x.hi, 92.33248261689366f));  // 64 / ln 2
    const int m = (int)nf;
    DF r = two_sum(__fmaf_rn(-nf, kLn2by64_1, x.hi), x.lo);  // x.hi - m L1 is exact
    const float p2 = __fmul_rn(nf, kLn2by64_2);
    r = r - DF{p2, __fmaf_rn(nf, kLn2by64_2, -p2)};
    r = add_f(r, __fmul_rn(-nf, kLn2by64_3));
    const float q = r.hi;
    float t = __fmaf_rn(q, 1.0f / 720.0f, 1.0f / 120.0f);
    t = __fmaf_rn(t, q, 1.0f / 24.0f);
    t = __fmaf_rn(t, q, 1.0f / 6.0f);
    t = __fmul_rn(__fmul_rn(t, q), __fmul_rn(q, q));
    const DF r2 = r * r;
    const DF em1 = add_f(r + DF{__fmul_rn(r2.hi, 0.5f), __fmul_rn(r2.lo, 0.5f)}, t);
    const float2 T2 = __ldg(&kExp2TableDF[m & 63]);
    const DF T{T2.x, T2.y};
    const DF v = T + T * em1;
    const float sc = __int_as_float(((m >> 6) + 127) << 23);  // 2^(m/64 integer part)
    return DF{__fmul_rn(v.hi, sc), __fmul_rn(v.lo, sc)};
}

// sin(pi x), cos(pi x) for |x| < 2^20.  x = n/128 + r, |r| <= 1/256
// (x.hi - n/128 exact), a = pi r: sin a = a - a (a^2/6 - a^4/120 + ...),
// cos a - 1 = -a^2/2 + a^4/24 - ... with the a^2 terms in DF and the rest in
// FP32, recombined with the table entry for n mod 256.
__device__ __forceinline__ void fast_sincospi(DF x, DF* s, DF* c) {
    const float nf = rintf(__fmul_rn(x.hi, 128.0f));
    const int n = (int)nf;
    const DF r = two_sum(__fmaf_rn(nf, -0.0078125f, x.hi), x.lo);
    const DF a = r * DF{kPiDFhi, kPiDFlo};
    const DF a2 = a * a;
    const float a2f = a2.hi;
    const float a4 = __fmul_rn(a2f, a2f);
    const float srest = __fmul_rn(a4, __fmaf_rn(a2f, 1.0f / 5040.0f, -1.0f / 120.0f));
    const DF q = add_f(a2 * DF{kSixthDFhi, kSixthDFlo}, srest);  // a^2/6 - a^4/120 + a^6/5040
    const DF sa = a - a * q;
    const float crest = __fmul_rn(a4, __fmaf_rn(a2f, -1.0f / 720.0f, 1.0f / 24.0f));
    const DF cm1 = add_f(DF{__fmul_rn(a2.hi, -0.5f), __fmul_rn(a2.lo, -0.5f)}, crest);
    const float4 T = __ldg(&kSinCosPiTableDF[n & 255]);
    const DF S{T.x, T.y}, C{T.z, T.w};
    *s = add_norm(S, S * cm1 + C * sa);
    *c = add_norm(C, C * cm1 - S * sa);
}

// The photon state after a step (ray_kernel.cuh), renormalised so that its
// error does not grow over the ray's steps; by two-sum, which is exact for
// any hi and lo (a momentum component through zero leaves |lo| > |hi|).
__device__ __forceinline__ DF renorm(DF a) { return two_sum(a.hi, a.lo); }

// trunc toward zero of hi + lo (the reference's (int) cast in Xtoij)
__device__ __forceinline__ int df_trunc(DF x) {
    const DF t = two_sum(x.hi, x.lo);
    int i = (int)t.hi;
    if ((float)i == t.hi) {
        if (t.hi > 0.0f && t.lo < 0.0f) i -= 1;
        else if (t.hi < 0.0f && t.lo > 0.0f) i += 1;
    }
    return i;
}

// A stage derivative times its RK weight, a power of two: two exact
// multiplies.
__device__ __forceinline__ DF stage_scale(DF f, float w) { return DF{__fmul_rn(f.hi, w), __fmul_rn(f.lo, w)}; }

// RK stage weights (1/2, 1, 2) in FP32 for DF states: exact, and a DF times
// an FP32 power of two is two multiplies.
template <>
struct StageWeight<DF> {
    using type = float;
};

}  // namespace raptor
