// Forward-mode dual numbers for the adjoint (VJP) kernels: a value of type
// T and N directional derivatives of type TD (default T) - double for the
// FP64 adjoint; a double value with FP32 tangents for the mixed adjoint; a DF
// value (df64.cuh) with FP32 tangents for the mixed-DF adjoint; FP32 values
// and tangents for both mixed samples - with the arithmetic and the libm
// functions the imaging path uses.  Comparisons act on the value, so every
// branch of the primal computation is taken as the primal takes it
// (derivatives of the taken branch).  Plain double constants are converted
// to T / TD first (scalar_cast), which folds at compile time for literals;
// values enter tangent expressions through tan_cast (the leading FP32 part
// of a DF value; an FP64 value rounded on the integer pipes by f32_of).
// With T = TD = double both are the identity.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>

#include <type_traits>

#include "df_type.cuh"
#include "fp64_math.cuh"

namespace raptor {

// the plain versions stay visible next to the Dual overloads below
using ::cbrt;
using ::exp;
using ::expm1;
using ::fabs;
using ::fma;
using ::fmax;
using ::fmin;
using ::log;
using ::log1p;
using ::pow;
using ::rsqrt;
using ::sincos;
using ::sincospi;
using ::sqrt;

// a value in the tangent type
template <class TD, class T>
struct TanCast {
    __host__ __device__ static TD of(const T& x) { return (TD)x; }
};
template <>
struct TanCast<float, DF> {
    __host__ __device__ static float of(const DF& x) { return x.hi; }
};
// off the FP64 pipe (fp32_math.cuh f32_of)
template <>
struct TanCast<float, double> {
    __device__ static float of(const double& x) { return f32_of(x); }
};
template <class TD, class T>
__host__ __device__ inline TD tan_cast(const T& x) {
    return TanCast<TD, T>::of(x);
}

template <int N, class T = double, class TD = T>
struct Dual {
    T v;
    TD d[N];
    __host__ __device__ Dual() {}
    __host__ __device__ Dual(T x) : v(x) {
#pragma unroll
        for (int i = 0; i < N; ++i) d[i] = scalar_cast<TD>(0.0);
    }
};

// the state after an RK step: the value renormalised as its type does it
template <int N, class T, class TD>
__device__ __forceinline__ Dual<N, T, TD> renorm(const Dual<N, T, TD>& x) {
    Dual<N, T, TD> r = x;
    r.v = renorm(x.v);
    return r;
}

// enabled for scalar types other than double (whose mixed operators are the
// double ones below)
template <class T>
using if_not_double = typename std::enable_if<!std::is_same<T, double>::value, int>::type;
// enabled for scalar types other than double and float (DF)
template <class T>
using if_df_like = typename std::enable_if<!std::is_same<T, double>::value && !std::is_same<T, float>::value, int>::type;

template <int N, class T, class TD>
__host__ __device__ inline Dual<N, T, TD> operator+(const Dual<N, T, TD>& a, const Dual<N, T, TD>& b) {
    Dual<N, T, TD> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int N, class T, class TD>
__host__ __device__ inline Dual<N, T, TD> operator-(const Dual<N, T, TD>& a, const Dual<N, T, TD>& b) {
    Dual<N, T, TD> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int N, class T, class TD>
__host__ __device__ inline Dual<N, T, TD> operator-(const Dual<N, T, TD>& a) {
    Dual<N, T, TD> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
    return r;
}
template <int N, class T, class TD>
__host__ __device__ inline Dual<N, T, TD> operator*(const Dual<N, T, TD>& a, const Dual<N, T, TD>& b) {
    Dual<N, T, TD> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * tan_cast<TD>(b.v) + tan_cast<TD>(a.v) * b.d[i];
    return r;
}
template <int N, class T, class TD>
__host__ __device__ inline Dual<N, T, TD> operator/(const Dual<N, T, TD>& a, const Dual<N, T, TD>& b) {
    const T ib = recip(b.v);
    Dual<N, T, TD> r;
    r.v = a.v * ib;
    const TD rv = tan_cast<TD>(r.v), ibd = tan_cast<TD>(ib);
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - rv * b.d[i]) * ibd;
    return r;
}

// mixed with plain doubles
template <int N, class T, class TD>
__host__ __device__ inline Dual<N, T, TD> operator+(const Dual<N, T, TD>& a, double b) {
    Dual<N, T, TD> r = a;
    r.v = r.v + scalar_cast<T>(b);
    return r;
}
template <int N, class T, class TD> __host__ __device__ inline Dual<N, T, TD> operator+(double a, const Dual<N, T, TD>& b) { return b + a; }
template <int N, class T, class TD>
__host__ __device__ inline Dual<N, T, TD> operator-(const Dual<N, T, TD>& a, double b) {
    Dual<N, T, TD> r = a;
    r.v = r.v - scalar_cast<T>(b);
    return r;
}
template <int N, class T, class TD> __host__ __device__ inline Dual<N, T, TD> operator-(double a, const Dual<N, T, TD>& b) { return -(b - a); }
template <int N, class T, class TD>
__host__ __device__ inline Dual<N, T, TD> operator*(const Dual<N, T, TD>& a, double b) {
    const T bb = scalar_cast<T>(b);
    // FP64 values with FP32 tangents: runtime constants (the geometry's) off
    // the FP64 pipe, as tan_cast
    const TD bd = std::is_same<T, double>::value ? tan_cast<TD>(b) : scalar_cast<TD>(b);
    Dual<N, T, TD> r;
    r.v = a.v * bb;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * bd;
    return r;
}
template <int N, class T, class TD> __host__ __device__ inline Dual<N, T, TD> operator*(double a, const Dual<N, T, TD>& b) { return b * a; }
template <int N, class T, class TD> __host__ __device__ inline Dual<N, T, TD> operator/(const Dual<N, T, TD>& a, double b) { return a * (1.0 / b); }
template <int N, class T, class TD> __host__ __device__ inline Dual<N, T, TD> operator/(double a, const Dual<N, T, TD>& b) { return Dual<N, T, TD>(scalar_cast<T>(a)) / b; }

// mixed with plain values of the scalar type (T other than double)
template <int N, class T, class TD, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T, TD> operator*(const Dual<N, T, TD>& a, const T& b) {
    Dual<N, T, TD> r;
    r.v = a.v * b;
    const TD bd = tan_cast<TD>(b);
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * bd;
    return r;
}
template <int N, class T, class TD, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T, TD> operator*(const T& a, const Dual<N, T, TD>& b) { return b * a; }
template <int N, class T, class TD, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T, TD> operator+(const Dual<N, T, TD>& a, const T& b) {
    Dual<N, T, TD> r = a;
    r.v = r.v + b;
    return r;
}
template <int N, class T, class TD, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T, TD> operator+(const T& a, const Dual<N, T, TD>& b) { return b + a; }
template <int N, class T, class TD, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T, TD> operator-(const Dual<N, T, TD>& a, const T& b) {
    Dual<N, T, TD> r = a;
    r.v = r.v - b;
    return r;
}
template <int N, class T, class TD, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T, TD> operator-(const T& a, const Dual<N, T, TD>& b) { return -(b - a); }
// by an FP32 weight (the RK stage weights of a DF state)
template <int N, class T, class TD, if_df_like<T> = 0>
__host__ __device__ inline Dual<N, T, TD> operator*(const Dual<N, T, TD>& a, float b) {
    Dual<N, T, TD> r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
    return r;
}

template <int N, class T, class TD> __host__ __device__ inline Dual<N, T, TD>& operator+=(Dual<N, T, TD>& a, const Dual<N, T, TD>& b) { a = a + b; return a; }
template <int N, class T, class TD> __host__ __device__ inline Dual<N, T, TD>& operator-=(Dual<N, T, TD>& a, const Dual<N, T, TD>& b) { a = a - b; return a; }
template <int N, class T, class TD> __host__ __device__ inline Dual<N, T, TD>& operator*=(Dual<N, T, TD>& a, const Dual<N, T, TD>& b) { a = a * b; return a; }

#define RAPTOR_DUAL_CMP(OP)                                                                                    \
    template <int N, class T, class TD>                                                                                  \
    __host__ __device__ inline bool operator OP(const Dual<N, T, TD>& a, const Dual<N, T, TD>& b) { return a.v OP b.v; } \
    template <int N, class T, class TD>                                                                                  \
    __host__ __device__ inline bool operator OP(const Dual<N, T, TD>& a, double b) { return a.v OP scalar_cast<T>(b); } \
    template <int N, class T, class TD>                                                                                  \
    __host__ __device__ inline bool operator OP(double a, const Dual<N, T, TD>& b) { return scalar_cast<T>(a) OP b.v; }
RAPTOR_DUAL_CMP(<)
RAPTOR_DUAL_CMP(>)
RAPTOR_DUAL_CMP(<=)
RAPTOR_DUAL_CMP(>=)
RAPTOR_DUAL_CMP(==)
RAPTOR_DUAL_CMP(!=)
#undef RAPTOR_DUAL_CMP

// f(a) with f'(a) given
template <int N, class T, class TD>
__host__ __device__ inline Dual<N, T, TD> chain(const Dual<N, T, TD>& a, T f, T fp) {
    Dual<N, T, TD> r;
    r.v = f;
    const TD fpd = tan_cast<TD>(fp);
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = fpd * a.d[i];
    return r;
}

// At 0 the argument's tangents are 0 too wherever it is identically 0 (a
// field-free region: b^2 = 0), so the tangent is taken as 0 there rather
// than 0.5/0 * 0 = NaN.
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> sqrt(const Dual<N, T, TD>& a) {
    const T s = fsqrt(a.v);
    return chain(a, s, s > scalar_cast<T>(0.0) ? scalar_cast<T>(0.5) * recip(s) : scalar_cast<T>(0.0));
}
// 1/sqrt(x) of an FP64 dual, its tangent -r^3/2 without a division
template <int N> __device__ inline Dual<N, double, double> rsqrt(const Dual<N, double, double>& a) {
    const double r = rsqrt(a.v);
    return chain(a, r, -0.5 * r * r * r);
}
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> log1p(const Dual<N, T, TD>& a) {
    return chain(a, log1p(a.v), recip(scalar_cast<T>(1.0) + a.v));
}
// a^b for a constant exponent b
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> pow(const Dual<N, T, TD>& a, double b) {
    const T p = pow(a.v, scalar_cast<T>(b));
    return chain(a, p, scalar_cast<T>(b) * p * recip(a.v));
}
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> exp(const Dual<N, T, TD>& a) { const T e = exp(a.v); return chain(a, e, e); }
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> log(const Dual<N, T, TD>& a) { return chain(a, log(a.v), scalar_cast<T>(1.0) / a.v); }
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> cbrt(const Dual<N, T, TD>& a) {
    const T c = cbrt(a.v);
    return chain(a, c, c != scalar_cast<T>(0.0) ? recip(scalar_cast<T>(3.0) * c * c) : scalar_cast<T>(0.0));
}
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> expm1(const Dual<N, T, TD>& a) { return chain(a, expm1(a.v), exp(a.v)); }
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> fabs(const Dual<N, T, TD>& a) { return a.v < scalar_cast<T>(0.0) ? -a : a; }
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> fmin(const Dual<N, T, TD>& a, const Dual<N, T, TD>& b) { return b.v < a.v ? b : a; }
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> fmax(const Dual<N, T, TD>& a, const Dual<N, T, TD>& b) { return b.v > a.v ? b : a; }
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> fmax(const Dual<N, T, TD>& a, double b) {
    return scalar_cast<T>(b) > a.v ? Dual<N, T, TD>(scalar_cast<T>(b)) : a;
}
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> fma(const Dual<N, T, TD>& a, const Dual<N, T, TD>& b, const Dual<N, T, TD>& c) { return a * b + c; }
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> fma(double a, const Dual<N, T, TD>& b, double c) { return a * b + c; }
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> fma(const Dual<N, T, TD>& a, const Dual<N, T, TD>& b, double c) { return a * b + c; }
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> fma(double a, const Dual<N, T, TD>& b, const Dual<N, T, TD>& c) { return a * b + c; }
template <int N, class T, class TD, if_not_double<T> = 0>
__device__ inline Dual<N, T, TD> fma(const T& a, const Dual<N, T, TD>& b, const Dual<N, T, TD>& c) { return a * b + c; }
template <int N, class T, class TD, if_not_double<T> = 0>
__device__ inline Dual<N, T, TD> fma(const T& a, const Dual<N, T, TD>& b, double c) { return a * b + c; }
template <int N, class T, class TD>
__device__ inline void sincos(const Dual<N, T, TD>& a, Dual<N, T, TD>* s, Dual<N, T, TD>* c) {
    T sv, cv;
    sincos(a.v, &sv, &cv);
    *s = chain(a, sv, cv);
    *c = chain(a, cv, -sv);
}
template <int N, class T, class TD>
__device__ inline void sincospi(const Dual<N, T, TD>& a, Dual<N, T, TD>* s, Dual<N, T, TD>* c) {
    T sv, cv;
    sincospi(a.v, &sv, &cv);
    *s = chain(a, sv, scalar_cast<T>(CUDART_PI) * cv);
    *c = chain(a, cv, -(scalar_cast<T>(CUDART_PI) * sv));
}
// the engine's table-driven point transcendentals (fp64_math.cuh, df64.cuh)
template <int N, class T, class TD> __device__ inline Dual<N, T, TD> fast_exp(const Dual<N, T, TD>& a) {
    const T e = fast_exp(a.v);
    return chain(a, e, e);
}
template <int N, class T, class TD>
__device__ inline void fast_sincospi(const Dual<N, T, TD>& a, Dual<N, T, TD>* s, Dual<N, T, TD>* c) {
    T sv, cv;
    fast_sincospi(a.v, &sv, &cv);
    *s = chain(a, sv, scalar_cast<T>(CUDART_PI) * cv);
    *c = chain(a, cv, -(scalar_cast<T>(CUDART_PI) * sv));
}

// RK stage weights for dual states follow their scalar type
template <int N, class T, class TD>
struct StageWeight<Dual<N, T, TD>> {
    using type = typename StageWeight<T>::type;
};

}  // namespace raptor
