// Forward-mode dual numbers for the adjoint (VJP) kernels: a value and N
// directional derivatives of a scalar type T - double for the FP64 adjoint,
// DF (df64.cuh) and float for the mixed-DF adjoint - with the arithmetic and
// the libm functions the imaging path uses.  Comparisons act on the value,
// so every branch of the primal computation is taken as the primal takes it
// (derivatives of the taken branch).  Plain double constants are converted
// to T first (scalar_cast), which folds at compile time for literals and is
// the identity for T = double.
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
using ::sincos;
using ::sincospi;
using ::sqrt;

template <int N, class T = double>
struct Dual {
    T v;
    T d[N];
    __host__ __device__ Dual() {}
    __host__ __device__ Dual(T x) : v(x) {
#pragma unroll
        for (int i = 0; i < N; ++i) d[i] = scalar_cast<T>(0.0);
    }
};

// enabled for scalar types other than double (whose mixed operators are the
// double ones below)
template <class T>
using if_not_double = typename std::enable_if<!std::is_same<T, double>::value, int>::type;
// enabled for scalar types other than double and float (DF)
template <class T>
using if_df_like = typename std::enable_if<!std::is_same<T, double>::value && !std::is_same<T, float>::value, int>::type;

template <int N, class T>
__host__ __device__ inline Dual<N, T> operator+(const Dual<N, T>& a, const Dual<N, T>& b) {
    Dual<N, T> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int N, class T>
__host__ __device__ inline Dual<N, T> operator-(const Dual<N, T>& a, const Dual<N, T>& b) {
    Dual<N, T> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int N, class T>
__host__ __device__ inline Dual<N, T> operator-(const Dual<N, T>& a) {
    Dual<N, T> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
    return r;
}
template <int N, class T>
__host__ __device__ inline Dual<N, T> operator*(const Dual<N, T>& a, const Dual<N, T>& b) {
    Dual<N, T> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <int N, class T>
__host__ __device__ inline Dual<N, T> operator/(const Dual<N, T>& a, const Dual<N, T>& b) {
    const T ib = scalar_cast<T>(1.0) / b.v;
    Dual<N, T> r;
    r.v = a.v * ib;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
    return r;
}

// mixed with plain doubles
template <int N, class T>
__host__ __device__ inline Dual<N, T> operator+(const Dual<N, T>& a, double b) {
    Dual<N, T> r = a;
    r.v = r.v + scalar_cast<T>(b);
    return r;
}
template <int N, class T> __host__ __device__ inline Dual<N, T> operator+(double a, const Dual<N, T>& b) { return b + a; }
template <int N, class T>
__host__ __device__ inline Dual<N, T> operator-(const Dual<N, T>& a, double b) {
    Dual<N, T> r = a;
    r.v = r.v - scalar_cast<T>(b);
    return r;
}
template <int N, class T> __host__ __device__ inline Dual<N, T> operator-(double a, const Dual<N, T>& b) { return -(b - a); }
template <int N, class T>
__host__ __device__ inline Dual<N, T> operator*(const Dual<N, T>& a, double b) {
    const T bb = scalar_cast<T>(b);
    Dual<N, T> r;
    r.v = a.v * bb;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * bb;
    return r;
}
template <int N, class T> __host__ __device__ inline Dual<N, T> operator*(double a, const Dual<N, T>& b) { return b * a; }
template <int N, class T> __host__ __device__ inline Dual<N, T> operator/(const Dual<N, T>& a, double b) { return a * (1.0 / b); }
template <int N, class T> __host__ __device__ inline Dual<N, T> operator/(double a, const Dual<N, T>& b) { return Dual<N, T>(scalar_cast<T>(a)) / b; }

// mixed with plain values of the scalar type (T other than double)
template <int N, class T, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T> operator*(const Dual<N, T>& a, const T& b) {
    Dual<N, T> r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
    return r;
}
template <int N, class T, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T> operator*(const T& a, const Dual<N, T>& b) { return b * a; }
template <int N, class T, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T> operator+(const Dual<N, T>& a, const T& b) {
    Dual<N, T> r = a;
    r.v = r.v + b;
    return r;
}
template <int N, class T, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T> operator+(const T& a, const Dual<N, T>& b) { return b + a; }
template <int N, class T, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T> operator-(const Dual<N, T>& a, const T& b) {
    Dual<N, T> r = a;
    r.v = r.v - b;
    return r;
}
template <int N, class T, if_not_double<T> = 0>
__host__ __device__ inline Dual<N, T> operator-(const T& a, const Dual<N, T>& b) { return -(b - a); }
// by an FP32 weight (the RK stage weights of a DF state)
template <int N, class T, if_df_like<T> = 0>
__host__ __device__ inline Dual<N, T> operator*(const Dual<N, T>& a, float b) {
    Dual<N, T> r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
    return r;
}

template <int N, class T> __host__ __device__ inline Dual<N, T>& operator+=(Dual<N, T>& a, const Dual<N, T>& b) { a = a + b; return a; }
template <int N, class T> __host__ __device__ inline Dual<N, T>& operator-=(Dual<N, T>& a, const Dual<N, T>& b) { a = a - b; return a; }
template <int N, class T> __host__ __device__ inline Dual<N, T>& operator*=(Dual<N, T>& a, const Dual<N, T>& b) { a = a * b; return a; }

#define RAPTOR_DUAL_CMP(OP)                                                                                    \
    template <int N, class T>                                                                                  \
    __host__ __device__ inline bool operator OP(const Dual<N, T>& a, const Dual<N, T>& b) { return a.v OP b.v; } \
    template <int N, class T>                                                                                  \
    __host__ __device__ inline bool operator OP(const Dual<N, T>& a, double b) { return a.v OP scalar_cast<T>(b); } \
    template <int N, class T>                                                                                  \
    __host__ __device__ inline bool operator OP(double a, const Dual<N, T>& b) { return scalar_cast<T>(a) OP b.v; }
RAPTOR_DUAL_CMP(<)
RAPTOR_DUAL_CMP(>)
RAPTOR_DUAL_CMP(<=)
RAPTOR_DUAL_CMP(>=)
RAPTOR_DUAL_CMP(==)
RAPTOR_DUAL_CMP(!=)
#undef RAPTOR_DUAL_CMP

// f(a) with f'(a) given
template <int N, class T>
__host__ __device__ inline Dual<N, T> chain(const Dual<N, T>& a, T f, T fp) {
    Dual<N, T> r;
    r.v = f;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = fp * a.d[i];
    return r;
}

// At 0 the argument's tangents are 0 too wherever it is identically 0 (a
// field-free region: b^2 = 0), so the tangent is taken as 0 there rather
// than 0.5/0 * 0 = NaN.
template <int N, class T> __device__ inline Dual<N, T> sqrt(const Dual<N, T>& a) {
    const T s = sqrt(a.v);
    return chain(a, s, s > scalar_cast<T>(0.0) ? scalar_cast<T>(0.5) / s : scalar_cast<T>(0.0));
}
template <int N, class T> __device__ inline Dual<N, T> exp(const Dual<N, T>& a) { const T e = exp(a.v); return chain(a, e, e); }
template <int N, class T> __device__ inline Dual<N, T> log(const Dual<N, T>& a) { return chain(a, log(a.v), scalar_cast<T>(1.0) / a.v); }
template <int N, class T> __device__ inline Dual<N, T> cbrt(const Dual<N, T>& a) {
    const T c = cbrt(a.v);
    return chain(a, c, c != scalar_cast<T>(0.0) ? scalar_cast<T>(1.0) / (scalar_cast<T>(3.0) * c * c) : scalar_cast<T>(0.0));
}
template <int N, class T> __device__ inline Dual<N, T> expm1(const Dual<N, T>& a) { return chain(a, expm1(a.v), exp(a.v)); }
template <int N, class T> __device__ inline Dual<N, T> fabs(const Dual<N, T>& a) { return a.v < scalar_cast<T>(0.0) ? -a : a; }
template <int N, class T> __device__ inline Dual<N, T> fmin(const Dual<N, T>& a, const Dual<N, T>& b) { return b.v < a.v ? b : a; }
template <int N, class T> __device__ inline Dual<N, T> fmax(const Dual<N, T>& a, const Dual<N, T>& b) { return b.v > a.v ? b : a; }
template <int N, class T> __device__ inline Dual<N, T> fmax(const Dual<N, T>& a, double b) {
    return scalar_cast<T>(b) > a.v ? Dual<N, T>(scalar_cast<T>(b)) : a;
}
template <int N, class T> __device__ inline Dual<N, T> fma(const Dual<N, T>& a, const Dual<N, T>& b, const Dual<N, T>& c) { return a * b + c; }
template <int N, class T> __device__ inline Dual<N, T> fma(double a, const Dual<N, T>& b, double c) { return a * b + c; }
template <int N, class T> __device__ inline Dual<N, T> fma(const Dual<N, T>& a, const Dual<N, T>& b, double c) { return a * b + c; }
template <int N, class T> __device__ inline Dual<N, T> fma(double a, const Dual<N, T>& b, const Dual<N, T>& c) { return a * b + c; }
template <int N, class T, if_not_double<T> = 0>
__device__ inline Dual<N, T> fma(const T& a, const Dual<N, T>& b, const Dual<N, T>& c) { return a * b + c; }
template <int N, class T, if_not_double<T> = 0>
__device__ inline Dual<N, T> fma(const T& a, const Dual<N, T>& b, double c) { return a * b + c; }
template <int N, class T>
__device__ inline void sincos(const Dual<N, T>& a, Dual<N, T>* s, Dual<N, T>* c) {
    T sv, cv;
    sincos(a.v, &sv, &cv);
    *s = chain(a, sv, cv);
    *c = chain(a, cv, -sv);
}
template <int N, class T>
__device__ inline void sincospi(const Dual<N, T>& a, Dual<N, T>* s, Dual<N, T>* c) {
    T sv, cv;
    sincospi(a.v, &sv, &cv);
    *s = chain(a, sv, scalar_cast<T>(CUDART_PI) * cv);
    *c = chain(a, cv, -(scalar_cast<T>(CUDART_PI) * sv));
}
// the engine's table-driven point transcendentals (fp64_math.cuh, df64.cuh)
template <int N, class T> __device__ inline Dual<N, T> fast_exp(const Dual<N, T>& a) {
    const T e = fast_exp(a.v);
    return chain(a, e, e);
}
template <int N, class T>
__device__ inline void fast_sincospi(const Dual<N, T>& a, Dual<N, T>* s, Dual<N, T>* c) {
    T sv, cv;
    fast_sincospi(a.v, &sv, &cv);
    *s = chain(a, sv, scalar_cast<T>(CUDART_PI) * cv);
    *c = chain(a, cv, -(scalar_cast<T>(CUDART_PI) * sv));
}

// RK stage weights for dual states follow their scalar type
template <int N, class T>
struct StageWeight<Dual<N, T>> {
    using type = typename StageWeight<T>::type;
};

}  // namespace raptor
