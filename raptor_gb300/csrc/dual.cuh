// Forward-mode dual numbers for the adjoint (VJP) kernel: a value and N
// directional derivatives, with the arithmetic and the libm functions the
// imaging path uses.  Comparisons act on the value, so every branch of the
// primal computation is taken as the primal takes it (derivatives of the
// taken branch).
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>

#include "fp64_math.cuh"

namespace raptor {

// the plain-double versions stay visible next to the Dual overloads below
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

template <int N>
struct Dual {
    double v;
    double d[N];
    __host__ __device__ Dual() {}
    __host__ __device__ Dual(double x) : v(x) {
#pragma unroll
        for (int i = 0; i < N; ++i) d[i] = 0.0;
    }
    // a value with derivative 1 in direction k
    __host__ __device__ static Dual seed(double x, int k) {
        Dual r(x);
        r.d[k] = 1.0;
        return r;
    }
};

template <class T> struct is_dual { static constexpr bool value = false; };
template <int N> struct is_dual<Dual<N>> { static constexpr bool value = true; };

__host__ __device__ inline double val(double x) { return x; }
template <int N> __host__ __device__ inline double val(const Dual<N>& x) { return x.v; }

template <int N>
__host__ __device__ inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator-(const Dual<N>& a) {
    Dual<N> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
    return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
    const double ib = 1.0 / b.v;
    Dual<N> r;
    r.v = a.v * ib;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
    return r;
}
// mixed with plain doubles
template <int N> __host__ __device__ inline Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v += b; return r; }
template <int N> __host__ __device__ inline Dual<N> operator+(double a, const Dual<N>& b) { return b + a; }
template <int N> __host__ __device__ inline Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v -= b; return r; }
template <int N> __host__ __device__ inline Dual<N> operator-(double a, const Dual<N>& b) { return -(b - a); }
template <int N>
__host__ __device__ inline Dual<N> operator*(const Dual<N>& a, double b) {
    Dual<N> r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
    return r;
}
template <int N> __host__ __device__ inline Dual<N> operator*(double a, const Dual<N>& b) { return b * a; }
template <int N> __host__ __device__ inline Dual<N> operator/(const Dual<N>& a, double b) { return a * (1.0 / b); }
template <int N> __host__ __device__ inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> __host__ __device__ inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { a = a + b; return a; }
template <int N> __host__ __device__ inline Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) { a = a - b; return a; }
template <int N> __host__ __device__ inline Dual<N>& operator*=(Dual<N>& a, const Dual<N>& b) { a = a * b; return a; }

#define RAPTOR_DUAL_CMP(OP)                                                                                    \
    template <int N> __host__ __device__ inline bool operator OP(const Dual<N>& a, const Dual<N>& b) { return a.v OP b.v; } \
    template <int N> __host__ __device__ inline bool operator OP(const Dual<N>& a, double b) { return a.v OP b; }          \
    template <int N> __host__ __device__ inline bool operator OP(double a, const Dual<N>& b) { return a OP b.v; }
RAPTOR_DUAL_CMP(<)
RAPTOR_DUAL_CMP(>)
RAPTOR_DUAL_CMP(<=)
RAPTOR_DUAL_CMP(>=)
RAPTOR_DUAL_CMP(==)
RAPTOR_DUAL_CMP(!=)
#undef RAPTOR_DUAL_CMP

// f(a) with f'(a) given
template <int N>
__host__ __device__ inline Dual<N> chain(const Dual<N>& a, double f, double fp) {
    Dual<N> r;
    r.v = f;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = fp * a.d[i];
    return r;
}

// At 0 the argument's tangents are 0 too wherever it is identically 0 (a
// field-free region: b^2 = 0), so the tangent is taken as 0 there rather
// than 0.5/0 * 0 = NaN.
template <int N> __device__ inline Dual<N> sqrt(const Dual<N>& a) {
    const double s = ::sqrt(a.v);
    return chain(a, s, s > 0.0 ? 0.5 / s : 0.0);
}
template <int N> __device__ inline Dual<N> exp(const Dual<N>& a) { const double e = ::exp(a.v); return chain(a, e, e); }
template <int N> __device__ inline Dual<N> log(const Dual<N>& a) { return chain(a, ::log(a.v), 1.0 / a.v); }
template <int N> __device__ inline Dual<N> cbrt(const Dual<N>& a) {
    const double c = ::cbrt(a.v);
    return chain(a, c, c != 0.0 ? 1.0 / (3.0 * c * c) : 0.0);
}
template <int N> __device__ inline Dual<N> expm1(const Dual<N>& a) { return chain(a, ::expm1(a.v), ::exp(a.v)); }
template <int N> __device__ inline Dual<N> fabs(const Dual<N>& a) { return a.v < 0.0 ? -a : a; }
template <int N> __device__ inline Dual<N> fmin(const Dual<N>& a, const Dual<N>& b) { return b.v < a.v ? b : a; }
template <int N> __device__ inline Dual<N> fmax(const Dual<N>& a, const Dual<N>& b) { return b.v > a.v ? b : a; }
template <int N> __device__ inline Dual<N> fmax(const Dual<N>& a, double b) { return b > a.v ? Dual<N>(b) : a; }
template <int N> __device__ inline Dual<N> fma(const Dual<N>& a, const Dual<N>& b, const Dual<N>& c) { return a * b + c; }
template <int N> __device__ inline Dual<N> fma(double a, const Dual<N>& b, double c) { return a * b + c; }
template <int N> __device__ inline Dual<N> fma(const Dual<N>& a, const Dual<N>& b, double c) { return a * b + c; }
template <int N>
__device__ inline void sincos(const Dual<N>& a, Dual<N>* s, Dual<N>* c) {
    double sv, cv;
    ::sincos(a.v, &sv, &cv);
    *s = chain(a, sv, cv);
    *c = chain(a, cv, -sv);
}
template <int N>
__device__ inline void sincospi(const Dual<N>& a, Dual<N>* s, Dual<N>* c) {
    double sv, cv;
    ::sincospi(a.v, &sv, &cv);
    *s = chain(a, sv, CUDART_PI * cv);
    *c = chain(a, cv, -CUDART_PI * sv);
}
template <int N> __device__ inline Dual<N> fma(double a, const Dual<N>& b, const Dual<N>& c) { return a * b + c; }
// the engine's table-driven point transcendentals (fp64_math.cuh)
template <int N> __device__ inline Dual<N> fast_exp(const Dual<N>& a) {
    const double e = fast_exp(a.v);
    return chain(a, e, e);
}
template <int N>
__device__ inline void fast_sincospi(const Dual<N>& a, Dual<N>* s, Dual<N>* c) {
    double sv, cv;
    fast_sincospi(a.v, &sv, &cv);
    *s = chain(a, sv, CUDART_PI * cv);
    *c = chain(a, cv, -CUDART_PI * sv);
}

}  // namespace raptor
