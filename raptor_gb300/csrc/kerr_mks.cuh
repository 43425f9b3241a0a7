// Kerr spacetime in modified Kerr-Schild (MKS) coordinates, device side.
//
// The reference evaluates metric_dd / metric_uu / connection_udd from
// scratch at every call (metric.c:94-137, 207-231, 538-638), each with its
// own exp, sin and cos.  On GB300 the FP64 pipe is the bottleneck, so the
// engine evaluates the transcendentals and the four reciprocals of a point
// once (MksPointT) and shares them between the radiative-transfer sample at
// the post-step position and the first RK stage of the next step, which is
// the same point (integrator.c:259,277-278 then 259 again).
//
// The formulas are the reference's MKS expressions; only their grouping
// changes (shared sub-expressions, reciprocals instead of repeated
// divisions, 40 unique Christoffel symbols contracted with the 10 symmetric
// products U^j U^k), which moves results by rounding only.
//
// Everything is templated on the scalar type R: double for the forward
// kernels, Dual<N> (dual.cuh) for the forward-mode tangents of the adjoint,
// DF (df64.cuh) for the mixed-DF form; and on the constants' type G: Geo
// (FP64) or GeoDF.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>


#include "df_type.cuh"
#include "fp64_math.cuh"

namespace raptor {

struct Geo {
    double a, a2, hslope, R0;
    double one_m_h;   // 1 - hslope
    double th_coef;   // (1 - hslope) / (2 pi): theta / pi = x2 + th_coef sin(2 pi x2)
};

// Quantities at one MKS position X = (x0, x1, x2, x3).
template <class R>
struct MksPointT {
    R rp;        // exp(x1) = dr/dx1
    R r;         // R0 + exp(x1)
    R s, c;      // sin(theta), cos(theta)
    R s2x, c2x;  // sin(2 pi x2), cos(2 pi x2)
    R irp;       // 1/rp
    R Sg, iS;    // Sigma = r^2 + a^2 cos^2 theta, 1/Sigma
    R thp, ithp; // d theta/d x2, its reciprocal
    R isn;       // 1/sin(theta)
};
using MksPoint = MksPointT<double>;

// The point's four reciprocals 1/Sigma, 1/r', 1/theta', 1/sin(theta) from
// one division: with q = r' theta' sin(theta) Sigma, each is 1/q times the
// other three factors, built from the running products (9 multiplications
// and 1 division instead of 4 divisions).  At the exact pole (sin = 0) all
// four are non-finite, where one division would leave only 1/sin infinite;
// the geodesic is singular there either way.
template <class R>
__device__ __forceinline__ void point_reciprocals(const R& Sg, const R& thp, MksPointT<R>& p) {
    p.Sg = Sg;
    p.thp = thp;
    const R q1 = p.rp * thp, q2 = q1 * p.s, q3 = q2 * Sg;
    const R iq3 = recip(q3);
    p.iS = iq3 * q2;
    const R iq2 = iq3 * Sg;
    p.isn = iq2 * q1;
    const R iq1 = iq2 * p.s;
    p.ithp = iq1 * p.rp;
    p.irp = iq1 * thp;
}

template <class R, class G>
__device__ __forceinline__ void mks_point(R x1, R x2, const G& g, MksPointT<R>& p) {
    p.rp = fast_exp(x1);
    p.r = g.R0 + p.rp;
    fast_sincospi(2.0 * x2, &p.s2x, &p.c2x);
    // theta = pi x2 + (1-h)/2 sin(2 pi x2) (metric.c:98), evaluated as sinpi/cospi of theta/pi
    fast_sincospi(fma(g.th_coef, p.s2x, x2), &p.s, &p.c);
    const R Sg = fma(p.r, p.r, g.a2 * p.c * p.c);
    const R thp = CUDART_PI * fma(g.one_m_h, p.c2x, 1.0);
    point_reciprocals(Sg, thp, p);
}

// mks_point with the two sincospi evaluations (of 2 x2, then of theta / pi)
// through one copy of the code: for the double-float types, whose sincospi
// is a few hundred FP32 instructions, the smaller loop body fetches faster.
template <class R, class G>
__device__ __forceinline__ void mks_point_rolled(R x1, R x2, const G& g, MksPointT<R>& p) {
    p.rp = fast_exp(x1);
    p.r = g.R0 + p.rp;
    R arg = 2.0 * x2, sv, cv;
#pragma unroll 1
    for (int k = 0;; ++k) {
        fast_sincospi(arg, &sv, &cv);
        if (k == 1) break;
        p.s2x = sv;
        p.c2x = cv;
        // theta = pi x2 + (1-h)/2 sin(2 pi x2) (metric.c:98), as theta / pi
        arg = fma(g.th_coef, sv, x2);
    }
    p.s = sv;
    p.c = cv;
    const R Sg = fma(p.r, p.r, g.a2 * p.c * p.c);
    const R thp = CUDART_PI * fma(g.one_m_h, p.c2x, 1.0);
    point_reciprocals(Sg, thp, p);
}

// d^2 x^i / d lambda^2 = -Gamma^i_jk U^j U^k  (integrator.c:126-146 with the
// MKS connection of metric.c:538-638).
template <class R, class G>
__device__ __forceinline__ void geodesic_accel(const MksPointT<R>& p, const G& g, const R U[4], R A[4]) {
    const auto a = g.a, a2 = g.a2;
    const R r = p.r, r2 = r * r;
    const R rp = p.rp, rp2 = rp * rp;
    const R thp = p.thp;
    const R thp2 = thp * thp;
    const R thpp = (-2.0 * CUDART_PI * CUDART_PI * g.one_m_h) * p.s2x;
    const R s = p.s, c = p.c;
    const R s2 = s * s;
    const R sc = s * c;
    const R s2th = 2.0 * sc;
    const R cot = c * p.isn;
    const R Sg = p.Sg, Sg2 = Sg * Sg;
    const R r2a2 = r2 + a2;
    const R two_r = 2.0 * r;
    const R Dl = r2a2 - two_r;
    const R Rr2 = two_r * r2a2;  // 2 r (r^2 + a^2)
    const R iS = p.iS, iS2 = iS * iS, iS3 = iS2 * iS;
    const R B = (2.0 * r2 - Sg) * iS3;
    const R riS = r * iS;
    const R as2 = a * s2;
    const R aB = a * B;
    const R C = riS - aB * as2;
    const R irp = p.irp, ithp = p.ithp;

    const R u0 = U[0], u1 = U[1], u2 = U[2], u3 = U[3];
    const R q00 = u0 * u0, q11 = u1 * u1, q22 = u2 * u2, q33 = u3 * u3;
    const R q01 = 2.0 * u0 * u1, q02 = 2.0 * u0 * u2, q03 = 2.0 * u0 * u3;
    const R q12 = 2.0 * u1 * u2, q13 = 2.0 * u1 * u3, q23 = 2.0 * u2 * u3;

    // The contraction with the symbols' common factors (B, iS^2 theta',
    // sin cos iS^3 / theta', C) taken out of the sums: a quarter fewer
    // multiplications than forming the 40 unique symbols first.  Term by
    // term it is sum_jk Gamma^i_jk q_jk with
    //   G0_00 = 2 r B, G0_01 = (Sigma + 2r) B r', G0_02 = -a^2 r sin2th iS^2 theta',
    //   G0_03 = -2 a r B s^2, G0_11 = 2 (Sigma + r) B r'^2, G0_12 = G0_02 r',
    //   G0_13 = -a s^2 G0_01, G0_22 = -2 r^2 iS theta'^2, G0_23 = -a s^2 G0_02,
    //   G0_33 = -2 r C s^2;
    //   G1_00 = Delta B / r', G1_01 = (Delta - Sigma) B, G1_03 = -a Delta B s^2 / r',
    //   G1_11 = 1 - (2 Sigma - Delta) B r', G1_12 = -a^2 s c iS theta',
    //   G1_13 = a (r iS + (Sigma - Delta) B) s^2, G1_22 = -r Delta iS theta'^2 / r',
    //   G1_33 = -Delta C s^2 / r', G1_02 = G1_23 = 0;
    //   G2_00 = iS G0_02 / theta'^2, G2_01 = G2_00 r', G2_11 = G2_00 r'^2,
    //   G2_03 = a r (r^2 + a^2) sin2th iS^3 / theta', G2_12 = r iS r',
    //   G2_13 = a s c (Aq + Sigma (Sigma - Delta)) iS^3 r' / theta',
    //   G2_22 = theta'' / theta' + G1_12,
    //   G2_33 = -s c (Delta Sigma^2 + 2 r (r^2 + a^2)^2) iS^3 / theta', G2_02 = G2_23 = 0;
    //   G3_00 = a B, G3_01 = G3_00 r', G3_11 = G3_00 r'^2, G3_02 = -2 a r cot iS^2 theta',
    //   G3_03 = -a^2 B s^2, G3_12 = -a (Sigma + 2r) cot iS^2 r' theta', G3_13 = C r',
    //   G3_22 = -a r iS theta'^2, G3_23 = (cot + a^2 r sin2th iS^2) theta', G3_33 = -a C s^2.
    // The double-float type gains as much (1024x1024 mixed-DF render 137 ->
    // 119 ms against compensated dot products over the 40 symbols), with the
    // same step counts and its geodesic as close to the FP64 one as before.
    const R Tr = (Sg + two_r) * rp;
    const R X0 = q00 - as2 * q03;
    const R X1 = q01 - as2 * q13;
    const R H = q00 + rp * (q01 + rp * q11);  // q00 + r' q01 + r'^2 q11
    const R iSthp = iS * thp;
    const R iS2thp = iS * iSthp;
    const R a2sc = a2 * sc;
    const R WpT = two_r * a2sc * iS2thp;      // -G0_02 = a^2 r sin 2theta iS^2 theta'
    const R riSthp2 = riS * thp2;
    const R M = riSthp2 * q22 + C * s2 * q33;  // shared by A0 and A1
    const R Dlirp = Dl * irp;
    const R G1_12 = -a2sc * iSthp;
    A[0] = -(B * (two_r * X0 + Tr * X1 + 2.0 * (Sg + r) * rp2 * q11) - WpT * (q02 + rp * q12 - as2 * q23) -
             two_r * M);
    A[1] = -(B * (Dlirp * X0 + (Dl - Sg) * X1 - (2.0 * Sg - Dl) * rp * q11) + q11 + riS * as2 * q13 +
             G1_12 * q12 - Dlirp * M);
    // Z = sin cos iS^3 / theta'; the G2_00 terms -iS Wp / theta' H are 2 a^2 r Z H,
    // and G2_13's Aq + Sigma (Sigma - Delta) with Aq = Sigma Delta + 2 r (r^2 + a^2)
    // is Sigma^2 + 2 r (r^2 + a^2)
    const R Z = sc * iS3 * ithp;
    A[2] = -(Z * (a * (Rr2 * q03 + (Sg2 + Rr2) * rp * q13) - (Dl * Sg2 + Rr2 * r2a2) * q33 - a2 * two_r * H) +
             riS * rp * q12 + (thpp * ithp + G1_12) * q22);
    const R K = a * cot * iS2thp;  // G3_02 = -2 r K, G3_12 = -(Sigma+2r) r' K
    A[3] = -(aB * (H - as2 * q03) - K * (two_r * q02 + Tr * q12) + C * (rp * q13 - as2 * q33) -
             a * riSthp2 * q22 + (cot * thp + WpT) * q23);
}

// Covariant metric (metric.c:94-137); the 7 independent entries.
template <class R>
struct MetricDDT {
    R g00, g01, g03, g11, g13, g22, g33;
};
// Contravariant metric (metric.c:207-231); the 6 independent entries.
template <class R>
struct MetricUUT {
    R g00, g01, g11, g13, g22, g33;
};
using MetricDD = MetricDDT<double>;
using MetricUU = MetricUUT<double>;

template <class R, class G>
__device__ __forceinline__ void mks_metric(const MksPointT<R>& p, const G& g, MetricDDT<R>& d, MetricUUT<R>& u) {
    const R r = p.r;
    const auto a = g.a;
    const R s2 = p.s * p.s;
    const R irho2 = p.iS;
    const R rfac = r - g.R0;
    const R hfac = p.thp;
    const R rho2 = p.Sg;
    const R z = 2.0 * r * irho2;
    const R mas2 = -a * s2;
    const R opz = 1.0 + z;
    const R opzr = opz * rfac;
    d.g00 = -1.0 + z;
    d.g01 = z * rfac;
    d.g03 = mas2 * z;
    d.g11 = opzr * rfac;
    d.g13 = mas2 * opzr;
    d.g22 = rho2 * hfac * hfac;
    d.g33 = s2 * (rho2 + g.a2 * s2 * opz);
    const R ir = (g.R0 == 0.0) ? p.irp : recip(r);  // r == rp exactly when R0 == 0
    u.g00 = -1.0 - z;
    u.g01 = 2.0 * irho2;
    u.g11 = irho2 * (r * (r - 2.0) + g.a2) * (ir * ir);
    u.g13 = a * irho2 * ir;
    u.g22 = irho2 * (p.ithp * p.ithp);
    u.g33 = irho2 * (p.isn * p.isn);
}

}  // namespace raptor
