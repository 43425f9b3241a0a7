// Kerr spacetime in modified Kerr-Schild (MKS) coordinates, device side.
//
// The reference evaluates metric_dd / metric_uu / connection_udd from
// scratch at every call (metric.c:94-137, 207-231, 538-638), each with its
// own exp, sin and cos.  On GB300 the FP64 pipe is the bottleneck, so the
// engine evaluates the transcendentals and the four reciprocals of a point
// once (MksPoint) and shares them between the radiative-transfer sample at
// the post-step position and the first RK stage of the next step, which is
// the same point (integrator.c:259,277-278 then 259 again).
//
// The formulas are the reference's MKS expressions; only their grouping
// changes (shared sub-expressions, reciprocals instead of repeated
// divisions, 40 unique Christoffel symbols contracted with the 10 symmetric
// products U^j U^k), which moves results by rounding only.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>

namespace raptor {

struct Geo {
    double a, a2, hslope, R0;
    double one_m_h;   // 1 - hslope
    double half_1mh;  // (1 - hslope)/2
};

// Quantities at one MKS position X = (x0, x1, x2, x3).
struct MksPoint {
    double rp;    // exp(x1) = dr/dx1
    double r;     // R0 + exp(x1)
    double s, c;  // sin(theta), cos(theta)
    double s2x, c2x;  // sin(2 pi x2), cos(2 pi x2)
    double irp;   // 1/rp
    double iS;    // 1/Sigma = 1/(r^2 + a^2 cos^2 theta)
    double ithp;  // 1/(d theta/d x2)
    double isn;   // 1/sin(theta)
};

__device__ __forceinline__ void mks_point(double x1, double x2, const Geo& g, MksPoint& p) {
    p.rp = exp(x1);
    p.r = g.R0 + p.rp;
    sincospi(2.0 * x2, &p.s2x, &p.c2x);
    const double th = CUDART_PI * x2 + g.half_1mh * p.s2x;
    sincos(th, &p.s, &p.c);
    const double Sg = fma(p.r, p.r, g.a2 * p.c * p.c);
    const double thp = CUDART_PI * fma(g.one_m_h, p.c2x, 1.0);
    p.iS = 1.0 / Sg;
    p.irp = 1.0 / p.rp;
    p.ithp = 1.0 / thp;
    p.isn = 1.0 / p.s;
}

// d^2 x^i / d lambda^2 = -Gamma^i_jk U^j U^k  (integrator.c:126-146 with the
// MKS connection of metric.c:538-638).
__device__ __forceinline__ void geodesic_accel(const MksPoint& p, const Geo& g, const double U[4],
                                               double A[4]) {
    const double a = g.a, a2 = g.a2;
    const double r = p.r, r2 = r * r;
    const double rp = p.rp, rp2 = rp * rp;
    const double thp = CUDART_PI * fma(g.one_m_h, p.c2x, 1.0);
    const double thp2 = thp * thp;
    const double thpp = -2.0 * CUDART_PI * CUDART_PI * g.one_m_h * p.s2x;
    const double s = p.s, c = p.c;
    const double s2 = s * s, c2 = c * c;
    const double sc = s * c;
    const double s2th = 2.0 * sc;
    const double cot = c * p.isn;
    const double Sg = r2 + a2 * c2;
    const double Dl = r2 - 2.0 * r + a2;
    const double r2a2 = r2 + a2;
    const double Aq = Sg * Dl + 2.0 * r * r2a2;
    const double iS = p.iS, iS2 = iS * iS, iS3 = iS2 * iS;
    const double B = (2.0 * r2 - Sg) * iS3;
    const double C = r * iS - a2 * B * s2;
    const double irp = p.irp, ithp = p.ithp;

    // Gamma^0
    const double G0_00 = 2.0 * r * B;
    const double G0_01 = (Sg + 2.0 * r) * B * rp;
    const double G0_02 = -a2 * r * s2th * iS2 * thp;
    const double G0_03 = -2.0 * a * r * B * s2;
    const double G0_11 = 2.0 * (Sg + r) * B * rp2;
    const double G0_12 = G0_02 * rp;
    const double G0_13 = -a * s2 * G0_01;
    const double G0_22 = -2.0 * r2 * iS * thp2;
    const double G0_23 = -a * s2 * G0_02;
    const double G0_33 = -2.0 * r * C * s2;
    // Gamma^1 (Gamma^1_02 = Gamma^1_23 = 0)
    const double G1_00 = Dl * B * irp;
    const double G1_01 = (Dl - Sg) * B;
    const double G1_03 = -a * Dl * B * s2 * irp;
    const double G1_11 = 1.0 - (2.0 * Sg - Dl) * B * rp;
    const double G1_12 = -a2 * sc * iS * thp;
    const double G1_13 = a * (r * iS + (Sg - Dl) * B) * s2;
    const double G1_22 = -r * Dl * iS * irp * thp2;
    const double G1_33 = -Dl * C * s2 * irp;
    // Gamma^2 (Gamma^2_02 = Gamma^2_23 = 0)
    const double G2_00 = iS * G0_02 * (ithp * ithp);
    const double G2_01 = G2_00 * rp;
    const double G2_03 = a * r * r2a2 * s2th * iS3 * ithp;
    const double G2_11 = G2_00 * rp2;
    const double G2_12 = r * iS * rp;
    const double G2_13 = a * sc * (Aq + Sg * (Sg - Dl)) * iS3 * rp * ithp;
    const double G2_22 = thpp * ithp + G1_12;
    const double G2_33 = -sc * (Dl * Sg * Sg + 2.0 * r * r2a2 * r2a2) * iS3 * ithp;
    // Gamma^3
    const double G3_00 = a * B;
    const double G3_01 = G3_00 * rp;
    const double G3_02 = -2.0 * a * r * cot * iS2 * thp;
    const double G3_03 = -a2 * B * s2;
    const double G3_11 = G3_00 * rp2;
    const double G3_12 = -a * (Sg + 2.0 * r) * cot * iS2 * rp * thp;
    const double G3_13 = C * rp;
    const double G3_22 = -a * r * iS * thp2;
    const double G3_23 = (cot + a2 * r * s2th * iS2) * thp;
    const double G3_33 = -a * C * s2;

    const double u0 = U[0], u1 = U[1], u2 = U[2], u3 = U[3];
    const double q00 = u0 * u0, q11 = u1 * u1, q22 = u2 * u2, q33 = u3 * u3;
    const double q01 = 2.0 * u0 * u1, q02 = 2.0 * u0 * u2, q03 = 2.0 * u0 * u3;
    const double q12 = 2.0 * u1 * u2, q13 = 2.0 * u1 * u3, q23 = 2.0 * u2 * u3;

    A[0] = -(G0_00 * q00 + G0_11 * q11 + G0_22 * q22 + G0_33 * q33 + G0_01 * q01 + G0_02 * q02 +
             G0_03 * q03 + G0_12 * q12 + G0_13 * q13 + G0_23 * q23);
    A[1] = -(G1_00 * q00 + G1_11 * q11 + G1_22 * q22 + G1_33 * q33 + G1_01 * q01 + G1_03 * q03 +
             G1_12 * q12 + G1_13 * q13);
    A[2] = -(G2_00 * q00 + G2_11 * q11 + G2_22 * q22 + G2_33 * q33 + G2_01 * q01 + G2_03 * q03 +
             G2_12 * q12 + G2_13 * q13);
    A[3] = -(G3_00 * q00 + G3_11 * q11 + G3_22 * q22 + G3_33 * q33 + G3_01 * q01 + G3_02 * q02 +
             G3_03 * q03 + G3_12 * q12 + G3_13 * q13 + G3_23 * q23);
}

// Covariant metric (metric.c:94-137); the 7 independent entries.
struct MetricDD {
    double g00, g01, g03, g11, g13, g22, g33;
};
// Contravariant metric (metric.c:207-231); the 6 independent entries.
struct MetricUU {
    double g00, g01, g11, g13, g22, g33;
};

__device__ __forceinline__ void mks_metric(const MksPoint& p, const Geo& g, MetricDD& d, MetricUU& u) {
    const double r = p.r, a = g.a;
    const double s2 = p.s * p.s;
    const double irho2 = p.iS;
    const double rfac = r - g.R0;
    const double hfac = CUDART_PI * fma(g.one_m_h, p.c2x, 1.0);
    const double rho2 = fma(r, r, g.a2 * p.c * p.c);
    const double z = 2.0 * r * irho2;
    d.g00 = -1.0 + z;
    d.g01 = z * rfac;
    d.g03 = -a * z * s2;
    d.g11 = (1.0 + z) * rfac * rfac;
    d.g13 = -a * s2 * (1.0 + z) * rfac;
    d.g22 = rho2 * hfac * hfac;
    d.g33 = s2 * (rho2 + g.a2 * s2 * (1.0 + z));
    const double ir = (g.R0 == 0.0) ? p.irp : 1.0 / r;  // r == rp exactly when R0 == 0
    u.g00 = -1.0 - z;
    u.g01 = 2.0 * irho2;
    u.g11 = irho2 * (r * (r - 2.0) + g.a2) * (ir * ir);
    u.g13 = a * irho2 * ir;
    u.g22 = irho2 * (p.ithp * p.ithp);
    u.g33 = irho2 * (p.isn * p.isn);
}

template <class T>
__device__ __forceinline__ void lower4(const MetricDD& g, const T v[4], T out[4]) {
    out[0] = T(g.g00) * v[0] + T(g.g01) * v[1] + T(g.g03) * v[3];
    out[1] = T(g.g01) * v[0] + T(g.g11) * v[1] + T(g.g13) * v[3];
    out[2] = T(g.g22) * v[2];
    out[3] = T(g.g03) * v[0] + T(g.g13) * v[1] + T(g.g33) * v[3];
}

}  // namespace raptor
