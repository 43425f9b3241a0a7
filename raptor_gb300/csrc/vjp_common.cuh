// Pieces shared by the adjoint kernels (vjp.cu: FP64; vjp_df.cu: mixed-DF
// and mixed): the inclination dual, the sample's three dual directions and
// the scalar factors that map them onto the parameters, and the launch
// interface.
#pragma once
#include "dual.cuh"
#include "ray_kernel.cuh"

namespace raptor {

using D1 = Dual<1>;

// The sample's dual directions: the inclination (through the geodesic), ln
// Theta_e and ln B.  Everything else reaches a sample through these and n_e,
// and n_e is a pure prefactor of j and a, so dS/d ln n_e = S and
// d delta/d ln n_e = delta:
//   rho_s:  n_e proportional to rho_s, and ln Theta_e by d ln Theta_e/d rho_s;
//   u_s, R_high, R_low:  ln Theta_e only (the R-beta model, thetae_log_derivs);
//   M_unit: n_e proportional to M_unit, B to sqrt(M_unit).
// Three tangents instead of one per parameter.
constexpr int kSIncl = 0, kSLnTh = 1, kSLnB = 2;

// The scalar factors that map a sample's (value, ln Theta_e) terms onto the
// per-cell and scalar parameters.
template <class T>
struct SampleScalarsT {
    T irho;      // 1 / rho_s
    T dlnth[4];  // d ln Theta_e / d(rho_s, u_s, R_high, R_low)
};

// d ln Theta_e / d(rho_s, u_s, R_high, R_low) of the R-beta electron
// temperature (raptor_harm_model.c:262-276, fluid_from_prims):
//   Theta_e = (u / rho) (gam(t) - 1) (m_p / m_e) / (1 + t),
//   t = (R_high b^2 + R_low) / (1 + b^2),  b = (1/3) u / (Bsq / 2),
//   gam(t) = ((1 + 2/3 (t + 1) / (t + 2)) + 4/3) / 2.
// Zero where Theta_e was clamped (u / rho ... < 0).
template <class T>
__device__ __forceinline__ void thetae_log_derivs(T rho, T uu, T bsq, T Rh, T Rl, T (&out)[4]) {
    const T tiny = (T)1.e-20;
    const T beta = fdiv(uu * (T(4) / T(3) - T(1)), T(0.5) * (bsq + tiny));
    const T b2 = beta * beta;
    const T i1b2 = fdiv(T(1), T(1) + b2);
    const T t = Rh * b2 * i1b2 + Rl * i1b2;
    const T gam = T(0.5) * ((T(1) + fdiv(T(2) / T(3) * (t + T(1)), t + T(2))) + T(4) / T(3));
    if (fdiv(uu, rho) * (gam - T(1)) < T(0)) {
        out[0] = out[1] = out[2] = out[3] = T(0);
        return;
    }
    // d ln((gam - 1) / (1 + t)) / dt and dt / d ln beta
    const T dlnTU = fdiv(fdiv(T(1) / T(3), (t + T(2)) * (t + T(2))), gam - T(1)) - fdiv(T(1), T(1) + t);
    const T dt_dlnb = T(2) * b2 * (Rh - Rl) * i1b2 * i1b2;
    out[0] = -fdiv(T(1), rho);
    out[1] = fdiv(T(1) + dlnTU * dt_dlnb, uu);
    out[2] = dlnTU * b2 * i1b2;
    out[3] = dlnTU * i1b2;
}

// thetae_log_derivs for FP64 arguments from three divisions instead of nine,
// in fluid_fast's variables: h = 2u/3, D = b^2 + tiny, Q = h^2 + D^2,
// A = R_high h^2 + R_low D^2 + Q, C = A + Q.  Then t + 1 = A/Q, t + 2 = C/Q,
// gam - 1 = (C + 2A)/(6C), b^2/(1 + b^2) = h^2/Q, 1/(1 + b^2) = D^2/Q, and
//   d ln((gam - 1)/(1 + t))/dt = 2Q^2/(C (C + 2A)) - Q/A
//                              = -Q^2 (3A^2 + 2AQ + Q^2) / (Q A C (C + 2A)),
//   dt/d ln beta = 2 (R_high - R_low) h^2 D^2 / Q^2,
// with 1/Q and the first quotient from one reciprocal of Q A C (C + 2A)
// (at least 6e-160: D^2 >= 1e-40).  gam - 1 > 0, so Theta_e's clamp is the
// sign of u / rho.
__device__ __forceinline__ void thetae_log_derivs_fp64(double irho, double uu, double bsq, double Rh, double Rl,
                                                       double (&out)[4]) {
    if (uu * irho < 0.0) {
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return;
    }
    const double h = uu * (2.0 / 3.0), D = bsq + 1.e-20;
    const double h2 = h * h, D2 = D * D;
    const double Q = h2 + D2;
    const double A = Rh * h2 + Rl * D2 + Q;
    const double C = A + Q;
    const double CE = C * (C + 2.0 * A);
    const double z = 1.0 / (Q * A * CE);
    const double iQ = z * A * CE;
    const double dlnTU = -(z * Q * Q) * (A * (3.0 * A + 2.0 * Q) + Q * Q);
    const double dt_dlnb = 2.0 * (Rh - Rl) * h2 * D2 * (iQ * iQ);
    out[0] = -irho;
    out[1] = (1.0 + dlnTU * dt_dlnb) / uu;
    out[2] = dlnTU * h2 * iQ;
    out[3] = dlnTU * D2 * iQ;
}

// A term's derivative along scalar parameter q (0 inclination, 1 ln M_unit,
// 2 R_high, 3 R_low) from its value and three tangents.
template <class Dl, class T>
__device__ __forceinline__ T scalar_tangent(const Dl& x, const SampleScalarsT<T>& ss, int q) {
    if (q == 0) return x.d[kSIncl];
    if (q == 1) return x.v + T(0.5) * x.d[kSLnB];
    return x.d[kSLnTh] * ss.dlnth[q];  // q = 2, 3: R_high, R_low
}

// A term's derivative along rho_s: (d/d ln n_e) / rho_s + (d ln Theta_e /
// d rho_s) d/d ln Theta_e.
template <class Dl, class T>
__device__ __forceinline__ T rho_tangent(const Dl& x, const SampleScalarsT<T>& ss) {
    return x.v * ss.irho + x.d[kSLnTh] * ss.dlnth[0];
}

constexpr int kVjpBlock = 128;
constexpr int kVjpRefill = 8;  // geodesic steps between lane refills of the mixed-DF adjoint

// The rays [begin, end) of an image (pixel x + y W) an adjoint pass covers.
struct RayRange {
    long long begin, end;
};

// The one-pass adjoint's record tape: lane l of the launch (block *
// kVjpBlock + thread) keeps its ray's records at rec + l * cap * stride,
// stride elements each (FP32 for the mixed and mixed-DF adjoints, FP64 for
// the FP64 one), and the pass writes its own image to out (image layout).
// A record: cell, two offsets, d ln Theta_e / d ln u, the two gated sums,
// and per frequency I before the sample and the two suffix coefficients.
// rec == nullptr: two passes.
struct VjpTape {
    void* rec;
    int cap;     // records per lane
    int stride;  // elements per record
    double* out;
};
// elements per record for nf frequencies, padded to 16 bytes
inline int vjp_tape_stride(int nf, bool fp64) {
    const int n = 6 + 3 * nf;
    return fp64 ? (n + 1) & ~1 : (n + 3) & ~3;
}

// Launch of the adjoint pass: grid blocks of kVjpBlock threads on stream st
// for image im (device pointer), camera constants with their inclination
// tangent, the forward image fwd (unused with a tape) and dL/dI dl (device,
// image layout); accumulates into counters, gscal[4] and the per-cell arrays
// (which may be null); lanes take new rays every refill steps; scratch is
// the sample pool's result buffer where the kernel has one; rr the rays to
// cover; tape the one-pass tape where the kernel has one.
using VjpLaunchFn = void (*)(int grid, cudaStream_t st, const DevImage* im, const CamT<D1>& cam, const double* fwd,
                             const double* dl, unsigned long long* counters, double* gscal, double* g_rho,
                             double* g_u, double* g_th, int refill, double* scratch, RayRange rr, VjpTape tape);
// the mixed-DF and the mixed adjoints for nf frequencies (vjp_df.cu), the
// one-pass (tape) or the two-pass kernel; *fn gets the kernel.  (The FP64
// adjoints' picker is pick_vjp_fp64, vjp.cu.)
VjpLaunchFn pick_vjp_df(int nf, const void** fn, bool kappa, bool tape);
VjpLaunchFn pick_vjp_mixed(int nf, const void** fn, bool kappa, bool tape);

}  // namespace raptor
