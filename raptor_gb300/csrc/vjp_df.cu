// The adjoint passes whose transfer sample runs in FP32: the derivative of
// what the mixed-DF form (ray_kernel_df) and the mixed form (ray_kernel<NF,
// true>) render.  Same method as vjp.cu (one forward sweep per ray, exact
// reverse-mode sample sensitivities from the suffix identity
// dI/d delta_k = -(I - I_<k) with the forward image's I, forward-mode
// tangents for the four scalars, per-cell atomic scatter), with the sample
// in FP32 as both forward forms compute it:
//  * the sample as Dual<3, float>, the FP32 transfer of the mixed forms
//    (rt_sample_fp32_core: emissivity without e2_c, absorptivity through
//    expm1) along the three directions of vjp_common.cuh (inclination, ln
//    Theta_e, ln B), accumulated per ray in FP32;
//  * the geodesic in the arithmetic of the form's forward render, through
//    the same templated code as every other form (step size, rolled RK4,
//    point transcendentals, Christoffels), so the path is the forward's:
//    - mixed-DF (vjp_kernel_df): DF values with FP32 inclination tangents
//      (Dual<1, DF, float>; the tangent needs ~1e-5, not the path's 1e-14);
//    - mixed (vjp_kernel_mixed): FP64 values with FP32 inclination tangents
//      (Dual<1, double, float>): the FP64 path of the mixed forward, with
//      the tangent's arithmetic off the FP64 pipe.
// FP64 is otherwise used once per ray (camera set-up, the forward image's I,
// the scalar gradients) and for the per-cell atomics.
#include <cuda_runtime.h>

#include "df64.cuh"
#include "engine_internal.h"
#include "vjp_common.cuh"

namespace raptor {
namespace {

using DD1 = Dual<1, DF, float>;  // DF value, FP32 inclination tangent
using F1 = Dual<1, float>;
using F3 = Dual<3, float>;
using SampleScalarsF = SampleScalarsT<float>;

// mks_point for the dual DF state: the rolled form (kerr_mks.cuh)
__device__ __forceinline__ void mks_point(DD1 x1, DD1 x2, const GeoDF& g, MksPointT<DD1>& p) {
    mks_point_rolled(x1, x2, g, p);
}

// A geodesic dual as FP32 value and tangent (the leading part of a DF value)
__device__ __forceinline__ F1 to_f1(const DD1& x) {
    F1 r(x.v.hi);
    r.d[0] = x.d[0];
    return r;
}
template <class TD>
__device__ __forceinline__ F1 to_f1(const Dual<1, double, TD>& x) {
    F1 r(f32_of(x.v));
    r.d[0] = tan_cast<float>(x.d[0]);
    return r;
}
__device__ __forceinline__ F3 liftf(const F1& a) {
    F3 r(a.v);
    r.d[kSIncl] = a.d[0];
    return r;
}

// The sample's metric (metric.c:94-137, 207-231) in FP32 with its
// inclination tangent, from the point's values rounded to FP32 (the DF
// point's leading parts, or the FP64 point), as the forward samples'
// metric_f32 (transfer.cuh).
template <class P>
__device__ __forceinline__ MetricT<F1> metric_f1(const MksPointT<P>& pd, const GeoDF& gd) {
    const float a = gd.a.hi, a2 = gd.a2.hi, R0 = gd.R0.hi;
    const F1 r = to_f1(pd.r), s = to_f1(pd.s), irho2 = to_f1(pd.iS);
    const F1 irp = to_f1(pd.irp), ithp = to_f1(pd.ithp), isn = to_f1(pd.isn);
    const F1 s2 = s * s;
    const F1 rfac = r - R0;
    const F1 hfac = to_f1(pd.thp);
    const F1 rho2 = to_f1(pd.Sg);
    const F1 z = 2.0f * (r * irho2);
    const F1 ir = (R0 == 0.0f) ? irp : F1(1.0f) / r;
    const F1 opz = 1.0f + z;
    MetricT<F1> g;
    g.d00 = -1.0f + z;
    g.d01 = z * rfac;
    g.d03 = (-a) * (z * s2);
    g.d11 = opz * rfac * rfac;
    g.d13 = (-a) * (s2 * opz * rfac);
    g.d22 = rho2 * hfac * hfac;
    g.d33 = s2 * (rho2 + a2 * (s2 * opz));
    g.u00 = -1.0f - z;
    g.u01 = 2.0f * irho2;
    g.u11 = irho2 * (r * (r - 2.0f) + a2) * (ir * ir);
    g.u13 = a * (irho2 * ir);
    g.u22 = irho2 * (ithp * ithp);
    g.u33 = irho2 * (isn * isn);
    return g;
}

// a F3 times an F1 (the second's ln Theta_e and ln B tangents are zero)
__device__ __forceinline__ F3 mul31f(const F3& a, const F1& b) {
    F3 r;
    r.v = a.v * b.v;
    r.d[kSIncl] = a.d[kSIncl] * b.v + a.v * b.d[0];
    r.d[kSLnTh] = a.d[kSLnTh] * b.v;
    r.d[kSLnB] = a.d[kSLnB] * b.v;
    return r;
}

// The frequency-independent part of one FP32 sample with three tangents.
struct SampleCommonF {
    F3 kU, nus, jpre, xpre, adl;
    SampleScalarsF ss;
    bool emits;
    int base;        // first of the four cells
    float d1, d2;    // bilinear offsets
    // kappa images (K): B in nus, Theta_e in xpre, n_e in jpre, and the pitch
    // angle's cosine, the inputs of kappa_sample_f
    F3 kcos;
};

// The FP32 sample (rt_sample_fp32_core's fluid, tetrad projection and
// emission prefactors) from its FP32 metric, the first of its four cells and
// the bilinear offsets, the wave vector and |d lambda|, each with its
// inclination tangent.  Everything up to the fluid's Theta_e and B depends
// on the inclination alone and is carried as single-direction duals (F1);
// Theta_e and B take their ln Theta_e and ln B directions, and only what
// depends on them is F3.
// K: the image takes the kappa fits (the adjoint kernels are instantiated
// apart for them, so that the thermal kernels carry none of their code).
template <bool K>
__device__ bool sample_common_f(const DevImage& im, const MetricT<F1>& g, int base, const F1& d1, const F1& d2,
                                const F1 (&k)[4], const F1& adl, SampleCommonF& out) {
    out.base = base;
    out.d1 = d1.v;
    out.d2 = d2.v;
    const F1 c0 = (1.0f - d1) * (1.0f - d2), c1 = (1.0f - d1) * d2, c2 = d1 * (1.0f - d2), c3 = d1 * d2;
    float a[8], b[8], e[8], f[8];
    const float* cp = im.cells32 + (size_t)base * 8;
    load_cell(cp, a);
    load_cell(cp + 8, b);
    load_cell(cp + (size_t)im.n2 * 8, e);
    load_cell(cp + (size_t)im.n2 * 8 + 8, f);
    F1 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = c0 * a[q] + c1 * b[q] + c2 * e[q] + c3 * f[q];

    const F1 B_unit(im.b_unit_f);
    Fluid<F1> fl;
    if (!fluid_from_prims(v, g, F1(im.ne_unit_f), B_unit, F1(im.r_high_f), F1(im.r_low_f), fl)) return false;
    out.ss.irho = fdiv(1.0f, v[0].v);
    thetae_log_derivs(v[0].v, v[1].v, fl.bsq.v, im.r_high_f, im.r_low_f, out.ss.dlnth);
    // |b| in code units for the pitch angle, which M_unit does not move:
    // formed before B takes its ln B direction
    const F1 Bcode = fl.B / B_unit;
    F3 thetae = liftf(fl.thetae), B = liftf(fl.B);
    thetae.d[kSLnTh] = fl.thetae.v;
    B.d[kSLnB] = fl.B.v - 1.e-20f;  // B = sqrt(Bsq) B_unit + tiny: the part that scales

    F1 kd[4];
    lowerT(g, k, kd);
    const F1* U = fl.ucon;
    const F1* Bc = fl.bcon;
    const F1 kU = kd[0] * U[0] + kd[1] * U[1] + kd[2] * U[2] + kd[3] * U[3];
    out.kU = liftf(kU);
    F1 pitch = (kd[0] * Bc[0] + kd[1] * Bc[1] + kd[2] * Bc[2] + kd[3] * Bc[3]) / (fabs(kU) * Bcode);
    if (fabsf(pitch.v) > 1.0f) pitch = F1(pitch.v > 0.0f ? 1.0f : -1.0f);
    out.adl = liftf(adl);
    if constexpr (K) {
        out.nus = B;
        out.xpre = thetae;
        out.jpre = liftf(fl.ne);
        out.kcos = liftf(pitch);
        out.emits = true;
        return true;
    }
    const F1 sth = sqrt(1.0f - pitch * pitch);
    const F3 nuc = (float)(kECharge / (2.0 * CUDART_PI * kEMass * kC)) * B;
    out.nus = mul31f((2.0f / 9.0f) * nuc * thetae * thetae, sth);
    out.emits = (fabsf(sth.v) >= 1.e-10f) && (fl.thetae.v > 1e-4f);
    out.jpre = mul31f(mul31f(nuc, fl.ne * (float)(1.4142135623730951 * CUDART_PI / 27.0)), sth);
    out.xpre = (float)(kPlanck / (kEMass * kC * kC)) / thetae;
    return true;
}

// A kappa image's terms at one frequency: the FP32 sample's kappa branch
// (transfer.cuh, sample_freq_fp32) on the same values, with tangents; out of
// line, the per-sample part recomputed per frequency.
__device__ __noinline__ bool kappa_terms_f(const DevImage& im, const F3& B, const F3& cosp, const F3& thetae,
                                           const F3& ne, const F3& nup, const F3& dlf, F3& S, F3& dtau) {
    const KappaSampleFT<F3> ks = kappa_sample_f(im.kapf, B, cosp, thetae, ne);
    F3 j, a;
    kappa_coeffs_f(im.kapf, ks, nup, j, a);
    if (j.v == 0.0f && a.v == 0.0f) return false;
    const F3 q = fdiv(fdiv(j, nup), nup);
    dtau = nup * a * dlf;
    S = q * dlf;
    return true;
}

// S and delta at frequency fi (rt_sample_fp32_core's arithmetic, emissivity
// without e2_c); false if the frequency does not emit.
template <bool K>
__device__ __forceinline__ bool sample_freq_f(const DevImage& im, const SampleCommonF& sc, int fi, F3& S, F3& dtau) {
    F3 nup = -sc.kU * im.freq_f[fi];
    if (nup.v <= 0.0f) nup = F3(1.0f);
    if constexpr (K)
        return kappa_terms_f(im, sc.nus, sc.kcos, sc.xpre, sc.jpre, nup, sc.adl * im.rg_over_nu_f[fi], S, dtau);
    if (!(sc.emits && nup.v != 1.0f)) return false;
    const F3 dlf = sc.adl * im.rg_over_nu_f[fi];
    const F3 X = nup / sc.nus;
    const F3 cb = cbrt(X);
    const F3 sq = sqrt(cb) * (cb + 1.8877486f);  // X^1/2 + 2^(11/12) X^1/6
    const F3 jh = sc.jpre * (sq * sq) * exp(-cb);
    const F3 q = (jh / nup) / nup;
    dtau = q * expm1(sc.xpre * nup) * (float)(kE2CH * kC * kC * 0.5) * dlf;
    S = q * dlf;
    return true;
}

// ------------------------------------------------------------ the two forms
// What the adjoint body needs of a form's geodesic: the state type (a value
// with its inclination tangent), its constants, the step size, the stopping
// and sampling tests in the forward kernel's arithmetic, and the sample's
// FP32 inputs from the state.

// Mixed-DF: the geodesic of ray_kernel_df.
struct FormDF {
    using S = DD1;
    using Th = float;  // d x2 / d lambda as the theta-turn test reads it
    static constexpr bool kMergeReplay = false;  // vjp_f32_body's record replay
    __device__ static const GeoDF& geo(const DevImage& im) { return im.geo_df; }
    __device__ static S from_camera(const D1& y) {
        S s(df_const(y.v));
        s.d[0] = (float)y.d[0];
        return s;
    }
    // stepsize (integrator.c:109-122) as step_size_df
    __device__ static S step(const DevImage& im, const S y[8]) {
        const DF t = df_const(1.e-40);
        const S m2 = fmin(y[2], 1.0 - y[2]);
        const S i13 = (fabs(y[5]) + t) + (fabs(y[7]) + t);
        const S i2 = fabs(y[6]) + t;
        return -fmax(m2 / ((m2 * i13 + i2) * im.inv_stepsize_df), 1e-12);
    }
    __device__ static bool alive(const DevImage& im, const MksPointT<S>& p, int steps, int stop) {
        const DF r = p.rp.v;
        return r < df_const(kCutoffOuter) && r > im.cutoff_inner_df && steps < (int)kMaxSteps && !stop;
    }
    __device__ static Th theta_rate(const S& y6) { return y6.v.hi; }
    __device__ static bool turned(Th prev, Th now) {
        return (prev < 0.0f && now > 0.0f) || (prev > 0.0f && now < 0.0f);
    }
    __device__ static bool escaped(const DevImage& im, const S y[8]) {
        return y[1].v > im.stopx1_df && y[5].v.hi < 0.0f;
    }
    // a finite photon state at the ray's end, as finish_ray tests it
    __device__ static bool finite(const MksPointT<S>& p, const S y[8]) {
        return p.rp.v.hi == p.rp.v.hi && isfinite(y[5].v.hi);
    }
    __device__ static bool in_grid(const DevImage& im, const S y[8]) {
        return y[1].v < im.stopx1_df && y[1].v > im.startx1_df && y[2].v > im.startx2_df && y[2].v < im.stopx2_df;
    }
    // rt_sample_df's inputs: Xtoij (grmhd.c:46-71) from the DF position,
    // the offsets carrying the inclination tangent unless clamped
    template <bool K>
    __device__ static bool sample(const DevImage& im, const S y[8], const MksPointT<S>& p, const S& adl,
                                  SampleCommonF& out) {
        const MetricT<F1> g = metric_f1(p, im.geo_df);
        const DF t1 = (y[1].v - im.startx1_df) * im.idx1_df - 0.5;
        const DF t2 = (y[2].v - im.startx2_df) * im.idx2_df - 0.5;
        int i = df_trunc(t1), j = df_trunc(t2);
        F1 d1(0.0f), d2(0.0f);
        if (i < 0) i = 0;
        else if (i > im.n1 - 2) { i = im.n1 - 2; d1 = F1(1.0f); }
        else { d1 = F1(df_value(add_f(t1, (float)-i))); d1.d[0] = y[1].d[0] * im.idx1_df.hi; }
        if (j < 0) j = 0;
        else if (j > im.n2 - 2) { j = im.n2 - 2; d2 = F1(1.0f); }
        else { d2 = F1(df_value(add_f(t2, (float)-j))); d2.d[0] = y[2].d[0] * im.idx2_df.hi; }
        if (!chk(i >= 0 && i <= im.n1 - 2 && j >= 0 && j <= im.n2 - 2, im.check_word, kChkCell,
                 (long long)i * im.n2 + j))
            i = j = 0;
        const F1 k[4] = {to_f1(y[4]), to_f1(y[5]), to_f1(y[6]), to_f1(y[7])};
        return sample_common_f<K>(im, g, i * im.n2 + j, d1, d2, k, to_f1(adl), out);
    }
};

// Mixed: the FP64 geodesic of ray_kernel<NF, true>, with the inclination
// tangent in TD.
template <class TD>
struct FormMixed {
    using S = Dual<1, double, TD>;
    using Th = double;
    static constexpr bool kMergeReplay = true;  // vjp_f32_body's record replay
    __device__ static const Geo& geo(const DevImage& im) { return im.geo; }
    __device__ static S from_camera(const D1& y) {
        S s(y.v);
        s.d[0] = (TD)y.d[0];
        return s;
    }
    __device__ static S step(const DevImage& im, const S y[8]) { return step_size(im, y); }
    // the while-condition of integrator.c:228-229, as advance_ray
    __device__ static bool alive(const DevImage& im, const MksPointT<S>& p, int steps, int stop) {
        const double r = p.rp.v;
        return r < kCutoffOuter && r > im.cutoff_inner && (double)steps < kMaxSteps && !stop;
    }
    __device__ static Th theta_rate(const S& y6) { return y6.v; }
    __device__ static bool turned(Th prev, Th now) { return prev * now < 0.0; }
    __device__ static bool escaped(const DevImage& im, const S y[8]) { return y[1].v > im.stopx1 && y[5].v < 0.0; }
    __device__ static bool in_grid(const DevImage& im, const S y[8]) {
        return y[1].v < im.stopx1 && y[1].v > im.startx1 && y[2].v > im.startx2 && y[2].v < im.stopx2;
    }
    __device__ static bool finite(const MksPointT<S>& p, const S y[8]) {
        return p.rp.v == p.rp.v && isfinite(y[5].v);
    }
    // rt_sample_fp32's inputs: the metric in FP32 from the FP64 point
    // rounded (with its tangent), Xtoij in FP64 (cell_coef), the wave vector
    // rounded to FP32
    template <bool K>
    __device__ static bool sample(const DevImage& im, const S y[8], const MksPointT<S>& p, const S& adl,
                                  SampleCommonF& out) {
        const MetricT<F1> g = metric_f1(p, im.geo_df);
        const CellCoef cc = cell_coef(im, y[1].v, y[2].v);
        const int i = cc.base / im.n2, j = cc.base - i * im.n2;
        F1 d1(f32_of(cc.d1)), d2(f32_of(cc.d2));
        const double t1 = (y[1].v - im.startx1) * im.idx1 - 0.5;
        const double t2 = (y[2].v - im.startx2) * im.idx2 - 0.5;
        if ((int)t1 == i) d1.d[0] = y[1].d[0] * im.idx1_df.hi;  // not clamped
        if ((int)t2 == j) d2.d[0] = y[2].d[0] * im.idx2_df.hi;
        const F1 k[4] = {to_f1(y[4]), to_f1(y[5]), to_f1(y[6]), to_f1(y[7])};
        return sample_common_f<K>(im, g, cc.base, d1, d2, k, to_f1(adl), out);
    }
};

template <int NF, class F>
struct AdjState {
    typename F::S y[8];
    MksPointT<typename F::S> p;
    typename F::Th thdot_prev;
    int bsign, steps, turns, stop, pix;
    float tau[NF], Ipart[NF], Itot[NF], w[NF];
    float dtg[NF][4];
    float dIw[4];
    int wexp;  // w[f] holds dL/dI_f * 2^-wexp; the ray's gradient terms are scaled back by 2^wexp
    int nrec;     // one-pass adjoint: records on the lane's tape
    bool full;    // one-pass adjoint: a record did not fit
    bool replay;  // one-pass adjoint: the ended ray's records wait for the warp
};

// 2^e as a double for e in [-1022, 1023] (built from the exponent field).
__device__ __forceinline__ double pow2_double(int e) {
    e = min(max(e, -1022), 1023);
    return __longlong_as_double((long long)(e + 1023) << 52);
}

// One sample's loss gradient with respect to the four cells' fields: Gr,
// Gt, Gu the derivatives with respect to ln rho, ln Theta_e and ln u at the
// sample (scaled by 2^-wexp), spread bilinearly over the cells.
__device__ __forceinline__ void scatter_sample(float Gr, float Gt, float Gu, int base, float d1, float d2, int n2,
                                               int wexp, double* __restrict__ g_rho, double* __restrict__ g_u,
                                               double* __restrict__ g_th) {
    if ((Gr != 0.0f || Gt != 0.0f) && isfinite(Gr) && isfinite(Gt) && isfinite(Gu)) {
        const float w0 = (1.0f - d1) * (1.0f - d2), w1 = (1.0f - d1) * d2;
        const float w2 = d1 * (1.0f - d2), w3 = d1 * d2;
        const long long c = base, cn = (long long)base + n2;
        const double un = pow2_double(wexp);
        const double gr = (double)Gr * un, gu = (double)Gu * un, gt = (double)Gt * un;
        atomicAdd(&g_rho[c], gr * w0);
        atomicAdd(&g_rho[c + 1], gr * w1);
        atomicAdd(&g_rho[cn], gr * w2);
        atomicAdd(&g_rho[cn + 1], gr * w3);
        atomicAdd(&g_u[c], gu * w0);
        atomicAdd(&g_u[c + 1], gu * w1);
        atomicAdd(&g_u[cn], gu * w2);
        atomicAdd(&g_u[cn + 1], gu * w3);
        atomicAdd(&g_th[c], gt * w0);
        atomicAdd(&g_th[c + 1], gt * w1);
        atomicAdd(&g_th[cn], gt * w2);
        atomicAdd(&g_th[cn + 1], gt * w3);
    }
}

// Per-cell sums m (d/d ln rho, d/d ln u, d/d ln Theta_e on the four cells
// from base; scaled by 2^-wexp) added to the gradient arrays.
__device__ __forceinline__ void flush_cells(const float (&m)[12], int base, int n2, int wexp,
                                            double* __restrict__ g_rho, double* __restrict__ g_u,
                                            double* __restrict__ g_th) {
    const double un = pow2_double(wexp);
    const long long c[4] = {base, (long long)base + 1, (long long)base + n2, (long long)base + n2 + 1};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        atomicAdd(&g_rho[c[q]], (double)m[q] * un);
        atomicAdd(&g_u[c[q]], (double)m[4 + q] * un);
        atomicAdd(&g_th[c[q]], (double)m[8 + q] * un);
    }
}

// The adjoint pass: lanes take rays from the queue and refill every
// refill_interval steps, as the forward kernels do.
//
// A sample's loss gradient with respect to its cells' fields takes, per
// frequency, the intensity the ray gathers after it (the suffix I - I_before
// of the transfer's exact derivative).  Two passes (TAPE false) read the
// ray's I from the forward render of the same form.  One pass (TAPE) has
// none: each sample inside the tau gate of some frequency writes a record to
// the lane's tape - cell, offsets, d ln Theta_e / d ln u, the gated parts of
// Gr and Gt, and per frequency I_before and the suffix coefficients - and
// when the ray ends its own I (the same sums) closes the records, which are
// then scattered; the pass also writes that I as the image.  Samples with
// every frequency past the gate need no record: tau does not decrease (the
// absorptivities are non-negative), so no later sample adds to I and their
// suffix is exactly 0.
template <int NF, class F, bool K, bool TAPE>
__device__ __forceinline__ void vjp_f32_body(const DevImage& im, const CamT<D1>& cam, const double* __restrict__ fwd,
                                             const double* __restrict__ dLdO, unsigned long long* __restrict__ counters,
                                             double* __restrict__ gscal, double* __restrict__ g_rho,
                                             double* __restrict__ g_u, double* __restrict__ g_th,
                                             int refill_interval, RayRange rr, VjpTape tape) {
    using S = typename F::S;
    using G = typename std::remove_cv<typename std::remove_reference<decltype(F::geo(im))>::type>::type;
    const int lane = threadIdx.x & 31;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    unsigned long long n_calls = 0, n_samples = 0, n_emit = 0, n_gate = 0, n_steps = 0, n_rays = 0;
    unsigned long long n_nan = 0, n_cap = 0, n_full = 0;
    // this lane's records (one pass, per-cell gradients asked for)
    const size_t lane_floats = (size_t)tape.cap * (size_t)tape.stride;
    float* const lane_tape =
        TAPE && g_rho ? static_cast<float*>(tape.rec) + ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * lane_floats
                      : nullptr;
    AdjState<NF, F> s;
    s.replay = false;
    bool active = false, live = true;
    while (true) {
        if constexpr (TAPE) {
            // The records of rays that ended, closed with their I and
            // scattered by the whole warp: replayed by their own lane they
            // would hold the warp for ~nrec record bodies, with the other
            // lanes idle.  F::kMergeReplay: each lane takes a contiguous run
            // of the ray's records and sums consecutive records of one cell
            // before its atomics (fewer atomics, the lanes of one atomic
            // instruction in different cells; uncoalesced record loads);
            // else lane l takes records l, l + 32, ... (coalesced loads).
            // 1024x1024, five frequencies: the mixed adjoint 529 -> 505 ms
            // merged, the issue-bound mixed-DF one 190 -> 210 ms.
            unsigned pend = __ballot_sync(kFull, s.replay);
            if (pend) __syncwarp();  // the owners' record stores before the loads
            while (pend) {
                const int owner = __ffs(pend) - 1;
                pend &= pend - 1;
                const int nrec = __shfl_sync(kFull, s.nrec, owner);
                const int wexp = __shfl_sync(kFull, s.wexp, owner);
                float itot[NF];
#pragma unroll
                for (int f = 0; f < NF; ++f) itot[f] = __shfl_sync(kFull, s.Ipart[f], owner);
                const float* otape = lane_tape + (long long)(owner - lane) * (long long)lane_floats;
                if constexpr (F::kMergeReplay) {
                    const int run = (nrec + 31) >> 5, rend = min(lane * run + run, nrec);
                    int cb = -1;
                    float m[12];
                    for (int r = lane * run; r < rend; ++r) {
                        const float* rq = otape + (size_t)r * (size_t)tape.stride;
                        float Gr = rq[4], Gt = rq[5];
#pragma unroll
                        for (int f = 0; f < NF; ++f) {
                            if (f >= im.nfreq) break;
                            const float suffix = itot[f] - rq[6 + 3 * f];
                            Gr -= rq[7 + 3 * f] * suffix;
                            Gt -= rq[8 + 3 * f] * suffix;
                        }
                        const float Gu = Gt * rq[3];
                        if (!((Gr != 0.0f || Gt != 0.0f) && isfinite(Gr) && isfinite(Gt) && isfinite(Gu))) continue;
                        const int base = __float_as_int(rq[0]);
                        if (base != cb) {
                            if (cb >= 0) flush_cells(m, cb, im.n2, wexp, g_rho, g_u, g_th);
                            cb = base;
#pragma unroll
                            for (int q = 0; q < 12; ++q) m[q] = 0.0f;
                        }
                        const float d1 = rq[1], d2 = rq[2];
                        const float wc[4] = {(1.0f - d1) * (1.0f - d2), (1.0f - d1) * d2, d1 * (1.0f - d2), d1 * d2};
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            m[q] += Gr * wc[q];
                            m[4 + q] += Gu * wc[q];
                            m[8 + q] += Gt * wc[q];
                        }
                    }
                    if (cb >= 0) flush_cells(m, cb, im.n2, wexp, g_rho, g_u, g_th);
                } else {
                    for (int r = lane; r < nrec; r += 32) {
                        const float* rq = otape + (size_t)r * (size_t)tape.stride;
                        float Gr = rq[4], Gt = rq[5];
#pragma unroll
                        for (int f = 0; f < NF; ++f) {
                            if (f >= im.nfreq) break;
                            const float suffix = itot[f] - rq[6 + 3 * f];
                            Gr -= rq[7 + 3 * f] * suffix;
                            Gt -= rq[8 + 3 * f] * suffix;
                        }
                        scatter_sample(Gr, Gt, Gt * rq[3], __float_as_int(rq[0]), rq[1], rq[2], im.n2, wexp, g_rho,
                                       g_u, g_th);
                    }
                }
            }
            s.replay = false;
        }
        const unsigned need = __ballot_sync(kFull, !active && live);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&counters[kCtrQueue], (unsigned long long)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (!active && live) {
                const long long rid = rr.begin + (long long)(base + __popc(need & ((1u << lane) - 1u)));
                if (rid < rr.end) {
                    s.pix = (int)rid;
                    const int px = s.pix % im.width, py = s.pix / im.width;
                    D1 y0[8];
                    double beta;
                    init_photon(im, cam, px, py, y0, beta);  // FP64 duals, once per ray
#pragma unroll
                    for (int i = 0; i < 8; ++i) s.y[i] = F::from_camera(y0[i]);
                    s.bsign = (beta < 0.0) ? -1 : ((beta > 0.0) ? 1 : 0);
                    mks_point(s.y[1], s.y[2], F::geo(im), s.p);
                    const PixelScale ps = pixel_scale(im, px);
                    // The loss weights dL/dO * dO/dI can sit far outside FP32's range (the
                    // log-polar camera's dO/dI carries 1/D^2); scale them by a power of two
                    // so the largest is in [0.5, 1) and undo the scale in FP64.
                    double wmax = 0.0;
                    for (int f = 0; f < im.nfreq && f < NF; ++f) {
                        const long long o = (long long)s.pix * im.nfreq + f;
                        const double wf = fabs(dLdO[o] * scale_output(im, ps, 1.0, f) * kE2C);
                        if (isfinite(wf)) wmax = fmax(wmax, wf);
                    }
                    s.wexp = 0;
                    if (wmax > 0.0) frexp(wmax, &s.wexp);
                    s.wexp = min(max(s.wexp, -1022), 1022);  // 2^wexp and 2^-wexp both normal
                    const double wscale = pow2_double(-s.wexp);
#pragma unroll
                    for (int f = 0; f < NF; ++f) {
                        s.tau[f] = 0.0f;
                        s.Ipart[f] = 0.0f;
                        s.Itot[f] = 0.0f;
                        s.w[f] = 0.0f;
#pragma unroll
                        for (int q = 0; q < 4; ++q) s.dtg[f][q] = 0.0f;
                        if (f < im.nfreq) {
                            // I in the units of the FP32 transfer (without e2_c)
                            const long long o = (long long)s.pix * im.nfreq + f;
                            const double dOdI = scale_output(im, ps, 1.0, f) * kE2C;
                            if constexpr (!TAPE) s.Itot[f] = (float)(fwd[o] / dOdI);
                            s.w[f] = (float)(dLdO[o] * dOdI * wscale);
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) s.dIw[q] = 0.0f;
                    s.steps = 0;
                    s.turns = 0;
                    s.stop = 0;
                    s.thdot_prev = 0;
                    s.nrec = 0;
                    s.full = false;
                    active = true;
                } else {
                    live = false;
                }
            }
        }
        if (!__any_sync(kFull, active)) break;
        if (!active) continue;
        for (int it = 0; it < refill_interval; ++it) {
            bool done = !F::alive(im, s.p, s.steps, s.stop);
            if (!done) {
                const typename F::Th th = F::theta_rate(s.y[6]);
                if (F::turned(s.thdot_prev, th) && s.steps > 2) s.turns += 1;
                s.thdot_prev = th;
                if ((s.bsign < 0 && s.turns > kMaxOrder) || (s.bsign > 0 && s.turns > kMaxOrder + 1)) s.stop = 1;
                const S dl = F::step(im, s.y);
                if (im.integrator == 2) rk2_step<S, G, false>(F::geo(im), s.y, s.p, dl);
                else rk4_step_rolled<S, G, false>(F::geo(im), s.y, s.p, dl);
                s.steps += 1;
                if (F::escaped(im, s.y)) {
                    done = true;
                } else if (F::in_grid(im, s.y)) {
                    ++n_calls;
                    SampleCommonF sc;
                    if (F::template sample<K>(im, s.y, s.p, fabs(dl), sc)) {
                        ++n_samples;
                        float Gr = 0.0f, Gt = 0.0f;
                        // one pass: this sample's record, if it has room
                        float* const rp = lane_tape && s.nrec < tape.cap
                                              ? lane_tape + (size_t)s.nrec * (size_t)tape.stride
                                              : nullptr;
                        bool live = false;
                        // one copy of the frequency body (the per-frequency
                        // state of a multi-frequency ray lives in local memory)
#pragma unroll 1
                        for (int f = 0; f < NF; ++f) {
                            if (f >= im.nfreq) break;
                            F3 S3, dt;
                            if (!sample_freq_f<K>(im, sc, f, S3, dt)) {
                                if (TAPE && rp) {
                                    rp[6 + 3 * f] = 0.0f;
                                    rp[7 + 3 * f] = 0.0f;
                                    rp[8 + 3 * f] = 0.0f;
                                }
                                continue;
                            }
                            ++n_emit;
                            s.tau[f] += dt.v;
#pragma unroll
                            for (int q = 0; q < 4; ++q) s.dtg[f][q] += scalar_tangent(dt, sc.ss, q);
                            const float e = expf(-s.tau[f]);
                            const bool gate = s.tau[f] < 6.9077553f && !(s.tau[f] < 0.0f);
                            const float eS = gate ? e : 0.0f;
                            if constexpr (TAPE) {
                                // the gated part now; the suffix part, with I,
                                // when the ray ends
                                Gr += s.w[f] * (eS * rho_tangent(S3, sc.ss));
                                Gt += s.w[f] * (eS * S3.d[kSLnTh]);
                                if (rp) {
                                    rp[6 + 3 * f] = s.Ipart[f];
                                    rp[7 + 3 * f] = s.w[f] * rho_tangent(dt, sc.ss);
                                    rp[8 + 3 * f] = s.w[f] * dt.d[kSLnTh];
                                }
                                live = live || gate;
                            } else {
                                const float suffix = s.Itot[f] - s.Ipart[f];
                                Gr += s.w[f] * (eS * rho_tangent(S3, sc.ss) - suffix * rho_tangent(dt, sc.ss));
                                Gt += s.w[f] * (eS * S3.d[kSLnTh] - suffix * dt.d[kSLnTh]);
                            }
                            if (gate) {
                                ++n_gate;
                                const float we = s.w[f] * e;
#pragma unroll
                                for (int q = 0; q < 4; ++q)
                                    s.dIw[q] += we * (scalar_tangent(S3, sc.ss, q) - S3.v * s.dtg[f][q]);
                                s.Ipart[f] += S3.v * e;
                            }
                        }
                        if constexpr (TAPE) {
                            if (live && lane_tape) {
                                if (rp) {
                                    rp[0] = __int_as_float(sc.base);
                                    rp[1] = sc.d1;
                                    rp[2] = sc.d2;
                                    rp[3] = sc.ss.dlnth[1];
                                    rp[4] = Gr;
                                    rp[5] = Gt;
                                    ++s.nrec;
                                } else {
                                    s.full = true;
                                }
                            }
                        } else if (g_rho) {
                            scatter_sample(Gr, Gt, Gt * sc.ss.dlnth[1], sc.base, sc.d1, sc.d2, im.n2, s.wexp, g_rho,
                                           g_u, g_th);
                        }
                    }
                }
            }
            if (done) {
                if constexpr (TAPE) {
                    // the ray's own I: the pass's image, and the suffixes
                    // that close its records
                    const long long oi = im.out_offset + (long long)s.pix * im.nfreq;
                    const bool in_bounds = chk(oi >= 0 && oi + im.nfreq <= im.out_end, im.check_word, kChkOutput, oi);
                    const PixelScale ps = pixel_scale(im, s.pix % im.width);
                    bool finite = F::finite(s.p, s.y);
#pragma unroll
                    for (int f = 0; f < NF; ++f) {
                        if (f >= im.nfreq || !in_bounds) break;
                        const double o = scale_output(im, ps, (double)s.Ipart[f] * kE2C, f);
                        tape.out[oi + f] = o;
                        finite = finite && isfinite(o);
                    }
                    if (!finite) ++n_nan;
                    if ((double)s.steps >= kMaxSteps) ++n_cap;
                    if (s.full) ++n_full;  // the call falls back to two passes
                    else s.replay = lane_tape && s.nrec > 0;  // at the warp's next refill
                }
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (isfinite(s.dIw[q])) acc[q] += (double)s.dIw[q] * pow2_double(s.wexp);
                n_steps += (unsigned long long)s.steps;
                n_rays += 1;
                active = false;
                break;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        n_steps += __shfl_xor_sync(kFull, n_steps, o);
        n_rays += __shfl_xor_sync(kFull, n_rays, o);
        n_calls += __shfl_xor_sync(kFull, n_calls, o);
        n_samples += __shfl_xor_sync(kFull, n_samples, o);
        n_emit += __shfl_xor_sync(kFull, n_emit, o);
        n_gate += __shfl_xor_sync(kFull, n_gate, o);
        if (TAPE) {
            n_nan += __shfl_xor_sync(kFull, n_nan, o);
            n_cap += __shfl_xor_sync(kFull, n_cap, o);
            n_full += __shfl_xor_sync(kFull, n_full, o);
        }
    }
    if (lane == 0) {
        atomicAdd(&counters[kCtrSteps], n_steps);
        atomicAdd(&counters[kCtrRays], n_rays);
        atomicAdd(&counters[kCtrRtCalls], n_calls);
        atomicAdd(&counters[kCtrRtSamples], n_samples);
        atomicAdd(&counters[kCtrVjpEmit], n_emit);
        atomicAdd(&counters[kCtrVjpGate], n_gate);
        if (TAPE) {
            atomicAdd(&counters[kCtrNonFinite], n_nan);
            atomicAdd(&counters[kCtrStepCap], n_cap);
            atomicAdd(&counters[kCtrTapeFull], n_full);
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        double v = acc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
        if (lane == 0) atomicAdd(&gscal[q], v);
    }
}

#ifndef RAPTOR_VJP_DF_MIN_BLOCKS
#define RAPTOR_VJP_DF_MIN_BLOCKS 2
#endif
#ifndef RAPTOR_VJP_MIXED_MIN_BLOCKS
#define RAPTOR_VJP_MIXED_MIN_BLOCKS 2
#endif
// The mixed adjoint's inclination tangent: FP32 (1), which keeps its
// arithmetic off the FP64 pipe, or FP64 (0).
#ifndef RAPTOR_VJP_MIXED_TANGENT_FP32
#define RAPTOR_VJP_MIXED_TANGENT_FP32 1
#endif
using MixedTangent = std::conditional<RAPTOR_VJP_MIXED_TANGENT_FP32 != 0, float, double>::type;

template <int NF, bool K, bool TAPE>
__global__ void __launch_bounds__(kVjpBlock, RAPTOR_VJP_DF_MIN_BLOCKS)
    vjp_kernel_df(const DevImage* __restrict__ imp, CamT<D1> cam, const double* __restrict__ fwd,
                  const double* __restrict__ dLdO, unsigned long long* __restrict__ counters,
                  double* __restrict__ gscal, double* __restrict__ g_rho, double* __restrict__ g_u,
                  double* __restrict__ g_th, int refill_interval, RayRange rr, VjpTape tape) {
    vjp_f32_body<NF, FormDF, K, TAPE>(*imp, cam, fwd, dLdO, counters, gscal, g_rho, g_u, g_th, refill_interval, rr,
                                      tape);
}

template <int NF, bool K, bool TAPE>
__global__ void __launch_bounds__(kVjpBlock, RAPTOR_VJP_MIXED_MIN_BLOCKS)
    vjp_kernel_mixed(const DevImage* __restrict__ imp, CamT<D1> cam, const double* __restrict__ fwd,
                     const double* __restrict__ dLdO, unsigned long long* __restrict__ counters,
                     double* __restrict__ gscal, double* __restrict__ g_rho, double* __restrict__ g_u,
                     double* __restrict__ g_th, int refill_interval, RayRange rr, VjpTape tape) {
    vjp_f32_body<NF, FormMixed<MixedTangent>, K, TAPE>(*imp, cam, fwd, dLdO, counters, gscal, g_rho, g_u, g_th,
                                                       refill_interval, rr, tape);
}

template <int NF, bool K, bool TAPE>
void launch_vjp_df(int grid, cudaStream_t st, const DevImage* im, const CamT<D1>& cam, const double* fwd,
                   const double* dl, unsigned long long* ctr, double* gs, double* gr, double* gu, double* gt,
                   int refill, double*, RayRange rr, VjpTape tape) {
    vjp_kernel_df<NF, K, TAPE><<<grid, kVjpBlock, 0, st>>>(im, cam, fwd, dl, ctr, gs, gr, gu, gt, refill, rr, tape);
}

template <int NF, bool K, bool TAPE>
void launch_vjp_mixed(int grid, cudaStream_t st, const DevImage* im, const CamT<D1>& cam, const double* fwd,
                      const double* dl, unsigned long long* ctr, double* gs, double* gr, double* gu, double* gt,
                      int refill, double*, RayRange rr, VjpTape tape) {
    vjp_kernel_mixed<NF, K, TAPE><<<grid, kVjpBlock, 0, st>>>(im, cam, fwd, dl, ctr, gs, gr, gu, gt, refill, rr,
                                                              tape);
}

template <bool TAPE>
VjpLaunchFn pick_df(int nf, const void** fn, bool kappa) {
    if (kappa) {
        *fn = (const void*)vjp_kernel_df<kMaxFreqs, true, TAPE>;
        return launch_vjp_df<kMaxFreqs, true, TAPE>;
    }
    if (nf <= 1) {
        *fn = (const void*)vjp_kernel_df<1, false, TAPE>;
        return launch_vjp_df<1, false, TAPE>;
    }
    *fn = (const void*)vjp_kernel_df<kMaxFreqs, false, TAPE>;
    return launch_vjp_df<kMaxFreqs, false, TAPE>;
}

template <bool TAPE>
VjpLaunchFn pick_mixed(int nf, const void** fn, bool kappa) {
    if (kappa) {
        *fn = (const void*)vjp_kernel_mixed<kMaxFreqs, true, TAPE>;
        return launch_vjp_mixed<kMaxFreqs, true, TAPE>;
    }
    if (nf <= 1) {
        *fn = (const void*)vjp_kernel_mixed<1, false, TAPE>;
        return launch_vjp_mixed<1, false, TAPE>;
    }
    *fn = (const void*)vjp_kernel_mixed<kMaxFreqs, false, TAPE>;
    return launch_vjp_mixed<kMaxFreqs, false, TAPE>;
}

}  // namespace

// kappa: the kappa fits' instantiation (any frequency count); tape: the
// one-pass kernel
VjpLaunchFn pick_vjp_df(int nf, const void** fn, bool kappa, bool tape) {
    return tape ? pick_df<true>(nf, fn, kappa) : pick_df<false>(nf, fn, kappa);
}

VjpLaunchFn pick_vjp_mixed(int nf, const void** fn, bool kappa, bool tape) {
    return tape ? pick_mixed<true>(nf, fn, kappa) : pick_mixed<false>(nf, fn, kappa);
}

}  // namespace raptor
