// Vector-Jacobian product of one image: raptor_gpu_vjp.
//
// Given dL/dO for the rendered image O (the nu^3-scaled intensities of
// core.c:136), returns dL/d(M_UNIT, R_HIGH, R_LOW, INCLINATION) and, per grid
// cell, dL/d rho, dL/d u and dL/d ln Theta_e (Theta_e of the samples scaled by
// a bilinear per-cell factor).
//
// Structure of the computation, per ray and frequency (radiative_transfer.c:
// 88-95): with delta_k = nu_p a dl and S_k = j / nu_p^2 dl at sample k,
//   tau_k = sum_{m<=k} delta_m,   I = sum_k g_k S_k exp(-tau_k),
// g_k the ln(1000) gate (held fixed).  Then
//   dI/dS_k     = g_k exp(-tau_k)
//   dI/ddelta_k = -sum_{k'>=k} g_k' S_k' exp(-tau_k') = -(I - I_<k)
// so one forward sweep over the ray, knowing the ray's final I from the
// forward render, gives the exact reverse-mode sensitivities of every sample
// without storing or re-walking the ray backwards.
//
// * The four scalars go forward mode: the ray carries d tau / d theta and
//   accumulates dI/d theta = sum_k g_k e^-tau_k (dS_k/d theta - S_k dtau_k/d theta).
// * The inclination moves the camera and so the whole geodesic: its tangent
//   runs through the camera constants (host, below) and every RK stage
//   (Dual<1> over the same templated FP64 code as the forward kernel).
// * The per-cell fields enter a sample only through the bilinear rho and u
//   (grmhd.c:35-44), so each sample scatters
//   w (g e^-tau dS/drho_s - (I - I_<k) ddelta/drho_s) times the four bilinear
//   weights into dL/drho with FP64 atomics.  u reaches the emission only
//   through Theta_e (raptor_harm_model.c:261-271), so the sample carries the
//   direction d/d ln Theta_e instead of d/du_s and scatters both it and
//   its product with d ln Theta_e/du_s.
// Discrete decisions (step count, gates, sigma cut, clamps) are those of the
// primal, as a finite difference of small step sees them.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine_internal.h"
#include "vjp_common.cuh"

using namespace raptor;

namespace {

// The FP64 adjoint's sample: value and the three directions of
// vjp_common.cuh (inclination, ln Theta_e, ln B) in FP64.
using D3 = Dual<3>;
using SampleScalars = SampleScalarsT<double>;

__device__ __forceinline__ D3 lift(const D1& a) {
    D3 r(a.v);
    r.d[kSIncl] = a.d[0];
    return r;
}

// A D3 times a D1, whose only direction is the inclination: the product's ln
// Theta_e and ln B tangents are a's scaled by b's value.  Equal to the D3
// product with b lifted (whose two zero tangents add exact zeros), at two
// FP64 operations fewer per direction.
__device__ __forceinline__ D3 mul31(const D3& a, const D1& b) {
    D3 r;
    r.v = a.v * b.v;
    r.d[kSIncl] = a.d[kSIncl] * b.v + a.v * b.d[0];
    r.d[kSLnTh] = a.d[kSLnTh] * b.v;
    r.d[kSLnB] = a.d[kSLnB] * b.v;
    return r;
}

// The frequency-independent part of one transfer sample, as value + three
// tangents: the same arithmetic as rt_sample_fp64 (get_fluid_params
// raptor_harm_model.c:190-290, pitch_angle radiative_transfer.c:32-47,
// j_nu.c:130-153, 188-200) up to the frequency loop.  Everything up to the
// fluid's Theta_e and B - metric, cell offsets, interpolated primitives,
// four-velocity, field, pitch angle - depends on the inclination alone and
// is carried as D1; Theta_e and B take their ln Theta_e and ln B directions,
// and only what depends on them is D3.
struct SampleCommon {
    D1 kU;        // k_mu u^mu
    D3 inus;      // 1 / nu_s
    D1 ikU2;      // 1 / (k.u)^2: 1/nu_p^2 = ikU2 / nu^2
    D3 pre;       // n_e sqrt(2) pi nu_s e2_c / (3 K2), the first factors of j
    D3 hkt;       // h / (k_B T): h nu / (k_B T) per Hz
    D1 adl;       // |d lambda|
    double nus;   // nu_s
    double ikU;   // 1 / (k.u)
    SampleScalars ss;
    bool emits;
    // kappa images (K): B in pre, Theta_e in hkt, and n_e and the pitch
    // angle's cosine, the inputs of kappa_sample
    D1 kne, kcos;
};

// K: the image takes the kappa fits (the adjoint kernels are instantiated
// apart for them, so that the thermal kernels carry none of their code).
template <bool K>
__device__ bool sample_common(const DevImage& im, const D1& x1, const D1& x2, const D1 k1[4], const MksPointT<D1>& p,
                              const D1& adl1, CellCoef& cc, SampleCommon& out) {
    MetricDDT<D1> gd1;
    MetricUUT<D1> gu1;
    mks_metric(p, im.geo, gd1, gu1);
    MetricT<D1> g;
    g.d00 = gd1.g00; g.d01 = gd1.g01; g.d03 = gd1.g03; g.d11 = gd1.g11;
    g.d13 = gd1.g13; g.d22 = gd1.g22; g.d33 = gd1.g33;
    g.u00 = gu1.g00; g.u01 = gu1.g01; g.u11 = gu1.g11; g.u13 = gu1.g13;
    g.u22 = gu1.g22; g.u33 = gu1.g33;

    // Xtoij with the fractional offsets carrying their inclination tangent
    cc = cell_coef(im, x1.v, x2.v);
    const int i = cc.base / im.n2, j = cc.base % im.n2;
    D1 d1 = D1(cc.d1), d2 = D1(cc.d2);
    {
        const double t1 = (x1.v - im.startx1) * im.idx1 - 0.5;
        const double t2 = (x2.v - im.startx2) * im.idx2 - 0.5;
        if ((int)t1 == i) d1.d[0] = x1.d[0] * im.idx1;  // not clamped
        if ((int)t2 == j) d2.d[0] = x2.d[0] * im.idx2;
    }
    const D1 c0 = (1.0 - d1) * (1.0 - d2), c1 = (1.0 - d1) * d2, c2 = d1 * (1.0 - d2), c3 = d1 * d2;
    double a[8], b[8], e[8], f[8];
    const double* cp = im.cells64 + (size_t)cc.base * 8;
    load_cell(cp, a);
    load_cell(cp + 8, b);
    load_cell(cp + (size_t)im.n2 * 8, e);
    load_cell(cp + (size_t)im.n2 * 8 + 8, f);
    D1 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = c0 * a[q] + c1 * b[q] + c2 * e[q] + c3 * f[q];

    Fluid<D1> fl;
    if (!fluid_fast(v, g, D1(im.Ne_unit), D1(im.B_unit), D1(im.r_high), D1(im.r_low), fl)) return false;
    out.ss.irho = fl.irho.v;
    thetae_log_derivs_fp64(fl.irho.v, v[1].v, fl.bsq.v, im.r_high, im.r_low, out.ss.dlnth);
    // pitch_angle divides by |k.u| B / B_unit, the field in code units, which
    // M_unit does not move: formed before B takes its ln B direction
    const D1 Bcode = fl.B * im.inv_B_unit;
    D3 thetae = lift(fl.thetae), B = lift(fl.B);
    thetae.d[kSLnTh] = fl.thetae.v;
    B.d[kSLnB] = fl.B.v - 1.e-20;  // B = sqrt(Bsq) B_unit + tiny: the part that scales

    D1 kd[4];
    lowerT(g, k1, kd);
    const D1* U = fl.ucon;
    const D1* Bc = fl.bcon;
    out.kU = kd[0] * U[0] + kd[1] * U[1] + kd[2] * U[2] + kd[3] * U[3];
    // 1/(k.u |B|) gives the cosine's 1/(|k.u| |B|) and 1/(k.u), as in the
    // FP64 sample (rt_terms_fp64)
    const D1 ikB = 1.0 / (out.kU * Bcode);
    D1 pitch = (kd[0] * Bc[0] + kd[1] * Bc[1] + kd[2] * Bc[2] + kd[3] * Bc[3]) * fabs(ikB);
    if (fabs(pitch.v) > 1.0) pitch = D1(pitch.v > 0 ? 1.0 : -1.0);
    const D1 ikU = ikB * Bcode;
    out.ikU = ikU.v;
    out.ikU2 = ikU * ikU;
    out.adl = adl1;
    if constexpr (K) {
        out.pre = B;
        out.hkt = thetae;
        out.kne = fl.ne;
        out.kcos = pitch;
        out.emits = true;
        return true;
    }
    const D1 s2 = 1.0 - pitch * pitch;
    const D1 sth = s2.v > 0.0 ? sqrt(s2) : D1(0.0);
    const D3 nuc = B * (kECharge / (2.0 * CUDART_PI * kEMass * kC));
    const D3 nus = mul31((2.0 / 9.0) * nuc * thetae * thetae, sth);
    out.emits = (fabs(sth.v) >= 1.e-10) && (fl.thetae.v > 1e-4);
    // n_e sqrt(2) pi nu_s e2_c / (3 K2) with K2 = 2 Theta^2 and nu_s / Theta^2
    // = (2/9) nu_c sin(theta)
    out.pre = mul31(mul31(nuc, sth), fl.ne * (1.4142135623730951 * CUDART_PI / 6.0 * (2.0 / 9.0) * kE2C));
    out.hkt = (kPlanck / (kEMass * kC * kC)) / thetae;
    out.inus = 1.0 / nus;
    out.nus = nus.v;
    return true;
}

// A kappa image's terms at one frequency: rt_terms_fp64's kappa branch
// (kappa_sample, kappa_coeffs; dtau = nu_p a_nu dl_f, S = j_nu / nu_p^2
// dl_f) on the same values, with tangents; out of line, the per-sample part
// recomputed per frequency.
// Returns sample_freq's kind: 1 if the frequency changes tau or I, else 0.
__device__ __noinline__ int kappa_terms(const DevImage& im, const D3& B, const D1& cosp, const D3& thetae,
                                        const D1& ne, const D1& nup, const D1& dlf, const D1& inup2, D3& S,
                                        D3& dtau) {
    const KappaSampleT<D3> ks = kappa_sample(im.kap, B, lift(cosp), thetae, lift(ne));
    D3 j, a;
    kappa_coeffs(im.kap, ks, lift(nup), j, a);
    if (j.v == 0.0 && a.v == 0.0) return 0;  // rt_apply_fp64 leaves tau and I as they are
    dtau = mul31(mul31(a, nup), dlf);
    S = mul31(mul31(j, inup2), dlf);
    return 1;
}

// The terms S and delta of the tau / I recurrence at frequency fi, in the
// FP64 sample's formulation (transfer.cuh, rt_terms_fp64): B_nu is never
// formed, a nu = j (e2_ch c^2 / (2 e2_c)) (e^{h nu / k T} - 1) / nu^2.
// Returns 1 if the frequency emits, 2 where the primal's tau turns NaN (B_nu
// underflowed to 0), else 0.
template <bool K>
__device__ __forceinline__ int sample_freq(const DevImage& im, const SampleCommon& sc, int fi, D3& S, D3& dtau) {
    D1 nup = -sc.kU * im.freq[fi];
    if (nup.v <= 0.0) nup = D1(1.0);
    if constexpr (K)
        return kappa_terms(im, sc.pre, sc.kcos, sc.hkt, sc.kne, nup, sc.adl * im.rg_over_nu[fi],
                           sc.ikU2 * im.inv_freq2[fi], S, dtau);
    if (sc.emits && nup.v != 1.0) {
        const D1 dlf = sc.adl * im.rg_over_nu[fi];
        const D3 X = mul31(sc.inus, nup);
        // the tangents of X^1/3 and X^1/6 through 1/X = nu_s / nu_p, 1/nu_p =
        // -nu / (k.u nu^2): d X^1/3 = X^1/3 / (3X), d sqrt(c) = sqrt(c) c^2 / (2X)
        const double iX = sc.nus * (-sc.ikU * (im.freq[fi] * im.inv_freq2[fi]));
        const double cv = cbrt(X.v);
        const D3 cb = chain(X, cv, cv * iX * (1.0 / 3.0));
        const double sv = sqrt(cv);
        const D3 sq = chain(cb, sv, 0.5 * sv * (cv * cv * iX)) * (cb + 1.8877486253633869);  // X^1/2 + 2^(11/12) X^1/6
        const D3 jn = sc.pre * (sq * sq) * fast_exp(-cb);
        const D3 ex = fast_exp(mul31(sc.hkt, nup)) - 1.0;
        const D1 inup2 = sc.ikU2 * im.inv_freq2[fi];
        dtau = mul31(mul31(jn * (kE2CH * kC * kC / (2.0 * kE2C)) * ex, inup2), dlf);
        S = mul31(mul31(jn, inup2), dlf);
        return 1;
    }
    const double ex = fast_exp(sc.hkt.v * nup.v) - 1.0;
    return !(ex < CUDART_INF) ? 2 : 0;
}

// One frequency's terms of a sample, consumed in step order: tau, the part
// of I accumulated so far, d tau / d(scalars), dL/dI dI/d(scalars) (dIw), and
// the sample's sums Gr, Gt of w (g e^-tau dS/dx - (I - I_<k) ddelta/dx) for
// x = rho_s and ln Theta_e.  kind is sample_freq's.  One pass (TAPE): Gr, Gt
// get the gated part only; the suffix part's I_<k and coefficients go to the
// record's three slots rec (when it has room), and live tells whether the
// sample is inside the gate (vjp_df.cu, vjp_f32_body, has the scheme).
template <bool TAPE = false>
__device__ __forceinline__ void consume_term(int kind, const D3& S, const D3& dt, const SampleScalars& ss, double w,
                                             double Itot, double& tau, double& Ipart, double (&dtg)[4],
                                             double (&dIw)[4], double& Gr, double& Gt,
                                             unsigned long long& n_emit, unsigned long long& n_gate,
                                             double* rec = nullptr, bool* live = nullptr) {
    if (TAPE && rec && kind != 1) {
        rec[0] = 0.0;
        rec[1] = 0.0;
        rec[2] = 0.0;
    }
    if (kind == 1) {
        ++n_emit;
        tau += dt.v;
#pragma unroll
        for (int q = 0; q < 4; ++q) dtg[q] += scalar_tangent(dt, ss, q);
        const double e = fast_exp(-tau);
        const bool gate = tau < 6.907755278982137 && !(tau < 0.0);
        const double eS = gate ? e : 0.0;
        if constexpr (TAPE) {
            if (rec) {
                rec[0] = Ipart;
                rec[1] = w * rho_tangent(dt, ss);
                rec[2] = w * dt.d[kSLnTh];
            }
            if (gate) {
                Gr += w * (eS * rho_tangent(S, ss));
                Gt += w * (eS * S.d[kSLnTh]);
                *live = true;
            }
        } else {
            const double suffix = Itot - Ipart;
            if (suffix != 0.0 || gate) {
                Gr += w * (eS * rho_tangent(S, ss) - suffix * rho_tangent(dt, ss));
                Gt += w * (eS * S.d[kSLnTh] - suffix * dt.d[kSLnTh]);
            }
        }
        if (gate) {
            ++n_gate;
            const double we = w * e;
#pragma unroll
            for (int q = 0; q < 4; ++q) dIw[q] += we * (scalar_tangent(S, ss, q) - S.v * dtg[q]);
            Ipart += S.v * e;
        }
    } else if (kind == 2) {
        tau = __longlong_as_double(0x7ff8000000000000ll);
    }
}

// A sample's per-cell gradients: Gr, Gu = Gt d ln Theta_e / d u_s and Gt on
// the four cells of its bilinear interpolation, with FP64 atomics.
__device__ __forceinline__ void scatter_cells(double* __restrict__ g_rho, double* __restrict__ g_u,
                                              double* __restrict__ g_th, long long base, int n2, double d1,
                                              double d2, double Gr, double Gt, double dlnth_du) {
    const double Gu = Gt * dlnth_du;
    if (!((Gr != 0.0 || Gt != 0.0) && isfinite(Gr) && isfinite(Gt) && isfinite(Gu) && g_rho)) return;
    const double w0 = (1.0 - d1) * (1.0 - d2), w1 = (1.0 - d1) * d2;
    const double w2 = d1 * (1.0 - d2), w3 = d1 * d2;
    const long long c = base, cn = base + n2;
    atomicAdd(&g_rho[c], Gr * w0);
    atomicAdd(&g_rho[c + 1], Gr * w1);
    atomicAdd(&g_rho[cn], Gr * w2);
    atomicAdd(&g_rho[cn + 1], Gr * w3);
    atomicAdd(&g_u[c], Gu * w0);
    atomicAdd(&g_u[c + 1], Gu * w1);
    atomicAdd(&g_u[cn], Gu * w2);
    atomicAdd(&g_u[cn + 1], Gu * w3);
    atomicAdd(&g_th[c], Gt * w0);
    atomicAdd(&g_th[c + 1], Gt * w1);
    atomicAdd(&g_th[cn], Gt * w2);
    atomicAdd(&g_th[cn + 1], Gt * w3);
}

// Inclination-dependent camera constants with their tangent per degree.
struct HD {
    double v, d;
};
HD operator+(HD a, HD b) { return {a.v + b.v, a.d + b.d}; }
HD operator-(HD a, HD b) { return {a.v - b.v, a.d - b.d}; }
HD operator*(HD a, HD b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
HD operator/(HD a, HD b) { return {a.v / b.v, (a.d - a.v / b.v * b.d) / b.v}; }
HD cst(double x) { return {x, 0.0}; }
HD hsin(HD a) { return {std::sin(a.v), std::cos(a.v) * a.d}; }
HD hcos(HD a) { return {std::cos(a.v), -std::sin(a.v) * a.d}; }
HD hsqrt(HD a) { const double s = std::sqrt(a.v); return {s, 0.5 / s * a.d}; }
HD hacos(HD a) { return {std::acos(a.v), -a.d / std::sqrt(1.0 - a.v * a.v)}; }

CamT<D1> camera_tangent(const DevImage& im, double inclination, double a, double hslope) {
    const HD incl{inclination, 1.0};
    const HD mu0 = hcos(incl * cst(M_PI / 180.));
    const HD thc = hacos(mu0);
    const HD sin_mu = hsqrt(cst(1.0) - mu0 * mu0);
    const HD mu0sq = mu0 * mu0;
    const HD sc2 = hsin(thc) * hsin(thc), cc2 = hcos(thc) * hcos(thc);
    const HD st = hsin(thc), ct = hcos(thc);
    const double r = kRcam;
    const HD sig = cst(r * r) + cst(a * a) * ct * ct;
    const double dl = r * r + a * a - 2. * r;
    const HD A = cst((r * r + a * a) * (r * r + a * a)) - cst(dl * a * a) * st * st;
    const HD g11 = sig / cst(dl) * cst(r * r);
    const HD gu00 = cst(-1.0) * A / (sig * cst(dl));
    const HD gu03 = cst(-2. * a * r) / (sig * cst(dl));
    const HD gu33 = (cst(dl) - cst(a * a) * st * st) / (sig * cst(dl) * st * st);
    const HD gu22 = cst(1.0) / sig;
    // x2 solves pi x + (1-h)/2 sin(2 pi x) = theta: dx2/dtheta = 1/(pi (1 + (1-h) cos 2 pi x2)) = 1/k2fac
    const double x2 = im.xcam[2];
    const bool clamped = (x2 <= 0.0 || x2 >= 1.0);
    const HD x2c{x2, clamped ? 0.0 : thc.d / im.k2fac};
    const HD k2fac{im.k2fac, -M_PI * (1. - hslope) * 2. * M_PI * std::sin(2. * M_PI * x2) * x2c.d};
    auto D = [](HD h) { D1 r(h.v); r.d[0] = h.d; return r; };
    CamT<D1> c;
    c.sin_mu = D(sin_mu);
    c.mu0sq = D(mu0sq);
    c.cc_over_sc = D(cc2 / sc2);
    c.cosc2 = D(cc2);
    c.g11 = D(g11);
    c.gu00 = D(gu00);
    c.gu03 = D(gu03);
    c.gu33 = D(gu33);
    c.gu22 = D(gu22);
    c.x2c = D(x2c);
    c.k2fac = D(k2fac);
    return c;
}

// One lane runs its ray to the end before taking the next: with the FP64
// duals' register footprint, keeping a ray's state across lane refills (as
// the mixed-DF adjoint does) spilled more and ran slower (5-frequency
// 2048x2048: 14.5 s against 11.7 s).
template <int NF, bool K>
__global__ void __launch_bounds__(kVjpBlock, 1)
    vjp_kernel(const DevImage* __restrict__ imp, CamT<D1> cam, const double* __restrict__ fwd,
               const double* __restrict__ dLdO, unsigned long long* __restrict__ counters,
               double* __restrict__ gscal, double* __restrict__ g_rho, double* __restrict__ g_u,
               double* __restrict__ g_th, RayRange rr) {
    const DevImage& im = *imp;
    const int lane = threadIdx.x & 31;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    unsigned long long n_calls = 0, n_samples = 0, n_emit = 0, n_gate = 0;
    bool live = true;
    while (true) {
        const unsigned want = __ballot_sync(kFull, live);
        if (!want) break;
        const int leader = __ffs(want) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(&counters[kCtrQueue], (unsigned long long)__popc(want));
        base = __shfl_sync(kFull, base, leader);
        long long rid = -1;
        if (live) {
            rid = rr.begin + (long long)(base + __popc(want & ((1u << lane) - 1u)));
            if (rid >= rr.end) {
                live = false;
                rid = -1;
            }
        }
        if (rid < 0) continue;

        const int pix = (int)rid;
        D1 y[8];
        double beta;
        init_photon(im, cam, pix % im.width, pix / im.width, y, beta);
        MksPointT<D1> p;
        mks_point(y[1], y[2], im.geo, p);
        const PixelScale ps = pixel_scale(im, pix % im.width);
        // per frequency: tau, the forward I, the part of I accumulated so far,
        // dL/dI and d tau / d(scalars); dIw = sum over frequencies of dL/dI dI/d(scalars)
        double tau[NF], Itot[NF], Ipart[NF], w[NF], dtg[NF][4], dIw[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            tau[f] = 0.0;
            Ipart[f] = 0.0;
            Itot[f] = 0.0;
            w[f] = 0.0;
#pragma unroll
            for (int q = 0; q < 4; ++q) dtg[f][q] = 0.0;
            if (f < im.nfreq) {
                const long long o = (long long)pix * im.nfreq + f;
                const double dOdI = scale_output(im, ps, 1.0, f);
                Itot[f] = fwd[o] / dOdI;
                w[f] = dLdO[o] * dOdI;
            }
        }
        int steps = 0, turns = 0, stop = 0;
        double thdot_prev = 0.0;
        while (true) {
            const double r = p.rp.v;
            if (!(r < kCutoffOuter && r > im.cutoff_inner && (double)steps < kMaxSteps && !stop)) break;
            if (thdot_prev * y[6].v < 0.0 && steps > 2) turns += 1;
            thdot_prev = y[6].v;
            if ((beta < 0.0 && turns > kMaxOrder) || (beta > 0.0 && turns > kMaxOrder + 1)) stop = 1;
            const D1 dl = step_size(im, y);
            if (im.integrator == 2) rk2_step<D1, Geo, false>(im.geo, y, p, dl);
            else rk4_step_rolled<D1, Geo, false>(im.geo, y, p, dl);
            steps += 1;
            if (y[1].v > im.stopx1 && y[5].v < 0.0) break;
            if (y[1].v < im.stopx1 && y[1].v > im.startx1 && y[2].v > im.startx2 && y[2].v < im.stopx2) {
                ++n_calls;
                SampleCommon sc;
                CellCoef cc;
                const D1 k1[4] = {y[4], y[5], y[6], y[7]};
                if (sample_common<K>(im, y[1], y[2], k1, p, fabs(dl), cc, sc)) {
                    ++n_samples;
                    double Gr = 0.0, Gt = 0.0;
                    // one copy of the frequency body: with NF > 1 the per-frequency
                    // state lives in local memory, and fewer registers spill
                    // (5 frequencies: 8 % faster than unrolled)
#pragma unroll 1
                    for (int f = 0; f < NF; ++f) {
                        if (f >= im.nfreq) break;
                        D3 S, dt;
                        const int kind = sample_freq<K>(im, sc, f, S, dt);
                        consume_term(kind, S, dt, sc.ss, w[f], Itot[f], tau[f], Ipart[f], dtg[f], dIw, Gr, Gt,
                                     n_emit, n_gate);
                    }
                    scatter_cells(g_rho, g_u, g_th, cc.base, im.n2, cc.d1, cc.d2, Gr, Gt, sc.ss.dlnth[1]);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (isfinite(dIw[q])) acc[q] += dIw[q];
        atomicAdd(&counters[kCtrSteps], (unsigned long long)steps);
        atomicAdd(&counters[kCtrRays], 1ull);
    }
    atomicAdd(&counters[kCtrRtCalls], n_calls);
    atomicAdd(&counters[kCtrRtSamples], n_samples);
    atomicAdd(&counters[kCtrVjpEmit], n_emit);
    atomicAdd(&counters[kCtrVjpGate], n_gate);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        double v = acc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
        if (lane == 0) atomicAdd(&gscal[q], v);
    }
}

// ------------------------------------------------------------ sample pool
//
// The dual sample at a post-step point (sample_common + sample_freq: fluid,
// emission and absorption with their six tangents) does not depend on the
// ray's history, so, as in the forward kernel's pool (ray_kernel_pool),
// lanes inside the sampling region append a ticket - the point, wave vector
// and |d lambda| with their inclination tangents - to the warp's ring in
// shared memory, every lane evaluates one once 32 wait, and the owners then
// consume their evaluated tickets in step order: tau, the suffix identity,
// the scalar tangents and the per-cell scatter, exactly as vjp_kernel does
// in place.  The evaluating lane recomputes the point's transcendentals from
// (x1, x2) rather than carrying them (16 more doubles per ticket).  A
// ticket's result is 7 + 8 NF doubles: with one frequency it overwrites the
// ticket in shared memory; with more it goes to the warp's slice of a
// scratch buffer in device memory (L2-resident: 24 KB per warp at five
// frequencies).
namespace vpool {
constexpr int C = kPoolCap;
// ticket rows, C doubles each.  In: 0-1 |dl|, 2-3 x1, 4-5 x2, 6-13 k^mu
// (value, tangent).  Out: 0 d1, 1 d2, 2 1/rho_s, 3-6 d ln Theta_e / d(rho_s,
// u_s, R_high, R_low), then per frequency f at 7 + 8 f: S (value, three
// tangents) and dtau.  Ints per entry: next ticket, first cell, per
// frequency the kind (sample_freq's; -1 at frequency 0: sigma cut).
constexpr int kIn = 14;
template <int NF>
struct Layout {
    static constexpr int kOut = 7 + 8 * NF;
    static constexpr bool kSharedOut = NF == 1;
    static constexpr int kSharedRows = kSharedOut ? (kOut > kIn ? kOut : kIn) : kIn;
    // + the ints (and in the checked build each entry's owner lane)
    static constexpr int kInts = (2 + NF + (kChecked ? 1 : 0)) * C;
    static constexpr int kWarpDoubles = kSharedRows * C + (kInts + 1) / 2;
    static constexpr int kScratchRows = kSharedOut ? 0 : kOut;  // per warp, in the scratch buffer
};
}  // namespace vpool

// TAPE: one pass, the ray's records on the lane's tape (consume_term).
template <int NF, bool K, bool TAPE>
__global__ void __launch_bounds__(kVjpBlock, 1)
    vjp_kernel_pool(const DevImage* __restrict__ imp, CamT<D1> cam, const double* __restrict__ fwd,
                    const double* __restrict__ dLdO, unsigned long long* __restrict__ counters,
                    double* __restrict__ gscal, double* __restrict__ g_rho, double* __restrict__ g_u,
                    double* __restrict__ g_th, int refill_interval, double* __restrict__ scratch, RayRange rr,
                    VjpTape tape) {
    using namespace vpool;
    using L = Layout<NF>;
    __shared__ double pool_mem[(kVjpBlock / 32) * L::kWarpDoubles];
    const DevImage& im = *imp;
    const int lane = threadIdx.x & 31;
    double* const fld = pool_mem + (threadIdx.x >> 5) * L::kWarpDoubles;
    int* const nxt = reinterpret_cast<int*>(fld + L::kSharedRows * C);
    int* const tbase = nxt + C;
    int* const tkind = tbase + C;  // [NF][C]
    int* const towner = tkind + NF * C;  // checked build only
    unsigned long long* const cw = imp->check_word;
    // evaluated results: the ticket rows themselves, or this warp's scratch slice
    double* const res = L::kSharedOut ? fld
                                      : scratch + (size_t)(blockIdx.x * (kVjpBlock / 32) + (threadIdx.x >> 5)) *
                                                      L::kScratchRows * C;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    unsigned long long n_calls = 0, n_samples = 0, n_emit = 0, n_gate = 0, n_steps = 0, n_rays = 0;
    unsigned long long n_nan = 0, n_cap = 0, n_full = 0;
    // one pass: this lane's records (per-cell gradients asked for)
    const size_t lane_elems = (size_t)tape.cap * (size_t)tape.stride;
    double* const lane_tape =
        TAPE && g_rho ? static_cast<double*>(tape.rec) + ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * lane_elems
                      : nullptr;
    int nrec = 0, pix = 0;
    bool full = false, replay = false;

    D1 y[8];
    MksPointT<D1> p;
    double beta = 0.0, thdot_prev = 0.0;
    int steps = 0, turns = 0, stop = 0;
    // per frequency: tau, the forward I, the part of I accumulated so far, dL/dI and
    // d tau / d(scalars); dIw = sum over frequencies of dL/dI dI/d(scalars)
    double tau[NF], Itot[NF], Ipart[NF], w[NF], dtg[NF][4], dIw[4];
    int mode = 0;  // 0 idle, 1 stepping, 2 ended with tickets outstanding
    bool live = true;
    TicketRing ring;
    int since_refill = refill_interval;

    while (true) {
        if constexpr (TAPE) {
            // the records of rays that ended, closed with their I and
            // scattered by the whole warp, 32 at a time (vjp_df.cu has the
            // reason)
            unsigned pend = __ballot_sync(kFull, replay);
            if (pend) __syncwarp();  // the owners' record stores before the loads
            while (pend) {
                const int owner = __ffs(pend) - 1;
                pend &= pend - 1;
                const int onrec = __shfl_sync(kFull, nrec, owner);
                double itot[NF];
#pragma unroll
                for (int f = 0; f < NF; ++f) itot[f] = __shfl_sync(kFull, Ipart[f], owner);
                const double* otape = lane_tape + (long long)(owner - lane) * (long long)lane_elems;
                for (int r = lane; r < onrec; r += 32) {
                    const double* rq = otape + (size_t)r * (size_t)tape.stride;
                    double Gr = rq[4], Gt = rq[5];
#pragma unroll
                    for (int f = 0; f < NF; ++f) {
                        if (f >= im.nfreq) break;
                        const double suffix = itot[f] - rq[6 + 3 * f];
                        Gr -= rq[7 + 3 * f] * suffix;
                        Gt -= rq[8 + 3 * f] * suffix;
                    }
                    scatter_cells(g_rho, g_u, g_th, (long long)rq[0], im.n2, rq[1], rq[2], Gr, Gt, rq[3]);
                }
            }
            replay = false;
        }
        const unsigned need = __ballot_sync(kFull, mode == 0 && live);
        if (need && (since_refill >= refill_interval || !__any_sync(kFull, mode != 0))) {
            since_refill = 0;
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&counters[kCtrQueue], (unsigned long long)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (mode == 0 && live) {
                const long long rid = rr.begin + (long long)(base + __popc(need & ((1u << lane) - 1u)));
                if (rid < rr.end) {
                    pix = (int)rid;
                    nrec = 0;
                    full = false;
                    init_photon(im, cam, pix % im.width, pix / im.width, y, beta);
                    mks_point(y[1], y[2], im.geo, p);
                    const PixelScale ps = pixel_scale(im, pix % im.width);
#pragma unroll
                    for (int f = 0; f < NF; ++f) {
                        tau[f] = 0.0;
                        Ipart[f] = 0.0;
                        Itot[f] = 0.0;
                        w[f] = 0.0;
#pragma unroll
                        for (int q = 0; q < 4; ++q) dtg[f][q] = 0.0;
                        if (f < im.nfreq) {
                            const long long o = (long long)pix * im.nfreq + f;
                            const double dOdI = scale_output(im, ps, 1.0, f);
                            if constexpr (!TAPE) Itot[f] = fwd[o] / dOdI;
                            w[f] = dLdO[o] * dOdI;
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) dIw[q] = 0.0;
                    steps = 0;
                    turns = 0;
                    stop = 0;
                    thdot_prev = 0.0;
                    mode = 1;
                } else {
                    live = false;
                }
            }
        }
        if (!__any_sync(kFull, mode != 0)) break;
        ++since_refill;

        bool want = false;
        D1 adl(0.0);
        if (mode == 1) {
            const double r = p.rp.v;
            bool done = !(r < kCutoffOuter && r > im.cutoff_inner && (double)steps < kMaxSteps && !stop);
            if (!done) {
                if (thdot_prev * y[6].v < 0.0 && steps > 2) turns += 1;
                thdot_prev = y[6].v;
                if ((beta < 0.0 && turns > kMaxOrder) || (beta > 0.0 && turns > kMaxOrder + 1)) stop = 1;
                const D1 dl = step_size(im, y);
                if (im.integrator == 2) rk2_step<D1, Geo, false>(im.geo, y, p, dl);
                else rk4_step_rolled<D1, Geo, false>(im.geo, y, p, dl);
                steps += 1;
                if (y[1].v > im.stopx1 && y[5].v < 0.0) {
                    done = true;
                } else if (y[1].v < im.stopx1 && y[1].v > im.startx1 && y[2].v > im.startx2 &&
                           y[2].v < im.stopx2) {
                    ++n_calls;
                    want = true;
                    adl = fabs(dl);
                }
            }
            if (done) {
                mode = 2;
                ring.ray_ended();
            }
        }
        const int t = ring.append(want, nxt, lane);
        if (kChecked) {
            chk(ring.tail - ring.head <= (unsigned)C, cw, kChkRing, (long long)(ring.tail - ring.head));
            chk(ring.qn >= 0 && ring.qn <= C, cw, kChkList, ring.qn);
            if (t >= 0) towner[t] = lane;
        }
        if (t >= 0) {
            double* e = fld + t;
            e[0] = adl.v;
            e[1 * C] = adl.d[0];
            e[2 * C] = y[1].v;
            e[3 * C] = y[1].d[0];
            e[4 * C] = y[2].v;
            e[5 * C] = y[2].d[0];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                e[(6 + 2 * i) * C] = y[4 + i].v;
                e[(7 + 2 * i) * C] = y[4 + i].d[0];
            }
        }

        const unsigned n = ring.batch(mode == 2, mode == 1);
        chk(n <= 32u, cw, kChkBatch, n);
        if (n) {
            __syncwarp();
            if ((unsigned)lane < n) {
                const int te = ring.slot(lane);
                double* e = fld + te;
                D1 a(e[0]), x1(e[2 * C]), x2(e[4 * C]), k1[4];
                a.d[0] = e[1 * C];
                x1.d[0] = e[3 * C];
                x2.d[0] = e[5 * C];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    k1[i] = D1(e[(6 + 2 * i) * C]);
                    k1[i].d[0] = e[(7 + 2 * i) * C];
                }
                MksPointT<D1> mp;
                mks_point(x1, x2, im.geo, mp);
                SampleCommon sc;
                CellCoef cc;
                double* const o = res + te;
                if (sample_common<K>(im, x1, x2, k1, mp, a, cc, sc)) {
                    ++n_samples;
#pragma unroll 1
                    for (int f = 0; f < NF; ++f) {
                        int kd = 0;
                        if (f < im.nfreq) {
                            D3 S, dt;
                            kd = sample_freq<K>(im, sc, f, S, dt);
                            if (kd == 1) {
                                double* of = o + (7 + 8 * f) * C;
                                of[0] = S.v;
                                of[4 * C] = dt.v;
#pragma unroll
                                for (int q = 0; q < 3; ++q) {
                                    of[(1 + q) * C] = S.d[q];
                                    of[(5 + q) * C] = dt.d[q];
                                }
                            }
                        }
                        tkind[f * C + te] = kd;
                    }
                    o[0] = cc.d1;
                    o[1 * C] = cc.d2;
                    o[2 * C] = sc.ss.irho;
#pragma unroll
                    for (int q = 0; q < 4; ++q) o[(3 + q) * C] = sc.ss.dlnth[q];
                    tbase[te] = cc.base;
                } else {
                    tkind[te] = -1;
                }
            }
            __syncwarp();
            ring.evaluated(n);
            // owners consume their evaluated tickets, oldest first
            while (true) {
                const int ta = ring.ready();
                if (!__any_sync(kFull, ta >= 0)) break;
                if (ta >= 0) {
                    if (kChecked) chk(towner[ta] == lane, cw, kChkList, ta);
                    const double* o = res + ta;
                    if (tkind[ta] >= 0) {
                        SampleScalars ss;
                        ss.irho = o[2 * C];
#pragma unroll
                        for (int q = 0; q < 4; ++q) ss.dlnth[q] = o[(3 + q) * C];
                        double Gr = 0.0, Gt = 0.0;
                        // one pass: this sample's record, if it has room
                        double* const rp = TAPE && lane_tape && nrec < tape.cap
                                               ? lane_tape + (size_t)nrec * (size_t)tape.stride
                                               : nullptr;
                        bool in_gate = false;
#pragma unroll 1
                        for (int f = 0; f < NF; ++f) {
                            if (f >= im.nfreq) break;
                            const int kd = tkind[f * C + ta];
                            D3 S, dt;
                            if (kd == 1) {
                                const double* of = o + (7 + 8 * f) * C;
                                S = D3(of[0]);
                                dt = D3(of[4 * C]);
#pragma unroll
                                for (int q = 0; q < 3; ++q) {
                                    S.d[q] = of[(1 + q) * C];
                                    dt.d[q] = of[(5 + q) * C];
                                }
                            }
                            consume_term<TAPE>(kd, S, dt, ss, w[f], Itot[f], tau[f], Ipart[f], dtg[f], dIw, Gr, Gt,
                                               n_emit, n_gate, rp ? rp + 6 + 3 * f : nullptr, &in_gate);
                        }
                        if constexpr (TAPE) {
                            if (in_gate && lane_tape) {
                                if (rp) {
                                    rp[0] = (double)tbase[ta];
                                    rp[1] = o[0];
                                    rp[2] = o[1 * C];
                                    rp[3] = ss.dlnth[1];
                                    rp[4] = Gr;
                                    rp[5] = Gt;
                                    ++nrec;
                                } else {
                                    full = true;
                                }
                            }
                        } else {
                            scatter_cells(g_rho, g_u, g_th, tbase[ta], im.n2, o[0], o[1 * C], Gr, Gt, ss.dlnth[1]);
                        }
                    }
                    ring.pop(nxt, ta);
                }
            }
            __syncwarp();
        }
        if (mode == 2 && ring.empty()) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (isfinite(dIw[q])) acc[q] += dIw[q];
            n_steps += (unsigned long long)steps;
            n_rays += 1;
            mode = 0;
            if constexpr (TAPE) {
                // the ray's own I: the pass's image, and the suffixes that
                // close its records (at the warp's next refill)
                const long long oi = im.out_offset + (long long)pix * im.nfreq;
                const bool in_bounds = chk(oi >= 0 && oi + im.nfreq <= im.out_end, cw, kChkOutput, oi);
                const PixelScale ps = pixel_scale(im, pix % im.width);
                bool finite = p.rp.v == p.rp.v && isfinite(y[5].v);
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    if (f >= im.nfreq || !in_bounds) break;
                    const double ov = scale_output(im, ps, Ipart[f], f);
                    tape.out[oi + f] = ov;
                    finite = finite && isfinite(ov);
                }
                if (!finite) ++n_nan;
                if ((double)steps >= kMaxSteps) ++n_cap;
                if (full) ++n_full;  // the call falls back to two passes
                else replay = lane_tape && nrec > 0;
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

template <int NF, bool K, bool TAPE>
void launch_vjp_pool(int grid, cudaStream_t st, const DevImage* im, const CamT<D1>& cam, const double* fwd,
                     const double* dl, unsigned long long* ctr, double* gs, double* gr, double* gu, double* gt,
                     int refill, double* scratch, RayRange rr, VjpTape tape) {
    vjp_kernel_pool<NF, K, TAPE><<<grid, kVjpBlock, 0, st>>>(im, cam, fwd, dl, ctr, gs, gr, gu, gt, refill, scratch,
                                                             rr, tape);
}

template <int NF, bool K>
void launch_vjp(int grid, cudaStream_t st, const DevImage* im, const CamT<D1>& cam, const double* fwd,
                const double* dl, unsigned long long* ctr, double* gs, double* gr, double* gu, double* gt,
                int, double*, RayRange rr, VjpTape) {
    vjp_kernel<NF, K><<<grid, kVjpBlock, 0, st>>>(im, cam, fwd, dl, ctr, gs, gr, gu, gt, rr);
}

// The pooled kernel for nf frequencies, one pass (TAPE) or two.
template <bool TAPE>
VjpLaunchFn pick_pool(int nf, const void** fn, int* scratch_rows, bool kappa) {
    if (kappa) {
        *fn = (const void*)vjp_kernel_pool<8, true, TAPE>;
        *scratch_rows = vpool::Layout<8>::kScratchRows;
        return launch_vjp_pool<8, true, TAPE>;
    }
#define PICK(NF)                                                  \
    if (nf <= NF) {                                               \
        *fn = (const void*)vjp_kernel_pool<NF, false, TAPE>;      \
        *scratch_rows = vpool::Layout<NF>::kScratchRows;          \
        return launch_vjp_pool<NF, false, TAPE>;                  \
    }
    PICK(1)
    PICK(2)
    PICK(4)
    PICK(5)
#undef PICK
    *fn = (const void*)vjp_kernel_pool<8, false, TAPE>;
    *scratch_rows = vpool::Layout<8>::kScratchRows;
    return launch_vjp_pool<8, false, TAPE>;
}

// pool: the sample-pool kernel (one pass with tape, two without); else the
// in-place kernel (two passes); *scratch_rows gets the scratch rows (of
// kPoolCap doubles) the pooled kernel needs per warp.  kappa: the kappa
// fits' instantiation (any frequency count).
VjpLaunchFn pick_vjp_fp64(int nf, const void** fn, bool pool, int* scratch_rows, bool kappa, bool tape) {
    *scratch_rows = 0;
    if (pool) return tape ? pick_pool<true>(nf, fn, scratch_rows, kappa) : pick_pool<false>(nf, fn, scratch_rows, kappa);
    if (kappa) {
        *fn = (const void*)vjp_kernel<8, true>;
        return launch_vjp<8, true>;
    }
#define PICK(NF)                                 \
    if (nf <= NF) {                              \
        *fn = (const void*)vjp_kernel<NF, false>; \
        return launch_vjp<NF, false>;            \
    }
    PICK(1)
    PICK(2)
    PICK(4)
    PICK(5)
#undef PICK
    *fn = (const void*)vjp_kernel<8, false>;
    return launch_vjp<8, false>;
}

}  // namespace

#define CK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return ctx_fail(ctx, RAPTOR_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));  \
    } while (0)

// Records per lane of the one-pass adjoint's tape unless the options say
// otherwise: above the largest sample count of a ray in the benchmark images
// (the longest rays take some 1600 steps).
constexpr int kVjpTapeRecords = 2048;

static int vjp_impl(raptor_gpu_ctx* ctx, const raptor_image_desc* img, int precision, long long ray_begin,
                    long long ray_count, const double* dL_dI, double* I_out, raptor_grad* grad) {
    if (!ctx) return RAPTOR_ERR_INVALID;
    ctx->err[0] = 0;
    if (!img || !dL_dI || !grad) return ctx_fail(ctx, RAPTOR_ERR_INVALID, "vjp: null image, dL_dI or grad");
    if (precision != RAPTOR_PREC_FP64 && precision != RAPTOR_PREC_MIXED && precision != RAPTOR_PREC_MIXED_DF)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "vjp: precision %d unknown", precision);
    auto t0 = std::chrono::steady_clock::now();
    CK(cudaSetDevice(ctx->device));
    cudaGetLastError();
    Batch& b = ctx->batch;
    int rc = prepare_batch(ctx, img, 1, b);
    if (rc) return rc;
    const DevImage& him = b.host[0];
    const GridSlot& gs = ctx->grids[img->grid];
    const long long ncell = (long long)gs.geom.n1 * gs.geom.n2;
    if (ray_begin < 0 || ray_count < 0 || ray_begin > b.total_rays)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "vjp: ray range [%lld, +%lld) outside the image", ray_begin,
                        ray_count);
    const long long rb = ray_begin, re = ray_count > b.total_rays - rb ? b.total_rays : rb + ray_count;

    const size_t nout = (size_t)b.out_len;
    rc = ensure_buffer(ctx, (void**)&ctx->d_dldi, &ctx->dldi_cap, sizeof(double) * nout);
    if (!rc) rc = ensure_buffer(ctx, (void**)&ctx->d_grad, &ctx->grad_cap, sizeof(double) * (4 + 3 * ncell));
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->d_dldi, dL_dI, sizeof(double) * nout, cudaMemcpyHostToDevice, ctx->stream));

    const CamT<D1> cam = camera_tangent(him, img->inclination, gs.geom.a, gs.geom.hslope);
    const bool kappa = img->emission == RAPTOR_EMISSION_KAPPA;
    // the per-cell scatter runs when any of the three fields is asked for
    const bool fields = grad->d_rho || grad->d_u || grad->d_lnthetae;
    double* gsc = ctx->d_grad;
    double* grho = fields ? ctx->d_grad + 4 : nullptr;
    double* gu = fields ? ctx->d_grad + 4 + ncell : nullptr;
    double* gth = fields ? ctx->d_grad + 4 + 2 * ncell : nullptr;
    // The adjoints run in one pass (their own I, records on a tape) unless
    // the options ask for two (or, in FP64, for the in-place kernel); a tape
    // too small for some ray, or one that cannot be allocated, falls back to
    // two passes.
    const bool fp64 = precision == RAPTOR_PREC_FP64;
    bool one_pass = ctx->opt.vjp_tape >= 0 && !(fp64 && ctx->opt.no_sample_pool);
    const int tape_cap = ctx->opt.vjp_tape > 0 ? ctx->opt.vjp_tape : kVjpTapeRecords;
    const int tape_stride = vjp_tape_stride(b.max_nf, fp64);
    const size_t tape_elem = fp64 ? sizeof(double) : sizeof(float);
    for (;;) {
        // two passes: the forward render of the range (its image is the I
        // of the suffix identity)
        float fwd_ms = 0.f;
        unsigned long long fwd_ctr[kCtrCount] = {};
        if (!one_pass) {
            const void* fnp = nullptr;
            RayLaunchFn fn = pick_ray_kernel(b.max_nf, precision, &fnp, !ctx->opt.no_sample_pool);
            LaunchShape ls = choose_shape(ctx, b, precision, fn, fnp);
            rc = enqueue_render(ctx, b, precision, rb, re, ls, fn, true);
            if (rc) return rc;
            CK(cudaMemcpyAsync(fwd_ctr, ctx->d_counters, sizeof fwd_ctr, cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            CK(cudaEventElapsedTime(&fwd_ms, ctx->evA, ctx->evB));
        } else {
            // pixels outside the range stay 0, as the forward render leaves them
            CK(cudaMemsetAsync(ctx->d_out, 0, sizeof(double) * nout, ctx->stream));
        }
        CK(cudaMemsetAsync(ctx->d_grad, 0, sizeof(double) * (4 + 3 * ncell), ctx->stream));
        CK(cudaMemsetAsync(ctx->d_counters, 0, kCtrCount * sizeof(unsigned long long), ctx->stream));

        // the adjoint of the form that rendered: FP64 duals for the FP64 form;
        // for the mixed and mixed-DF forms their own geodesic with FP32
        // tangents and the FP32 dual sample (vjp_df.cu)
        int occ = 1;
        const void* kp = nullptr;
        int scratch_rows = 0;
        const VjpLaunchFn vfn =
            precision == RAPTOR_PREC_MIXED_DF ? pick_vjp_df(b.max_nf, &kp, kappa, one_pass)
            : precision == RAPTOR_PREC_MIXED
                ? pick_vjp_mixed(b.max_nf, &kp, kappa, one_pass)
                : pick_vjp_fp64(b.max_nf, &kp, !ctx->opt.no_sample_pool, &scratch_rows, kappa, one_pass);
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kp, kVjpBlock, 0));
        const int grid = ctx->num_sms * std::max(occ, 1);
        // the pooled adjoint's per-warp result slices (several frequencies)
        if (scratch_rows > 0) {
            rc = ensure_buffer(ctx, (void**)&ctx->d_vjp_scratch, &ctx->vjp_scratch_cap,
                               sizeof(double) * (size_t)grid * (kVjpBlock / 32) * scratch_rows * kPoolCap);
            if (rc) return rc;
        }
        VjpTape tape{nullptr, tape_cap, tape_stride, ctx->d_out};
        if (one_pass && fields) {
            const size_t bytes = tape_elem * (size_t)grid * kVjpBlock * (size_t)tape_cap * (size_t)tape_stride;
            if (ensure_buffer(ctx, (void**)&ctx->d_vjp_tape, &ctx->vjp_tape_cap, bytes)) {
                ctx->err[0] = 0;  // no room for the tape: two passes
                one_pass = false;
                continue;
            }
            tape.rec = ctx->d_vjp_tape;
        }
        CK(cudaEventRecord(ctx->ev0, ctx->stream));
        // one pass: no forward image (the pass writes its own to tape.out)
        vfn(grid, ctx->stream, ctx->d_imgs, cam, one_pass ? nullptr : ctx->d_out, ctx->d_dldi, ctx->d_counters, gsc,
            grho, gu, gth, kVjpRefill, ctx->d_vjp_scratch, RayRange{rb, re}, tape);
        CK(cudaGetLastError());
        CK(cudaEventRecord(ctx->ev1, ctx->stream));
        unsigned long long ctr[kCtrCount];
        CK(cudaMemcpyAsync(ctr, ctx->d_counters, sizeof ctr, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if (one_pass && ctr[kCtrTapeFull] > 0 && !ctr[kCtrCheck]) {
            one_pass = false;  // some ray's records did not fit: two passes
            continue;
        }
        double scal[4];
        CK(cudaMemcpyAsync(scal, gsc, sizeof scal, cudaMemcpyDeviceToHost, ctx->stream));
        if (grad->d_rho)
            CK(cudaMemcpyAsync(grad->d_rho, grho, sizeof(double) * ncell, cudaMemcpyDeviceToHost, ctx->stream));
        if (grad->d_u)
            CK(cudaMemcpyAsync(grad->d_u, gu, sizeof(double) * ncell, cudaMemcpyDeviceToHost, ctx->stream));
        if (grad->d_lnthetae)
            CK(cudaMemcpyAsync(grad->d_lnthetae, gth, sizeof(double) * ncell, cudaMemcpyDeviceToHost, ctx->stream));
        if (I_out)
            CK(cudaMemcpyAsync(I_out, ctx->d_out, sizeof(double) * nout, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        float vjp_ms = 0.f;
        CK(cudaEventElapsedTime(&vjp_ms, ctx->ev0, ctx->ev1));

        grad->d_inclination = scal[0];
        grad->d_m_unit = scal[1] / img->m_unit;  // the kernel differentiates with respect to ln M_unit
        grad->d_r_high = scal[2];
        grad->d_r_low = scal[3];

        // the render's counters: the forward pass's, or the one pass's own
        const unsigned long long* rctr = one_pass ? ctr : fwd_ctr;
        raptor_gpu_stats& s = ctx->stats;
        memset(&s, 0, sizeof s);
        s.kernel_ms = vjp_ms;
        s.device_ms = fwd_ms + vjp_ms;
        // counters of the adjoint pass (the forward pass takes the same steps)
        s.rays = (long long)ctr[kCtrRays];
        s.steps = (long long)ctr[kCtrSteps];
        s.rt_calls = (long long)ctr[kCtrRtCalls];
        s.rt_samples = (long long)ctr[kCtrRtSamples];
        s.vjp_terms = (long long)ctr[kCtrVjpEmit];
        s.vjp_gated_terms = (long long)ctr[kCtrVjpGate];
        s.n_nonfinite = (long long)rctr[kCtrNonFinite];
        s.n_stepcap = (long long)rctr[kCtrStepCap];
        const unsigned long long check = fwd_ctr[kCtrCheck] ? fwd_ctr[kCtrCheck] : ctr[kCtrCheck];
        s.block_size = kVjpBlock;
        s.grid_blocks = grid;
        s.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (check) return render_status(ctx, re - rb, re - rb, 0, 0, check);
        if ((long long)ctr[kCtrRays] != re - rb)
            return ctx_fail(ctx, RAPTOR_ERR_DEVICE, "vjp kernel retired %lld rays, expected %lld",
                            (long long)ctr[kCtrRays], re - rb);
        // the render's status: its non-finite rays make the gradients
        // meaningless, its step-capped rays are the reference's own behaviour
        return render_status(ctx, (long long)(one_pass ? ctr[kCtrRays] : fwd_ctr[kCtrRays]), re - rb,
                             s.n_nonfinite, s.n_stepcap, 0);
    }
}

extern "C" int raptor_gpu_vjp(raptor_gpu_ctx* ctx, const raptor_image_desc* img, int precision, const double* dL_dI,
                              double* I_out, raptor_grad* grad) {
    return vjp_impl(ctx, img, precision, 0, (long long)1 << 62, dL_dI, I_out, grad);
}

extern "C" int raptor_gpu_vjp_range(raptor_gpu_ctx* ctx, const raptor_image_desc* img, int precision,
                                    long long ray_begin, long long ray_count, const double* dL_dI, double* I_out,
                                    raptor_grad* grad) {
    if (ray_begin < 0 || ray_count < 0) return ctx_fail(ctx, RAPTOR_ERR_INVALID, "vjp: negative ray range");
    return vjp_impl(ctx, img, precision, ray_begin, ray_count, dL_dI, I_out, grad);
}
