// The adjoint pass of the mixed-DF form: the derivative of what
// ray_kernel_df renders.  Same method as vjp.cu (one forward sweep per ray,
// exact reverse-mode sample sensitivities from the suffix identity
// dI/d delta_k = -(I - I_<k) with the forward image's I, forward-mode
// tangents for the four scalars, per-cell atomic scatter), in GB300's fast
// arithmetic:
//  * the geodesic as DF with its inclination tangent in FP32 (Dual<1, DF,
//    float>; the tangent needs ~1e-5, not the path's 1e-14) through the same
//    templated code as every other form (step size, rolled RK4, point
//    transcendentals, Christoffels), so the path is ray_kernel_df's;
//  * the sample as Dual<3, float>, the FP32 transfer of the mixed forms
//    (rt_sample_fp32_core: emissivity without e2_c, absorptivity through
//    expm1) along the three directions of vjp_common.cuh (inclination, ln
//    Theta_e, ln B), accumulated per ray in FP32.
// FP64 is used once per ray (camera set-up, the forward image's I, the
// scalar gradients) and for the per-cell atomics.
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

__device__ __forceinline__ F1 to_f1(const DD1& x) {
    F1 r(x.v.hi);
    r.d[0] = x.d[0];
    return r;
}
__device__ __forceinline__ F3 liftf(const F1& a) {
    F3 r(a.v);
    r.d[kSIncl] = a.d[0];
    return r;
}

// The sample's metric (metric.c:94-137, 207-231) in FP32 with its
// inclination tangent, from the point's leading parts (as metric_f32 in
// ray_kernel_df.cu).
__device__ __forceinline__ MetricT<F3> metric_f3(const MksPointT<DD1>& pd, const GeoDF& gd) {
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
    MetricT<F3> g;
    g.d00 = liftf(-1.0f + z);
    g.d01 = liftf(z * rfac);
    g.d03 = liftf((-a) * (z * s2));
    g.d11 = liftf(opz * rfac * rfac);
    g.d13 = liftf((-a) * (s2 * opz * rfac));
    g.d22 = liftf(rho2 * hfac * hfac);
    g.d33 = liftf(s2 * (rho2 + a2 * (s2 * opz)));
    g.u00 = liftf(-1.0f - z);
    g.u01 = liftf(2.0f * irho2);
    g.u11 = liftf(irho2 * (r * (r - 2.0f) + a2) * (ir * ir));
    g.u13 = liftf(a * (irho2 * ir));
    g.u22 = liftf(irho2 * (ithp * ithp));
    g.u33 = liftf(irho2 * (isn * isn));
    return g;
}

// trunc toward zero of hi + lo (the reference's (int) cast in Xtoij)
__device__ __forceinline__ int df_trunc_i(DF t) {
    int i = (int)t.hi;
    if ((float)i == t.hi) {
        if (t.hi > 0.0f && t.lo < 0.0f) i -= 1;
        else if (t.hi < 0.0f && t.lo > 0.0f) i += 1;
    }
    return i;
}

// The frequency-independent part of one FP32 sample with three tangents.
struct SampleCommonF {
    F3 kU, nus, jpre, xpre, adl;
    SampleScalarsF ss;
    bool emits;
    int base;        // first of the four cells
    float d1, d2;    // bilinear offsets
};

__device__ bool sample_common_f(const DevImage& im, const DD1 y[8], const MksPointT<DD1>& pd, const DD1& adl,
                                SampleCommonF& out) {
    const MetricT<F3> g = metric_f3(pd, im.geo_df);
    // Xtoij (grmhd.c:46-71) from the DF position; the offsets carry the
    // inclination tangent unless clamped
    const DF t1 = (y[1].v - im.startx1_df) * im.idx1_df - 0.5;
    const DF t2 = (y[2].v - im.startx2_df) * im.idx2_df - 0.5;
    int i = df_trunc_i(t1), j = df_trunc_i(t2);
    F3 d1(0.0f), d2(0.0f);
    if (i < 0) i = 0;
    else if (i > im.n1 - 2) { i = im.n1 - 2; d1 = F3(1.0f); }
    else { d1 = F3(add_f(t1, (float)-i).hi); d1.d[kSIncl] = y[1].d[0] * im.idx1_df.hi; }
    if (j < 0) j = 0;
    else if (j > im.n2 - 2) { j = im.n2 - 2; d2 = F3(1.0f); }
    else { d2 = F3(add_f(t2, (float)-j).hi); d2.d[kSIncl] = y[2].d[0] * im.idx2_df.hi; }
    out.base = i * im.n2 + j;
    out.d1 = d1.v;
    out.d2 = d2.v;
    const F3 c0 = (1.0f - d1) * (1.0f - d2), c1 = (1.0f - d1) * d2, c2 = d1 * (1.0f - d2), c3 = d1 * d2;
    float a[8], b[8], e[8], f[8];
    const float* cp = im.cells32 + (size_t)out.base * 8;
    load_cell(cp, a);
    load_cell(cp + 8, b);
    load_cell(cp + (size_t)im.n2 * 8, e);
    load_cell(cp + (size_t)im.n2 * 8 + 8, f);
    F3 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = c0 * a[q] + c1 * b[q] + c2 * e[q] + c3 * f[q];

    const F3 B_unit(im.b_unit_f);
    Fluid<F3> fl;
    if (!fluid_from_prims(v, g, F3(im.ne_unit_f), B_unit, F3(im.r_high_f), F3(im.r_low_f), fl)) return false;
    out.ss.irho = 1.0f / v[0].v;
    thetae_log_derivs(v[0].v, v[1].v, fl.bsq.v, im.r_high_f, im.r_low_f, out.ss.dlnth);
    // |b| in code units for the pitch angle, which M_unit does not move:
    // formed before B takes its ln B direction
    const F3 Bcode = fl.B / B_unit;
    fl.thetae.d[kSLnTh] = fl.thetae.v;
    fl.B.d[kSLnB] = fl.B.v - 1.e-20f;  // B = sqrt(Bsq) B_unit + tiny: the part that scales

    const F3 k[4] = {liftf(to_f1(y[4])), liftf(to_f1(y[5])), liftf(to_f1(y[6])), liftf(to_f1(y[7]))};
    F3 kd[4];
    lowerT(g, k, kd);
    const F3* U = fl.ucon;
    const F3* Bc = fl.bcon;
    out.kU = kd[0] * U[0] + kd[1] * U[1] + kd[2] * U[2] + kd[3] * U[3];
    F3 pitch = (kd[0] * Bc[0] + kd[1] * Bc[1] + kd[2] * Bc[2] + kd[3] * Bc[3]) / (fabs(out.kU) * Bcode);
    if (fabsf(pitch.v) > 1.0f) pitch = F3(pitch.v > 0.0f ? 1.0f : -1.0f);
    const F3 sth = sqrt(1.0f - pitch * pitch);
    const F3 nuc = (float)(kECharge / (2.0 * CUDART_PI * kEMass * kC)) * fl.B;
    out.nus = (2.0f / 9.0f) * nuc * fl.thetae * fl.thetae * sth;
    out.emits = (fabsf(sth.v) >= 1.e-10f) && (fl.thetae.v > 1e-4f);
    out.jpre = fl.ne * (float)(1.4142135623730951 * CUDART_PI / 27.0) * nuc * sth;
    out.xpre = (float)(kPlanck / (kEMass * kC * kC)) / fl.thetae;
    out.adl = liftf(to_f1(adl));
    return true;
}

// S and delta at frequency fi (rt_sample_fp32_core's arithmetic, emissivity
// without e2_c); false if the frequency does not emit.
__device__ __forceinline__ bool sample_freq_f(const DevImage& im, const SampleCommonF& sc, int fi, F3& S, F3& dtau) {
    F3 nup = -sc.kU * im.freq_f[fi];
    if (nup.v <= 0.0f) nup = F3(1.0f);
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

// stepsize (integrator.c:109-122) for the dual DF state
__device__ __forceinline__ DD1 step_size_dd1(const DevImage& im, const DD1 y[8]) {
    const DF t = df_const(1.e-40);
    const DD1 m2 = fmin(y[2], 1.0 - y[2]);
    const DD1 i13 = (fabs(y[5]) + t) + (fabs(y[7]) + t);
    const DD1 i2 = fabs(y[6]) + t;
    return -fmax(m2 / ((m2 * i13 + i2) * im.inv_stepsize_df), 1e-12);
}

template <int NF>
struct AdjState {
    DD1 y[8];
    MksPointT<DD1> p;
    float thdot_prev;
    int bsign, steps, turns, stop, pix;
    float tau[NF], Ipart[NF], Itot[NF], w[NF];
    float dtg[NF][4];
    float dIw[4];
    int wexp;  // w[f] holds dL/dI_f * 2^-wexp; the ray's gradient terms are scaled back by 2^wexp
};

// 2^e as a double for e in [-1022, 1023] (built from the exponent field).
__device__ __forceinline__ double pow2_double(int e) {
    e = min(max(e, -1022), 1023);
    return __longlong_as_double((long long)(e + 1023) << 52);
}

#ifndef RAPTOR_VJP_DF_MIN_BLOCKS
#define RAPTOR_VJP_DF_MIN_BLOCKS 2
#endif

template <int NF>
__global__ void __launch_bounds__(kVjpBlock, RAPTOR_VJP_DF_MIN_BLOCKS)
    vjp_kernel_df(const DevImage* __restrict__ imp, CamT<D1> cam, const double* __restrict__ fwd,
                  const double* __restrict__ dLdO, unsigned long long* __restrict__ counters,
                  double* __restrict__ gscal, double* __restrict__ g_rho, double* __restrict__ g_u,
                  double* __restrict__ g_th, int refill_interval) {
    const DevImage& im = *imp;
    const int lane = threadIdx.x & 31;
    const long long nrays = (long long)im.width * im.height;
    const DF cut_outer = df_const(kCutoffOuter);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    unsigned long long n_calls = 0, n_samples = 0, n_emit = 0, n_gate = 0, n_steps = 0, n_rays = 0;
    AdjState<NF> s;
    bool active = false, live = true;
    while (true) {
        const unsigned need = __ballot_sync(kFull, !active && live);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&counters[kCtrQueue], (unsigned long long)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (!active && live) {
                const long long rid = (long long)(base + __popc(need & ((1u << lane) - 1u)));
                if (rid < nrays) {
                    s.pix = (int)rid;
                    const int px = s.pix % im.width, py = s.pix / im.width;
                    D1 y0[8];
                    double beta;
                    init_photon(im, cam, px, py, y0, beta);  // FP64 duals, once per ray
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        s.y[i] = DD1(df_const(y0[i].v));
                        s.y[i].d[0] = (float)y0[i].d[0];
                    }
                    s.bsign = (beta < 0.0) ? -1 : ((beta > 0.0) ? 1 : 0);
                    mks_point(s.y[1], s.y[2], im.geo_df, s.p);
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
                            s.Itot[f] = (float)(fwd[o] / dOdI);
                            s.w[f] = (float)(dLdO[o] * dOdI * wscale);
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) s.dIw[q] = 0.0f;
                    s.steps = 0;
                    s.turns = 0;
                    s.stop = 0;
                    s.thdot_prev = 0.0f;
                    active = true;
                } else {
                    live = false;
                }
            }
        }
        if (!__any_sync(kFull, active)) break;
        if (!active) continue;
        for (int it = 0; it < refill_interval; ++it) {
            const DF r = s.p.rp.v;
            bool done = !(r < cut_outer && r > im.cutoff_inner_df && s.steps < (int)kMaxSteps && !s.stop);
            if (!done) {
                const float th = s.y[6].v.hi;
                if (((s.thdot_prev < 0.0f && th > 0.0f) || (s.thdot_prev > 0.0f && th < 0.0f)) && s.steps > 2)
                    s.turns += 1;
                s.thdot_prev = th;
                if ((s.bsign < 0 && s.turns > kMaxOrder) || (s.bsign > 0 && s.turns > kMaxOrder + 1)) s.stop = 1;
                const DD1 dl = step_size_dd1(im, s.y);
                if (im.integrator == 2) rk2_step<DD1, GeoDF, false>(im.geo_df, s.y, s.p, dl);
                else rk4_step_rolled<DD1, GeoDF, false>(im.geo_df, s.y, s.p, dl);
                s.steps += 1;
                if (s.y[1].v > im.stopx1_df && s.y[5].v.hi < 0.0f) {
                    done = true;
                } else if (s.y[1].v < im.stopx1_df && s.y[1].v > im.startx1_df && s.y[2].v > im.startx2_df &&
                           s.y[2].v < im.stopx2_df) {
                    ++n_calls;
                    SampleCommonF sc;
                    if (sample_common_f(im, s.y, s.p, fabs(dl), sc)) {
                        ++n_samples;
                        float Gr = 0.0f, Gt = 0.0f;
                        // one copy of the frequency body (the per-frequency
                        // state of a multi-frequency ray lives in local memory)
#pragma unroll 1
                        for (int f = 0; f < NF; ++f) {
                            if (f >= im.nfreq) break;
                            F3 S, dt;
                            if (!sample_freq_f(im, sc, f, S, dt)) continue;
                            ++n_emit;
                            s.tau[f] += dt.v;
#pragma unroll
                            for (int q = 0; q < 4; ++q) s.dtg[f][q] += scalar_tangent(dt, sc.ss, q);
                            const float e = expf(-s.tau[f]);
                            const bool gate = s.tau[f] < 6.9077553f && !(s.tau[f] < 0.0f);
                            const float suffix = s.Itot[f] - s.Ipart[f];
                            const float eS = gate ? e : 0.0f;
                            Gr += s.w[f] * (eS * rho_tangent(S, sc.ss) - suffix * rho_tangent(dt, sc.ss));
                            Gt += s.w[f] * (eS * S.d[kSLnTh] - suffix * dt.d[kSLnTh]);
                            if (gate) {
                                ++n_gate;
                                const float we = s.w[f] * e;
#pragma unroll
                                for (int q = 0; q < 4; ++q)
                                    s.dIw[q] += we * (scalar_tangent(S, sc.ss, q) - S.v * s.dtg[f][q]);
                                s.Ipart[f] += S.v * e;
                            }
                        }
                        const float Gu = Gt * sc.ss.dlnth[1];
                        if ((Gr != 0.0f || Gt != 0.0f) && isfinite(Gr) && isfinite(Gt) && isfinite(Gu) && g_rho) {
                            const float w0 = (1.0f - sc.d1) * (1.0f - sc.d2), w1 = (1.0f - sc.d1) * sc.d2;
                            const float w2 = sc.d1 * (1.0f - sc.d2), w3 = sc.d1 * sc.d2;
                            const long long c = sc.base, cn = sc.base + im.n2;
                            const double un = pow2_double(s.wexp);
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
                }
            }
            if (done) {
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
    }
    if (lane == 0) {
        atomicAdd(&counters[kCtrSteps], n_steps);
        atomicAdd(&counters[kCtrRays], n_rays);
        atomicAdd(&counters[kCtrRtCalls], n_calls);
        atomicAdd(&counters[kCtrRtSamples], n_samples);
        atomicAdd(&counters[kCtrVjpEmit], n_emit);
        atomicAdd(&counters[kCtrVjpGate], n_gate);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        double v = acc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
        if (lane == 0) atomicAdd(&gscal[q], v);
    }
}

template <int NF>
void launch_vjp_df(int grid, cudaStream_t st, const DevImage* im, const CamT<D1>& cam, const double* fwd,
                   const double* dl, unsigned long long* ctr, double* gs, double* gr, double* gu, double* gt,
                   int refill, double*) {
    vjp_kernel_df<NF><<<grid, kVjpBlock, 0, st>>>(im, cam, fwd, dl, ctr, gs, gr, gu, gt, refill);
}

}  // namespace

VjpLaunchFn pick_vjp_df(int nf, const void** fn) {
    if (nf <= 1) { *fn = (const void*)vjp_kernel_df<1>; return launch_vjp_df<1>; }
    *fn = (const void*)vjp_kernel_df<kMaxFreqs>;
    return launch_vjp_df<kMaxFreqs>;
}

}  // namespace raptor
