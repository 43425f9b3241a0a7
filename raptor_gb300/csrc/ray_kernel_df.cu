// The mixed-DF form: the geodesic (RK steps, step size, point
// transcendentals, Christoffels, the sample's metric) in double-float
// arithmetic (df64.cuh, 48-bit significand on the FP32 pipes), the transfer
// sample in FP32 with compensated sums exactly as the mixed form's.
//
// Same loop as ray_kernel (ray_kernel.cuh, integrator.c:149-289): the
// persistent grid, the ray queue with warp-aggregated refills, termination,
// theta-turn limit and transfer gating.  FP64 is used only per ray: the
// camera set-up (init_photon) and the output write.
#include <cuda_runtime.h>

#include "df64.cuh"
#include "engine_internal.h"
#include "ray_kernel.cuh"

namespace raptor {
namespace {

template <int NF>
struct RayStateDF {
    DF y[8];
    MksPointT<DF> p;
    float thdot_prev;
    long long rid;
    int bsign, steps, turns, stop, img, pix;
    float tf[NF], tc[NF], If[NF], Ic[NF];
};

// stepsize (integrator.c:109-122), as step_size in ray_kernel.cuh
__device__ __forceinline__ DF step_size_df(const DevImage& im, const DF y[8]) {
    const float t = 1.e-40f;
    const DF m2 = fmin(y[2], 1.0 - y[2]);
    const DF i13 = add_f(fabs(y[5]), t) + add_f(fabs(y[7]), t);
    const DF i2 = add_f(fabs(y[6]), t);
    return -fmax(m2 / ((m2 * i13 + i2) * im.inv_stepsize_df), df_const(1e-12));
}

// mks_point for DF states: the rolled form (kerr_mks.cuh)
__device__ __forceinline__ void mks_point(DF x1, DF x2, const GeoDF& g, MksPointT<DF>& p) {
    mks_point_rolled(x1, x2, g, p);
}

// A sample's inputs from the DF state: |d lambda|, the cell coordinates x1,
// x2 in DF, k^mu and the point's leading parts, all the sample reads.
struct SampleInDF {
    float adl;
    DF x1, x2;
    float k[4];
    float r, s, iS, thp, Sg, irp, ithp, isn;
};

__device__ __forceinline__ SampleInDF sample_in_df(const DF y[8], const MksPointT<DF>& p, float adl) {
    SampleInDF in;
    in.adl = adl;
    in.x1 = y[1];
    in.x2 = y[2];
#pragma unroll
    for (int i = 0; i < 4; ++i) in.k[i] = y[4 + i].hi;
    in.r = p.r.hi;
    in.s = p.s.hi;
    in.iS = p.iS.hi;
    in.thp = p.thp.hi;
    in.Sg = p.Sg.hi;
    in.irp = p.irp.hi;
    in.ithp = p.ithp.hi;
    in.isn = p.isn.hi;
    return in;
}

// The sample's metric in FP32 from the point's leading parts (transfer.cuh)
__device__ __forceinline__ MetricT<float> metric_f32(const SampleInDF& in, const GeoDF& gd) {
    return metric_f32(PointF32{in.r, in.s, in.iS, in.thp, in.Sg, in.irp, in.ithp, in.isn}, gd.a.hi, gd.a2.hi,
                      gd.R0.hi);
}

// The frequency-independent part of one transfer sample: Xtoij
// (grmhd.c:46-71) from the DF position, the metric in FP32 from the
// point's leading parts, the rest as the mixed form's FP32 sample.  false
// at the sigma cut.
__device__ __forceinline__ bool sample_common_df(const DevImage& im, const SampleInDF& in, SampleF32& sc) {
    const MetricT<float> g = metric_f32(in, im.geo_df);
    const DF t1 = (in.x1 - im.startx1_df) * im.idx1_df - 0.5;
    const DF t2 = (in.x2 - im.startx2_df) * im.idx2_df - 0.5;
    int i = df_trunc(t1), j = df_trunc(t2);
    float d1, d2;
    if (i < 0) { i = 0; d1 = 0.0f; }
    else if (i > im.n1 - 2) { i = im.n1 - 2; d1 = 1.0f; }
    else d1 = df_value(add_f(t1, (float)-i));
    if (j < 0) { j = 0; d2 = 0.0f; }
    else if (j > im.n2 - 2) { j = im.n2 - 2; d2 = 1.0f; }
    else d2 = df_value(add_f(t2, (float)-j));
    if (!chk(i >= 0 && i <= im.n1 - 2 && j >= 0 && j <= im.n2 - 2, im.check_word, kChkCell,
             (long long)i * im.n2 + j))
        i = j = 0;
    float v[8];
    interp_prims_at(im.cells32, im.n2, i * im.n2 + j, d1, d2, v);
    return sample_common_fp32(im, g, v, in.k, sc);
}

// One transfer sample in place (the in-place kernel and traces).
template <int NF>
__device__ __forceinline__ bool rt_sample_df(const DevImage& im, const SampleInDF& in, float (&tau)[NF],
                                             float (&tauc)[NF], float (&I)[NF], float (&Ic)[NF]) {
    SampleF32 sc;
    if (!sample_common_df(im, in, sc)) return false;
    // one copy of the frequency body (mixed-DF, 5 frequencies: 12 % faster)
#pragma unroll 1
    for (int f = 0; f < NF; ++f) {
        if (f >= im.nfreq) break;
        const float dlf = in.adl * im.rg_over_nu_f[f];
        float dtau, q;
        if (sample_freq_fp32(im, sc, f, dlf, dtau, q)) sample_apply_fp32(dtau, q, dlf, tau[f], tauc[f], I[f], Ic[f]);
    }
    return true;
}

// Per-step record of the traced ray (the layout of trace_record in
// ray_kernel.cuh), the DF state written as doubles.
template <int NF>
__device__ __forceinline__ void trace_record_df(const TraceSpec& tr, const RayStateDF<NF>& s, double dl, int event) {
    if (s.steps >= tr.cap) return;
    double* r = tr.out + (long long)s.steps * kTraceWidth;
#pragma unroll
    for (int i = 0; i < 8; ++i) r[i] = df_to_double(s.y[i]);
    r[8] = dl;
    r[9] = (double)s.tf[0] + (double)s.tc[0];
    r[10] = ((double)s.If[0] + (double)s.Ic[0]) * kE2C;
    r[11] = s.steps;
    r[12] = s.turns;
    r[13] = event;
    r[14] = s.stop;
    r[15] = 0.0;
}

// A lane takes ray rid: camera set-up in FP64 (once per ray), then the DF
// state.  Null where the checked build finds the ray outside the batch.
template <int NF>
__device__ __forceinline__ const DevImage* start_ray_df(const DevImage* __restrict__ imgs, int n_imgs, long long rid,
                                                        RayStateDF<NF>& s) {
    s.img = find_image(imgs, n_imgs, rid);
    if (!chk(s.img >= 0 && s.img < n_imgs, imgs[0].check_word, kChkImage, s.img)) return nullptr;
    const DevImage* im = imgs + s.img;
    s.pix = (int)(rid - im->ray_begin);
    if (!chk(rid >= im->ray_begin && rid - im->ray_begin < (long long)im->width * im->height, im->check_word,
             kChkPixel, rid))
        return nullptr;
    s.rid = rid;
    double y0[8], beta;
    init_photon(*im, camera_of(*im), s.pix % im->width, s.pix / im->width, y0, beta);
#pragma unroll
    for (int i = 0; i < 8; ++i) s.y[i] = df_const(y0[i]);
    s.bsign = (beta < 0.0) ? -1 : ((beta > 0.0) ? 1 : 0);
    mks_point(s.y[1], s.y[2], im->geo_df, s.p);
    s.steps = 0;
    s.turns = 0;
    s.stop = 0;
    s.thdot_prev = 0.0f;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        s.tf[f] = 0.f; s.tc[f] = 0.f; s.If[f] = 0.f; s.Ic[f] = 0.f;
    }
    return im;
}

// One step of integrate_geodesic's loop (integrator.c:228-285), as
// advance_ray in ray_kernel.cuh: -1 the while-condition ended the ray, 0
// stepped outside the sampling region, 1 inside it, 3 escaped outward.
template <int NF, bool TPhi>
__device__ __forceinline__ int advance_ray_df(const DevImage& im, RayStateDF<NF>& s, DF& dl) {
    const DF r = s.p.rp;
    if (!(r < df_const(kCutoffOuter) && r > im.cutoff_inner_df && s.steps < (int)kMaxSteps && !s.stop)) return -1;
    // theta turning points (integrator.c:243-247)
    const float th = s.y[6].hi;
    if (((s.thdot_prev < 0.0f && th > 0.0f) || (s.thdot_prev > 0.0f && th < 0.0f)) && s.steps > 2) s.turns += 1;
    s.thdot_prev = th;
    if ((s.bsign < 0 && s.turns > kMaxOrder) || (s.bsign > 0 && s.turns > kMaxOrder + 1)) s.stop = 1;
    dl = step_size_df(im, s.y);
    if (im.integrator == 2) rk2_step<DF, GeoDF, TPhi>(im.geo_df, s.y, s.p, dl);
    else rk4_step_rolled<DF, GeoDF, TPhi>(im.geo_df, s.y, s.p, dl);
    s.steps += 1;
    if (s.y[1] > im.stopx1_df && s.y[5].hi < 0.0f) return 3;
    if (s.y[1] < im.stopx1_df && s.y[1] > im.startx1_df && s.y[2] > im.startx2_df && s.y[2] < im.stopx2_df) return 1;
    return 0;
}

// |k.k| / k0^2 at the final state (null_drift of ray_kernel.cuh) in DF
// arithmetic from the point the last RK step left: the terms carry ~1e-14 of
// k0^2, far below the drift itself (~1e-4).  In FP64 this per-ray work ran
// at the FP64 pipe's rate on the one or two lanes that finish together.
__device__ __forceinline__ double null_drift_df(const MksPointT<DF>& p, const GeoDF& g, const DF y[8]) {
    MetricDDT<DF> d;
    MetricUUT<DF> u;
    mks_metric(p, g, d, u);
    const DF k0 = y[4], k1 = y[5], k2 = y[6], k3 = y[7];
    const DF kk = d.g00 * k0 * k0 + d.g11 * k1 * k1 + d.g22 * k2 * k2 + d.g33 * k3 * k3 +
                  2.0 * (d.g01 * k0 * k1 + d.g03 * k0 * k3 + d.g13 * k1 * k3);
    const double k0d = df_to_double(k0);
    return fabs(df_to_double(kk)) / (k0d * k0d);
}

// The ray has ended: write I nu^3 (core.c:121-137) and the ray's statistics,
// with the k.k drift at the final state.
template <int NF>
__device__ __forceinline__ void finish_ray_df(const DevImage& im, const RayStateDF<NF>& s, double* __restrict__ out,
                                              RayCounters& c) {
    const long long oi = im.out_offset + (long long)s.pix * im.nfreq;
    const bool in_bounds = chk(oi >= 0 && oi + im.nfreq <= im.out_end, im.check_word, kChkOutput, oi);
    double* o = out + oi;
    const PixelScale ps = pixel_scale(im, s.pix % im.width);
    bool finite = s.p.rp.hi == s.p.rp.hi && isfinite(s.y[5].hi);
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        if (f >= im.nfreq || !in_bounds) break;
        o[f] = scale_output(im, ps, ((double)s.If[f] + (double)s.Ic[f]) * kE2C, f);
        finite = finite && isfinite(o[f]);
    }
    c.steps += (unsigned long long)s.steps;
    c.rays += 1;
    if ((double)s.steps >= kMaxSteps) ++c.cap;
    if (!finite) ++c.nan;  // a non-finite photon state or intensity
    c.max_steps = max(c.max_steps, (unsigned long long)s.steps);
    const double kk = null_drift_df(s.p, im.geo_df, s.y);
    if (kk == kk) c.kk_max = fmax(c.kk_max, kk);
}

// 3 blocks of 128 per SM: 168 registers a thread and no spills.  The DF
// arithmetic wants warps to hide FP32 latency, but 4 blocks (128 registers,
// a few hundred bytes of spills) were 2 % slower at 1024x1024, and 2 blocks
// (8 warps at 196 registers) ran 1.4x slower.
#ifndef RAPTOR_RAY_DF_MIN_BLOCKS
#define RAPTOR_RAY_DF_MIN_BLOCKS 3
#endif

// Each lane samples its own ray in place.  A sample pool as in the FP64
// form (ray_kernel_pool: tickets of the sample's inputs in a per-warp
// shared-memory ring, evaluated 32 at a time, applied in step order) gave
// bit-identical images but ran slower here: 1024x1024, 83 against 68 ms (one
// frequency) and 109 against 81 ms (five).  The FP32 sample is a fifth of
// this kernel's time, and the ring's bookkeeping and ticket traffic cost
// more issue slots than the sample's half-empty warps waste.
// TRACE: the per-step trace kernel (t and phi integrated, records written)
template <int NF, bool TRACE>
__global__ void __launch_bounds__(kRayMaxBlock, RAPTOR_RAY_DF_MIN_BLOCKS)
    ray_kernel_df(const DevImage* __restrict__ imgs, int n_imgs, long long ray_begin, long long ray_end,
                  unsigned long long* __restrict__ counters, double* __restrict__ out, int refill_interval,
                  TraceSpec tr) {
    const int lane = threadIdx.x & 31;
    RayStateDF<NF> s;
    bool active = false, live = true;
    const DevImage* im = imgs;
    RayCounters c;

    while (true) {
        const unsigned need = __ballot_sync(kFull, !active && live);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&counters[kCtrQueue], (unsigned long long)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (!active && live) {
                const long long rid = ray_begin + (long long)(base + __popc(need & ((1u << lane) - 1u)));
                if (rid < ray_end) {
                    const DevImage* ri = start_ray_df(imgs, n_imgs, rid, s);
                    if (ri) {
                        im = ri;
                        active = true;
                        if (TRACE && rid == tr.ray) trace_record_df<NF>(tr, s, 0.0, 0);
                    }
                } else {
                    live = false;
                }
            }
        }
        if (!__any_sync(kFull, active)) break;
        if (active) {
            for (int it = 0; it < refill_interval; ++it) {
                DF dl = df_const(0.0);
                int event = advance_ray_df<NF, TRACE>(*im, s, dl);
                const bool done = event == -1 || event == 3;
                if (event == 1) {
                    ++c.rt_calls;
                    const bool sampled =
                        rt_sample_df<NF>(*im, sample_in_df(s.y, s.p, -dl.hi), s.tf, s.tc, s.If, s.Ic);
                    c.rt_samples += sampled ? 1 : 0;
                    event = sampled ? 2 : 1;
                }
                if (TRACE && event != -1 && s.rid == tr.ray) trace_record_df<NF>(tr, s, df_to_double(dl), event);
                if (done) {
                    finish_ray_df(*im, s, out, c);
                    active = false;
                    break;
                }
            }
        }
    }
    c.publish(counters, lane);
}

// renders; a trace (any frequency count) takes the 8-frequency trace kernel
template <int NF>
void launch_ray_df(const LaunchShape& ls, cudaStream_t st, const DevImage* imgs, int n, long long b, long long e,
                   unsigned long long* ctr, double* out, TraceSpec tr) {
    if (tr.out) ray_kernel_df<kMaxFreqs, true><<<ls.grid, ls.block, 0, st>>>(imgs, n, b, e, ctr, out, ls.refill, tr);
    else ray_kernel_df<NF, false><<<ls.grid, ls.block, 0, st>>>(imgs, n, b, e, ctr, out, ls.refill, tr);
}

}  // namespace
}  // namespace raptor

using namespace raptor;

RayLaunchFn pick_ray_kernel_df(int nf, const void** fn) {
    if (nf <= 1) { *fn = (const void*)ray_kernel_df<1, false>; return launch_ray_df<1>; }
    if (nf <= 2) { *fn = (const void*)ray_kernel_df<2, false>; return launch_ray_df<2>; }
    if (nf <= 4) { *fn = (const void*)ray_kernel_df<4, false>; return launch_ray_df<4>; }
    *fn = (const void*)ray_kernel_df<8, false>;
    return launch_ray_df<8>;
}
