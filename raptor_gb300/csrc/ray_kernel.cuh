// Persistent ray kernel: the per-pixel loop of calculate_image
// (core.c:107-114) and integrate_geodesic (integrator.c:149-289) for every
// pixel of every image in a batch.
//
// Launch shape: one grid of (SM count x resident blocks) that stays
// resident.  Each lane owns one ray; when a lane's ray terminates it takes
// the next ray index from a device-wide counter (warp-aggregated atomicAdd,
// one per warp per refill) so horizon-captured rays (~200 steps) and
// photon-ring rays (thousands) share the SMs without tail imbalance.  Rays
// are numbered image by image, pixel x + y*W within an image, so a warp's
// lanes start on neighbouring pixels.  There are no spin-waits: the only
// inter-thread communication is the atomic counter, so every launch ends.
#pragma once
#include "transfer.cuh"

namespace raptor {

constexpr unsigned kFull = 0xffffffffu;

// Stats slots in the counters buffer (counters[0] is the ray queue).
enum : int {
    kCtrQueue = 0,
    kCtrSteps = 1,
    kCtrRtCalls = 2,
    kCtrRtSamples = 3,
    kCtrRays = 4,
    kCtrStepCap = 5,
    kCtrNonFinite = 6,
    kCtrMaxSteps = 7,
    kCtrKkMax = 8,  // bits of a non-negative double, atomicMax as integer
    kCtrVjpEmit = 9,  // adjoint pass: emitting (sample, frequency) pairs
    kCtrVjpGate = 10, // adjoint pass: terms inside the tau gate
    kCtrCheck = 11,   // the checked build's first failed check (checked.cuh), 0 if none
    kCtrTapeFull = 12,  // one-pass adjoint: rays whose records did not fit the lane's tape
    kCtrCount = 16
};

__device__ __forceinline__ int find_image(const DevImage* __restrict__ imgs, int n_imgs, long long ray) {
    int lo = 0, hi = n_imgs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&imgs[mid].ray_begin) <= ray) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The inclination-dependent camera constants of initialize_photon
// (metric.c:652-692, 722-725): plain values for the forward kernels, values
// with their inclination tangent for the adjoint.
template <class R>
struct CamT {
    R sin_mu, mu0sq, cc_over_sc, cosc2;
    R g11, gu00, gu03, gu33, gu22;
    R x2c, k2fac;
};

__device__ __forceinline__ CamT<double> camera_of(const DevImage& im) {
    return CamT<double>{im.sin_mu, im.mu0sq, im.cc_over_sc, im.cosc2, im.g11, im.gu00,
                        im.gu03,   im.gu33,  im.gu22,       im.xcam[2], im.k2fac};
}

// Output factor of a pixel (core.c:121-137): the image holds I nu^3 for the
// linear camera and I nu^3 r_i d_r d_theta / D^2 for the log-polar one,
// multiplied in the reference's order.
struct PixelScale {
    double r_i = 0.0, d_r = 0.0;
};

__device__ __forceinline__ PixelScale pixel_scale(const DevImage& im, int x) {
    PixelScale p;
    if (im.camera == kCamLog) {
        p.r_i = exp(__ddiv_rn(__dmul_rn(im.ln20, x + 0.5), (double)im.width)) - 1.0;
        p.d_r = __ddiv_rn(__dmul_rn(__dmul_rn(im.rgrav, p.r_i + 1.0), im.ln20), (double)im.width);
    }
    return p;
}

__device__ __forceinline__ double scale_output(const DevImage& im, const PixelScale& ps, double v, int f) {
    double o = v * im.nu3[f];
    if (im.camera == kCamLog)
        o = __ddiv_rn(__dmul_rn(__dmul_rn(__dmul_rn(o, ps.r_i), ps.d_r), im.dtheta_px), im.dist2);
    return o;
}

// Initial photon (metric.c:650-727, GRmath.c:135-184, newtonraphson.c:76-97);
// the pixel-independent part lives in DevImage / CamT.
template <class R>
__device__ __forceinline__ void init_photon(const DevImage& im, const CamT<R>& cam, int x, int yy, R y[8],
                                            double& beta) {
    // Impact parameters with every operation rounded separately, as the
    // reference computes them (C99 without FMA contraction): on the middle
    // row of an odd-height linear image beta is then exactly 0, and
    // sign(beta) = 0 selects k_theta = 0 (metric.c:669).
    double alpha;
    if (im.camera == kCamLog) {  // integrator.c:192-198
        const double r_i = exp(__ddiv_rn(__dmul_rn(im.ln20, x + 0.5), (double)im.width)) - 1.0;
        const double th = __ddiv_rn(__dmul_rn(kTwoPi, yy + 0.5), (double)im.height);
        double sn, cs;
        sincos(th, &sn, &cs);
        alpha = r_i * cs;
        beta = r_i * sn;
    } else {  // integrator.c:187-190
        alpha = __dadd_rn(-im.half_x, __dmul_rn(x + 0.5, im.stepx));
        beta = __dadd_rn(-im.half_y, __dmul_rn(yy + 0.5, im.stepy));
    }
    const R ll = -alpha * cam.sin_mu;
    const R qq = beta * beta + cam.mu0sq * (alpha * alpha - 1.0);
    const double sg = (beta < 0.0) ? -1.0 : ((beta > 0.0) ? 1.0 : 0.0);
    const R kd2 = sg * sqrt(fabs(qq - ll * ll * cam.cc_over_sc + cam.cosc2));
    const double kd0 = -1.0;
    const R kd3 = ll;
    const R ku0 = cam.gu00 * kd0 + cam.gu03 * kd3;
    const R ku3 = cam.gu33 * kd3 + cam.gu03 * kd0;
    const R ku2 = cam.gu22 * kd2;
    const R ku1 = sqrt((-ku0 * kd0 - ku2 * kd2 - ku3 * kd3) / cam.g11);
    y[0] = im.xcam[0];
    y[1] = im.xcam[1];
    y[2] = cam.x2c;
    y[3] = im.xcam[3];
    y[4] = ku0 + im.t01 * ku1;
    y[5] = ku1;
    y[6] = ku2 / cam.k2fac;
    y[7] = im.t31 * ku1 + ku3;
}

// stepsize (integrator.c:109-122) with the reciprocals folded:
// 1/(eps/|k|) = |k|/eps; the tiny^2 guards keep the reference's limits.
// 1 / (i1 + i2/m2 + i3) is formed as m2 / (m2 (i1 + i3) + i2), one
// reciprocal.
template <class R>
__device__ __forceinline__ R step_size(const DevImage& im, const R y[8]) {
    const double t = 1.e-40;
    const R m2 = fmin(y[2], 1.0 - y[2]);
    const R i13 = (fabs(y[5]) + t) + (fabs(y[7]) + t);
    const R i2 = fabs(y[6]) + t;
    return -fmax(m2 * recip((m2 * i13 + i2) * im.inv_stepsize), 1e-12);
}

template <class R, class G>
__device__ __forceinline__ void rhs(const MksPointT<R>& p, const G& g, const R ys[8], R f[8]) {
    f[0] = ys[4];
    f[1] = ys[5];
    f[2] = ys[6];
    f[3] = ys[7];
    geodesic_accel(p, g, ys + 4, f + 4);
}

// Whether an RK step updates state component i.  The metric does not depend
// on t or phi, so x^0 and x^3 feed nothing the image, its derivatives or the
// stopping tests read; kernels that do not record traces (TPhi = false)
// leave them at their initial values.
template <bool TPhi>
__device__ __forceinline__ constexpr bool rk_updates(int i) {
    return TPhi || (i != 0 && i != 3);
}

// One RK4 step (integrator.c:13-41): stage weights 1/2, 1/2, 1 and
// y += dt (f1 + 2 f2 + 2 f3 + f4) / 6.  dt multiplies the stage offsets and
// the final sum instead of each stage's derivatives (the reference forms
// k_i = dt f_i first): 8 multiplications fewer per stage, the same step to
// rounding.  p holds the point at y on entry and at the new y on exit.
// Stages 2-4 run as one rolled loop: the stage body (point transcendentals,
// the connection, contraction) is large, and one copy of it instead of
// three keeps the kernel's hot loop inside the instruction cache.
template <class R, class G, bool TPhi = true>
__device__ __forceinline__ void rk4_step(const G& g, R y[8], MksPointT<R>& p, R dt) {
    using W = typename StageWeight<R>::type;
    R acc[8], ys[8], f[8];
    rhs(p, g, y, f);
    const R hdt = dt * 0.5;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        acc[i] = f[i];
        ys[i] = rk_updates<TPhi>(i) ? y[i] + hdt * f[i] : y[i];
    }
#pragma unroll 1
    for (int q = 1; q < 4; ++q) {
        MksPointT<R> qp;
        mks_point(ys[1], ys[2], g, qp);
        rhs(qp, g, ys, f);
        const W wacc = (q == 3) ? W(1.0) : W(2.0);  // f2, f3 count twice
        const R dnext = (q == 1) ? hdt : dt;          // stage offsets dt/2, dt/2, dt
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            if (!rk_updates<TPhi>(i)) continue;
            acc[i] = acc[i] + f[i] * wacc;
            ys[i] = y[i] + dnext * f[i];
        }
    }
    const R dt6 = dt * (1.0 / 6.0);
#pragma unroll
    for (int i = 0; i < 8; ++i)
        if (rk_updates<TPhi>(i)) y[i] = renorm(y[i] + dt6 * acc[i]);
    mks_point(y[1], y[2], g, p);
}

// f times a stage weight (1 or 2); exact scaling for the double-float state
// (df64.cuh).
template <class R, class W>
__device__ __forceinline__ R stage_scale(const R& f, W w) {
    return f * w;
}

// The same RK4 step with all four stages and the end point's evaluation in
// one rolled loop, so the stage body (point transcendentals, connection,
// contraction) exists once.  Same operations in the same order as rk4_step.
// For the double-float state, where each operation is about ten FP32
// instructions, the single copy keeps the hot loop from stalling on
// instruction fetch.
template <class R, class G, bool TPhi = true>
__device__ __forceinline__ void rk4_step_rolled(const G& g, R y[8], MksPointT<R>& p, R dt) {
    using W = typename StageWeight<R>::type;
    R acc[8], ys[8], f[8];
    const R hdt = dt * 0.5;
#pragma unroll
    for (int i = 0; i < 8; ++i) ys[i] = y[i];
    MksPointT<R> qp = p;
#pragma unroll 1
    for (int q = 0;; ++q) {
        if (q > 0) mks_point(ys[1], ys[2], g, qp);
        if (q == 4) break;
        rhs(qp, g, ys, f);
        if (q < 3) {
            const W wacc = (q == 0) ? W(1.0) : W(2.0);  // f2, f3 count twice
            const R dnext = (q < 2) ? hdt : dt;         // stage offsets dt/2, dt/2, dt
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                if (!rk_updates<TPhi>(i)) continue;
                acc[i] = (q == 0) ? f[i] : acc[i] + stage_scale(f[i], wacc);
                ys[i] = y[i] + dnext * f[i];
            }
        } else {
            const R dt6 = dt * (1.0 / 6.0);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                if (!rk_updates<TPhi>(i)) continue;
                y[i] = renorm(y[i] + dt6 * (acc[i] + f[i]));
                ys[i] = y[i];
            }
        }
    }
    p = qp;
}

// RK2 midpoint step (integrator.c:44-70).
template <class R, class G, bool TPhi = true>
__device__ __forceinline__ void rk2_step(const G& g, R y[8], MksPointT<R>& p, R dt) {
    R ys[8], f[8];
    rhs(p, g, y, f);
#pragma unroll
    for (int i = 0; i < 8; ++i) ys[i] = rk_updates<TPhi>(i) ? y[i] + dt * f[i] * 0.5 : y[i];
    MksPointT<R> q;
    mks_point(ys[1], ys[2], g, q);
    rhs(q, g, ys, f);
#pragma unroll
    for (int i = 0; i < 8; ++i)
        if (rk_updates<TPhi>(i)) y[i] = renorm(y[i] + dt * f[i]);
    mks_point(y[1], y[2], g, p);
}

__device__ __forceinline__ double null_drift(const MksPoint& p, const Geo& g, const double y[8]) {
    MetricDD d;
    MetricUU u;
    mks_metric(p, g, d, u);
    const double k0 = y[4], k1 = y[5], k2 = y[6], k3 = y[7];
    const double kk = d.g00 * k0 * k0 + d.g11 * k1 * k1 + d.g22 * k2 * k2 + d.g33 * k3 * k3 +
                      2.0 * (d.g01 * k0 * k1 + d.g03 * k0 * k3 + d.g13 * k1 * k3);
    return fabs(kk) / (k0 * k0);
}

template <int NF, bool MIXED>
struct RayState {
    double y[8];
    MksPoint p;
    double beta, thdot_prev;
    long long rid;
    int steps, turns, stop, img, pix;
    double tau[NF], I[NF];  // FP64 form
    float tf[NF], tc[NF], If[NF], Ic[NF];  // FP32 form (tau, tau compensation, I, I compensation)
};

template <int NF, bool MIXED>
__device__ __forceinline__ void trace_record(const TraceSpec& tr, const RayState<NF, MIXED>& s, double dl, int event) {
    if (s.steps >= tr.cap) return;
    double* r = tr.out + (long long)s.steps * kTraceWidth;
#pragma unroll
    for (int i = 0; i < 8; ++i) r[i] = s.y[i];
    r[8] = dl;
    if constexpr (MIXED) {
        r[9] = (double)s.tf[0] + (double)s.tc[0];
        r[10] = ((double)s.If[0] + (double)s.Ic[0]) * kE2C;
    } else {
        r[9] = s.tau[0];
        r[10] = s.I[0];
    }
    r[11] = s.steps;
    r[12] = s.turns;
    r[13] = event;
    r[14] = s.stop;
    r[15] = 0.0;
}

// Launch bounds: blocks of at most 128 threads, at least kRayMinBlocks
// resident per SM, so the register budget (<= 168 per thread at 3) keeps
// 12 warps per SM to hide FP64 latency.
#ifndef RAPTOR_RAY_MIN_BLOCKS
#define RAPTOR_RAY_MIN_BLOCKS 3
#endif
constexpr int kRayMaxBlock = 128;
constexpr int kRayMinBlocks = RAPTOR_RAY_MIN_BLOCKS;

// Per-launch statistics of the ray kernels, folded over the warp and added
// to the counters buffer by one lane per warp.
struct RayCounters {
    unsigned long long steps = 0, rt_calls = 0, rt_samples = 0, rays = 0, cap = 0, nan = 0, max_steps = 0;
    double kk_max = 0.0;

    __device__ __forceinline__ void publish(unsigned long long* __restrict__ counters, int lane) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            steps += __shfl_xor_sync(kFull, steps, o);
            rt_calls += __shfl_xor_sync(kFull, rt_calls, o);
            rt_samples += __shfl_xor_sync(kFull, rt_samples, o);
            rays += __shfl_xor_sync(kFull, rays, o);
            cap += __shfl_xor_sync(kFull, cap, o);
            nan += __shfl_xor_sync(kFull, nan, o);
            max_steps = max(max_steps, __shfl_xor_sync(kFull, max_steps, o));
            kk_max = fmax(kk_max, __shfl_xor_sync(kFull, kk_max, o));
        }
        if (lane == 0) {
            atomicAdd(&counters[kCtrSteps], steps);
            atomicAdd(&counters[kCtrRtCalls], rt_calls);
            atomicAdd(&counters[kCtrRtSamples], rt_samples);
            atomicAdd(&counters[kCtrRays], rays);
            atomicAdd(&counters[kCtrStepCap], cap);
            atomicAdd(&counters[kCtrNonFinite], nan);
            atomicMax(&counters[kCtrMaxSteps], max_steps);
            atomicMax(&counters[kCtrKkMax], (unsigned long long)__double_as_longlong(kk_max));
        }
    }
};

// A lane takes ray rid: its image, pixel, initial photon and zeroed transfer
// state.  Returns the image, or null where the checked build finds the ray
// outside the batch (the lane then drops it).
template <int NF, bool MIXED>
__device__ __forceinline__ const DevImage* start_ray(const DevImage* __restrict__ imgs, int n_imgs, long long rid,
                                                     RayState<NF, MIXED>& s) {
    s.img = find_image(imgs, n_imgs, rid);
    if (!chk(s.img >= 0 && s.img < n_imgs, imgs[0].check_word, kChkImage, s.img)) return nullptr;
    const DevImage* im = imgs + s.img;
    s.pix = (int)(rid - im->ray_begin);
    if (!chk(rid >= im->ray_begin && rid - im->ray_begin < (long long)im->width * im->height, im->check_word,
             kChkPixel, rid))
        return nullptr;
    s.rid = rid;
    const int px = s.pix % im->width, py = s.pix / im->width;
    init_photon(*im, camera_of(*im), px, py, s.y, s.beta);
    s.p = im->cam_point;  // mks_point at (xcam[1], xcam[2]), once per image
    s.steps = 0;
    s.turns = 0;
    s.stop = 0;
    s.thdot_prev = 0.0;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        s.tau[f] = 0.0; s.I[f] = 0.0;
        s.tf[f] = 0.f; s.tc[f] = 0.f; s.If[f] = 0.f; s.Ic[f] = 0.f;
    }
    return im;
}

// The ray has ended: write intensityfield[pix][f] * nu^3 (core.c:121-137) and
// its statistics.
template <int NF, bool MIXED>
__device__ __forceinline__ void finish_ray(const DevImage& im, const RayState<NF, MIXED>& s,
                                           double* __restrict__ out, RayCounters& c) {
    const long long oi = im.out_offset + (long long)s.pix * im.nfreq;
    const bool in_bounds = chk(oi >= 0 && oi + im.nfreq <= im.out_end, im.check_word, kChkOutput, oi);
    double* o = out + oi;
    const PixelScale ps = pixel_scale(im, s.pix % im.width);
    bool finite = s.p.rp == s.p.rp && isfinite(s.y[5]);
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        if (f >= im.nfreq || !in_bounds) break;
        double v;
        if constexpr (MIXED) v = ((double)s.If[f] + (double)s.Ic[f]) * kE2C;
        else v = s.I[f];
        o[f] = scale_output(im, ps, v, f);
        finite = finite && isfinite(o[f]);
    }
    c.steps += (unsigned long long)s.steps;
    c.rays += 1;
    if ((double)s.steps >= kMaxSteps) ++c.cap;
    if (!finite) ++c.nan;  // a non-finite photon state or intensity
    c.max_steps = max(c.max_steps, (unsigned long long)s.steps);
    const double kk = null_drift(s.p, im.geo, s.y);
    if (kk == kk) c.kk_max = fmax(c.kk_max, kk);
}

// The step of integrate_geodesic's loop body (integrator.c:228-285) for a
// ray that has not ended: theta-turn count, step size, RK step.  Returns the
// event: 0 stepped outside the sampling region, 1 inside it (sample due),
// 3 escaped outward (integrator.c:271-272), -1 the while-condition ended the
// ray before the step.  dl is the step taken.
template <int NF, bool MIXED, bool TPhi = true>
__device__ __forceinline__ int advance_ray(const DevImage& im, RayState<NF, MIXED>& s, double& dl) {
    // while-condition of integrator.c:228-229 (r = exp(x1), no R0)
    const double r = s.p.rp;
    if (!(r < kCutoffOuter && r > im.cutoff_inner && (double)s.steps < kMaxSteps && !s.stop)) return -1;
    // theta turning points limit the lensed-image order (integrator.c:243-247)
    if (s.thdot_prev * s.y[6] < 0.0 && s.steps > 2) s.turns += 1;
    s.thdot_prev = s.y[6];
    if ((s.beta < 0.0 && s.turns > kMaxOrder) || (s.beta > 0.0 && s.turns > kMaxOrder + 1)) s.stop = 1;
    dl = step_size(im, s.y);
    if (im.integrator == 2) rk2_step<double, Geo, TPhi>(im.geo, s.y, s.p, dl);
    else rk4_step<double, Geo, TPhi>(im.geo, s.y, s.p, dl);
    s.steps += 1;
    if (s.y[1] > im.stopx1 && s.y[5] < 0.0) return 3;
    if (s.y[1] < im.stopx1 && s.y[1] > im.startx1 && s.y[2] > im.startx2 && s.y[2] < im.stopx2) return 1;
    return 0;
}

// TRACE: the per-step trace kernel (t and phi integrated, records written)
template <int NF, bool MIXED, bool TRACE>
__global__ void __launch_bounds__(kRayMaxBlock, kRayMinBlocks)
    ray_kernel(const DevImage* __restrict__ imgs, int n_imgs, long long ray_begin, long long ray_end,
               unsigned long long* __restrict__ counters, double* __restrict__ out, int refill_interval,
               TraceSpec tr) {
    const int lane = threadIdx.x & 31;
    RayState<NF, MIXED> s;
    bool active = false, live = true;
    const DevImage* im = imgs;
    RayCounters c;

    while (true) {
        // refill idle lanes from the device-wide ray queue
        const unsigned need = __ballot_sync(kFull, !active && live);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&counters[kCtrQueue], (unsigned long long)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (!active && live) {
                const long long rid = ray_begin + (long long)(base + __popc(need & ((1u << lane) - 1u)));
                if (rid < ray_end) {
                    const DevImage* ri = start_ray(imgs, n_imgs, rid, s);
                    if (ri) {
                        im = ri;
                        active = true;
                        if (TRACE && rid == tr.ray) trace_record<NF, MIXED>(tr, s, 0.0, 0);
                    }
                } else {
                    live = false;
                }
            }
        }
        if (!__any_sync(kFull, active)) break;
        if (active) {
            for (int it = 0; it < refill_interval; ++it) {
                double dl = 0.0;
                int event = advance_ray<NF, MIXED, TRACE>(*im, s, dl);
                const bool done = event == -1 || event == 3;
                if (event == 1) {
                    ++c.rt_calls;
                    bool sampled;
                    if constexpr (MIXED) sampled = rt_sample_fp32<NF>(*im, s.y, s.p, fabs(dl), s.tf, s.tc, s.If, s.Ic);
                    else sampled = rt_sample_fp64<NF>(*im, s.y, s.p, fabs(dl), s.tau, s.I);
                    c.rt_samples += sampled ? 1 : 0;
                    event = sampled ? 2 : 1;
                }
                if (TRACE && event != -1 && s.rid == tr.ray) trace_record<NF, MIXED>(tr, s, dl, event);
                if (done) {
                    finish_ray(*im, s, out, c);
                    active = false;
                    break;
                }
            }
        }
    }
    c.publish(counters, lane);
}

// ------------------------------------------------- FP64 form, sample pool
//
// In the FP64 form a warp's lanes are seldom all inside the sampling region
// at once (on a 1024x1024 image of the torus, 92 % of warp steps run the
// sample with 60 % of their lanes taking part), so the in-place sample runs
// at little more than half width.  ray_kernel_pool evaluates the
// order-free part of the sample (rt_terms_fp64: fluid, emissivity,
// absorptivity) at full width: each step, lanes inside the region append a
// ticket - the sample's inputs - to a per-warp ring in shared memory; once 32
// tickets wait, every lane evaluates one, and each owner then applies its
// evaluated tickets in step order (rt_apply_fp64).  A ray that has ended waits
// for its outstanding tickets before it writes its pixel; a partial batch is
// evaluated when such a ray has waited kPoolDrainWait steps or no lane of the
// warp is stepping.  Per ray the operations and their order are those of
// ray_kernel: the images agree bit for bit wherever the compiler contracts
// the two kernels' arithmetic alike (the 1-, 2- and 4-frequency
// instantiations), and to rounding elsewhere.
constexpr int kPoolCap = 64;  // ring entries per warp: up to 31 waiting + 32 appended in one step
// at least this many 128-thread blocks per SM: 2 gives 192 registers a
// thread and 8 warps, 1 % faster at 1024x1024 than 3 (168 registers, 12
// warps; 4 blocks spill)
#ifndef RAPTOR_POOL_MIN_BLOCKS
#define RAPTOR_POOL_MIN_BLOCKS 2
#endif
#ifndef RAPTOR_POOL_DRAIN_WAIT
#define RAPTOR_POOL_DRAIN_WAIT 4
#endif
constexpr int kPoolDrainWait = RAPTOR_POOL_DRAIN_WAIT;

// A warp's ring of sample tickets.  head (oldest unevaluated ticket) and
// tail (next free sequence number) are the same in every lane; each lane
// keeps its own outstanding tickets as a list - oldest qh, newest ql, count
// qn - linked through nxt[] in shared memory.  Tickets are evaluated in ring
// order, so a lane's evaluated tickets are always the oldest of its list and
// it applies them oldest first.  Every member that votes (append, batch) is
// called by all 32 lanes together.
struct TicketRing {
    unsigned head = 0, tail = 0;
    unsigned qh = 0, ql = 0;
    int qn = 0, wait = 0;

    // Lanes with want take consecutive slots in lane order; returns this
    // lane's slot, or -1.
    __device__ __forceinline__ int append(bool want, int* nxt, int lane) {
        const unsigned wm = __ballot_sync(kFull, want);
        int t = -1;
        if (want) {
            const unsigned seq = tail + __popc(wm & ((1u << lane) - 1u));
            t = (int)(seq & (kPoolCap - 1));
            if (qn > 0) nxt[ql & (kPoolCap - 1)] = (int)seq;
            else qh = seq;
            ql = seq;
            ++qn;
        }
        tail += (unsigned)__popc(wm);
        return t;
    }
    // How many tickets to evaluate now: a warp's worth once 32 wait, or all
    // that wait once a lane whose ray has ended (ended) has waited
    // kPoolDrainWait steps for its tickets, or no lane is stepping; else 0.
    __device__ __forceinline__ unsigned batch(bool ended, bool stepping) {
        if (ended && qn > 0) ++wait;
        const unsigned cnt = tail - head;
        const bool flush = __any_sync(kFull, ended && qn > 0 && wait > kPoolDrainWait) || !__any_sync(kFull, stepping);
        if (cnt >= 32u) return 32u;
        return (cnt > 0u && flush) ? cnt : 0u;
    }
    // the slot a lane evaluates in the current batch
    __device__ __forceinline__ int slot(int lane) const { return (int)((head + (unsigned)lane) & (kPoolCap - 1)); }
    __device__ __forceinline__ void evaluated(unsigned n) { head += n; }
    // this lane's oldest ticket if it has been evaluated, else -1
    __device__ __forceinline__ int ready() const {
        return (qn > 0 && (int)(qh - head) < 0) ? (int)(qh & (kPoolCap - 1)) : -1;
    }
    __device__ __forceinline__ void pop(const int* nxt, int t) {
        if (--qn > 0) qh = (unsigned)nxt[t];
    }
    __device__ __forceinline__ bool empty() const { return qn == 0; }
    __device__ __forceinline__ void ray_ended() { wait = 0; }
};

template <int NF>
struct PoolLayout {
    // ticket fields, one row of kPoolCap doubles each: 0 |dl|, 1-2 x1 x2,
    // 3-6 k^mu, 7-15 the point (r, s, c, Sigma, theta', iS, irp, ithp, isn);
    // evaluated, rows 1..NF hold dtau and NF+1..2NF j / nu_p^2
    static constexpr int kIn = 16;
    static constexpr int kOut = 1 + 2 * NF;
    static constexpr int kFields = kIn > kOut ? kIn : kOut;
    // + the next-ticket links and image indices (two ints per entry), and in
    // the checked build the owner lane of each entry
    static constexpr int kWarpDoubles = kFields * kPoolCap + kPoolCap + (kChecked ? kPoolCap / 2 : 0);
};

template <int NF>
__global__ void __launch_bounds__(kRayMaxBlock, RAPTOR_POOL_MIN_BLOCKS)
    ray_kernel_pool(const DevImage* __restrict__ imgs, int n_imgs, long long ray_begin, long long ray_end,
                    unsigned long long* __restrict__ counters, double* __restrict__ out, int refill_interval) {
    using L = PoolLayout<NF>;
    constexpr int C = kPoolCap;
    __shared__ double pool_mem[(kRayMaxBlock / 32) * L::kWarpDoubles];
    const int lane = threadIdx.x & 31;
    double* const fld = pool_mem + (threadIdx.x >> 5) * L::kWarpDoubles;
    int* const nxt = reinterpret_cast<int*>(fld + L::kFields * C);
    int* const timg = nxt + C;
    int* const towner = timg + C;  // checked build only
    unsigned long long* const cw = imgs[0].check_word;
    RayState<NF, false> s;
    int mode = 0;  // 0 idle, 1 stepping, 2 ended with tickets outstanding
    bool live = true;
    TicketRing ring;
    int since_refill = refill_interval;
    const DevImage* im = imgs;
    RayCounters c;

    while (true) {
        // refill idle lanes every refill_interval steps, or at once when the warp has nothing to do
        const unsigned need = __ballot_sync(kFull, mode == 0 && live);
        if (need && (since_refill >= refill_interval || !__any_sync(kFull, mode != 0))) {
            since_refill = 0;
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&counters[kCtrQueue], (unsigned long long)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (mode == 0 && live) {
                const long long rid = ray_begin + (long long)(base + __popc(need & ((1u << lane) - 1u)));
                if (rid < ray_end) {
                    const DevImage* ri = start_ray(imgs, n_imgs, rid, s);
                    if (ri) {
                        im = ri;
                        mode = 1;
                    }
                } else {
                    live = false;
                }
            }
        }
        if (!__any_sync(kFull, mode != 0)) break;
        ++since_refill;

        // one geodesic step per stepping lane; a step inside the region appends a ticket
        bool want = false;
        double dl = 0.0;
        if (mode == 1) {
            const int event = advance_ray<NF, false, false>(*im, s, dl);
            if (event == 1) {
                ++c.rt_calls;
                want = true;
            }
            if (event == -1 || event == 3) {
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
            e[0] = fabs(dl);
            e[1 * C] = s.y[1];
            e[2 * C] = s.y[2];
#pragma unroll
            for (int i = 0; i < 4; ++i) e[(3 + i) * C] = s.y[4 + i];
            e[7 * C] = s.p.r;
            e[8 * C] = s.p.s;
            e[9 * C] = s.p.c;
            e[10 * C] = s.p.Sg;
            e[11 * C] = s.p.thp;
            e[12 * C] = s.p.iS;
            e[13 * C] = s.p.irp;
            e[14 * C] = s.p.ithp;
            e[15 * C] = s.p.isn;
            timg[t] = s.img;
        }

        const unsigned n = ring.batch(mode == 2, mode == 1);
        chk(n <= 32u, cw, kChkBatch, n);
        if (n) {
            __syncwarp();
            if ((unsigned)lane < n) {
                const int te = ring.slot(lane);
                double* e = fld + te;
                double y[8];
                MksPoint mp;
                y[0] = 0.0;
                y[1] = e[1 * C];
                y[2] = e[2 * C];
                y[3] = 0.0;
#pragma unroll
                for (int i = 0; i < 4; ++i) y[4 + i] = e[(3 + i) * C];
                mp.rp = 0.0;  // the metric does not read rp, s2x, c2x
                mp.s2x = 0.0;
                mp.c2x = 0.0;
                mp.r = e[7 * C];
                mp.s = e[8 * C];
                mp.c = e[9 * C];
                mp.Sg = e[10 * C];
                mp.thp = e[11 * C];
                mp.iS = e[12 * C];
                mp.irp = e[13 * C];
                mp.ithp = e[14 * C];
                mp.isn = e[15 * C];
                double dtau[NF], jn[NF];
                const bool ok = rt_terms_fp64<NF>(imgs[timg[te]], y, mp, e[0], dtau, jn);
                c.rt_samples += ok ? 1 : 0;
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    e[(1 + f) * C] = ok ? dtau[f] : 0.0;
                    e[(1 + NF + f) * C] = ok ? jn[f] : 0.0;
                }
            }
            __syncwarp();
            ring.evaluated(n);
            // owners apply their evaluated tickets, oldest first
            while (true) {
                const int ta = ring.ready();
                if (!__any_sync(kFull, ta >= 0)) break;
                if (ta >= 0) {
                    if (kChecked) chk(towner[ta] == lane, cw, kChkList, ta);
                    const double* e = fld + ta;
                    double dtau[NF], jn[NF];
#pragma unroll
                    for (int f = 0; f < NF; ++f) {
                        dtau[f] = e[(1 + f) * C];
                        jn[f] = e[(1 + NF + f) * C];
                    }
                    rt_apply_fp64<NF>(*im, e[0], dtau, jn, s.tau, s.I);
                    ring.pop(nxt, ta);
                }
            }
            __syncwarp();
        }
        if (mode == 2 && ring.empty()) {
            finish_ray(*im, s, out, c);
            mode = 0;
        }
    }
    c.publish(counters, lane);
}

// Spectrum: core.c:146-150 sums intensityfield over pixels per frequency.
// One block per (image, frequency) in a fixed-order tree, so the result is
// deterministic.  spec_img[s], spec_f[s] map spectrum slot s to its source.
// The camera's point quantities (mks_point at xcam[1], xcam[2], the same for
// every ray of an image), once per image after the images are uploaded and
// before any ray kernel reads them: per ray, the FP64 pipe evaluated them on
// the one or two lanes that a refill starts, at the cost of a full warp.
static __global__ void camera_point_kernel(DevImage* __restrict__ imgs, int n_imgs) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n_imgs) {
        MksPoint p;
        mks_point(imgs[k].xcam[1], imgs[k].xcam[2], imgs[k].geo, p);
        imgs[k].cam_point = p;
    }
}

static __global__ void spectrum_kernel(const DevImage* __restrict__ imgs, const int* __restrict__ spec_img,
                                const int* __restrict__ spec_f, const double* __restrict__ out,
                                double* __restrict__ spectrum) {
    __shared__ double red[256];
    const int sidx = blockIdx.x;
    const DevImage& im = imgs[spec_img[sidx]];
    const int f = spec_f[sidx];
    const long long npix = (long long)im.width * im.height;
    const double* o = out + im.out_offset + f;
    double acc = 0.0;
    for (long long k = threadIdx.x; k < npix; k += blockDim.x) acc += o[k * im.nfreq];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) spectrum[sidx] = red[0];
}

}  // namespace raptor
