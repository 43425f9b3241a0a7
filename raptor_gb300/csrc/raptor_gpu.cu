// C ABI of the engine (include/raptor_gpu.h): context, grid upload, batched
// render, statistics.  Host code here builds the per-image constants in
// FP64 and drives the persistent ray kernel on the context's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "raptor_gpu.h"
#include "engine_internal.h"
#include "ray_kernel.cuh"

using namespace raptor;

// ------------------------------------------------------------------ errors
int ctx_fail(raptor_gpu_ctx* ctx, int code, const char* fmt, ...) {
    if (ctx) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->err, sizeof ctx->err, fmt, ap);
        va_end(ap);
    }
    return code;
}

#define CK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return ctx_fail(ctx, RAPTOR_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));  \
    } while (0)

// ------------------------------------------------------------ grid packing
// [8][n1][n2] (HARM primitive-major, the reference's p[q][i][j]) ->
// [n1][n2][8] cells in FP64 and FP32, so one bilinear sample reads two
// 128-byte (FP64) / 64-byte (FP32) runs instead of 32 scattered words.
__global__ void pack_cells_kernel(const double* __restrict__ prims, long long ncell, double* __restrict__ c64,
                                  float* __restrict__ c32, int* __restrict__ bad) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ncell) return;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const double v = prims[q * ncell + k];
        if (!isfinite(v)) atomicExch(bad, 1);
        c64[k * 8 + q] = v;
        c32[k * 8 + q] = (float)v;
    }
}

// ------------------------------------------------------------- host math
static double camera_x2(double theta, double h) {
    // root of pi x + (1-h)/2 sin(2 pi x) = theta (newtonraphson.c:11-18,
    // 49-72), monotone for 0 <= h <= 2; Newton to convergence, clamped as
    // newtonraphson.c:71.
    double x = theta / M_PI;
    for (int it = 0; it < 100; ++it) {
        const double f = M_PI * x + 0.5 * (1. - h) * sin(2. * M_PI * x) - theta;
        const double fp = M_PI + M_PI * (1. - h) * cos(2. * M_PI * x);
        const double nx = x - f / fp;
        const bool conv = (nx == x) || fabs(nx - x) <= 1e-16 * fabs(nx);
        x = nx;
        if (conv) break;
    }
    return fmin(1., fmax(x, 0.));
}

static bool finite_all(std::initializer_list<double> v) {
    for (double x : v)
        if (!std::isfinite(x)) return false;
    return true;
}

int build_dev_image(raptor_gpu_ctx* ctx, const raptor_image_desc& d, DevImage& im) {
    if (d.grid < 0 || d.grid >= RAPTOR_MAX_GRIDS || !ctx->grids[d.grid].used)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "image refers to grid %d, which is not uploaded", d.grid);
    if (d.width <= 0 || d.height <= 0 || (long long)d.width * d.height > (1ll << 31) - 1)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "image size %dx%d out of range", d.width, d.height);
    if (d.n_freq < 1 || d.n_freq > RAPTOR_MAX_FREQS)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "n_freq %d out of range 1..%d", d.n_freq, RAPTOR_MAX_FREQS);
    if (d.integrator != RAPTOR_RK4 && d.integrator != RAPTOR_RK2)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "integrator %d is neither RK4 (4) nor RK2 (2)", d.integrator);
    if (d.camera != RAPTOR_CAM_LINEAR && d.camera != RAPTOR_CAM_LOG)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "camera %d is neither linear (0) nor log-polar (1)", d.camera);
    if (d.emission != RAPTOR_EMISSION_THERMAL && d.emission != RAPTOR_EMISSION_KAPPA)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "emission %d is neither thermal (0) nor kappa (1)", d.emission);
    if (!finite_all({d.cam_size_x, d.cam_size_y, d.inclination, d.mbh, d.m_unit, d.r_high, d.r_low, d.stepsize}) ||
        !(d.stepsize > 0) || !(d.mbh > 0) || !(d.m_unit > 0))
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "non-finite or non-positive image parameter");
    for (int f = 0; f < d.n_freq; ++f)
        if (!(d.freq[f] > 0) || !std::isfinite(d.freq[f]))
            return ctx_fail(ctx, RAPTOR_ERR_INVALID, "frequency %d is not a positive number", f);
    const GridSlot& gs = ctx->grids[d.grid];
    const raptor_grid_geom& g = gs.geom;
    memset(&im, 0, sizeof im);
    im.width = d.width;
    im.height = d.height;
    im.nfreq = d.n_freq;
    im.integrator = d.integrator;
    im.cells64 = gs.c64;
    im.cells32 = gs.c32;
    im.n1 = g.n1;
    im.n2 = g.n2;
    im.startx1 = g.startx1;
    im.startx2 = g.startx2;
    im.stopx1 = g.startx1 + g.n1 * g.dx1;  // raptor_harm_model.c:127-128
    im.stopx2 = g.startx2 + g.n2 * g.dx2;
    im.idx1 = 1.0 / g.dx1;
    im.idx2 = 1.0 / g.dx2;
    const double a = g.a;
    im.geo.a = a;
    im.geo.a2 = a * a;
    im.geo.hslope = g.hslope;
    im.geo.R0 = g.R0;
    im.geo.one_m_h = 1.0 - g.hslope;
    im.geo.th_coef = (1.0 - g.hslope) / (2.0 * M_PI);

    // camera grid (integrator.c:188-191)
    im.stepx = d.cam_size_x / (double)d.width;
    im.stepy = d.cam_size_y / (double)d.height;
    im.half_x = d.cam_size_x * 0.5;
    im.half_y = d.cam_size_y * 0.5;
    // pixel-independent part of initialize_photon (metric.c:652-692)
    const double mu0 = cos(d.inclination / 180. * M_PI);
    const double thc = acos(mu0);
    im.sin_mu = sqrt(1. - mu0 * mu0);
    im.mu0sq = mu0 * mu0;
    const double sinc2 = sin(thc) * sin(thc), cosc2 = cos(thc) * cos(thc);
    im.cc_over_sc = cosc2 / sinc2;
    im.cosc2 = cosc2;
    const double r = kRcam, rf = r;
    const double st = sin(thc), ct = cos(thc);
    const double sig = r * r + a * a * ct * ct;
    const double dl = r * r + a * a - 2. * r;
    const double A = (r * r + a * a) * (r * r + a * a) - dl * a * a * st * st;
    im.g11 = sig / dl * rf * rf;
    im.gu00 = -A / (sig * dl);
    im.gu03 = -2. * a * r / (sig * dl);
    im.gu33 = (dl - a * a * st * st) / (sig * dl * st * st);
    im.gu22 = 1. / sig;
    // BL -> KS at the camera (GRmath.c:151-177)
    const double x1c = log(kRcam);
    const double rc = exp(x1c);
    const double dc = rc * rc - 2. * rc + a * a;
    im.t01 = 2. * rc / dc * rc;
    im.t31 = a / dc * rc;
    const double rplus = 1. + sqrt(1. - a * a), rmin = 1. - sqrt(1. - a * a);
    im.xcam[0] = 0. + (log(dc) + 1. / sqrt(1. - a * a) * log((rc - rplus) / (rc - rmin)));
    im.xcam[1] = x1c;
    im.xcam[2] = camera_x2(thc, g.hslope);
    im.xcam[3] = 90. / 180. * M_PI + (a / (2. * sqrt(1. - a * a)) * log((rc - rplus) / (rc - rmin)));
    im.k2fac = M_PI * (1. + (1. - g.hslope) * cos(2. * M_PI * im.xcam[2]));

    // units and cut-offs (grmhd.c:17-33, utilities.c:19-21, radiative_transfer.c:56)
    const double L = kGGrav * d.mbh / (kC * kC);
    const double rho_unit = d.m_unit / pow(L, 3);
    im.B_unit = kC * sqrt(4. * M_PI * rho_unit);
    im.inv_B_unit = 1.0 / im.B_unit;
    im.Ne_unit = rho_unit / (kPMass + kEMass);
    im.r_high = d.r_high;
    im.r_low = d.r_low;
    im.stepsize = d.stepsize;
    im.inv_stepsize = 1.0 / d.stepsize;
    im.cutoff_inner = (1. + sqrt(1. - a * a)) * (1. + 1e-1);
    const double Rg = kGGrav * d.mbh / kC / kC;
    // log-polar camera constants (integrator.c:192-198, core.c:123-133, utilities.c:20)
    im.camera = d.camera;
    im.ln20 = log(20.);
    im.rgrav = Rg;
    im.dtheta_px = Rg * 2. * M_PI / (double)d.height;
    im.dist2 = kSourceDist * kSourceDist;
    for (int f = 0; f < d.n_freq; ++f) {
        im.freq[f] = d.freq[f];
        im.nu3[f] = pow(d.freq[f], 3.);
        im.rg_over_nu[f] = Rg / d.freq[f];
        im.inv_freq2[f] = 1.0 / (d.freq[f] * d.freq[f]);
        im.freq_f[f] = (float)im.freq[f];
        im.rg_over_nu_f[f] = (float)im.rg_over_nu[f];
    }
    // kappa-distribution fits (j_nu.c:28-106): the constant factors, in the
    // reference's own expressions, as logarithms
    im.emission = d.emission;
    if (d.emission == RAPTOR_EMISSION_KAPPA) {
        const double k = kKappa;
        KappaConst& kc = im.kap;
        kc.ln_jlow = log(4. * M_PI * std::tgamma(k - 4. / 3.) / (pow(3., 7. / 3.) * std::tgamma(k - 2.)));
        kc.ln_jhigh = log(pow(3., (k - 1) / 2.) * (k - 2.) * (k - 1.) / 4. * std::tgamma(k / 4. - 1. / 3.) *
                          std::tgamma(k / 4. + 4. / 3.));
        kc.xj = 3 * pow(k, -3. / 2.);
        kc.ln_alow = log(pow(3, 1. / 6.) * (10. / 41.) * pow(2 * M_PI, 2) * (k - 2.) * (k - 1.) * k / (3. * k - 1.) *
                         std::tgamma(5. / 3.));
        kc.ln_ahigh = log((pow(M_PI, 5. / 2.) / 3.) * ((k - 2.) * (k - 1.) * k) *
                          (2 * std::tgamma(2. + k / 2.) / (2. + k) - 1.) * (pow(3. / k, 19. / 4.) + 3. / 5.));
        kc.xa = pow(-7. / 4. + 8. * k / 5., -43. / 50.);
        const double ka = k - 1. / 3., kb = k + 1., kcc = k + 2. / 3.;
        kc.g1 = std::tgamma(kcc) * std::tgamma(kb - ka) / (std::tgamma(kb) * std::tgamma(kcc - ka));
        kc.g2 = std::tgamma(kcc) * std::tgamma(ka - kb) / (std::tgamma(ka) * std::tgamma(kcc - kb));
        im.kapf = KappaConstF{(float)kc.ln_jlow, (float)kc.ln_jhigh, (float)kc.xj,  (float)kc.ln_alow,
                              (float)kc.ln_ahigh, (float)kc.xa,     (float)kc.g1, (float)kc.g2};
    }
    im.ne_unit_f = (float)im.Ne_unit;
    im.b_unit_f = (float)im.B_unit;
    im.inv_b_unit_f = (float)im.inv_B_unit;
    im.r_high_f = (float)im.r_high;
    im.r_low_f = (float)im.r_low;
    // DF copies for the mixed-DF geodesic
    im.geo_df = GeoDF{df_const(im.geo.a),  df_const(im.geo.a2),      df_const(im.geo.hslope),
                      df_const(im.geo.R0), df_const(im.geo.one_m_h), df_const(im.geo.th_coef)};
    im.inv_stepsize_df = df_const(im.inv_stepsize);
    im.cutoff_inner_df = df_const(im.cutoff_inner);
    im.startx1_df = df_const(im.startx1);
    im.startx2_df = df_const(im.startx2);
    im.stopx1_df = df_const(im.stopx1);
    im.stopx2_df = df_const(im.stopx2);
    im.idx1_df = df_const(im.idx1);
    im.idx2_df = df_const(im.idx2);
    return RAPTOR_OK;
}

// ---------------------------------------------------------------- context
extern "C" int raptor_gpu_init(const raptor_gpu_options* options, raptor_gpu_ctx** out) {
    if (!out) return RAPTOR_ERR_INVALID;
    *out = nullptr;
    raptor_gpu_ctx* ctx = new (std::nothrow) raptor_gpu_ctx();
    if (!ctx) return RAPTOR_ERR_NOMEM;
    if (options) ctx->opt = *options;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= ctx->opt.device || ctx->opt.device < 0) {
        cudaGetLastError();
        delete ctx;
        return RAPTOR_ERR_NODEVICE;
    }
    ctx->device = ctx->opt.device;
    cudaDeviceProp prop;
    if (cudaSetDevice(ctx->device) != cudaSuccess || cudaGetDeviceProperties(&prop, ctx->device) != cudaSuccess) {
        delete ctx;
        return RAPTOR_ERR_NODEVICE;
    }
    if (prop.major < 10) {
        delete ctx;
        return RAPTOR_ERR_NODEVICE;
    }
    ctx->num_sms = prop.multiProcessorCount;
    snprintf(ctx->device_name, sizeof ctx->device_name, "%s", prop.name);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
        cudaEventCreate(&ctx->evA) != cudaSuccess || cudaEventCreate(&ctx->evB) != cudaSuccess ||
        cudaMalloc(&ctx->d_counters, kCtrCount * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&ctx->d_flag, sizeof(int)) != cudaSuccess) {
        raptor_gpu_destroy(ctx);
        return RAPTOR_ERR_CUDA;
    }
    *out = ctx;
    return RAPTOR_OK;
}

extern "C" void raptor_gpu_destroy(raptor_gpu_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto& g : ctx->grids) {
        cudaFree(g.c64);
        cudaFree(g.c32);
        cudaFree(g.staging);
    }
    cudaFree(ctx->d_imgs);
    cudaFree(ctx->d_out);
    cudaFree(ctx->d_spec);
    cudaFree(ctx->d_spec_map);
    cudaFree(ctx->d_counters);
    cudaFree(ctx->d_flag);
    cudaFree(ctx->d_grad);
    cudaFree(ctx->d_dldi);
    cudaFree(ctx->d_vjp_scratch);
    cudaFree(ctx->d_vjp_tape);
    cudaFree(ctx->d_trace);
    cudaFreeHost(ctx->h_imgs);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->evA) cudaEventDestroy(ctx->evA);
    if (ctx->evB) cudaEventDestroy(ctx->evB);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" const char* raptor_gpu_last_error(const raptor_gpu_ctx* ctx) { return ctx ? ctx->err : "no context"; }

extern "C" int raptor_gpu_get_stats(const raptor_gpu_ctx* ctx, raptor_gpu_stats* out) {
    if (!ctx || !out) return RAPTOR_ERR_INVALID;
    *out = ctx->stats;
    out->device_bytes = ctx->device_bytes;
    out->peak_device_bytes = ctx->peak_device_bytes;
    return RAPTOR_OK;
}

// FP64 cells, FP32 cells and the FP64 upload staging area
constexpr long long kGridBytesPerCell = 8 * (8 + 4 + 8);

void account_bytes(raptor_gpu_ctx* ctx, long long delta) {
    ctx->device_bytes += delta;
    ctx->peak_device_bytes = std::max(ctx->peak_device_bytes, ctx->device_bytes);
}

int ensure_buffer(raptor_gpu_ctx* ctx, void** ptr, size_t* cap, size_t bytes) {
    if (*cap >= bytes && *ptr) return RAPTOR_OK;
    cudaFree(*ptr);
    account_bytes(ctx, -(long long)*cap);
    *ptr = nullptr;
    *cap = 0;
    size_t want = std::max<size_t>(bytes, 256);
    if (cudaMalloc(ptr, want) != cudaSuccess) {
        cudaGetLastError();
        return ctx_fail(ctx, RAPTOR_ERR_NOMEM, "device allocation of %zu bytes failed", want);
    }
    *cap = want;
    account_bytes(ctx, (long long)want);
    return RAPTOR_OK;
}

extern "C" int raptor_gpu_upload_grid(raptor_gpu_ctx* ctx, const double* prims, const raptor_grid_geom* geom,
                                      int* grid_id) {
    if (!ctx) return RAPTOR_ERR_INVALID;
    ctx->err[0] = 0;
    if (!prims || !geom || !grid_id) return ctx_fail(ctx, RAPTOR_ERR_INVALID, "null argument");
    const raptor_grid_geom& g = *geom;
    if (g.n1 < 2 || g.n2 < 2 || (long long)g.n1 * g.n2 > (1ll << 30))
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "grid %dx%d out of range (need >= 2x2)", g.n1, g.n2);
    if (!finite_all({g.startx1, g.startx2, g.dx1, g.dx2, g.a, g.hslope, g.R0}) || !(g.dx1 > 0) || !(g.dx2 > 0))
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "non-finite or non-positive grid geometry");
    if (!(fabs(g.a) < 1.0)) return ctx_fail(ctx, RAPTOR_ERR_INVALID, "spin |a| = %g must be below 1", g.a);
    if (!(g.hslope >= 0.0 && g.hslope < 2.0))
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "hslope %g outside [0, 2): theta(x2) would not be monotone", g.hslope);
    auto t0 = std::chrono::steady_clock::now();
    CK(cudaSetDevice(ctx->device));
    cudaGetLastError();  // a failed earlier call must not fail this one
    int id = *grid_id;
    if (id >= 0) {
        if (id >= RAPTOR_MAX_GRIDS || !ctx->grids[id].used)
            return ctx_fail(ctx, RAPTOR_ERR_INVALID, "grid id %d is not in use", id);
        if (ctx->grids[id].geom.n1 != g.n1 || ctx->grids[id].geom.n2 != g.n2) {
            GridSlot& s = ctx->grids[id];
            cudaFree(s.c64);
            cudaFree(s.c32);
            cudaFree(s.staging);
            account_bytes(ctx, -kGridBytesPerCell * s.cap_cells);
            s = GridSlot();
        }
    } else {
        for (int k = 0; k < RAPTOR_MAX_GRIDS; ++k)
            if (!ctx->grids[k].used) {
                id = k;
                break;
            }
        if (id < 0) return ctx_fail(ctx, RAPTOR_ERR_INVALID, "all %d grid slots are in use", RAPTOR_MAX_GRIDS);
    }
    GridSlot& s = ctx->grids[id];
    const long long ncell = (long long)g.n1 * g.n2;
    if (s.c64 && s.cap_cells < ncell) {  // a released slot keeps its buffers; grow them if too small
        cudaFree(s.c64);
        cudaFree(s.c32);
        cudaFree(s.staging);
        account_bytes(ctx, -kGridBytesPerCell * s.cap_cells);
        s = GridSlot();
    }
    if (!s.c64) {
        if (cudaMalloc(&s.c64, ncell * 8 * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&s.c32, ncell * 8 * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&s.staging, ncell * 8 * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(s.c64);
            cudaFree(s.c32);
            cudaFree(s.staging);
            s = GridSlot();
            return ctx_fail(ctx, RAPTOR_ERR_NOMEM, "grid allocation failed");
        }
        s.cap_cells = ncell;
        account_bytes(ctx, kGridBytesPerCell * ncell);
    }
    s.used = true;
    s.geom = g;
    CK(cudaMemcpyAsync(s.staging, prims, ncell * 8 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
    const int tpb = 256;
    pack_cells_kernel<<<(unsigned)((ncell + tpb - 1) / tpb), tpb, 0, ctx->stream>>>(s.staging, ncell, s.c64, s.c32,
                                                                                     ctx->d_flag);
    CK(cudaGetLastError());
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    auto t1 = std::chrono::steady_clock::now();
    ctx->last_upload_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    if (bad) {
        s.used = false;
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "grid holds non-finite primitive values");
    }
    *grid_id = id;
    return RAPTOR_OK;
}

extern "C" long long raptor_gpu_output_size(const raptor_image_desc* imgs, int n_imgs) {
    long long n = 0;
    for (int k = 0; k < n_imgs; ++k) n += (long long)imgs[k].width * imgs[k].height * imgs[k].n_freq;
    return n;
}

extern "C" long long raptor_gpu_spectrum_size(const raptor_image_desc* imgs, int n_imgs) {
    long long n = 0;
    for (int k = 0; k < n_imgs; ++k) n += imgs[k].n_freq;
    return n;
}

// ----------------------------------------------------------------- render
// Renders take ray_kernel<NF, MIXED, false>; a trace (any frequency count)
// takes the 8-frequency trace kernel, which also integrates t and phi.
template <int NF, bool MIXED>
static void launch_ray(const LaunchShape& ls, cudaStream_t st, const DevImage* imgs, int n, long long b, long long e,
                       unsigned long long* ctr, double* out, TraceSpec tr) {
    if (tr.out) ray_kernel<kMaxFreqs, MIXED, true><<<ls.grid, ls.block, 0, st>>>(imgs, n, b, e, ctr, out, ls.refill, tr);
    else ray_kernel<NF, MIXED, false><<<ls.grid, ls.block, 0, st>>>(imgs, n, b, e, ctr, out, ls.refill, tr);
}

// The FP64 form's pooled kernel; a trace (per-step records of tau and I)
// needs the in-place sample and takes the trace kernel.
template <int NF>
static void launch_ray_pool(const LaunchShape& ls, cudaStream_t st, const DevImage* imgs, int n, long long b,
                            long long e, unsigned long long* ctr, double* out, TraceSpec tr) {
    if (tr.out) ray_kernel<kMaxFreqs, false, true><<<ls.grid, ls.block, 0, st>>>(imgs, n, b, e, ctr, out, ls.refill, tr);
    else ray_kernel_pool<NF><<<ls.grid, ls.block, 0, st>>>(imgs, n, b, e, ctr, out, ls.refill);
}

RayLaunchFn pick_ray_kernel(int nf, int form, const void** fn, bool pool) {
    if (form == RAPTOR_PREC_MIXED_DF) return pick_ray_kernel_df(nf, fn);
    const bool mixed = form == RAPTOR_PREC_MIXED;
    // one instantiation per frequency-count bucket so tau/I stay in registers
#define PICK(NF)                                                        \
    if (nf <= NF) {                                                     \
        if (mixed) { *fn = (const void*)ray_kernel<NF, true, false>; return launch_ray<NF, true>; } \
        if (pool) { *fn = (const void*)ray_kernel_pool<NF>; return launch_ray_pool<NF>; } \
        *fn = (const void*)ray_kernel<NF, false, false>;               \
        return launch_ray<NF, false>;                                   \
    }
    PICK(1)
    PICK(2)
    PICK(4)
    PICK(8)
#undef PICK
    return nullptr;
}

int prepare_batch(raptor_gpu_ctx* ctx, const raptor_image_desc* imgs, int n_imgs, Batch& b) {
    if (!imgs || n_imgs <= 0) return ctx_fail(ctx, RAPTOR_ERR_INVALID, "no images");
    b.n = n_imgs;
    b.total_rays = 0;
    b.out_len = 0;
    b.spec_len = 0;
    b.max_nf = 1;
    b.host.resize(n_imgs);
    b.spec_img.clear();
    b.spec_f.clear();
    for (int k = 0; k < n_imgs; ++k) {
        int rc = build_dev_image(ctx, imgs[k], b.host[k]);
        if (rc) return rc;
        b.host[k].ray_begin = b.total_rays;
        b.host[k].out_offset = b.out_len;
        b.total_rays += (long long)imgs[k].width * imgs[k].height;
        b.out_len += (long long)imgs[k].width * imgs[k].height * imgs[k].n_freq;
        for (int f = 0; f < imgs[k].n_freq; ++f) {
            b.spec_img.push_back(k);
            b.spec_f.push_back(f);
        }
        b.spec_len += imgs[k].n_freq;
        b.max_nf = std::max(b.max_nf, imgs[k].n_freq);
    }
    int rc = ensure_buffer(ctx, (void**)&ctx->d_imgs, &ctx->imgs_cap, sizeof(DevImage) * n_imgs);
    if (!rc) rc = ensure_buffer(ctx, (void**)&ctx->d_out, &ctx->out_cap, sizeof(double) * b.out_len);
    if (!rc) rc = ensure_buffer(ctx, (void**)&ctx->d_spec, &ctx->spec_cap, sizeof(double) * b.spec_len);
    if (!rc) rc = ensure_buffer(ctx, (void**)&ctx->d_spec_map, &ctx->spec_map_cap, sizeof(int) * 2 * b.spec_len);
    if (rc) return rc;
    if (ctx->h_imgs_cap < (size_t)n_imgs) {
        cudaFreeHost(ctx->h_imgs);
        ctx->h_imgs = nullptr;
        ctx->h_imgs_cap = 0;
        if (cudaMallocHost(&ctx->h_imgs, sizeof(DevImage) * n_imgs) != cudaSuccess) {
            cudaGetLastError();
            return ctx_fail(ctx, RAPTOR_ERR_NOMEM, "pinned allocation failed");
        }
        ctx->h_imgs_cap = n_imgs;
    }
    for (int k = 0; k < n_imgs; ++k) {
        b.host[k].out_end = b.out_len;
        b.host[k].check_word = ctx->d_counters + kCtrCheck;
    }
    memcpy(ctx->h_imgs, b.host.data(), sizeof(DevImage) * n_imgs);
    std::vector<int> map(2 * b.spec_len);
    for (int s = 0; s < b.spec_len; ++s) {
        map[s] = b.spec_img[s];
        map[b.spec_len + s] = b.spec_f[s];
    }
    CK(cudaMemcpyAsync(ctx->d_imgs, ctx->h_imgs, sizeof(DevImage) * n_imgs, cudaMemcpyHostToDevice, ctx->stream));
    camera_point_kernel<<<(n_imgs + 127) / 128, 128, 0, ctx->stream>>>(ctx->d_imgs, n_imgs);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ctx->d_spec_map, map.data(), sizeof(int) * 2 * b.spec_len, cudaMemcpyHostToDevice,
                       ctx->stream));
    b.h2d_bytes = sizeof(DevImage) * n_imgs + sizeof(int) * 2 * b.spec_len;
    return RAPTOR_OK;
}

LaunchShape default_shape(raptor_gpu_ctx* ctx, const void* fn, int form) {
    LaunchShape ls;
    ls.block = ctx->opt.block_size > 0 ? ctx->opt.block_size : kRayMaxBlock;
    ls.block = std::max(32, std::min(kRayMaxBlock, ls.block / 32 * 32));
    int occ = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, ls.block, 0);
    occ = std::max(occ, 1);
    int bps = ctx->opt.blocks_per_sm > 0 ? std::min(ctx->opt.blocks_per_sm, occ) : occ;
    ls.grid = ctx->num_sms * bps;
    ls.bps = bps;
    ls.refill = ctx->opt.refill_interval > 0 ? ctx->opt.refill_interval
                                             : (form == RAPTOR_PREC_MIXED_DF ? kDefaultRefillDF : kDefaultRefill);
    return ls;
}

// Enqueue the whole render (counters reset, ray kernel, spectrum) on the
// context stream; used directly and under stream capture.
int enqueue_render(raptor_gpu_ctx* ctx, const Batch& b, int form, long long rb, long long re,
                   const LaunchShape& ls, RayLaunchFn fn, bool timed, TraceSpec tr) {
    if (timed) CK(cudaEventRecord(ctx->evA, ctx->stream));
    CK(cudaMemsetAsync(ctx->d_counters, 0, kCtrCount * sizeof(unsigned long long), ctx->stream));
    if (rb > 0 || re < b.total_rays) CK(cudaMemsetAsync(ctx->d_out, 0, sizeof(double) * b.out_len, ctx->stream));
    if (timed) CK(cudaEventRecord(ctx->ev0, ctx->stream));
    fn(ls, ctx->stream, ctx->d_imgs, b.n, rb, re, ctx->d_counters, ctx->d_out, tr);
    CK(cudaGetLastError());
    if (timed) CK(cudaEventRecord(ctx->ev1, ctx->stream));
    spectrum_kernel<<<(unsigned)b.spec_len, 256, 0, ctx->stream>>>(ctx->d_imgs, ctx->d_spec_map,
                                                                   ctx->d_spec_map + b.spec_len, ctx->d_out,
                                                                   ctx->d_spec);
    CK(cudaGetLastError());
    if (timed) CK(cudaEventRecord(ctx->evB, ctx->stream));
    return RAPTOR_OK;
}

int collect_stats(raptor_gpu_ctx* ctx, bool timed) {
    unsigned long long c[kCtrCount];
    CK(cudaMemcpy(c, ctx->d_counters, sizeof c, cudaMemcpyDeviceToHost));
    raptor_gpu_stats& s = ctx->stats;
    s.steps = (long long)c[kCtrSteps];
    s.rt_calls = (long long)c[kCtrRtCalls];
    s.rt_samples = (long long)c[kCtrRtSamples];
    s.rays = (long long)c[kCtrRays];
    s.n_stepcap = (long long)c[kCtrStepCap];
    s.n_nonfinite = (long long)c[kCtrNonFinite];
    s.max_ray_steps = (long long)c[kCtrMaxSteps];
    ctx->check_word = c[kCtrCheck];
    s.vjp_terms = 0;  // render statistics: no adjoint terms
    s.vjp_gated_terms = 0;
    double kk;
    memcpy(&kk, &c[kCtrKkMax], sizeof kk);
    s.kk_max = kk;
    if (timed) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        s.kernel_ms = ms;
        CK(cudaEventElapsedTime(&ms, ctx->evA, ctx->evB));
        s.device_ms = ms;
    }
    return RAPTOR_OK;
}

// Status of a finished render from its counters: a failed check of the
// checked build, or a ray count other than expected, is a device error;
// rays that ended non-finite make it an error, rays stopped by the step cap
// a warning; the outputs are complete in these last two cases.
int render_status(raptor_gpu_ctx* ctx, long long rays, long long expected, long long n_nonfinite,
                  long long n_stepcap, unsigned long long check) {
    if (check)
        return ctx_fail(ctx, RAPTOR_ERR_DEVICE, "checked build: %s (value %lld)", check_name(check),
                        (long long)(check & 0x00ffffffffffffffull));
    if (rays != expected)
        return ctx_fail(ctx, RAPTOR_ERR_DEVICE, "ray kernel retired %lld rays, expected %lld", rays, expected);
    if (n_nonfinite > 0)
        return ctx_fail(ctx, RAPTOR_ERR_NONFINITE,
                        "%lld of %lld rays ended with a non-finite photon state or intensity", n_nonfinite, rays);
    if (n_stepcap > 0)
        return ctx_fail(ctx, RAPTOR_WARN_STEPCAP, "%lld of %lld rays stopped at the step cap of %.0f steps",
                        n_stepcap, rays, kMaxSteps);
    return RAPTOR_OK;
}

// Replay the device part of a render (counter reset, ray kernel, spectrum)
// as one CUDA graph.  The graph is captured once per batch signature - image
// count, ray and output extents, kernel instantiation, launch shape and the
// buffers it touches - and relaunched while the signature repeats; the
// per-image descriptors are uploaded before every launch, so their contents
// (angles, frequencies, units, grids of the same size) may change freely.
int graph_render(raptor_gpu_ctx* ctx, const Batch& b, int form, const LaunchShape& ls, RayLaunchFn fn,
                 bool* replayed) {
    char key[512];
    snprintf(key, sizeof key, "%d|%lld|%lld|%d|%d|%d|%d|%d|%d|%p|%p|%p|%p|%p|%p", b.n, b.total_rays, b.out_len,
             b.spec_len, b.max_nf, form, ls.grid, ls.block, ls.refill, (void*)fn, (void*)ctx->d_imgs,
             (void*)ctx->d_out, (void*)ctx->d_spec, (void*)ctx->d_spec_map, (void*)ctx->d_counters);
    *replayed = ctx->graph_exec && ctx->graph_key == key;
    if (!*replayed) {
        if (ctx->graph_exec) {
            cudaGraphExecDestroy(ctx->graph_exec);
            ctx->graph_exec = nullptr;
        }
        cudaGraph_t graph = nullptr;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_render(ctx, b, form, 0, b.total_rays, ls, fn, false);
        cudaError_t ec = cudaStreamEndCapture(ctx->stream, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (ec != cudaSuccess) return ctx_fail(ctx, RAPTOR_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ec));
        ec = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ec != cudaSuccess) {
            ctx->graph_exec = nullptr;
            return ctx_fail(ctx, RAPTOR_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ec));
        }
        ctx->graph_key = key;
    }
    // the whole graph is the timed region: kernel and device times coincide
    CK(cudaEventRecord(ctx->evA, ctx->stream));
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaEventRecord(ctx->evB, ctx->stream));
    return RAPTOR_OK;
}

static int render_impl(raptor_gpu_ctx* ctx, const raptor_image_desc* imgs, int n_imgs, int precision,
                       long long ray_begin, long long ray_count, double* I_out, double* spectrum_out) {
    if (!ctx) return RAPTOR_ERR_INVALID;
    ctx->err[0] = 0;
    auto t0 = std::chrono::steady_clock::now();
    if (precision != RAPTOR_PREC_FP64 && precision != RAPTOR_PREC_MIXED && precision != RAPTOR_PREC_MIXED_DF)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "precision %d unknown", precision);
    CK(cudaSetDevice(ctx->device));
    cudaGetLastError();  // a failed earlier call must not fail this one
    Batch& b = ctx->batch;
    int rc = prepare_batch(ctx, imgs, n_imgs, b);
    if (rc) return rc;
    long long rb = ray_begin < 0 ? 0 : ray_begin;
    long long re = ray_count < 0 ? b.total_rays : std::min(b.total_rays, rb + ray_count);
    if (rb > b.total_rays) return ctx_fail(ctx, RAPTOR_ERR_INVALID, "ray range starts past the batch");
    const int form = precision;
    const void* fnp = nullptr;
    RayLaunchFn fn = pick_ray_kernel(b.max_nf, form, &fnp, !ctx->opt.no_sample_pool);
    LaunchShape ls = choose_shape(ctx, b, form, fn, fnp);
    bool replayed = false;
    if (ctx->opt.use_graph && rb == 0 && re == b.total_rays) {
        rc = graph_render(ctx, b, form, ls, fn, &replayed);
    } else {
        rc = enqueue_render(ctx, b, form, rb, re, ls, fn, true);
    }
    if (rc) return rc;
    size_t d2h = 0;
    if (I_out) {
        CK(cudaMemcpyAsync(I_out, ctx->d_out, sizeof(double) * b.out_len, cudaMemcpyDeviceToHost, ctx->stream));
        d2h += sizeof(double) * b.out_len;
    }
    if (spectrum_out) {
        CK(cudaMemcpyAsync(spectrum_out, ctx->d_spec, sizeof(double) * b.spec_len, cudaMemcpyDeviceToHost,
                           ctx->stream));
        d2h += sizeof(double) * b.spec_len;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    rc = collect_stats(ctx, true);
    if (rc) return rc;
    raptor_gpu_stats& s = ctx->stats;
    s.h2d_bytes = (double)b.h2d_bytes;
    s.d2h_bytes = (double)d2h;
    s.block_size = ls.block;
    s.blocks_per_sm = ls.bps;
    s.refill_interval = ls.refill;
    s.grid_blocks = ls.grid;
    s.graph_replayed = replayed ? 1 : 0;
    s.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return render_status(ctx, s.rays, re - rb, s.n_nonfinite, s.n_stepcap, ctx->check_word);
}

extern "C" int raptor_gpu_render(raptor_gpu_ctx* ctx, const raptor_image_desc* imgs, int n_imgs, int precision,
                                 double* I_out, double* spectrum_out) {
    return render_impl(ctx, imgs, n_imgs, precision, 0, -1, I_out, spectrum_out);
}

extern "C" int raptor_gpu_render_range(raptor_gpu_ctx* ctx, const raptor_image_desc* imgs, int n_imgs,
                                       int precision, long long ray_begin, long long ray_count, double* I_out,
                                       double* spectrum_out) {
    if (ray_begin < 0 || ray_count < 0) return ctx_fail(ctx, RAPTOR_ERR_INVALID, "negative ray range");
    return render_impl(ctx, imgs, n_imgs, precision, ray_begin, ray_count, I_out, spectrum_out);
}

extern "C" int raptor_gpu_trace_ray(raptor_gpu_ctx* ctx, const raptor_image_desc* img, int precision, int pixel,
                                    int max_records, double* records, int* n_records) {
    if (!ctx) return RAPTOR_ERR_INVALID;
    ctx->err[0] = 0;
    if (!img || !records || !n_records || max_records <= 0)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "trace_ray: null output or non-positive max_records");
    if (precision != RAPTOR_PREC_FP64 && precision != RAPTOR_PREC_MIXED && precision != RAPTOR_PREC_MIXED_DF)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "precision %d unknown", precision);
    if (pixel < 0 || (long long)pixel >= (long long)img->width * img->height)
        return ctx_fail(ctx, RAPTOR_ERR_INVALID, "pixel %d outside the %dx%d image", pixel, img->width, img->height);
    CK(cudaSetDevice(ctx->device));
    cudaGetLastError();  // a failed earlier call must not fail this one
    Batch& b = ctx->batch;
    int rc = prepare_batch(ctx, img, 1, b);
    if (rc) return rc;
    const size_t bytes = sizeof(double) * (size_t)max_records * kTraceWidth;
    rc = ensure_buffer(ctx, (void**)&ctx->d_trace, &ctx->trace_cap, bytes);
    if (rc) return rc;
    CK(cudaMemsetAsync(ctx->d_trace, 0, bytes, ctx->stream));
    const void* fnp = nullptr;
    RayLaunchFn fn = pick_ray_kernel(b.max_nf, precision, &fnp, false);
    LaunchShape ls = default_shape(ctx, fnp, precision);
    ls.grid = 1;
    ls.block = 32;
    TraceSpec tr{pixel, ctx->d_trace, max_records};
    rc = enqueue_render(ctx, b, precision, pixel, pixel + 1, ls, fn, true, tr);
    if (rc) return rc;
    CK(cudaMemcpyAsync(records, ctx->d_trace, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    rc = collect_stats(ctx, true);
    if (rc) return rc;
    const long long steps = ctx->stats.steps;
    *n_records = (int)std::min<long long>(steps + 1, max_records);
    return RAPTOR_OK;
}
