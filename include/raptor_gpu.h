/* raptor_gpu.h - C ABI of the GB300 (sm_103a) engine for RAPTOR's per-pixel
 * imaging hot path.
 *
 * The engine replaces the body of the reference's calculate_image
 * (core.c:74-152, declared at functions.h:70): for every camera pixel it
 * traces the null geodesic backward through Kerr spacetime in MKS
 * coordinates (integrator.c:149-289, metric.c:94-137,207-231,538-638),
 * samples the HARM primitives (raptor_harm_model.c:190-320, grmhd.c:35-71)
 * and accumulates thermal-synchrotron transfer (radiative_transfer.c:49-119,
 * j_nu.c:130-153,188-200).  Everything outside that loop - read_model,
 * init_harm_data, set_units, set_constants, output_files - stays in the
 * caller, with its model.in and file formats unchanged.
 *
 * Plain C types only.  The caller owns every host buffer; device memory
 * belongs to the context and never crosses this interface.  Every call
 * blocks until its results are on the host, returns RAPTOR_OK (0), a
 * positive warning (the results are complete) or a negative error, and never
 * exits the process (unlike core.c:15 or raptor_harm_model.c:84).  One
 * context per host thread.
 */
#ifndef RAPTOR_GPU_H
#define RAPTOR_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RAPTOR_GPU_ABI_VERSION 1
#define RAPTOR_MAX_FREQS 8  /* frequencies per image in one render */
#define RAPTOR_MAX_GRIDS 16 /* dumps resident in one context */

/* status codes */
#define RAPTOR_OK 0
#define RAPTOR_ERR_INVALID (-1)  /* bad argument (sizes, ids, non-finite input) */
#define RAPTOR_ERR_CUDA (-2)     /* a CUDA runtime call failed */
#define RAPTOR_ERR_DEVICE (-3)   /* the kernels flagged an error (see last_error) */
#define RAPTOR_ERR_NOMEM (-4)    /* device or pinned allocation failed */
#define RAPTOR_ERR_NODEVICE (-5) /* no usable sm_103 device */
/* (-6 is RAPTOR_ERR_NOALLOC_LIMIT, below) */
#define RAPTOR_ERR_NONFINITE (-7) /* a render finished, but rays ended with a non-finite photon
                                     state or intensity (the stats count them in n_nonfinite).
                                     The outputs are written, each such pixel as its ray left
                                     it; the reference renders these without notice (a camera
                                     at inclination exactly 0 gives NaN wave vectors at
                                     metric.c:662-668, 0 * inf, and an empty image). */
#define RAPTOR_WARN_STEPCAP 1 /* a warning, not an error: the render is complete, but rays
                                 stopped at the step cap (max_steps, parameters.h:182), as the
                                 reference stops them without notice (integrator.c:228); the
                                 stats count them in n_stepcap.  Text in last_error. */

/* arithmetic forms */
#define RAPTOR_PREC_FP64 0  /* everything FP64, the reference's arithmetic */
#define RAPTOR_PREC_MIXED 1 /* FP64 geodesic + metric, FP32 fluid/emission/transfer */
#define RAPTOR_PREC_MIXED_DF 2 /* geodesic + metric in double-float (pairs of FP32, 48-bit
                                  significand) on the FP32 pipes, transfer as RAPTOR_PREC_MIXED */

/* integrators (parameters.h:186-189) */
#define RAPTOR_RK4 4
#define RAPTOR_RK2 2

/* emission models: the fits that emission_coeff (j_nu.c:20-26) returns */
#define RAPTOR_EMISSION_THERMAL 0 /* thermal synchrotron, j_nu.c:130-153, 188-200 (the reference's) */
#define RAPTOR_EMISSION_KAPPA 1   /* kappa distribution, kappa = 3.5, j_nu.c:28-106 (defined in the
                                     reference but not called by it); renders, traces and
                                     adjoints in every form */

/* camera maps (parameters.h:54-55) */
#define RAPTOR_CAM_LINEAR 0 /* LINEAR_IMPACT_CAM: uniform grid of impact parameters (integrator.c:186-190) */
#define RAPTOR_CAM_LOG 1    /* LOG_IMPACT_CAM: log-polar grid, x -> radius, y -> angle (integrator.c:191-198) */

typedef struct raptor_gpu_options {
    int device;          /* CUDA device ordinal */
    int block_size;      /* threads per block of the ray kernel; 0 = default/tuned */
    int blocks_per_sm;   /* resident blocks per SM of the persistent grid; 0 = default/tuned */
    int refill_interval; /* geodesic steps between lane refills ("steps per chunk"); 0 = 1 */
    int autotune;        /* 1: tune block size / refill interval on a ray sample once per
                            (device, batch signature) and reuse the result */
    int use_graph;       /* 1: replay a render through a captured CUDA graph when the batch
                            signature repeats */
    int no_sample_pool;  /* FP64 form and FP64 adjoint: 1 = each lane evaluates its own ray's
                            samples in place; 0 (default) = a warp evaluates them 32 at a time
                            from a shared-memory pool.  The same arithmetic per ray: the images
                            agree bit for bit or to rounding. */
    int vjp_tape;        /* raptor_gpu_vjp: 0 (default) = one adjoint pass that keeps each ray's
                            per-cell terms on a per-lane device tape of 2048 records and takes
                            the ray's I from its own sums; n > 0 = n records per lane; -1 = two
                            passes (the forward render, then the adjoint reading each pixel's I
                            from it).  A ray with more records than fit, or a tape that cannot
                            be allocated, makes the call fall back to two passes; the in-place
                            FP64 adjoint (no_sample_pool) always takes two.  The tape (resident
                            lanes x records x 48 to 240 bytes: 14 GB at five frequencies in
                            FP64) stays allocated on the context for later calls. */
    int reserved[6];
} raptor_gpu_options;

/* Grid geometry: the HARM header fields the hot path uses
 * (raptor_harm_model.c:90-115).  stopx = startx + n*dx is derived inside,
 * as raptor_harm_model.c:127-128 does. */
typedef struct raptor_grid_geom {
    int n1, n2;
    double startx1, startx2;
    double dx1, dx2;
    double a;      /* black-hole spin */
    double hslope; /* MKS theta compression */
    double R0;     /* MKS radial offset */
} raptor_grid_geom;

/* One image: the model.in + argv values that calculate_image reads through
 * globals (core.c:22-42, parameters.h). */
typedef struct raptor_image_desc {
    int width, height;            /* IMG_WIDTH, IMG_HEIGHT */
    double cam_size_x, cam_size_y; /* CAM_SIZE_X/Y, in Rg */
    double inclination;           /* INCLINATION, degrees */
    double mbh;                   /* MBH, g */
    double m_unit;                /* M_UNIT, g */
    double r_high, r_low;         /* R_HIGH, R_LOW (R-beta electron temperature) */
    double stepsize;              /* STEPSIZE */
    int integrator;               /* RAPTOR_RK4 or RAPTOR_RK2 */
    int grid;                     /* id from raptor_gpu_upload_grid */
    int n_freq;                   /* 1..RAPTOR_MAX_FREQS */
    double freq[RAPTOR_MAX_FREQS]; /* Hz */
    int camera;                   /* RAPTOR_CAM_LINEAR (0) or RAPTOR_CAM_LOG */
    int emission;                 /* RAPTOR_EMISSION_THERMAL (0) or RAPTOR_EMISSION_KAPPA */
} raptor_image_desc;

typedef struct raptor_gpu_stats {
    double kernel_ms;  /* ray kernel, CUDA events on the context stream */
    double device_ms;  /* all device work of the render (reset, ray kernel, spectrum), same events */
    double total_ms;   /* whole call, host wall time */
    double h2d_bytes, d2h_bytes;
    long long rays;
    long long steps;      /* geodesic (RK) steps */
    long long rt_calls;   /* steps inside the grid (radiative_transfer calls) */
    long long rt_samples; /* calls that passed the sigma cut (emission evaluated) */
    long long max_ray_steps;
    long long n_stepcap;  /* rays stopped by max_steps (parameters.h:182) */
    long long n_nonfinite; /* rays that ended with a non-finite photon state or intensity */
    double kk_max;        /* max |g k k| / (k^t)^2 over rays at termination */
    int block_size, blocks_per_sm, refill_interval, grid_blocks;
    int graph_replayed;
    long long device_bytes;      /* device memory the context holds now */
    long long peak_device_bytes; /* the most it has held */
    long long vjp_terms;         /* raptor_gpu_vjp: (sample, frequency) terms that emitted */
    long long vjp_gated_terms;   /* raptor_gpu_vjp: of those, inside the tau < ln 1000 gate */
} raptor_gpu_stats;

/* Gradients of a scalar loss L(I) of the output image, given dL/dI. */
typedef struct raptor_grad {
    double d_m_unit;      /* dL/dM_UNIT */
    double d_r_high;      /* dL/dR_HIGH */
    double d_r_low;       /* dL/dR_LOW  (dL/d(T_p/T_e) = d_r_high + d_r_low when equal) */
    double d_inclination; /* dL/dINCLINATION, per degree */
    double *d_rho;        /* [n1*n2] dL/d rho per cell (caller-allocated, may be NULL) */
    double *d_u;          /* [n1*n2] dL/d u per cell (caller-allocated, may be NULL) */
    double *d_lnthetae;   /* [n1*n2] dL/d ln f per cell, f a per-cell factor on the electron
                             temperature Theta_e of every sample, interpolated bilinearly as
                             rho and u are (f = 1 renders the reference's image; may be NULL) */
} raptor_grad;

typedef struct raptor_gpu_ctx raptor_gpu_ctx;

/* Create a context on options->device (NULL: defaults).  Replaces the
 * OpenACC data region set-up of core.c:78. */
int raptor_gpu_init(const raptor_gpu_options *options, raptor_gpu_ctx **out);
void raptor_gpu_destroy(raptor_gpu_ctx *ctx);
/* Text of the last error on this context ("" if none). */
const char *raptor_gpu_last_error(const raptor_gpu_ctx *ctx);

/* Upload a dump's eight primitives, float64 [8][n1][n2] in HARM order
 * (rho, u, U1, U2, U3, B1, B2, B3) - the contiguous form of the
 * reference's p[NPRIM][N1][N2][1] (grmhd.c:76-91, copied in at core.c:78).
 * Returns the grid id in *grid_id.  Re-uploading to an existing id
 * (*grid_id >= 0 on entry and geometry unchanged) reuses its memory. */
int raptor_gpu_upload_grid(raptor_gpu_ctx *ctx, const double *prims, const raptor_grid_geom *geom,
                           int *grid_id);

/* Render n_imgs images in one persistent launch (core.c:97-142 for each).
 * I_out: concatenation over images of intensityfield[W*H][n_freq]
 * (pixel x + y*W, frequency fastest), already multiplied by nu^3 as
 * core.c:136 does (by nu^3 r dr dtheta / D^2 for RAPTOR_CAM_LOG, core.c:123-133).  spectrum_out: [sum over images of n_freq], the plain
 * pixel sum of core.c:146-150 (the caller applies JANSKY_FACTOR when
 * writing, core.c:177,192,195).  Either output may be NULL. */
int raptor_gpu_render(raptor_gpu_ctx *ctx, const raptor_image_desc *imgs, int n_imgs, int precision,
                      double *I_out, double *spectrum_out);

/* Same, restricted to the global ray range [ray_begin, ray_begin+ray_count)
 * of the batch (rays numbered image by image, pixel x + y*W within one).
 * Pixels outside the range are written as 0 and left out of the spectrum.
 * Lets a caller split one batch across processes or devices. */
int raptor_gpu_render_range(raptor_gpu_ctx *ctx, const raptor_image_desc *imgs, int n_imgs,
                            int precision, long long ray_begin, long long ray_count,
                            double *I_out, double *spectrum_out);

/* Number of doubles raptor_gpu_render writes to I_out / spectrum_out. */
long long raptor_gpu_output_size(const raptor_image_desc *imgs, int n_imgs);
long long raptor_gpu_spectrum_size(const raptor_image_desc *imgs, int n_imgs);

/* Statistics of the last render or VJP on this context (for a VJP: the
 * adjoint pass's counters, with n_stepcap and n_nonfinite of the image it
 * returns; kernel_ms is the adjoint pass, device_ms all of the call's
 * device work: the adjoint pass in one pass, forward plus adjoint in two). */
int raptor_gpu_get_stats(const raptor_gpu_ctx *ctx, raptor_gpu_stats *out);

/* Per-step record of one ray, the engine's form of the reference's GEOD
 * switch (integrator.c:172-184,208-210,238-240, which writes x1,x2,x3 per
 * step to geod/geodesic_x_y.dat).  records[k*16 + c] after step k (k = 0 is
 * the initial photon): c = 0..7 photon_u, 8 d lambda, 9 tau of the first
 * frequency, 10 its intensity before the nu^3 scaling, 11 steps, 12 theta
 * turns, 13 event (0 no transfer, 1 sigma cut, 2 sampled, 3 escaped), 14 the
 * order-limit stop flag, 15 unused.  *n_records = records written. */
#define RAPTOR_TRACE_WIDTH 16
int raptor_gpu_trace_ray(raptor_gpu_ctx *ctx, const raptor_image_desc *img, int precision, int pixel,
                         int max_records, double *records, int *n_records);

/* Vector-Jacobian product of one image: given dL_dI [W*H][n_freq] (same
 * layout and nu^3 scaling as I_out), returns dL/d(M_UNIT, R_HIGH, R_LOW,
 * INCLINATION) and, if the pointers are set, the per-cell gradients on the
 * image's grid.  precision selects the form and its adjoint pass (FP64:
 * FP64 tangents and dual sample; mixed: the FP64 geodesic with FP32 tangents
 * and the FP32 dual sample; mixed-DF: the double-float geodesic with FP32
 * tangents and sample).  By default the adjoint runs in one pass, taking
 * each ray's I from its own sums and keeping the ray's per-cell terms on a
 * device tape until the ray ends (raptor_gpu_options.vjp_tape); I_out
 * (may be NULL) then receives the image that pass renders, equal to
 * raptor_gpu_render's to rounding (1e-11 of the largest pixel in FP64, 1e-5
 * with the FP32 transfers).  In two passes (vjp_tape = -1, the in-place FP64
 * adjoint, or a tape too small) the form's forward render runs first and
 * I_out receives it.
 * No counterpart in the reference, which has no derivatives. */
int raptor_gpu_vjp(raptor_gpu_ctx *ctx, const raptor_image_desc *img, int precision,
                   const double *dL_dI, double *I_out, raptor_grad *grad);

/* The same, restricted to the image's rays [ray_begin, ray_begin+ray_count)
 * (pixel x + y*W): the forward image holds those pixels only (0 elsewhere)
 * and the gradients are those rays' contributions.  Gradients are sums over
 * rays, so the gradients of disjoint ranges add up to raptor_gpu_vjp's; a
 * caller splitting one image across processes or devices sums them (scalars
 * and per-cell arrays alike).  No counterpart in the reference. */
int raptor_gpu_vjp_range(raptor_gpu_ctx *ctx, const raptor_image_desc *img, int precision,
                         long long ray_begin, long long ray_count, const double *dL_dI, double *I_out,
                         raptor_grad *grad);

/* ---- Render without allocating device memory ----
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc - an application that embeds the renderer and owns all device
 * memory through its own pool (a GRMHD code imaging its grid in place between
 * time steps under a fixed memory budget), or a latency-critical loop that
 * must not take the allocator's lock and implicit device synchronisation.
 *
 * Renders n_imgs (1..RAPTOR_NOALLOC_MAX_IMAGES) FP64 images of one grid, as
 * raptor_gpu_render does, without a context and without allocating:
 *   d_cells         device memory, the grid as float64 [n1][n2][8] (the eight
 *                   primitives of a cell contiguous, in HARM order)
 *   geom            the grid geometry (imgs[k].grid is ignored)
 *   d_I_out         device memory, raptor_gpu_output_size(imgs, n_imgs) doubles
 *   d_spectrum_out  device memory, raptor_gpu_spectrum_size doubles, or NULL
 *   stream          a cudaStream_t, or NULL for the default stream
 * The call synchronises `stream` and returns when the results are in device
 * memory, with raptor_gpu_render's statuses.  It makes `device` current while
 * it runs and gives the caller's current device back before it returns.  Its
 * scratch (ray queue, counters, descriptors: RAPTOR_NOALLOC_SCRATCH_BYTES) is
 * one fixed device array in the library that every GPU loading the library
 * keeps until exit.  The first call on each device (and the first after that
 * device's context was re-created, e.g. by cudaDeviceReset) looks up the
 * array's device address with cudaGetSymbolAddress.  Being synchronous, no
 * call may be made while a stream is being captured.  All calls share the array, which keeps
 * the last call's contents (each call clears its counters first): calls whose
 * GPU work overlaps race on it and must be serialised by the caller.  A batch
 * larger than RAPTOR_NOALLOC_MAX_IMAGES is rejected with
 * RAPTOR_ERR_NOALLOC_LIMIT; other bad arguments with RAPTOR_ERR_INVALID. */
#define RAPTOR_NOALLOC_MAX_IMAGES 16
#define RAPTOR_NOALLOC_SCRATCH_BYTES 20480
#define RAPTOR_ERR_NOALLOC_LIMIT (-6)
int raptor_gpu_render_noalloc(int device, const double *d_cells, const raptor_grid_geom *geom,
                              const raptor_image_desc *imgs, int n_imgs, double *d_I_out, double *d_spectrum_out,
                              void *stream);

#ifdef __cplusplus
}
#endif
#endif
