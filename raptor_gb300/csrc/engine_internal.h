// Internal state shared by the engine's translation units (not part of the
// C ABI).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "image_desc.cuh"
#include "raptor_gpu.h"

// geodesic steps between lane refills of the persistent ray kernels when
// the caller sets none: 8 for the FP64 and mixed forms (1.3 % faster than
// every step on the 1024x1024 image), 16 for mixed-DF (2 % faster than 8)
constexpr int kDefaultRefill = 8;
constexpr int kDefaultRefillDF = 16;

struct LaunchShape {
    int block = 128;   // threads per block
    int bps = 1;       // resident blocks per SM
    int grid = 0;      // blocks in the persistent grid
    int refill = 1;    // steps between lane refills
};

using RayLaunchFn = void (*)(const LaunchShape&, cudaStream_t, const raptor::DevImage*, int, long long, long long,
                             unsigned long long*, double*, raptor::TraceSpec);

struct GridSlot {
    bool used = false;
    raptor_grid_geom geom{};
    double* c64 = nullptr;
    float* c32 = nullptr;
    double* staging = nullptr;
    long long cap_cells = 0;  // cells the buffers hold
};

struct Batch {
    int n = 0;
    long long total_rays = 0, out_len = 0;
    int spec_len = 0, max_nf = 1;
    size_t h2d_bytes = 0;
    std::vector<raptor::DevImage> host;
    std::vector<int> spec_img, spec_f;
};

struct raptor_gpu_ctx {
    raptor_gpu_options opt{};
    int device = 0;
    int num_sms = 0;
    char device_name[256] = {0};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evA = nullptr, evB = nullptr;  // ray kernel / whole render
    GridSlot grids[RAPTOR_MAX_GRIDS];
    raptor::DevImage* d_imgs = nullptr;
    size_t imgs_cap = 0;
    raptor::DevImage* h_imgs = nullptr;
    size_t h_imgs_cap = 0;
    double* d_out = nullptr;
    size_t out_cap = 0;
    double* d_spec = nullptr;
    size_t spec_cap = 0;
    int* d_spec_map = nullptr;
    size_t spec_map_cap = 0;
    unsigned long long* d_counters = nullptr;
    int* d_flag = nullptr;
    double* d_grad = nullptr;
    size_t grad_cap = 0;
    double* d_dldi = nullptr;
    size_t dldi_cap = 0;
    double* d_vjp_scratch = nullptr;  // the pooled FP64 adjoint's per-warp results (several frequencies)
    size_t vjp_scratch_cap = 0;
    void* d_vjp_tape = nullptr;  // the one-pass adjoint's per-lane records
    size_t vjp_tape_cap = 0;
    double* d_trace = nullptr;
    size_t trace_cap = 0;
    Batch batch;
    raptor_gpu_stats stats{};
    double last_upload_ms = 0.0;
    std::map<std::string, LaunchShape> tuned;  // autotuner cache, keyed by batch signature
    bool tune_file_loaded = false;
    long long device_bytes = 0, peak_device_bytes = 0;  // cudaMalloc'd by this context
    cudaGraphExec_t graph_exec = nullptr;       // captured render, replayed while graph_key repeats
    std::string graph_key;
    unsigned long long check_word = 0;  // the last render's check word (checked build)
    char err[512] = {0};
};

int ctx_fail(raptor_gpu_ctx* ctx, int code, const char* fmt, ...);
int ensure_buffer(raptor_gpu_ctx* ctx, void** ptr, size_t* cap, size_t bytes);
int build_dev_image(raptor_gpu_ctx* ctx, const raptor_image_desc& d, raptor::DevImage& im);
int prepare_batch(raptor_gpu_ctx* ctx, const raptor_image_desc* imgs, int n_imgs, Batch& b);
// form: RAPTOR_PREC_FP64, RAPTOR_PREC_MIXED or RAPTOR_PREC_MIXED_DF
// pool: the FP64 form's sample-pool kernel (ray_kernel_pool) instead of ray_kernel
RayLaunchFn pick_ray_kernel(int nf, int form, const void** fn, bool pool = true);
RayLaunchFn pick_ray_kernel_df(int nf, const void** fn);
LaunchShape default_shape(raptor_gpu_ctx* ctx, const void* fn, int form);
LaunchShape choose_shape(raptor_gpu_ctx* ctx, const Batch& b, int form, RayLaunchFn fn, const void* fnp);
int enqueue_render(raptor_gpu_ctx* ctx, const Batch& b, int form, long long rb, long long re,
                   const LaunchShape& ls, RayLaunchFn fn, bool timed, raptor::TraceSpec tr = {-1, nullptr, 0});
int collect_stats(raptor_gpu_ctx* ctx, bool timed);
// RAPTOR_ERR_DEVICE if the checked build recorded a failed check (check,
// the counters' check word) or the kernel retired other than `expected`
// rays, else RAPTOR_ERR_NONFINITE / RAPTOR_WARN_STEPCAP / RAPTOR_OK from the
// counts
int render_status(raptor_gpu_ctx* ctx, long long rays, long long expected, long long n_nonfinite,
                  long long n_stepcap, unsigned long long check);
