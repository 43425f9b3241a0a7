// raptor_gpu_render_noalloc: the batched FP64 render for callers that
// cannot allocate device memory.
//
// Who needs it: a host application that embeds the renderer inside its own
// GPU program and owns every byte of device memory through its own pool
// (for example a GRMHD code that images its grid in place between time
// steps, with a fixed memory budget), or a time-critical loop that must not
// call cudaMalloc/cudaFree, because they take the driver's allocation lock
// and synchronise the device.  Such a caller already holds the grid and the
// output buffers in device memory; this entry point uses them as they are
// and keeps its own small scratch (the ray-queue and statistics counters,
// the image descriptors and the spectrum map) in a fixed file-scope device
// array instead of allocating it.
//
// The scratch array is part of the loaded module: every GPU that loads this
// library holds RAPTOR_NOALLOC_SCRATCH_BYTES of it until the process exits.
// All calls share it, so two calls whose work overlaps on the GPU (on
// different streams, or from different host threads) race on it and must
// be serialised by the caller.
#include <cuda.h>  // CUcontext and CUresult only: the driver is reached through cudart
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "engine_internal.h"
#include "ray_kernel.cuh"

using namespace raptor;

namespace {

constexpr size_t kCountersBytes = 256;  // kCtrCount 64-bit counters, padded
constexpr size_t kDescBytes = sizeof(DevImage) * RAPTOR_NOALLOC_MAX_IMAGES;
constexpr size_t kMapBytes = sizeof(int) * 2 * RAPTOR_NOALLOC_MAX_IMAGES * RAPTOR_MAX_FREQS;
static_assert(kCountersBytes >= kCtrCount * sizeof(unsigned long long), "counters do not fit");
static_assert(kCountersBytes + kDescBytes + kMapBytes <= RAPTOR_NOALLOC_SCRATCH_BYTES,
              "no-alloc scratch too small for its stated limits");

// The scratch.  In host code this name is only a host-side handle: the
// device address comes from cudaGetSymbolAddress, taken once per device
// context (below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[RAPTOR_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;

// The symbol's device address, looked up once per device and again whenever
// that device's context is a different one (the primary context was reset
// and re-created, which reloads the module and may move the array).  The
// context is told apart by its process-unique id, read through the driver
// entry points cudart exposes, so the library needs no link to the driver.
struct ScratchSlot {
    unsigned long long ctx_id = 0;
    unsigned char* addr = nullptr;
};
std::mutex g_setup_mu;
ScratchSlot g_scratch[kMaxDevices];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// The current context's id, or 0 if it cannot be read.
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {  // under g_setup_mu
        looked_up = true;
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
            get_id = reinterpret_cast<CtxGetIdFn>(f2);
        }
        cudaGetLastError();
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (get_current && get_id && get_current(&c) == CUDA_SUCCESS && c && get_id(c, &id) == CUDA_SUCCESS) return id;
    return 0;
}

// Device address of the scratch on `device`, which must be current: the
// set-up on the first call on a device (and on the first call after its
// context was re-created), a cached pointer on every other call.  Where
// the context id cannot be read, the address is looked up on every call.
cudaError_t scratch_address(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    const unsigned long long id = current_context_id();
    ScratchSlot& s = g_scratch[device];
    if (id == 0 || s.ctx_id != id || !s.addr) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        s.addr = static_cast<unsigned char*>(p);
        s.ctx_id = id;
    }
    *out = s.addr;
    return cudaSuccess;
}

// Makes `device` current for the call and gives the caller's current device
// back on every return path.
struct DeviceGuard {
    int saved = -1;
    bool ok = false;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&saved) != cudaSuccess) saved = -1;
        ok = cudaSetDevice(device) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (saved >= 0) cudaSetDevice(saved);
    }
};

}  // namespace

extern "C" int raptor_gpu_render_noalloc(int device, const double* d_cells, const raptor_grid_geom* geom,
                                         const raptor_image_desc* imgs, int n_imgs, double* d_I_out,
                                         double* d_spectrum_out, void* stream) {
    if (!d_cells || !geom || !imgs || !d_I_out || n_imgs < 1) return RAPTOR_ERR_INVALID;
    if (n_imgs > RAPTOR_NOALLOC_MAX_IMAGES) return RAPTOR_ERR_NOALLOC_LIMIT;
    if (device < 0 || device >= kMaxDevices) return RAPTOR_ERR_INVALID;
    DeviceGuard guard(device);
    if (!guard.ok) {
        cudaGetLastError();
        return RAPTOR_ERR_NODEVICE;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // Per-image constants, built on the host exactly as raptor_gpu_render
    // builds them, in a stack-only context that points at the caller's grid.
    static thread_local raptor_gpu_ctx shim;  // holds no device memory
    shim.grids[0].used = true;
    shim.grids[0].geom = *geom;
    shim.grids[0].c64 = const_cast<double*>(d_cells);
    shim.grids[0].c32 = nullptr;
    DevImage h_desc[RAPTOR_NOALLOC_MAX_IMAGES];
    int h_map[2 * RAPTOR_NOALLOC_MAX_IMAGES * RAPTOR_MAX_FREQS];
    long long rays = 0, outlen = 0;
    int nspec = 0, max_nf = 1;
    for (int k = 0; k < n_imgs; ++k) {
        raptor_image_desc d = imgs[k];
        d.grid = 0;
        if (build_dev_image(&shim, d, h_desc[k]) != RAPTOR_OK) return RAPTOR_ERR_INVALID;
        h_desc[k].ray_begin = rays;
        h_desc[k].out_offset = outlen;
        rays += (long long)d.width * d.height;
        outlen += (long long)d.width * d.height * d.n_freq;
        for (int f = 0; f < d.n_freq; ++f) h_map[nspec++] = k;
        max_nf = d.n_freq > max_nf ? d.n_freq : max_nf;
    }
    for (int s = 0, k = 0; k < n_imgs; ++k)
        for (int f = 0; f < imgs[k].n_freq; ++f) h_map[nspec + s++] = f;

    unsigned char* scratch = nullptr;
    if (scratch_address(device, &scratch) != cudaSuccess) {
        cudaGetLastError();
        return RAPTOR_ERR_CUDA;
    }
    unsigned long long* d_ctr = reinterpret_cast<unsigned long long*>(scratch);
    DevImage* d_desc = reinterpret_cast<DevImage*>(scratch + kCountersBytes);
    int* d_map = reinterpret_cast<int*>(scratch + kCountersBytes + kDescBytes);
    for (int k = 0; k < n_imgs; ++k) {
        h_desc[k].out_end = outlen;
        h_desc[k].check_word = d_ctr + kCtrCheck;
    }

    // the counters (ray queue first) must start at zero on every call
    if (cudaMemsetAsync(d_ctr, 0, kCountersBytes, st) != cudaSuccess ||
        cudaMemcpyAsync(d_desc, h_desc, sizeof(DevImage) * n_imgs, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(d_map, h_map, sizeof(int) * 2 * nspec, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return RAPTOR_ERR_CUDA;
    // the camera's point quantities, which the ray kernel reads from each image
    camera_point_kernel<<<(n_imgs + 127) / 128, 128, 0, st>>>(d_desc, n_imgs);
    if (cudaGetLastError() != cudaSuccess) return RAPTOR_ERR_CUDA;

    // the FP64 form's default kernel and launch shape, as raptor_gpu_render
    // picks them without tuning
    const void* fnp = nullptr;
    RayLaunchFn fn = pick_ray_kernel(max_nf, RAPTOR_PREC_FP64, &fnp);
    int occ = 1, sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fnp, kRayMaxBlock, 0) != cudaSuccess)
        return RAPTOR_ERR_CUDA;
    LaunchShape ls;
    ls.block = kRayMaxBlock;
    ls.bps = occ > 0 ? occ : 1;
    ls.grid = sms * ls.bps;
    ls.refill = kDefaultRefill;
    fn(ls, st, d_desc, n_imgs, 0, rays, d_ctr, d_I_out, TraceSpec{-1, nullptr, 0});
    if (cudaGetLastError() != cudaSuccess) return RAPTOR_ERR_CUDA;
    if (d_spectrum_out) {
        spectrum_kernel<<<nspec, 256, 0, st>>>(d_desc, d_map, d_map + nspec, d_I_out, d_spectrum_out);
        if (cudaGetLastError() != cudaSuccess) return RAPTOR_ERR_CUDA;
    }
    unsigned long long ctr[kCtrCount];
    if (cudaMemcpyAsync(ctr, d_ctr, sizeof ctr, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return RAPTOR_ERR_CUDA;
    return render_status(nullptr, (long long)ctr[kCtrRays], rays, (long long)ctr[kCtrNonFinite],
                         (long long)ctr[kCtrStepCap], ctr[kCtrCheck]);
}
