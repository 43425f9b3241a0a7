// Measurement helpers for bench.py (not part of the engine's C ABI):
// FP64 and FP32 FMA throughput probes (the roofline denominators of the
// FP64-pipe-bound ray kernel and of the FP32-issue-bound mixed-DF kernel)
// and an L2 flush between timed renders.
#include <cuda_runtime.h>

#include <cstdio>

namespace {

constexpr int kChains = 8;

// kChains independent DFMA chains per thread; values stay near 1 so no
// overflow or denormal slows the pipe.
__global__ void dfma_probe(double* out, int iters, double b, double c) {
    double x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) x[k] = fma(x[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += x[k];
    if (s == 12345.678) out[0] = s;  // keeps the chains live
}

// The same with FP32 FFMA chains: 16 independent chains per thread cover the
// FP32 pipe's latency at 8 warps per scheduler.
constexpr int kChainsF = 16;
__global__ void ffma_probe(float* out, int iters, float b, float c) {
    float x[kChainsF];
#pragma unroll
    for (int k = 0; k < kChainsF; ++k) x[k] = 1.0f + 1e-3f * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChainsF; ++k) x[k] = fmaf(x[k], b, c);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kChainsF; ++k) s += x[k];
    if (s == 12345.678f) out[0] = s;  // keeps the chains live
}

__global__ void flush_kernel(int4* buf, long long n, int v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        buf[i] = make_int4(v, v, v, v);
}

int4* g_flush = nullptr;
long long g_flush_n = 0;

}  // namespace

// Measured DFMA throughput in TFLOP/s (2 FLOP per FMA), best of `reps`.
extern "C" int raptor_bench_fp64_peak(int device, int reps, double* tflops) {
    if (cudaSetDevice(device) != cudaSuccess) return -1;
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, device);
    double* out = nullptr;
    cudaMalloc(&out, sizeof(double));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int block = 256, blocks = p.multiProcessorCount * 8, iters = 4096;
    dfma_probe<<<blocks, block>>>(out, 64, 0.9999999, 1e-7);
    double best = 0.0;
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(a);
        dfma_probe<<<blocks, block>>>(out, iters, 0.9999999, 1e-7);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        const double flop = 2.0 * kChains * (double)iters * block * (double)blocks;
        if (ms > 0) best = fmax(best, flop / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    *tflops = best;
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

// Measured FFMA throughput in FP32 thread-instructions per second (1e12),
// best of `reps` (2 FLOP per FFMA: TFLOP/s is twice this).
extern "C" int raptor_bench_fp32_peak(int device, int reps, double* tinst) {
    if (cudaSetDevice(device) != cudaSuccess) return -1;
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, device);
    float* out = nullptr;
    cudaMalloc(&out, sizeof(float));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int block = 256, blocks = p.multiProcessorCount * 8, iters = 16384;
    ffma_probe<<<blocks, block>>>(out, 64, 0.9999999f, 1e-7f);
    double best = 0.0;
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(a);
        ffma_probe<<<blocks, block>>>(out, iters, 0.9999999f, 1e-7f);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        const double inst = (double)kChainsF * (double)iters * block * (double)blocks;
        if (ms > 0) best = fmax(best, inst / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    *tinst = best;
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

// Overwrite `bytes` of device memory (more than L2) and wait for it.
extern "C" int raptor_bench_flush_l2(int device, long long bytes) {
    if (cudaSetDevice(device) != cudaSuccess) return -1;
    const long long n = bytes / (long long)sizeof(int4);
    if (n > g_flush_n) {
        cudaFree(g_flush);
        g_flush = nullptr;
        if (cudaMalloc(&g_flush, n * sizeof(int4)) != cudaSuccess) return -2;
        g_flush_n = n;
    }
    static int v = 0;
    flush_kernel<<<1024, 256>>>(g_flush, n, ++v);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -3;
}
