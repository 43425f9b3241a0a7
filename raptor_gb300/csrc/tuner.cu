// Launch-shape autotuner for the persistent ray kernel.
//
// The shape of the persistent launch - threads per block (at the resident
// blocks per SM that the kernel's registers allow) and how many geodesic
// steps a lane runs between queue refills ("steps per chunk") - trades
// warp granularity against lane idling at ray ends.  With options.autotune
// set, the first render of a batch
// signature (device, precision, frequency bucket, size class) times each
// candidate on a sample of that batch's rays - a contiguous range from its
// middle, about six rays per lane - and keeps the fastest.  Results live in
// the context and, if RAPTOR_TUNE_CACHE names a file, are appended there and
// read back by later contexts.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "engine_internal.h"
#include "ray_kernel.cuh"

using raptor::kCtrCount;
using raptor::TraceSpec;

namespace {

std::string signature(const raptor_gpu_ctx* ctx, const Batch& b, int form) {
    char k[384];
    const int size_class = (int)std::log2((double)std::max<long long>(b.total_rays, 1));
    const char* name = form == RAPTOR_PREC_MIXED_DF ? "mixed_df"
                       : form == RAPTOR_PREC_MIXED  ? "mixed"
                       : ctx->opt.no_sample_pool    ? "fp64_inplace"
                                                    : "fp64";
    snprintf(k, sizeof k, "%s|%s|nf%d|2^%d", ctx->device_name, name, b.max_nf, size_class);
    std::string s(k);
    for (char& c : s)
        if (c == ' ') c = '_';
    return s;
}

void load_file_cache(raptor_gpu_ctx* ctx) {
    const char* path = getenv("RAPTOR_TUNE_CACHE");
    if (!path || ctx->tune_file_loaded) return;
    ctx->tune_file_loaded = true;
    FILE* f = fopen(path, "r");
    if (!f) return;
    char key[384];
    LaunchShape ls;
    while (fscanf(f, "%383s %d %d %d", key, &ls.block, &ls.bps, &ls.refill) == 4) ctx->tuned[key] = ls;
    fclose(f);
}

void save_file_cache(const std::string& key, const LaunchShape& ls) {
    const char* path = getenv("RAPTOR_TUNE_CACHE");
    if (!path) return;
    FILE* f = fopen(path, "a");
    if (!f) return;
    fprintf(f, "%s %d %d %d\n", key.c_str(), ls.block, ls.bps, ls.refill);
    fclose(f);
}

}  // namespace

LaunchShape choose_shape(raptor_gpu_ctx* ctx, const Batch& b, int form, RayLaunchFn fn, const void* fnp) {
    LaunchShape base = default_shape(ctx, fnp, form);
    if (!ctx->opt.autotune) return base;
    load_file_cache(ctx);
    const std::string key = signature(ctx, b, form);
    auto it = ctx->tuned.find(key);
    if (it != ctx->tuned.end()) {
        LaunchShape ls = it->second;
        int occ = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fnp, ls.block, 0);
        ls.bps = std::max(1, std::min(ls.bps, occ));
        ls.grid = ctx->num_sms * ls.bps;
        return ls;
    }
    // Candidates run at full occupancy.  The timed sample has a few rays per
    // lane, where a smaller grid wins by balancing the tail; on whole batches
    // (~100 rays per lane) full occupancy is faster (64 images: 2 blocks of 128
    // per SM 3545 ms, 1 block 3630 ms), so only the block size and the refill
    // interval are tuned.
    std::vector<LaunchShape> cands;
    for (int block : {64, 128}) {
        int occ = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fnp, block, 0);
        occ = std::max(occ, 1);
        for (int refill : {1, 4, 8, 16}) {
            LaunchShape ls;
            ls.block = block;
            ls.bps = occ;
            ls.grid = ctx->num_sms * occ;
            ls.refill = refill;
            cands.push_back(ls);
        }
    }
    const long long lanes = (long long)ctx->num_sms * 3 * 128;
    const long long n = std::min<long long>(b.total_rays, 6 * lanes);
    const long long rb = (b.total_rays - n) / 2, re = rb + n;
    LaunchShape best = base;
    float best_ms = 1e30f;
    const TraceSpec none{-1, nullptr, 0};
    for (size_t k = 0; k <= cands.size(); ++k) {
        // k == 0 is a warm-up of the default shape
        const LaunchShape& ls = k == 0 ? base : cands[k - 1];
        cudaMemsetAsync(ctx->d_counters, 0, kCtrCount * sizeof(unsigned long long), ctx->stream);
        cudaEventRecord(ctx->ev0, ctx->stream);
        fn(ls, ctx->stream, ctx->d_imgs, b.n, rb, re, ctx->d_counters, ctx->d_out, none);
        cudaEventRecord(ctx->ev1, ctx->stream);
        if (cudaEventSynchronize(ctx->ev1) != cudaSuccess) {
            cudaGetLastError();
            return base;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        if (k > 0 && ms < best_ms) {
            best_ms = ms;
            best = ls;
        }
    }
    ctx->tuned[key] = best;
    save_file_cache(key, best);
    return best;
}
