// The checked build (compiled with -DRAPTOR_CHECKED into
// libraptor_gpu_checked.so): device-side checks of the indices the kernels
// compute - the image and pixel of a ray taken from the queue, the grid
// cells of a transfer sample, the output offset a ray writes, and the
// slots, counts and links of the per-warp sample-pool rings.  A failed
// check records its code and the offending value in the batch's check word
// (the first failure wins), makes the access safe - clamped, skipped or the
// ray retired - and the host fails the call with RAPTOR_ERR_DEVICE, naming
// the check in last_error.  Nothing traps or asserts, so the context stays
// usable.  In the normal build every check compiles to nothing.
#pragma once
#include <cuda_runtime.h>

namespace raptor {

enum CheckCode : unsigned {
    kChkImage = 1,   // a ray's image index outside the batch
    kChkPixel = 2,   // a ray's pixel outside its image
    kChkCell = 3,    // a sample's cell block outside the grid
    kChkOutput = 4,  // an output offset past the batch's output
    kChkRing = 5,    // a pool ring holding more tickets than its slots
    kChkList = 6,    // a lane's ticket list: count out of range or a ticket it does not own
    kChkBatch = 7,   // a pool evaluation batch larger than a warp
};

#ifdef RAPTOR_CHECKED
constexpr bool kChecked = true;
#else
constexpr bool kChecked = false;
#endif

// ok, after recording a failure in *word when ok is false (checked build).
__device__ __forceinline__ bool chk(bool ok, unsigned long long* word, unsigned code, long long value) {
#ifdef RAPTOR_CHECKED
    if (!ok && word)
        atomicCAS(word, 0ull, ((unsigned long long)code << 56) | ((unsigned long long)value & 0x00ffffffffffffffull));
    return ok;
#else
    (void)word;
    (void)code;
    (void)value;
    return true;
#endif
}

// Host side: the text of a recorded check word.
inline const char* check_name(unsigned long long word) {
    switch ((unsigned)(word >> 56)) {
        case kChkImage: return "image index outside the batch";
        case kChkPixel: return "pixel outside its image";
        case kChkCell: return "sample cell outside the grid";
        case kChkOutput: return "output offset past the batch's output";
        case kChkRing: return "sample-pool ring over capacity";
        case kChkList: return "sample-pool ticket list inconsistent";
        case kChkBatch: return "sample-pool batch larger than a warp";
        default: return "unknown check";
    }
}

}  // namespace raptor
