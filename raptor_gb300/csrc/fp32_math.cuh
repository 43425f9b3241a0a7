// FP32 quotient and square root for the FP32 transfer samples (the mixed
// and mixed-DF forms and their adjoints).
//
// CUDA's IEEE-rounded FP32 division and square root carry a branch to an
// out-of-line slow path at every use.  The samples run between geodesic
// steps whose loop already fills the instruction cache; with some twenty
// such operations the mixed-DF kernel's sample was 6 % of its instructions
// and 30 % of its time.  The PTX instructions div.full.f32 and
// sqrt.approx.f32 have no slow path: with them the 1024x1024 mixed-DF render
// went from 79.5 to 69 ms.  On the GPU they are within 2 ulp of the IEEE
// quotient (subnormal results included) and 1 ulp of the IEEE square root,
// with IEEE's special values (tests/test_gpu_math.py): a few ulp in a
// transfer whose tolerance is 1e-4 in flux.
//
// Templated code (the sample's fluid, shared with FP32 duals) calls fdiv and
// fsqrt; for other types they are the type's own division and sqrt.
#pragma once
#include <cuda_runtime.h>

namespace raptor {

__device__ __forceinline__ float fdiv(float a, float b) {
    float q;
    asm("div.full.f32 %0, %1, %2;" : "=f"(q) : "f"(a), "f"(b));
    return q;
}
__device__ __forceinline__ float fsqrt(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

template <class T>
__device__ __forceinline__ T fdiv(const T& a, const T& b) {
    return a / b;
}
template <class T>
__device__ __forceinline__ T fsqrt(const T& x) {
    return sqrt(x);
}

}  // namespace raptor
