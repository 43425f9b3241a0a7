// Pieces shared by the two adjoint kernels (vjp.cu: FP64; vjp_df.cu:
// mixed-DF): the inclination dual, the tangent directions of the mixed-DF
// adjoint's six-direction sample, and the launch interface.
#pragma once
#include "dual.cuh"
#include "ray_kernel.cuh"

namespace raptor {

using D1 = Dual<1>;
// tangent directions of the mixed-DF adjoint's sample: 0 inclination, 1 rho_s,
// 2 ln Theta_e (u_s), 3 ln M_unit, 4 R_high, 5 R_low
constexpr int kDirIncl = 0, kDirRho = 1, kDirU = 2, kDirLnM = 3, kDirRh = 4, kDirRl = 5;
// the four scalar parameters' directions: 0 -> incl, 1 -> ln M, 2 -> R_high, 3 -> R_low
__host__ __device__ __forceinline__ int gdir(int q) { return q == 0 ? kDirIncl : q + 2; }

constexpr int kVjpBlock = 128;
constexpr int kVjpRefill = 8;  // geodesic steps between lane refills of the mixed-DF adjoint

// Launch of the adjoint pass: grid blocks of kVjpBlock threads on stream st
// for image im (device pointer), camera constants with their inclination
// tangent, the forward image fwd and dL/dI dl (device, image layout);
// accumulates into counters, gscal[4] and the per-cell arrays (which may be
// null); lanes take new rays every refill steps; scratch is the sample
// pool's result buffer where the kernel has one.
using VjpLaunchFn = void (*)(int grid, cudaStream_t st, const DevImage* im, const CamT<D1>& cam, const double* fwd,
                             const double* dl, unsigned long long* counters, double* gscal, double* g_rho,
                             double* g_u, double* g_th, int refill, double* scratch);
// the mixed-DF adjoint for nf frequencies (vjp_df.cu); *fn gets the kernel
VjpLaunchFn pick_vjp_df(int nf, const void** fn);

}  // namespace raptor
