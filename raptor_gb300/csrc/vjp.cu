// Vector-Jacobian product entry point (forward-mode tangent of the
// geodesic plus reverse accumulation of the transfer).
#include "engine_internal.h"

extern "C" int raptor_gpu_vjp(raptor_gpu_ctx* ctx, const raptor_image_desc* img, int precision, const double* dL_dI,
                              double* I_out, raptor_grad* grad) {
    (void)img; (void)precision; (void)dL_dI; (void)I_out; (void)grad;
    return ctx_fail(ctx, RAPTOR_ERR_INVALID, "raptor_gpu_vjp: not built yet");
}
