// Launch-shape selection for the persistent ray kernel.
#include "engine_internal.h"

LaunchShape choose_shape(raptor_gpu_ctx* ctx, const Batch& b, bool mixed, RayLaunchFn fn, const void* fnp) {
    (void)b;
    (void)mixed;
    (void)fn;
    return default_shape(ctx, fnp);
}
