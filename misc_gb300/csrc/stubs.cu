// Entry points whose GPU implementations are not part of this build yet.  Each returns
// ASTRO_ERR_UNSUPPORTED with a message; none falls back to a CPU computation.
#include "astro_internal.h"

extern "C" int astro_drdd_complex(astro_ctx *ctx, int32_t, double, const astro_state *, double *, double *) {
    return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "complex-step sensitivities not available in this build");
}
