// Entry points whose GPU implementations are not part of this build yet.  Each returns
// ASTRO_ERR_UNSUPPORTED with a message; none falls back to a CPU computation.
#include "astro_internal.h"

extern "C" int astro_convert_to_ltri(astro_ctx *ctx, double *) {
    return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "convert_to_ltri not available in this build");
}
extern "C" int astro_ldl_fact(astro_ctx *ctx, double *, int32_t, const int32_t *, int32_t) {
    return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "ldl_fact not available in this build");
}
extern "C" int astro_ldl_fact_resident(astro_ctx *ctx) {
    return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "ldl_fact_resident not available in this build");
}
extern "C" int astro_ldl_solve(astro_ctx *ctx, double *, const double *, const double *, int32_t, const int32_t *,
                               int32_t, double *) {
    return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "ldl_solve not available in this build");
}
extern "C" int astro_gmres(astro_ctx *ctx, double *, const double *, const int32_t *, const int32_t *, int32_t, int32_t,
                           const double *, const int32_t *, const int32_t *, int32_t, int32_t, const double *,
                           const int32_t *, int32_t, const double *, int32_t, int32_t) {
    return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "gmres not available in this build");
}
extern "C" int astro_drdd_complex(astro_ctx *ctx, int32_t, double, const astro_state *, double *, double *) {
    return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "complex-step sensitivities not available in this build");
}
