// PHR refinement on the device (pkg/pt/phr.go).  Filled in below.
#include "gbt_internal.cuh"

int gbt_phr_run(gbt_ctx *ctx, gbt_bvh *aux, double alpha, double delta, int bf, gbt_bvh *out) {
    (void)aux; (void)alpha; (void)delta; (void)bf; (void)out;
    return gbt_fail(ctx, GBT_EUNSUPPORTED, "phr_build: not built yet");
}
