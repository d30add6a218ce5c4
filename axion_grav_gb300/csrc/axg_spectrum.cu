// axg_spectrum.cu -- field spectrum (spectrum.f90).  Filled in below.
#include "axg_internal.h"

extern "C" {
int axg_spectrum_estimation(axg_ctx *ctx, double, double *, double *, double *, double *) {
  return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "not built yet");
}
int axg_compute_crho(axg_ctx *ctx, double *) { return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "not built yet"); }
}
