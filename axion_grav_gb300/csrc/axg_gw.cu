// axg_gw.cu -- gravitational waves (grav_waves.f90).  Filled in below.
#include "axg_internal.h"

int axg_gw_init(axg_ctx *ctx) { return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "GW green not built yet"); }
int axg_gw_integration(axg_ctx *ctx, double, double) {
  return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "GW green not built yet");
}
extern "C" {
int axg_grav_spec_estimation(axg_ctx *ctx, double, double *, double *, double *, double *) {
  return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "not built yet");
}
int axg_grav_spec_log(axg_ctx *ctx, double, double *, double *, double *, double *) {
  return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "not built yet");
}
}
