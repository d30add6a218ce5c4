// axg_defects.cu -- defect identification (defects_3d.f90).  Filled in below.
#include "axg_internal.h"

extern "C" {
int axg_classify_cells(axg_ctx *ctx, int, int64_t *) { return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "not built yet"); }
int axg_download_defect_flags(axg_ctx *ctx, int8_t *) { return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "not built yet"); }
int axg_string_winding(axg_ctx *ctx, int64_t *) { return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "not built yet"); }
int axg_id_defects(axg_ctx *ctx, int64_t, double, double *, double *, double *, int64_t *) {
  return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "not built yet");
}
int axg_download_defect_lists(axg_ctx *ctx, double *, int64_t, double *, int64_t) {
  return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "not built yet");
}
}
