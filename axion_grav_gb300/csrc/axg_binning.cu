// axg_binning.cu -- host-built |k|^2 -> shell-bin tables (see axg_binning.h).
#include <cmath>
#include <vector>

#include "axg_binning.h"

namespace {

// the device expressions of the GW and spectrum bins, evaluated on the host
// with the same IEEE operations (no contraction)
int gw_bin(double q, double dq, int nb, int logmode, const double *edges) {
  if (!(q > 0.0)) return -1;
  if (!logmode) {
    const double id = std::round(q / dq + 0.5);
    return (id >= 1 && id <= nb) ? (int)id - 1 : -1;
  }
  if (q < edges[0] || q > edges[nb]) return -1;
  // the unique b with edges[b] <= q < edges[b + 1] (top edge inclusive)
  int lo = 0, hi = nb - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (q >= edges[mid]) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

int spectrum_bin(double q, double dq, int nb) {
  const double id = std::round(q / dq + 0.5);
  return (id >= 1 && id <= nb) ? (int)id - 1 : -1;
}

}  // namespace

int axg_bin_table(axg_ctx *ctx, int kind, int m, double dwav, double dq, int nb, int logmode, const double *edges,
                  const int16_t **d_tab) {
  if (nb < 1 || nb > 32767) return axg_set_error(ctx, AXG_ERR_ARG, "bin count out of range");
  auto &c = ctx->bin_cache;
  const int slot = kind == AXG_BIN_GW ? (logmode ? 1 : 0) : 2;
  auto &e = c[slot];
  std::vector<double> ev;
  if (logmode) ev.assign(edges, edges + nb + 1);
  if (e.tab && e.m == m && e.dwav == dwav && e.dq == dq && e.nb == nb && e.edges == ev) {
    *d_tab = e.tab;
    return AXG_OK;
  }
  const int64_t h = m / 2, top = 3 * h * h;
  std::vector<int16_t> t((size_t)top + 1);
  for (int64_t k2 = 0; k2 <= top; ++k2) {
    const double q = std::sqrt((double)k2) * dwav;
    t[(size_t)k2] = (int16_t)(kind == AXG_BIN_GW ? gw_bin(q, dq, nb, logmode, edges) : spectrum_bin(q, dq, nb));
  }
  if (e.tab && e.cap < (size_t)(top + 1)) axg_free(ctx, (void **)&e.tab);
  if (!e.tab) {
    AXG_TRY(axg_alloc(ctx, (void **)&e.tab, sizeof(int16_t) * (size_t)(top + 1), "bin table"));
    e.cap = (size_t)(top + 1);
  }
  AXG_CUDA_TRY(ctx, cudaMemcpyAsync(e.tab, t.data(), sizeof(int16_t) * t.size(), cudaMemcpyHostToDevice, ctx->stream));
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  e.m = m;
  e.dwav = dwav;
  e.dq = dq;
  e.nb = nb;
  e.edges = ev;
  *d_tab = e.tab;
  return AXG_OK;
}
