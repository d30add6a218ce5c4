// axg_ensemble.cu -- batched ensembles of lattices of uneven sizes.
//
// An ensemble owns M member contexts (each a full axg_ctx: IC, defects,
// spectra and transfers go through the member handle) on one shared stream.
// The leapfrog of all members runs as one launch per step (k_fused_batch in
// axg_evolve.cu): work items are (member, column, z-chunk),
// coefficients come from a device table, and the whole step sequence of an
// interval -- coefficient upload, first half drifts, nsteps batched steps --
// is captured once into a CUDA graph and replayed for later intervals with
// the same shape.  The tile shape is shared by all members; it and the
// launch mode (resident CTAs walking the items, or one CTA per item) are
// chosen by axg_ensemble_autotune.
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "axg_internal.h"

struct axg_ensemble {
  std::vector<axg_ctx *> m;
  cudaStream_t stream = nullptr;
  axg_ens_member_dev *d_mem = nullptr;
  std::vector<axg_ens_member_dev> h_mem;
  axg_ens_coef *d_coef = nullptr;
  axg_ens_coef *h_coef = nullptr;  // pinned (graph memcpy source)
  int64_t coef_cap = 0;
  int *d_err = nullptr;
  long long total_items = 0;
  int cfg = -1;
  bool persistent = false;
  int cur = 0;
  bool fp32 = true, uij = false;
  double dspa = 1.0;
  std::map<std::tuple<int64_t, int, int, int, uint64_t>, cudaGraphExec_t> graphs;
  int64_t launches = 0;
  std::string err;
};

namespace {

int ens_error(axg_ensemble *e, int code, const std::string &msg) {
  if (e) e->err = msg;
  return code;
}

bool tile_ok_all(axg_ensemble *e, int cfg) {
  for (auto *c : e->m)
    if (!axg_evo_tile_supported(c, cfg)) return false;
  return true;
}

void clear_graphs(axg_ensemble *e) {
  for (auto &kv : e->graphs) cudaGraphExecDestroy(kv.second);
  e->graphs.clear();
}

// (re)build the device descriptors for tile configuration cfg
int build_descriptors(axg_ensemble *e, int cfg) {
  const axg_tile_cfg t = axg_evo_tile(cfg);
  e->h_mem.assign(e->m.size(), axg_ens_member_dev{});
  long long items = 0;
  for (size_t i = 0; i < e->m.size(); ++i) {
    axg_ctx *c = e->m[i];
    int rc = axg_evo_build_tmaps(c, cfg);
    if (rc != AXG_OK) return ens_error(e, rc, "member " + std::to_string(i) + ": " + c->err);
    axg_ens_member_dev &d = e->h_mem[i];
    for (int b = 0; b < 2; ++b) {
      d.tm[b][0] = c->tm.phi_row[b];
      d.tm[b][1] = c->tm.phi_body[b];
      d.tm[b][2] = c->tm.phi_halo[b];
      d.tm[b][3] = c->tm.u_row[b];
      d.tm[b][4] = c->tm.u_body[b];
      d.tm[b][5] = c->tm.u_halo[b];
      for (int q = 0; q < 4; ++q) d.pw[q] = c->tm.pw[q];
      d.phi[b] = c->phi[b];
      d.u[b] = c->u[b];
    }
    d.phid = c->phid;
    d.cphi = c->cphi;
    d.ud = c->ud;
    d.cu = c->cu;
    d.n3 = c->n3;
    d.n = (int32_t)c->n;
    d.ncols = (int32_t)((c->n / t.tx) * (c->n / t.ty));
    d.item_begin = items;
    items += (long long)d.ncols * (c->n / t.zc);
  }
  e->total_items = items;
  if (cudaMemcpy(e->d_mem, e->h_mem.data(), sizeof(axg_ens_member_dev) * e->m.size(), cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return ens_error(e, AXG_ERR_CUDA, "descriptor upload");
  e->cfg = cfg;
  clear_graphs(e);
  return AXG_OK;
}

int ensure_coef(axg_ensemble *e, int64_t nsteps) {
  if (nsteps <= e->coef_cap) return AXG_OK;
  if (e->d_coef) cudaFree(e->d_coef);
  if (e->h_coef) cudaFreeHost(e->h_coef);
  e->d_coef = nullptr;
  e->h_coef = nullptr;
  e->coef_cap = 0;
  if (cudaMalloc(&e->d_coef, sizeof(axg_ens_coef) * nsteps) != cudaSuccess ||
      cudaMallocHost(&e->h_coef, sizeof(axg_ens_coef) * nsteps) != cudaSuccess) {
    cudaGetLastError();
    return ens_error(e, AXG_ERR_NOMEM, "coefficient table");
  }
  e->coef_cap = nsteps;
  clear_graphs(e);  // graphs reference the old table
  return AXG_OK;
}

// Enqueue one interval on the ensemble stream (plain launches, or inside a
// capture when `count` is false).
int enqueue_interval(axg_ensemble *e, double dt, int64_t nsteps, int first_half, int cur0, bool count = true) {
  if (cudaMemcpyAsync(e->d_coef, e->h_coef, sizeof(axg_ens_coef) * nsteps, cudaMemcpyHostToDevice, e->stream) !=
      cudaSuccess)
    return ens_error(e, AXG_ERR_CUDA, "coefficient upload");
  int cur = cur0;
  if (first_half) {
    for (size_t i = 0; i < e->m.size(); ++i) {
      axg_ctx *c = e->m[i];
      c->cur = cur;
      const bool kt = c->ktiming;
      c->ktiming = false;
      const int rc = axg_evo_drift(c, dt / 2);
      c->ktiming = kt;
      if (count) e->launches++;
      if (rc != AXG_OK) return ens_error(e, rc, c->err);
    }
  }
  for (int64_t s = 0; s < nsteps; ++s) {
    const int rc = axg_evo_batch_step(e->m[0], e->stream, e->d_mem, (int)e->m.size(), e->total_items, cur, e->d_coef,
                                      (int)s, e->cfg, e->d_err, e->fp32, e->uij, e->dspa, e->persistent);
    if (count) e->launches++;
    if (rc != AXG_OK) return ens_error(e, rc, e->m[0]->err);
    cur = 1 - cur;
  }
  return AXG_OK;
}

int check_error(axg_ensemble *e) {
  int h = 0;
  if (cudaMemcpyAsync(&h, e->d_err, sizeof(int), cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
      cudaStreamSynchronize(e->stream) != cudaSuccess)
    return ens_error(e, AXG_ERR_CUDA, "synchronize");
  if (h != 0) {
    cudaMemsetAsync(e->d_err, 0, sizeof(int), e->stream);
    return ens_error(e, AXG_ERR_TIMEOUT, "batched kernel reported error " + std::to_string(h));
  }
  return AXG_OK;
}

}  // namespace

extern "C" {

int axg_ensemble_create(const axg_params *members, int32_t count, axg_ensemble **out) {
  if (!members || count < 1 || !out) return AXG_ERR_ARG;
  *out = nullptr;
  axg_ensemble *e = new axg_ensemble();
  const axg_params &p0 = members[0];
  for (int i = 0; i < count; ++i) {
    const axg_params &p = members[i];
    if (p.precision == AXG_PREC_FP64_PLAIN || p.precision != p0.precision || p.gw_mode == AXG_GW_GREEN ||
        p.gw_mode != p0.gw_mode || p.dspa != p0.dspa || p.sigma_cr != p0.sigma_cr || p.potential != p0.potential ||
        p.kappa != p0.kappa || p.lambda != p0.lambda || p.vev != p0.vev || p.ma2_0 != p0.ma2_0 ||
        p.n_dw != p0.n_dw || p.device != p0.device || (p.flags & AXG_F_INITIAL_LOOP) != (p0.flags & AXG_F_INITIAL_LOOP)) {
      delete e;
      return axg_set_error(nullptr, AXG_ERR_ARG,
                           "ensemble members must share a fused precision, a non-Green gw_mode, dspa and the "
                           "potential (member " + std::to_string(i) + ")");
    }
  }
  e->fp32 = p0.precision == AXG_PREC_FP32_MIXED;
  e->uij = p0.gw_mode == AXG_GW_UIJ;
  e->dspa = p0.dspa;
  int rc = AXG_OK;
  cudaSetDevice(p0.device);
  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete e;
    return axg_set_error(nullptr, AXG_ERR_CUDA, "stream create");
  }
  for (int i = 0; i < count && rc == AXG_OK; ++i) {
    axg_ctx *c = nullptr;
    rc = axg_create(&members[i], &c);
    if (rc != AXG_OK) break;
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
    c->stream = e->stream;  // all members work on the ensemble stream
    e->m.push_back(c);
  }
  if (rc == AXG_OK) {
    if (cudaMalloc(&e->d_mem, sizeof(axg_ens_member_dev) * count) != cudaSuccess ||
        cudaMalloc(&e->d_err, 64) != cudaSuccess) {
      rc = axg_set_error(nullptr, AXG_ERR_NOMEM, "ensemble descriptors");
    } else {
      cudaMemset(e->d_err, 0, 64);
      int cfg = -1;
      for (int k = 0; k < axg_evo_tile_count() && cfg < 0; ++k) {
        const int c = axg_evo_tile_preference(e->fp32, k);
        if (tile_ok_all(e, c)) cfg = c;
      }
      if (cfg < 0) rc = axg_set_error(nullptr, AXG_ERR_UNSUPPORTED, "no fused tile fits every member");
      else if ((rc = build_descriptors(e, cfg)) != AXG_OK) axg_set_error(nullptr, rc, e->err);
    }
  }
  if (rc != AXG_OK) {
    axg_ensemble_destroy(e);
    return rc;
  }
  *out = e;
  return AXG_OK;
}

int axg_ensemble_destroy(axg_ensemble *e) {
  if (!e) return AXG_OK;
  if (e->stream) cudaStreamSynchronize(e->stream);
  clear_graphs(e);
  for (auto *c : e->m) {
    c->stream = nullptr;  // the shared stream is destroyed below
    axg_destroy(c);
  }
  if (e->d_mem) cudaFree(e->d_mem);
  if (e->d_coef) cudaFree(e->d_coef);
  if (e->h_coef) cudaFreeHost(e->h_coef);
  if (e->d_err) cudaFree(e->d_err);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return AXG_OK;
}

const char *axg_ensemble_last_error(const axg_ensemble *e) { return e ? e->err.c_str() : axg_last_error(nullptr); }

int axg_ensemble_size(const axg_ensemble *e, int32_t *count) {
  if (!e || !count) return AXG_ERR_ARG;
  *count = (int32_t)e->m.size();
  return AXG_OK;
}

int axg_ensemble_member(axg_ensemble *e, int32_t i, axg_ctx **member) {
  if (!e || !member || i < 0 || i >= (int32_t)e->m.size()) return AXG_ERR_ARG;
  *member = e->m[i];
  return AXG_OK;
}

int axg_ensemble_launch_count(const axg_ensemble *e, int64_t *launches) {
  if (!e || !launches) return AXG_ERR_ARG;
  *launches = e->launches;
  return AXG_OK;
}

int axg_ensemble_leapfrog(axg_ensemble *e, double t1, double dt, int64_t nsteps, int first_half, int last_half,
                          int use_graph) {
  if (!e || nsteps < 1 || !(dt > 0) || !(t1 > 0)) return AXG_ERR_ARG;
  for (auto *c : e->m)
    if (c->cur != e->cur) return ens_error(e, AXG_ERR_STATE, "members' buffers out of step");
  AXG_TRY(ensure_coef(e, nsteps));
  // kick times and coefficients in the step order of axg_leapfrog
  double t = t1;
  if (first_half) t = t + dt / 2;
  for (int64_t it = 1; it <= nsteps; ++it) {
    const double h = (it == nsteps && last_half) ? dt / 2 : dt;
    axg_ens_coef &k = e->h_coef[it - 1];
    axg_kick_coeffs(&e->m[0]->p, t, dt, k.f, k.pot);
    k.dtd = h;
    t = t + h;
  }
  const int cur0 = e->cur;
  uint64_t dtbits;
  std::memcpy(&dtbits, &dt, 8);
  const auto key = std::make_tuple(nsteps, first_half, last_half, cur0, dtbits);
  auto it = use_graph ? e->graphs.find(key) : e->graphs.end();
  if (use_graph && it != e->graphs.end()) {
    // replay: the graph's first node copies this call's coefficient table
    if (cudaGraphLaunch(it->second, e->stream) != cudaSuccess) return ens_error(e, AXG_ERR_CUDA, "graph launch");
    e->launches += nsteps + (first_half ? (int64_t)e->m.size() : 0);
  } else {
    // eager run (this also loads the kernels outside any capture) ...
    AXG_TRY(enqueue_interval(e, dt, nsteps, first_half, cur0));
    if (use_graph) {
      // ... then capture the same sequence once for later intervals of this shape
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return ens_error(e, AXG_ERR_CUDA, "begin capture");
      const int rc = enqueue_interval(e, dt, nsteps, first_half, cur0, false);
      const cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
      if (rc != AXG_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (ce != cudaSuccess) return ens_error(e, AXG_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(ce));
      cudaGraphExec_t ex = nullptr;
      const cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) return ens_error(e, AXG_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(ie));
      e->graphs.emplace(key, ex);
    }
  }
  AXG_TRY(check_error(e));
  e->cur = (int)((cur0 + nsteps) & 1);
  for (auto *c : e->m) {
    c->cur = e->cur;
    c->flags_valid = false;
  }
  return AXG_OK;
}

int axg_ensemble_set_tile(axg_ensemble *e, int cfg) {
  if (!e || cfg < 0 || cfg >= axg_evo_tile_count()) return AXG_ERR_ARG;
  if (!tile_ok_all(e, cfg)) return ens_error(e, AXG_ERR_UNSUPPORTED, "tile shape does not fit every member");
  return build_descriptors(e, cfg);
}

int axg_ensemble_set_launch_mode(axg_ensemble *e, int persistent) {
  if (!e) return AXG_ERR_ARG;
  if (e->persistent != (persistent != 0)) {
    e->persistent = persistent != 0;
    clear_graphs(e);  // captured launches carry the grid
  }
  return AXG_OK;
}

int axg_ensemble_launch_mode(const axg_ensemble *e, int *persistent) {
  if (!e || !persistent) return AXG_ERR_ARG;
  *persistent = e->persistent ? 1 : 0;
  return AXG_OK;
}

int axg_ensemble_autotune(axg_ensemble *e, int steps, int *best_cfg, double *best_ms) {
  if (!e || steps < 1) return AXG_ERR_ARG;
  // snapshot everything a step modifies
  struct Buf {
    void *src;
    size_t bytes;
    void *copy;
  };
  std::vector<Buf> bufs;
  for (auto *c : e->m) {
    const size_t rs = c->elem, n3 = (size_t)c->n3;
    bufs.push_back({c->phi[c->cur], n3 * 2 * rs, nullptr});
    bufs.push_back({c->phid, n3 * 2 * rs, nullptr});
    if (c->cphi) bufs.push_back({c->cphi, n3 * 2 * rs, nullptr});
    if (c->p.gw_mode == AXG_GW_UIJ) {
      bufs.push_back({c->u[c->cur], n3 * 6 * rs, nullptr});
      bufs.push_back({c->ud, n3 * 6 * rs, nullptr});
      if (c->cu) bufs.push_back({c->cu, n3 * 6 * rs, nullptr});
    }
  }
  int rc = AXG_OK;
  for (auto &b : bufs) {
    if (cudaMalloc(&b.copy, b.bytes) != cudaSuccess) {
      cudaGetLastError();
      rc = ens_error(e, AXG_ERR_NOMEM, "autotune snapshot");
      break;
    }
    cudaMemcpyAsync(b.copy, b.src, b.bytes, cudaMemcpyDeviceToDevice, e->stream);
  }
  const int cur0 = e->cur, cfg0 = e->cfg;
  const bool mode0 = e->persistent;
  int best = -1;
  bool best_mode = mode0;
  double bt = 1e300;
  cudaEvent_t a, z;
  cudaEventCreate(&a);
  cudaEventCreate(&z);
  for (int cfg = 0; rc == AXG_OK && cfg < axg_evo_tile_count(); ++cfg) {
    if (!tile_ok_all(e, cfg)) continue;
    if ((rc = build_descriptors(e, cfg)) != AXG_OK) break;
    for (int mode = 0; rc == AXG_OK && mode < 2; ++mode) {
      e->persistent = mode == 1;
      if ((rc = axg_ensemble_leapfrog(e, 10.0, 1e-3, 1, 0, 0, 0)) != AXG_OK) break;  // warm-up
      cudaEventRecord(a, e->stream);
      rc = axg_ensemble_leapfrog(e, 10.0, 1e-3, steps, 0, 0, 0);
      cudaEventRecord(z, e->stream);
      cudaEventSynchronize(z);
      float ms = 0;
      cudaEventElapsedTime(&ms, a, z);
      if (rc == AXG_OK && ms / steps < bt) {
        bt = ms / steps;
        best = cfg;
        best_mode = e->persistent;
      }
      e->cur = cur0;
      for (auto *c : e->m) c->cur = cur0;
      for (auto &b : bufs) cudaMemcpyAsync(b.src, b.copy, b.bytes, cudaMemcpyDeviceToDevice, e->stream);
    }
  }
  cudaStreamSynchronize(e->stream);
  cudaEventDestroy(a);
  cudaEventDestroy(z);
  for (auto &b : bufs)
    if (b.copy) cudaFree(b.copy);
  const int chosen = (rc == AXG_OK && best >= 0) ? best : cfg0;
  e->persistent = (rc == AXG_OK && best >= 0) ? best_mode : mode0;
  const int rc2 = build_descriptors(e, chosen);
  if (rc != AXG_OK) return rc;
  AXG_TRY(rc2);
  if (best_cfg) *best_cfg = best;
  if (best_ms) *best_ms = bt;
  return AXG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Ensemble outputs: per-realisation results of the members' own calls,
// averaged bin by bin / component by component on the host.
// ---------------------------------------------------------------------------
namespace {
// mean and standard error of the mean of v[0..n), n >= 1
void mean_sem(const std::vector<double> &v, double *mean, double *sem) {
  double s = 0.0;
  for (double x : v) s += x;
  const double m = s / (double)v.size();
  double q = 0.0;
  for (double x : v) q += (x - m) * (x - m);
  *mean = m;
  *sem = v.size() > 1 ? std::sqrt(q / (double)(v.size() - 1) / (double)v.size()) : 0.0;
}
}  // namespace

extern "C" {

int axg_ensemble_grav_spec_mean(axg_ensemble *e, double tau, double *wave, double *power_mean, double *power_sem,
                                double *denom) {
  if (!e || !power_mean) return AXG_ERR_ARG;
  if (!e->uij) return ens_error(e, AXG_ERR_STATE, "ensemble GW spectrum: members run gw_mode NONE");
  const int nb = e->m[0]->p.num_bin_grav;
  for (auto *c : e->m)
    if (c->p.num_bin_grav != nb) return ens_error(e, AXG_ERR_ARG, "members differ in num_bin_grav");
  std::vector<std::vector<double>> per(nb);
  std::vector<double> w(nb), pw(nb), nu(nb), de(nb), dsum(nb, 0.0);
  for (auto *c : e->m) {
    const int rc = axg_grav_spec_estimation(c, tau, w.data(), pw.data(), nu.data(), de.data());
    if (rc != AXG_OK) return ens_error(e, rc, std::string("member spectrum: ") + c->err);
    for (int k = 0; k < nb; ++k) {
      dsum[k] += de[k];
      if (de[k] > 0) per[k].push_back(pw[k]);
    }
  }
  for (int k = 0; k < nb; ++k) {
    double m = 0.0, s = 0.0;
    if (!per[k].empty()) mean_sem(per[k], &m, &s);
    power_mean[k] = m;
    if (power_sem) power_sem[k] = s;
    if (denom) denom[k] = dsum[k];
    if (wave) wave[k] = w[k];  // the members share dspa, so the linear bins coincide
  }
  return AXG_OK;
}

int axg_ensemble_defect_mean(axg_ensemble *e, int64_t idx, double tau, double xi_mean[3], double xi_sem[3],
                             double area_mean[3], double area_sem[3]) {
  if (!e || !xi_mean || !(tau > 0)) return AXG_ERR_ARG;
  std::vector<std::vector<double>> xi(3), ar(3);
  for (auto *c : e->m) {
    double sl[3], wa[3], sv[3];
    int64_t counts[3];
    const int rc = axg_id_defects(c, idx, tau, sl, wa, sv, counts);
    if (rc != AXG_OK) return ens_error(e, rc, std::string("member id_defects: ") + c->err);
    // defects_and_spectrum (evolve.f90:191-192): xi = (tau/dx)^2 sl / N^3 / 4, A = (tau/dx) wa / N^3 / 2
    const double h = tau / c->p.dspa, n3 = (double)c->n3;
    for (int k = 0; k < 3; ++k) {
      xi[k].push_back(h * h * sl[k] / n3 / 4);
      ar[k].push_back(h * wa[k] / n3 / 2);
    }
  }
  for (int k = 0; k < 3; ++k) {
    double m, s;
    mean_sem(xi[k], &m, &s);
    xi_mean[k] = m;
    if (xi_sem) xi_sem[k] = s;
    mean_sem(ar[k], &m, &s);
    if (area_mean) area_mean[k] = m;
    if (area_sem) area_sem[k] = s;
  }
  return AXG_OK;
}

}  // extern "C"
