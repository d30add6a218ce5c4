// axg_capi.cu -- C-ABI entry points of libaxgpu (declared in include/axgpu.h).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <vector>

#include "axg_internal.h"

namespace {
std::string g_create_error;

// potential.f90:8, 26-30
constexpr double kRefPi = 3.14159265359;
constexpr double kRefTwoPi = 2 * kRefPi;
constexpr double kThrmSigma = 2.449489742783178;
constexpr double kNAxion = 6.68, kCTAxion = 6.26, kC0Axion = 1.0;

double msquared(double thrm) { return (thrm * thrm - kThrmSigma * kThrmSigma) / 3; }

double maxion2(double thrm, double kappa) {
  double thrm12 = kappa * std::pow(kCTAxion / kC0Axion, 1.0 / kNAxion);
  double m = thrm > thrm12 ? kCTAxion * std::pow(kappa / thrm, kNAxion) : kC0Axion;
  double k2 = kappa * kappa;
  return m * (k2 * k2);
}

// ---- conversion kernels between complex128 staging and the field storage ----
__global__ void k_c128_to_f32(const double2 *__restrict__ src, float2 *__restrict__ dst,
                              float2 *__restrict__ comp, int64_t count) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const double2 v = src[i];
    const float2 f = make_float2((float)v.x, (float)v.y);
    dst[i] = f;
    // Kahan compensation carries the rounding of the upload: c = f - v
    if (comp) comp[i] = make_float2((float)((double)f.x - v.x), (float)((double)f.y - v.y));
  }
}
__global__ void k_f32_to_c128(const float2 *__restrict__ src, const float2 *__restrict__ comp,
                              double2 *__restrict__ dst, int64_t count) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const float2 v = src[i];
    double2 o = make_double2((double)v.x, (double)v.y);
    if (comp) {
      const float2 c = comp[i];
      o.x -= (double)c.x;
      o.y -= (double)c.y;
    }
    dst[i] = o;
  }
}
__global__ void k_r64_to_f32(const double *__restrict__ src, float *__restrict__ dst,
                             float *__restrict__ comp, int64_t count) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const double v = src[i];
    const float f = (float)v;
    dst[i] = f;
    if (comp) comp[i] = (float)((double)f - v);
  }
}
__global__ void k_f32_to_r64(const float *__restrict__ src, const float *__restrict__ comp,
                             double *__restrict__ dst, int64_t count) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    double o = (double)src[i];
    if (comp) o -= (double)comp[i];
    dst[i] = o;
  }
}

int grid_for(int64_t count) {
  int64_t b = (count + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (int)b;
}

constexpr int64_t kChunkBytes = 64ll << 20;  // staging chunk for precision conversion

// Copy a complex field between host and device in z-plane chunks, converting
// precision on the device when the storage is FP32.
// Creates the copy stream, events and the two staging buffers on first use.
int xfer_init(axg_ctx *ctx) {
  if (ctx->xstream) return AXG_OK;
  for (int b = 0; b < 2; ++b) AXG_TRY(axg_alloc(ctx, &ctx->xstage[b], (size_t)kChunkBytes, "transfer staging"));
  AXG_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->xstream, cudaStreamNonBlocking));
  for (int b = 0; b < 2; ++b) {
    AXG_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->xev_copied[b], cudaEventDisableTiming));
    AXG_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->xev_done[b], cudaEventDisableTiming));
  }
  AXG_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->xev_start, cudaEventDisableTiming));
  return AXG_OK;
}

// Chunked transfer with precision conversion through two staging buffers.
// Upload: the copy stream moves chunk i into stage[i % 2] while the library
// stream converts chunk i - 1; download: the library stream converts chunk i
// while the copy stream drains chunk i - 1 to the host.  Returns after the
// host buffer is no longer touched.
using XferFn = std::function<cudaError_t(int64_t chunk, void *stage, cudaStream_t s)>;
int xfer_pipelined(axg_ctx *ctx, bool to_device, int64_t nchunks, const XferFn &copy, const XferFn &convert) {
  AXG_TRY(xfer_init(ctx));
  cudaError_t e = cudaEventRecord(ctx->xev_start, ctx->stream);  // earlier work on the library stream
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->xstream, ctx->xev_start, 0);
  for (int64_t i = 0; i < nchunks && e == cudaSuccess; ++i) {
    const int b = (int)(i & 1);
    void *st = ctx->xstage[b];
    if (to_device) {
      if (i >= 2) e = cudaStreamWaitEvent(ctx->xstream, ctx->xev_done[b], 0);  // conversion of i-2 read it
      if (e == cudaSuccess) e = copy(i, st, ctx->xstream);
      if (e == cudaSuccess) e = cudaEventRecord(ctx->xev_copied[b], ctx->xstream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ctx->xev_copied[b], 0);
      if (e == cudaSuccess) e = convert(i, st, ctx->stream);
      if (e == cudaSuccess) e = cudaEventRecord(ctx->xev_done[b], ctx->stream);
    } else {
      if (i >= 2) e = cudaStreamWaitEvent(ctx->stream, ctx->xev_copied[b], 0);  // copy of i-2 drained it
      if (e == cudaSuccess) e = convert(i, st, ctx->stream);
      if (e == cudaSuccess) e = cudaEventRecord(ctx->xev_done[b], ctx->stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->xstream, ctx->xev_done[b], 0);
      if (e == cudaSuccess) e = copy(i, st, ctx->xstream);
      if (e == cudaSuccess) e = cudaEventRecord(ctx->xev_copied[b], ctx->xstream);
    }
  }
  // the library stream must not run ahead of the last copy (staging reuse)
  if (e == cudaSuccess) e = cudaEventRecord(ctx->xev_start, ctx->xstream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ctx->xev_start, 0);
  const cudaError_t s1 = cudaStreamSynchronize(ctx->xstream);
  const cudaError_t s2 = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = s1 != cudaSuccess ? s1 : s2;
  if (e != cudaSuccess) return axg_set_error(ctx, AXG_ERR_CUDA, std::string("transfer: ") + cudaGetErrorString(e));
  return AXG_OK;
}

int xfer_complex(axg_ctx *ctx, bool to_device, double *host, int64_t plane_stride,
                 int64_t first_plane, void *dev, void *comp) {
  const int64_t n = ctx->n, n2 = n * n;
  const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
  if (plane_stride < n2) return axg_set_error(ctx, AXG_ERR_ARG, "plane_stride < N*N");
  if (first_plane < 0) return axg_set_error(ctx, AXG_ERR_ARG, "first_plane < 0");
  if (!fp32) {
    const cudaError_t e =
        to_device ? cudaMemcpy2DAsync(dev, (size_t)(n2 * 16), host + 2 * first_plane * plane_stride,
                                      (size_t)(plane_stride * 16), (size_t)(n2 * 16), (size_t)n,
                                      cudaMemcpyHostToDevice, ctx->stream)
                  : cudaMemcpy2DAsync(host + 2 * first_plane * plane_stride, (size_t)(plane_stride * 16), dev,
                                      (size_t)(n2 * 16), (size_t)(n2 * 16), (size_t)n, cudaMemcpyDeviceToHost,
                                      ctx->stream);
    if (e != cudaSuccess) return axg_set_error(ctx, AXG_ERR_CUDA, std::string("transfer: ") + cudaGetErrorString(e));
    AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return AXG_OK;
  }
  // whole z-planes per chunk when a plane fits, else runs of rows
  const int64_t zchunk = std::max<int64_t>(1, kChunkBytes / (n2 * 16));
  if (n2 * 16 > kChunkBytes) {
    const int64_t rows = std::max<int64_t>(1, kChunkBytes / (n * 16));
    const int64_t per_plane = (n + rows - 1) / rows;
    return xfer_pipelined(
        ctx, to_device, n * per_plane,
        [&](int64_t i, void *st, cudaStream_t s) {
          const int64_t z = i / per_plane, y0 = (i % per_plane) * rows, ny = std::min(rows, n - y0);
          double *h = host + 2 * ((first_plane + z) * plane_stride + y0 * n);
          return to_device ? cudaMemcpyAsync(st, h, (size_t)(ny * n * 16), cudaMemcpyHostToDevice, s)
                           : cudaMemcpyAsync(h, st, (size_t)(ny * n * 16), cudaMemcpyDeviceToHost, s);
        },
        [&](int64_t i, void *st, cudaStream_t s) {
          const int64_t z = i / per_plane, y0 = (i % per_plane) * rows, ny = std::min(rows, n - y0);
          const int64_t o = z * n2 + y0 * n, m = ny * n;
          if (to_device)
            k_c128_to_f32<<<grid_for(m), 256, 0, s>>>((const double2 *)st, (float2 *)dev + o,
                                                      comp ? (float2 *)comp + o : nullptr, m);
          else
            k_f32_to_c128<<<grid_for(m), 256, 0, s>>>((const float2 *)dev + o,
                                                      comp ? (const float2 *)comp + o : nullptr, (double2 *)st, m);
          ctx->launches++;
          return cudaGetLastError();
        });
  }
  const int64_t nch = (n + zchunk - 1) / zchunk;
  return xfer_pipelined(
      ctx, to_device, nch,
      [&](int64_t i, void *st, cudaStream_t s) {
        const int64_t z0 = i * zchunk, nz = std::min(zchunk, n - z0);
        double *h = host + 2 * (first_plane + z0) * plane_stride;
        return to_device ? cudaMemcpy2DAsync(st, (size_t)(n2 * 16), h, (size_t)(plane_stride * 16),
                                             (size_t)(n2 * 16), (size_t)nz, cudaMemcpyHostToDevice, s)
                         : cudaMemcpy2DAsync(h, (size_t)(plane_stride * 16), st, (size_t)(n2 * 16),
                                             (size_t)(n2 * 16), (size_t)nz, cudaMemcpyDeviceToHost, s);
      },
      [&](int64_t i, void *st, cudaStream_t s) {
        const int64_t z0 = i * zchunk, nz = std::min(zchunk, n - z0);
        const int64_t o = z0 * n2, m = nz * n2;
        if (to_device)
          k_c128_to_f32<<<grid_for(m), 256, 0, s>>>((const double2 *)st, (float2 *)dev + o,
                                                    comp ? (float2 *)comp + o : nullptr, m);
        else
          k_f32_to_c128<<<grid_for(m), 256, 0, s>>>((const float2 *)dev + o,
                                                    comp ? (const float2 *)comp + o : nullptr, (double2 *)st, m);
        ctx->launches++;
        return cudaGetLastError();
      });
}

int xfer_real6(axg_ctx *ctx, bool to_device, double *host, void *dev, void *comp) {
  const int64_t count = 6 * ctx->n3;
  const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
  if (!fp32) {
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(to_device ? dev : host, to_device ? (void *)host : dev,
                                      (size_t)count * 8,
                                      to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                                      ctx->stream));
    AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return AXG_OK;
  }
  const int64_t chunk = kChunkBytes / 8;
  return xfer_pipelined(
      ctx, to_device, (count + chunk - 1) / chunk,
      [&](int64_t i, void *st, cudaStream_t s) {
        const int64_t o = i * chunk, m = std::min(chunk, count - o);
        return to_device ? cudaMemcpyAsync(st, host + o, (size_t)m * 8, cudaMemcpyHostToDevice, s)
                         : cudaMemcpyAsync(host + o, st, (size_t)m * 8, cudaMemcpyDeviceToHost, s);
      },
      [&](int64_t i, void *st, cudaStream_t s) {
        const int64_t o = i * chunk, m = std::min(chunk, count - o);
        if (to_device)
          k_r64_to_f32<<<grid_for(m), 256, 0, s>>>((const double *)st, (float *)dev + o,
                                                   comp ? (float *)comp + o : nullptr, m);
        else
          k_f32_to_r64<<<grid_for(m), 256, 0, s>>>((const float *)dev + o, comp ? (const float *)comp + o : nullptr,
                                                   (double *)st, m);
        ctx->launches++;
        return cudaGetLastError();
      });
}

// CRC-32 (IEEE 802.3 polynomial, reflected), table driven.
uint32_t crc32_update(uint32_t crc, const unsigned char *buf, size_t len) {
  static uint32_t table[256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    init = true;
  }
  crc = ~crc;
  for (size_t i = 0; i < len; ++i) crc = table[(crc ^ buf[i]) & 0xff] ^ (crc >> 8);
  return ~crc;
}

bool valid_ctx(const axg_ctx *ctx) { return ctx != nullptr; }
}  // namespace

// ===========================================================================
// shared internal helpers
// ===========================================================================
int axg_set_error(axg_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->err = msg;
  else g_create_error = msg;
  return code;
}

int axg_alloc(axg_ctx *ctx, void **ptr, size_t bytes, const char *what) {
  *ptr = nullptr;
  if (bytes == 0) return AXG_OK;
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    cudaGetLastError();
    return axg_set_error(ctx, AXG_ERR_NOMEM,
                         std::string("cudaMalloc ") + what + " (" + std::to_string(bytes) +
                             " B): " + cudaGetErrorString(e));
  }
  ctx->bytes += (int64_t)bytes;
  return AXG_OK;
}

void axg_free(axg_ctx *ctx, void **ptr) {
  if (*ptr) {
    cudaFree(*ptr);
    *ptr = nullptr;
  }
  (void)ctx;
}

void axg_kt_begin(axg_ctx *ctx, const char *name) {
  if (!ctx->ktiming) return;
  auto it = ctx->kid.find(name);
  int id;
  if (it == ctx->kid.end()) {
    id = (int)ctx->kstats.size();
    ctx->kid[name] = id;
    axg_kernel_stat s;
    s.name = name;
    ctx->kstats.push_back(s);
  } else {
    id = it->second;
  }
  cudaEvent_t a, b;
  if (ctx->ev_pool.size() >= 2) {
    a = ctx->ev_pool.back();
    ctx->ev_pool.pop_back();
    b = ctx->ev_pool.back();
    ctx->ev_pool.pop_back();
  } else {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  cudaEventRecord(a, ctx->stream);
  ctx->pending.push_back({id, {a, b}});
}

void axg_kt_end(axg_ctx *ctx) {
  if (!ctx->ktiming || ctx->pending.empty()) return;
  cudaEventRecord(ctx->pending.back().second.second, ctx->stream);
  if (ctx->pending.size() > 8192) axg_kt_flush(ctx);
}

int axg_kt_flush(axg_ctx *ctx) {
  if (ctx->pending.empty()) return AXG_OK;
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  for (auto &pe : ctx->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, pe.second.first, pe.second.second);
    ctx->kstats[pe.first].launches += 1;
    ctx->kstats[pe.first].total_ms += ms;
    ctx->ev_pool.push_back(pe.second.first);
    ctx->ev_pool.push_back(pe.second.second);
  }
  ctx->pending.clear();
  return AXG_OK;
}

// evolve.f90:291-305 (reference potential) and the quartic model; identical
// expression order to the CPU restatement so the coefficients agree bitwise.
void axg_kick_coeffs(const axg_params *p, double t, double dt, double f[4], double pot[4]) {
  double hubble = 1 / t;
  double fact0 = 1 + dt * hubble;
  double fact1 = 1 - dt * hubble;
  double fact2 = dt / (p->dspa * p->dspa);
  double fact3 = -(dt * (t * t) * (p->sigma_cr * p->sigma_cr));
  double facts = dt * (p->sigma_cr * p->sigma_cr);
  f[0] = fact1 / fact0;
  f[1] = fact2 / fact0;
  f[2] = fact3 / fact0;
  f[3] = facts / fact0;
  if (p->potential == AXG_POT_REFERENCE) {
    double thrm = (p->flags & AXG_F_INITIAL_LOOP) ? 0.0 : kThrmSigma / t;
    double m2 = msquared(thrm);
    double ma2 = maxion2(thrm, p->kappa);
    pot[0] = 2.0;
    pot[1] = m2;
    pot[2] = -(ma2 / 2);
    pot[3] = 0.0;
  } else {
    double v2 = p->vev * p->vev;
    pot[0] = p->lambda / 2;
    pot[1] = -(p->lambda * v2 / 2);
    pot[2] = 0.0;
    pot[3] = 0.0;
    if (p->ma2_0 != 0.0 && t >= p->tau_axion_on) {
      double ma2 = p->ma2_0 * std::pow(t / p->tau_axion_on, p->ma2_power);
      if (p->n_dw == 2) {
        pot[1] += ma2 / 4;
        pot[3] = -(ma2 / 4);
      } else {
        pot[2] = -(ma2 * p->vev / 2);
      }
    }
  }
}

int axg_phi_to_fp64(axg_ctx *ctx, double2 *dst) {
  if (ctx->p.precision == AXG_PREC_FP32_MIXED) {
    k_f32_to_c128<<<grid_for(ctx->n3), 256, 0, ctx->stream>>>(
        (const float2 *)ctx->phi[ctx->cur], (const float2 *)ctx->cphi, dst, ctx->n3);
    ctx->launches++;
    AXG_CUDA_TRY(ctx, cudaGetLastError());
  } else {
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(dst, ctx->phi[ctx->cur], (size_t)ctx->n3 * 16,
                                      cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return AXG_OK;
}

int axg_phid_to_fp64(axg_ctx *ctx, double2 *dst) {
  if (ctx->p.precision == AXG_PREC_FP32_MIXED) {
    k_f32_to_c128<<<grid_for(ctx->n3), 256, 0, ctx->stream>>>((const float2 *)ctx->phid, nullptr,
                                                              dst, ctx->n3);
    ctx->launches++;
    AXG_CUDA_TRY(ctx, cudaGetLastError());
  } else {
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(dst, ctx->phid, (size_t)ctx->n3 * 16, cudaMemcpyDeviceToDevice,
                                      ctx->stream));
  }
  return AXG_OK;
}

// ===========================================================================
// C-ABI
// ===========================================================================
extern "C" {

int axg_version(void) { return 100; }

int axg_params_default(axg_params *p) {
  if (!p) return AXG_ERR_ARG;
  std::memset(p, 0, sizeof(*p));
  p->ngrid = 64;
  p->precision = AXG_PREC_FP64_PLAIN;
  p->gw_mode = AXG_GW_NONE;
  p->num_bin = 50;       // settings.f90:158
  p->num_bin_grav = 25;  // grav_waves.f90:6
  p->degrade_spec = 0;
  p->flags = AXG_F_ID_STRINGS | AXG_F_ID_WALLS | AXG_F_SPEC_EST;
  p->compat = AXG_COMPAT_REF;
  p->potential = AXG_POT_REFERENCE;
  p->n_dw = 1;
  p->gw_log_bins = 64;
  p->dspa = 1.0;
  p->sigma_cr = 1.0;
  p->kappa = 1.0;
  p->tau_cr = 1.0;
  p->a_now = 1.0;
  p->width_cr = 1.0 / std::sqrt(2.0);
  p->thickness_cr = 1.0;
  p->lambda = 1.0;
  p->vev = 1.0;
  p->ma2_power = 2.0;
  p->seed = 1;
  return AXG_OK;
}

const char *axg_last_error(const axg_ctx *ctx) {
  return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

int axg_create(const axg_params *pin, axg_ctx **out) {
  if (!pin || !out) return axg_set_error(nullptr, AXG_ERR_ARG, "null argument");
  *out = nullptr;
  const axg_params &p = *pin;
  if (p.ngrid < 4 || (p.ngrid & 1)) return axg_set_error(nullptr, AXG_ERR_ARG, "ngrid must be even and >= 4");
  if (p.ngrid > 2048) return axg_set_error(nullptr, AXG_ERR_ARG, "ngrid > 2048");
  if (p.precision < 0 || p.precision > 2) return axg_set_error(nullptr, AXG_ERR_ARG, "precision");
  if (p.gw_mode < 0 || p.gw_mode > 2) return axg_set_error(nullptr, AXG_ERR_ARG, "gw_mode");
  if (p.num_bin < 1 || p.num_bin_grav < 1) return axg_set_error(nullptr, AXG_ERR_ARG, "bins");
  if (!(p.dspa > 0) || !(p.sigma_cr > 0)) return axg_set_error(nullptr, AXG_ERR_ARG, "dspa/sigma_cr");
  if (p.degrade_spec < 0 || (p.ngrid >> p.degrade_spec) < 2 || ((p.ngrid >> p.degrade_spec) << p.degrade_spec) != p.ngrid)
    return axg_set_error(nullptr, AXG_ERR_ARG, "degrade_spec");
  // Green's mode runs on the GW grid ngrid / 2^degrade_spec (grav_waves.f90:37-45);
  // its half-spectrum accumulators need that side even and >= 4
  if (p.gw_mode == AXG_GW_GREEN && (((p.ngrid >> p.degrade_spec) & 1) || (p.ngrid >> p.degrade_spec) < 4))
    return axg_set_error(nullptr, AXG_ERR_UNSUPPORTED,
                         "gw_mode GREEN needs ngrid / 2^degrade_spec even and >= 4 (the GW grid of init_grav)");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return axg_set_error(nullptr, AXG_ERR_CUDA, "no CUDA device");
  }
  if (p.device < 0 || p.device >= ndev) return axg_set_error(nullptr, AXG_ERR_ARG, "device ordinal");
  if (cudaSetDevice(p.device) != cudaSuccess) return axg_set_error(nullptr, AXG_ERR_CUDA, "cudaSetDevice");
  axg_ctx *ctx = new axg_ctx();
  ctx->p = p;
  ctx->n = p.ngrid;
  ctx->n3 = (int64_t)p.ngrid * p.ngrid * p.ngrid;
  cudaGetDevice(&ctx->device);
  int rc = AXG_OK;
  auto fail = [&](int code) {
    g_create_error = ctx->err;
    axg_destroy(ctx);
    return code;
  };
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(axg_set_error(ctx, AXG_ERR_CUDA, "stream create"));
  for (auto &e : ctx->user_ev) cudaEventCreate(&e);
  const bool fp32 = p.precision == AXG_PREC_FP32_MIXED;
  const bool fused = p.precision != AXG_PREC_FP64_PLAIN;
  const bool uij = p.gw_mode == AXG_GW_UIJ;
  const size_t rs = fp32 ? 4 : 8;
  ctx->elem = rs;
  const size_t n3 = (size_t)ctx->n3;
  if ((rc = axg_alloc(ctx, &ctx->phi[0], n3 * 2 * rs, "phi"))) return fail(rc);
  if (fused && (rc = axg_alloc(ctx, &ctx->phi[1], n3 * 2 * rs, "phi pong"))) return fail(rc);
  if ((rc = axg_alloc(ctx, &ctx->phid, n3 * 2 * rs, "phidot"))) return fail(rc);
  if (fp32 && (rc = axg_alloc(ctx, &ctx->cphi, n3 * 2 * rs, "phi compensation"))) return fail(rc);
  if (uij) {
    if ((rc = axg_alloc(ctx, &ctx->u[0], n3 * 6 * rs, "u"))) return fail(rc);
    if (fused && (rc = axg_alloc(ctx, &ctx->u[1], n3 * 6 * rs, "u pong"))) return fail(rc);
    if ((rc = axg_alloc(ctx, &ctx->ud, n3 * 6 * rs, "udot"))) return fail(rc);
    if (fp32 && (rc = axg_alloc(ctx, &ctx->cu, n3 * 6 * rs, "u compensation"))) return fail(rc);
  }
  ctx->red_cap = 4096;
  if ((rc = axg_alloc(ctx, (void **)&ctx->d_red, ctx->red_cap * 8, "reduction"))) return fail(rc);
  if ((rc = axg_alloc(ctx, (void **)&ctx->d_cnt, 64 * 8, "counters"))) return fail(rc);
  if ((rc = axg_alloc(ctx, (void **)&ctx->d_err, 64, "error flag"))) return fail(rc);
  cudaMemsetAsync(ctx->d_err, 0, 64, ctx->stream);
  // zero state
  cudaMemsetAsync(ctx->phi[0], 0, n3 * 2 * rs, ctx->stream);
  if (ctx->phi[1]) cudaMemsetAsync(ctx->phi[1], 0, n3 * 2 * rs, ctx->stream);
  cudaMemsetAsync(ctx->phid, 0, n3 * 2 * rs, ctx->stream);
  if (ctx->cphi) cudaMemsetAsync(ctx->cphi, 0, n3 * 2 * rs, ctx->stream);
  for (void *q : {ctx->u[0], ctx->u[1], ctx->ud, ctx->cu})
    if (q) cudaMemsetAsync(q, 0, n3 * 6 * rs, ctx->stream);
  if (p.gw_mode == AXG_GW_GREEN && (rc = axg_gw_init(ctx))) return fail(rc);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    return fail(axg_set_error(ctx, AXG_ERR_CUDA, "initial memset"));
  *out = ctx;
  return AXG_OK;
}

int axg_destroy(axg_ctx *ctx) {
  if (!ctx) return AXG_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (void **q : {&ctx->phi[0], &ctx->phi[1], &ctx->phid, &ctx->cphi, &ctx->u[0], &ctx->u[1],
                   &ctx->ud, &ctx->cu, (void **)&ctx->acc, (void **)&ctx->gsrc, (void **)&ctx->gw_omega,
                   (void **)&ctx->gw_pol, (void **)&ctx->ff_tw, (void **)&ctx->gsrcF, (void **)&ctx->flags,
                   (void **)&ctx->phase, (void **)&ctx->phase64, (void **)&ctx->d_strings, (void **)&ctx->d_walls, (void **)&ctx->spec_mat,
                   (void **)&ctx->spec_largeq0, (void **)&ctx->spec_dq, (void **)&ctx->spec_buf,
                   &ctx->ubuf, (void **)&ctx->d_red, (void **)&ctx->d_cnt, (void **)&ctx->d_err})
    axg_free(ctx, q);
  if (ctx->plan_gsrc_ok) cufftDestroy(ctx->plan_gsrc);
  if (ctx->plan_spec_ok) cufftDestroy(ctx->plan_spec);
  if (ctx->plan_window_ok) cufftDestroy(ctx->plan_window);
  if (ctx->plan_u_ok) cufftDestroy(ctx->plan_u);
  for (auto &e : ctx->user_ev)
    if (e) cudaEventDestroy(e);
  for (auto &pe : ctx->pending) {
    cudaEventDestroy(pe.second.first);
    cudaEventDestroy(pe.second.second);
  }
  for (auto e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->xstream) {
    cudaStreamSynchronize(ctx->xstream);
    cudaStreamDestroy(ctx->xstream);
  }
  for (int b = 0; b < 2; ++b) {
    if (ctx->xev_copied[b]) cudaEventDestroy(ctx->xev_copied[b]);
    if (ctx->xev_done[b]) cudaEventDestroy(ctx->xev_done[b]);
    axg_free(ctx, &ctx->xstage[b]);
  }
  if (ctx->xev_start) cudaEventDestroy(ctx->xev_start);
  for (auto &e : ctx->bin_cache) axg_free(ctx, (void **)&e.tab);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return AXG_OK;
}

int axg_memory_bytes(const axg_ctx *ctx, int64_t *bytes) {
  if (!ctx || !bytes) return AXG_ERR_ARG;
  *bytes = ctx->bytes;
  return AXG_OK;
}

int axg_upload(axg_ctx *ctx, const double *phi, const double *phidot, int64_t plane_stride,
               int64_t first_plane) {
  if (!valid_ctx(ctx)) return AXG_ERR_ARG;
  if (phi) {
    AXG_TRY(xfer_complex(ctx, true, const_cast<double *>(phi), plane_stride, first_plane,
                         ctx->phi[ctx->cur], ctx->cphi));
  }
  if (phidot)
    AXG_TRY(xfer_complex(ctx, true, const_cast<double *>(phidot), plane_stride, first_plane,
                         ctx->phid, nullptr));
  ctx->flags_valid = false;
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return AXG_OK;
}

int axg_download(axg_ctx *ctx, double *phi, double *phidot, int64_t plane_stride,
                 int64_t first_plane) {
  if (!valid_ctx(ctx)) return AXG_ERR_ARG;
  AXG_TRY(axg_evo_check_error(ctx));
  if (phi) AXG_TRY(xfer_complex(ctx, false, phi, plane_stride, first_plane, ctx->phi[ctx->cur], ctx->cphi));
  if (phidot) AXG_TRY(xfer_complex(ctx, false, phidot, plane_stride, first_plane, ctx->phid, nullptr));
  return AXG_OK;
}

int axg_upload_uij(axg_ctx *ctx, const double *u, const double *udot) {
  if (!valid_ctx(ctx)) return AXG_ERR_ARG;
  if (ctx->p.gw_mode != AXG_GW_UIJ) return axg_set_error(ctx, AXG_ERR_STATE, "gw_mode is not UIJ");
  if (u) AXG_TRY(xfer_real6(ctx, true, const_cast<double *>(u), ctx->u[ctx->cur], ctx->cu));
  if (udot) AXG_TRY(xfer_real6(ctx, true, const_cast<double *>(udot), ctx->ud, nullptr));
  return AXG_OK;
}

int axg_download_uij(axg_ctx *ctx, double *u, double *udot) {
  if (!valid_ctx(ctx)) return AXG_ERR_ARG;
  if (ctx->p.gw_mode != AXG_GW_UIJ) return axg_set_error(ctx, AXG_ERR_STATE, "gw_mode is not UIJ");
  AXG_TRY(axg_evo_check_error(ctx));
  if (u) AXG_TRY(xfer_real6(ctx, false, u, ctx->u[ctx->cur], ctx->cu));
  if (udot) AXG_TRY(xfer_real6(ctx, false, udot, ctx->ud, nullptr));
  return AXG_OK;
}

// The device holds the accumulators of the stored half spectrum plus the
// Nyquist-row mirrors (axg_gw_acc_entries); the site of -k in the other half
// is the conjugate of its entry.  The host side is always the full
// complex128 [4][N^3] array: download fills the other half by conjugation,
// upload takes the stored half and the Nyquist-row mirrors (the reference's
// accumulators are conjugate-symmetric, so nothing is lost).  FP32-mixed and
// the float-float FP64 paths keep each component as a float-float pair.
}  // extern "C"
namespace {
// for each device entry, the full-lattice site it holds
template <typename F>
void gw_acc_sites(int n, F f) {
  const int nh = n / 2 + 1;
  const int64_t nhalf = (int64_t)n * n * nh;
  for (int hz = 0; hz < n; ++hz)
    for (int hy = 0; hy < n; ++hy)
      for (int hx = 0; hx < nh; ++hx) {
        const int64_t h = ((int64_t)hz * n + hy) * nh + hx;
        const int64_t s1 = ((int64_t)hz * n + hy) * n + hx;
        const int64_t s2 = ((int64_t)(hz == 0 ? 0 : n - hz) * n + (hy == 0 ? 0 : n - hy)) * n + (n - hx);
        const bool mirror = hx > 0 && hx < n / 2, nyq = mirror && (hy == n / 2 || hz == n / 2);
        f(h, s1, mirror && !nyq ? s2 : -1);  // s2: the conjugate site
        if (nyq) f(nhalf + gw_nyq_extra(hx, hy, hz, n), s2, -1);
      }
}
}  // namespace
extern "C" {

int axg_upload_gw_green(axg_ctx *ctx, const double *acc) {
  if (!valid_ctx(ctx) || !acc) return AXG_ERR_ARG;
  if (!ctx->acc) return axg_set_error(ctx, AXG_ERR_STATE, "gw_mode is not GREEN");
  const int n = ctx->gw_n;  // the GW grid (ngrid / 2^degrade_spec)
  const int64_t n3 = (int64_t)n * n * n, as = ctx->acc_stride;
  for (int a = 0; a < 4; ++a) {
    const double *src = acc + 2 * (size_t)a * n3;
    if (ctx->acc_ff) {
      std::vector<float4> buf((size_t)as);
      gw_acc_sites(n, [&](int64_t e, int64_t s, int64_t) {
        const double re = src[2 * s], im = src[2 * s + 1];
        const float rh = (float)re, ih = (float)im;
        buf[e] = make_float4(rh, (float)(re - (double)rh), ih, (float)(im - (double)ih));
      });
      AXG_CUDA_TRY(ctx, cudaMemcpy((float4 *)ctx->acc + a * as, buf.data(), (size_t)as * sizeof(float4),
                                   cudaMemcpyHostToDevice));
    } else {
      std::vector<double2> buf((size_t)as);
      gw_acc_sites(n, [&](int64_t e, int64_t s, int64_t) { buf[e] = make_double2(src[2 * s], src[2 * s + 1]); });
      AXG_CUDA_TRY(ctx, cudaMemcpy((double2 *)ctx->acc + a * as, buf.data(), (size_t)as * sizeof(double2),
                                   cudaMemcpyHostToDevice));
    }
  }
  return AXG_OK;
}

int axg_download_gw_green(axg_ctx *ctx, double *acc) {
  if (!valid_ctx(ctx) || !acc) return AXG_ERR_ARG;
  if (!ctx->acc) return axg_set_error(ctx, AXG_ERR_STATE, "gw_mode is not GREEN");
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  const int n = ctx->gw_n;  // the GW grid (ngrid / 2^degrade_spec)
  const int64_t n3 = (int64_t)n * n * n, as = ctx->acc_stride;
  for (int a = 0; a < 4; ++a) {
    double *dst = acc + 2 * (size_t)a * n3;
    auto put = [&](int64_t s, int64_t s2, double re, double im) {
      dst[2 * s] = re;
      dst[2 * s + 1] = im;
      if (s2 >= 0) {
        dst[2 * s2] = re;
        dst[2 * s2 + 1] = -im;
      }
    };
    if (ctx->acc_ff) {
      std::vector<float4> buf((size_t)as);
      AXG_CUDA_TRY(ctx, cudaMemcpy(buf.data(), (const float4 *)ctx->acc + a * as, (size_t)as * sizeof(float4),
                                   cudaMemcpyDeviceToHost));
      gw_acc_sites(n, [&](int64_t e, int64_t s, int64_t s2) {
        put(s, s2, (double)buf[e].x + (double)buf[e].y, (double)buf[e].z + (double)buf[e].w);
      });
    } else {
      std::vector<double2> buf((size_t)as);
      AXG_CUDA_TRY(ctx, cudaMemcpy(buf.data(), (const double2 *)ctx->acc + a * as, (size_t)as * sizeof(double2),
                                   cudaMemcpyDeviceToHost));
      gw_acc_sites(n, [&](int64_t e, int64_t s, int64_t s2) { put(s, s2, buf[e].x, buf[e].y); });
    }
  }
  return AXG_OK;
}

// evolve.f90:10-24
int axg_get_dtau(const axg_params *p, double tau1, double tau2, double eps_dtau, double *dtau,
                 int64_t *nsteps) {
  if (!p || !dtau || !nsteps || !(tau2 > tau1) || !(eps_dtau > 0)) return AXG_ERR_ARG;
  double dwav = kRefTwoPi / p->dspa / p->ngrid;  // settings.f90:295
  double mass = p->potential == AXG_POT_REFERENCE ? kThrmSigma : std::sqrt(2 * p->lambda) * p->vev;
  double omega = mass * tau2 * p->sigma_cr;
  double kmax = dwav * p->ngrid;
  omega = std::sqrt(kmax * kmax + omega * omega);
  double dt = eps_dtau / omega;
  int64_t nt = (int64_t)std::ceil((tau2 - tau1) / dt);
  if (nt < 1) nt = 1;
  *dtau = (tau2 - tau1) / nt;
  *nsteps = nt;
  return AXG_OK;
}

// evolve.f90:259-281
int axg_evolve_phi(axg_ctx *ctx, double *t, double dt) {
  if (!valid_ctx(ctx) || !t) return AXG_ERR_ARG;
  AXG_TRY(axg_evo_drift(ctx, dt));
  *t = *t + dt;
  return AXG_OK;
}

// evolve.f90:283-339
int axg_evolve_phidot(axg_ctx *ctx, double t, double dt) {
  if (!valid_ctx(ctx)) return AXG_ERR_ARG;
  if (ctx->p.precision == AXG_PREC_FP32_MIXED)
    return axg_set_error(ctx, AXG_ERR_UNSUPPORTED,
                         "FP32-mixed runs kick and drift fused: use axg_symplectic_integration or axg_leapfrog");
  AXG_TRY(axg_evo_kick_plain(ctx, t, dt));
  if (ctx->p.gw_mode == AXG_GW_GREEN) AXG_TRY(axg_gw_integration(ctx, t, dt));
  return AXG_OK;
}

int axg_leapfrog(axg_ctx *ctx, double t1, double dt, int64_t nsteps, int first_half,
                 int last_half) {
  if (!valid_ctx(ctx) || nsteps < 0 || !(dt != 0) || !std::isfinite(dt) || !(t1 > 0) ||
      !(t1 + (double)nsteps * dt > 0))
    return AXG_ERR_ARG;
  double t = t1;
  if (first_half) {
    AXG_TRY(axg_evo_drift(ctx, dt / 2));
    t = t + dt / 2;
  }
  for (int64_t it = 1; it <= nsteps; ++it) {
    const double h = (it == nsteps && last_half) ? dt / 2 : dt;
    if (ctx->p.precision == AXG_PREC_FP64_PLAIN) {
      AXG_TRY(axg_evo_kick_plain(ctx, t, dt));
      if (ctx->p.gw_mode == AXG_GW_GREEN) AXG_TRY(axg_gw_integration(ctx, t, dt));
      AXG_TRY(axg_evo_drift(ctx, h));
    } else {
      AXG_TRY(axg_evo_kick_drift(ctx, t, dt, h));
      if (ctx->p.gw_mode == AXG_GW_GREEN) {
        // the Green's-function source uses phi at the kick time, which the
        // fused pass left intact in the other ping-pong buffer
        ctx->cur = 1 - ctx->cur;
        int rc = axg_gw_integration(ctx, t, dt);
        ctx->cur = 1 - ctx->cur;
        AXG_TRY(rc);
      }
    }
    t = t + h;
  }
  ctx->flags_valid = false;
  return AXG_OK;
}

// evolve.f90:238-257
int axg_symplectic_integration(axg_ctx *ctx, double t1, double t2, double eps_dtau,
                               int64_t *nsteps_out) {
  if (!valid_ctx(ctx)) return AXG_ERR_ARG;
  double dt;
  int64_t nt;
  AXG_TRY(axg_get_dtau(&ctx->p, t1, t2, eps_dtau, &dt, &nt));
  if (nsteps_out) *nsteps_out = nt;
  return axg_leapfrog(ctx, t1, dt, nt, 1, 1);
}

int axg_synchronize(axg_ctx *ctx) {
  if (!valid_ctx(ctx)) return AXG_ERR_ARG;
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return axg_evo_check_error(ctx);
}

int axg_event_record(axg_ctx *ctx, int slot) {
  if (!valid_ctx(ctx) || slot < 0 || slot >= 8) return AXG_ERR_ARG;
  AXG_CUDA_TRY(ctx, cudaEventRecord(ctx->user_ev[slot], ctx->stream));
  return AXG_OK;
}

int axg_event_elapsed(axg_ctx *ctx, int a, int b, float *ms) {
  if (!valid_ctx(ctx) || a < 0 || a >= 8 || b < 0 || b >= 8 || !ms) return AXG_ERR_ARG;
  AXG_CUDA_TRY(ctx, cudaEventSynchronize(ctx->user_ev[b]));
  AXG_CUDA_TRY(ctx, cudaEventElapsedTime(ms, ctx->user_ev[a], ctx->user_ev[b]));
  return AXG_OK;
}

int axg_set_kernel_timing(axg_ctx *ctx, int on) {
  if (!valid_ctx(ctx)) return AXG_ERR_ARG;
  AXG_TRY(axg_kt_flush(ctx));
  ctx->ktiming = on != 0;
  if (on) {
    for (auto &s : ctx->kstats) {
      s.launches = 0;
      s.total_ms = 0;
    }
  }
  return AXG_OK;
}

int axg_kernel_timing(axg_ctx *ctx, int i, char *name, int64_t name_len, int64_t *launches,
                      double *total_ms) {
  if (!valid_ctx(ctx)) return AXG_ERR_ARG;
  AXG_TRY(axg_kt_flush(ctx));
  if (i < 0 || i >= (int)ctx->kstats.size()) return AXG_ERR_ARG;
  const auto &s = ctx->kstats[i];
  if (name && name_len > 0) {
    std::strncpy(name, s.name.c_str(), (size_t)name_len - 1);
    name[name_len - 1] = 0;
  }
  if (launches) *launches = s.launches;
  if (total_ms) *total_ms = s.total_ms;
  return AXG_OK;
}

int axg_launch_count(const axg_ctx *ctx, int64_t *launches) {
  if (!ctx || !launches) return AXG_ERR_ARG;
  *launches = ctx->launches;
  return AXG_OK;
}

// ---------------------------------------------------------------------------
// checkpoint (evolve.f90:401-546): raw complex128 phi block then phidot block
// in global x-fastest order, as io_chk writes them; u_ij blocks appended when
// the context evolves u_ij; CRC-32 of the whole file in path+".crc".
// ---------------------------------------------------------------------------
namespace {
// FP32-mixed sidecar path+".fp32": the raw device state (phi and its Kahan
// compensation, phi'; u, its compensation and u' when present) so that a
// resumed FP32 run continues bit for bit; the complex128 file alone fixes
// only the compensated value phi - c.  Layout: "AXGFP32" NUL, int64 N, int64
// uij, int64 CRC-32 of the complex128 checkpoint it belongs to, the arrays,
// CRC-32 of everything before it.  A sidecar whose recorded checkpoint CRC
// differs from the checkpoint being read belongs to another checkpoint
// (one rewritten since, by this library or another writer) and is ignored.
struct RawField {
  void *dev;
  size_t bytes;
};
std::vector<RawField> fp32_fields(axg_ctx *ctx) {
  const size_t n3 = (size_t)ctx->n3;
  std::vector<RawField> f = {{ctx->phi[ctx->cur], n3 * 8}, {ctx->cphi, n3 * 8}, {ctx->phid, n3 * 8}};
  if (ctx->p.gw_mode == AXG_GW_UIJ) {
    f.push_back({ctx->u[ctx->cur], n3 * 24});
    f.push_back({ctx->cu, n3 * 24});
    f.push_back({ctx->ud, n3 * 24});
  }
  return f;
}
const char kFp32Magic[8] = {'A', 'X', 'G', 'F', 'P', '3', '2', 0};

int write_fp32_sidecar(axg_ctx *ctx, const std::string &path, uint32_t chk_crc) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) return axg_set_error(ctx, AXG_ERR_IO, "cannot open " + path);
  const int64_t hdr[3] = {ctx->n, ctx->p.gw_mode == AXG_GW_UIJ ? 1 : 0, (int64_t)chk_crc};
  uint32_t crc = crc32_update(0, (const unsigned char *)kFp32Magic, 8);
  crc = crc32_update(crc, (const unsigned char *)hdr, sizeof(hdr));
  int rc = AXG_OK;
  if (std::fwrite(kFp32Magic, 1, 8, f) != 8 || std::fwrite(hdr, 1, sizeof(hdr), f) != sizeof(hdr))
    rc = axg_set_error(ctx, AXG_ERR_IO, "short write");
  std::vector<unsigned char> buf;
  for (const RawField &r : fp32_fields(ctx)) {
    if (rc != AXG_OK) break;
    buf.resize(r.bytes);
    if (cudaMemcpy(buf.data(), r.dev, r.bytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = axg_set_error(ctx, AXG_ERR_CUDA, "sidecar download");
      break;
    }
    if (std::fwrite(buf.data(), 1, r.bytes, f) != r.bytes) rc = axg_set_error(ctx, AXG_ERR_IO, "short write");
    crc = crc32_update(crc, buf.data(), r.bytes);
  }
  if (rc == AXG_OK && std::fwrite(&crc, 1, 4, f) != 4) rc = axg_set_error(ctx, AXG_ERR_IO, "short write");
  if (std::fclose(f) != 0 && rc == AXG_OK) rc = axg_set_error(ctx, AXG_ERR_IO, "close failed");
  return rc;
}

// 1: restored, 0: no sidecar of this checkpoint, < 0: error (a sidecar of
// this checkpoint must verify)
int read_fp32_sidecar(axg_ctx *ctx, const std::string &path, uint32_t chk_crc) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return 0;
  char magic[8];
  int64_t hdr[3];
  int rc = AXG_OK;
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kFp32Magic, 8) != 0 ||
      std::fread(hdr, 1, sizeof(hdr), f) != sizeof(hdr)) {
    std::fclose(f);
    return axg_set_error(ctx, AXG_ERR_IO, "FP32 sidecar: bad header");
  }
  if (hdr[0] != ctx->n || hdr[1] != (ctx->p.gw_mode == AXG_GW_UIJ ? 1 : 0)) {
    std::fclose(f);
    return axg_set_error(ctx, AXG_ERR_IO, "FP32 sidecar: lattice or u_ij mismatch");
  }
  if (hdr[2] != (int64_t)chk_crc) {  // written beside an older checkpoint of this path
    std::fclose(f);
    return 0;
  }
  uint32_t crc = crc32_update(0, (const unsigned char *)magic, 8);
  crc = crc32_update(crc, (const unsigned char *)hdr, sizeof(hdr));
  const std::vector<RawField> fields = fp32_fields(ctx);
  std::vector<std::vector<unsigned char>> data(fields.size());
  for (size_t k = 0; k < fields.size() && rc == AXG_OK; ++k) {
    data[k].resize(fields[k].bytes);
    if (std::fread(data[k].data(), 1, fields[k].bytes, f) != fields[k].bytes)
      rc = axg_set_error(ctx, AXG_ERR_IO, "FP32 sidecar too short");
    else
      crc = crc32_update(crc, data[k].data(), fields[k].bytes);
  }
  uint32_t want = 0;
  if (rc == AXG_OK && std::fread(&want, 1, 4, f) != 4) rc = axg_set_error(ctx, AXG_ERR_IO, "FP32 sidecar too short");
  std::fclose(f);
  if (rc != AXG_OK) return rc;
  if (want != crc) return axg_set_error(ctx, AXG_ERR_IO, "FP32 sidecar CRC mismatch");
  for (size_t k = 0; k < fields.size(); ++k)
    AXG_CUDA_TRY(ctx, cudaMemcpy(fields[k].dev, data[k].data(), fields[k].bytes, cudaMemcpyHostToDevice));
  return 1;
}
}  // namespace

int axg_write_chk(axg_ctx *ctx, const char *path) {
  if (!valid_ctx(ctx) || !path) return AXG_ERR_ARG;
  const int64_t n3 = ctx->n3;
  std::vector<double> buf((size_t)(2 * n3));
  FILE *f = std::fopen(path, "wb");
  if (!f) return axg_set_error(ctx, AXG_ERR_IO, std::string("cannot open ") + path);
  uint32_t crc = 0;
  int rc = AXG_OK;
  for (int which = 0; which < 2 && rc == AXG_OK; ++which) {
    rc = which == 0 ? axg_download(ctx, buf.data(), nullptr, ctx->n * ctx->n, 0)
                    : axg_download(ctx, nullptr, buf.data(), ctx->n * ctx->n, 0);
    if (rc == AXG_OK) {
      size_t bytes = buf.size() * sizeof(double);
      if (std::fwrite(buf.data(), 1, bytes, f) != bytes) rc = axg_set_error(ctx, AXG_ERR_IO, "short write");
      crc = crc32_update(crc, (const unsigned char *)buf.data(), bytes);
    }
  }
  if (rc == AXG_OK && ctx->p.gw_mode == AXG_GW_UIJ) {
    std::vector<double> ub((size_t)(6 * n3)), udb((size_t)(6 * n3));
    rc = axg_download_uij(ctx, ub.data(), udb.data());
    for (auto *v : {&ub, &udb}) {
      if (rc != AXG_OK) break;
      size_t bytes = v->size() * sizeof(double);
      if (std::fwrite(v->data(), 1, bytes, f) != bytes) rc = axg_set_error(ctx, AXG_ERR_IO, "short write");
      crc = crc32_update(crc, (const unsigned char *)v->data(), bytes);
    }
  }
  if (std::fclose(f) != 0 && rc == AXG_OK) rc = axg_set_error(ctx, AXG_ERR_IO, "close failed");
  if (rc != AXG_OK) return rc;
  std::string cpath = std::string(path) + ".crc";
  FILE *c = std::fopen(cpath.c_str(), "w");
  if (!c) return axg_set_error(ctx, AXG_ERR_IO, "cannot open " + cpath);
  std::fprintf(c, "%08x %lld\n", crc, (long long)ctx->n);
  std::fclose(c);
  if (ctx->p.precision == AXG_PREC_FP32_MIXED) {
    AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return write_fp32_sidecar(ctx, std::string(path) + ".fp32", crc);
  }
  // an FP32 sidecar left by an earlier checkpoint of this path is stale
  std::remove((std::string(path) + ".fp32").c_str());
  return AXG_OK;
}

int axg_read_chk(axg_ctx *ctx, const char *path) {
  if (!valid_ctx(ctx) || !path) return AXG_ERR_ARG;
  const int64_t n3 = ctx->n3;
  FILE *f = std::fopen(path, "rb");
  if (!f) return axg_set_error(ctx, AXG_ERR_IO, std::string("cannot open ") + path);
  std::vector<double> phi((size_t)(2 * n3)), phid((size_t)(2 * n3));
  uint32_t crc = 0;
  int rc = AXG_OK;
  for (auto *v : {&phi, &phid}) {
    size_t bytes = v->size() * sizeof(double);
    if (std::fread(v->data(), 1, bytes, f) != bytes) {
      rc = axg_set_error(ctx, AXG_ERR_IO, "checkpoint too short");
      break;
    }
    crc = crc32_update(crc, (const unsigned char *)v->data(), bytes);
  }
  std::vector<double> ub, udb;
  if (rc == AXG_OK && ctx->p.gw_mode == AXG_GW_UIJ) {
    ub.resize((size_t)(6 * n3));
    udb.resize((size_t)(6 * n3));
    for (auto *v : {&ub, &udb}) {
      size_t bytes = v->size() * sizeof(double);
      if (std::fread(v->data(), 1, bytes, f) != bytes) {
        rc = axg_set_error(ctx, AXG_ERR_IO, "checkpoint too short (u_ij)");
        break;
      }
      crc = crc32_update(crc, (const unsigned char *)v->data(), bytes);
    }
  }
  std::fclose(f);
  if (rc != AXG_OK) return rc;
  std::string cpath = std::string(path) + ".crc";
  FILE *c = std::fopen(cpath.c_str(), "r");
  if (c) {
    unsigned int want = 0;
    long long nn = 0;
    int got = std::fscanf(c, "%x %lld", &want, &nn);
    std::fclose(c);
    if (got >= 1 && want != crc) return axg_set_error(ctx, AXG_ERR_IO, "checkpoint CRC mismatch");
    if (got == 2 && nn != ctx->n) return axg_set_error(ctx, AXG_ERR_IO, "checkpoint lattice size mismatch");
  }
  AXG_TRY(axg_upload(ctx, phi.data(), phid.data(), ctx->n * ctx->n, 0));
  if (ctx->p.gw_mode == AXG_GW_UIJ) AXG_TRY(axg_upload_uij(ctx, ub.data(), udb.data()));
  if (ctx->p.precision == AXG_PREC_FP32_MIXED) {
    // the raw FP32 state, when its sidecar is there, replaces the converted one
    AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    const int r = read_fp32_sidecar(ctx, std::string(path) + ".fp32", crc);
    if (r < 0) return r;
  }
  return AXG_OK;
}

int axg_write_param_chk(const char *path, int64_t idx, double tau, int flag_defects) {
  if (!path) return AXG_ERR_ARG;
  FILE *f = std::fopen(path, "w");
  if (!f) return AXG_ERR_IO;
  // write_chk (evolve.f90:410): idx, tau, flag  ('(I,E,L)')
  std::fprintf(f, "%lld %.17E %c\n", (long long)idx, tau, flag_defects ? 'T' : 'F');
  std::fclose(f);
  return AXG_OK;
}

int axg_read_param_chk(const char *path, int64_t *idx, double *tau, int *flag_defects) {
  if (!path || !idx || !tau || !flag_defects) return AXG_ERR_ARG;
  FILE *f = std::fopen(path, "r");
  if (!f) return AXG_ERR_IO;
  long long i = 0;
  double t = 0;
  char fl[8] = {0};
  int got = std::fscanf(f, "%lld %lf %7s", &i, &t, fl);
  std::fclose(f);
  if (got < 2) return AXG_ERR_IO;
  *idx = i;
  *tau = t;
  *flag_defects = (got == 3 && (fl[0] == 'T' || fl[0] == 't' || fl[0] == '1')) ? 1 : 0;
  return AXG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// tile selection and autotuning of the fused kernel
// ---------------------------------------------------------------------------
extern "C" {

int axg_tile_count(void) { return axg_evo_tile_count(); }

int axg_tile_info(int i, int32_t *tx, int32_t *ty, int32_t *zc, int32_t *pointwise_tma) {
  if (i < 0 || i >= axg_evo_tile_count() || !tx || !ty || !zc) return AXG_ERR_ARG;
  axg_tile_cfg t = axg_evo_tile(i);
  *tx = t.tx;
  *ty = t.ty;
  *zc = t.zc;
  if (pointwise_tma) *pointwise_tma = t.pw;
  return AXG_OK;
}

int axg_set_tile(axg_ctx *ctx, int cfg) {
  if (!ctx) return AXG_ERR_ARG;
  if (cfg == -1) {
    ctx->tile_cfg = -1;
    return AXG_OK;
  }
  if (!axg_evo_tile_supported(ctx, cfg))
    return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "tile " + std::to_string(cfg) + " unsupported for this lattice");
  ctx->tile_cfg = cfg;
  return AXG_OK;
}

int axg_autotune(axg_ctx *ctx, int steps, int *best_cfg, double *best_ms) {
  if (!ctx || steps < 1) return AXG_ERR_ARG;
  if (ctx->p.precision == AXG_PREC_FP64_PLAIN)
    return axg_set_error(ctx, AXG_ERR_STATE, "the FP64-plain path has no tiled kernel");
  const size_t rs = ctx->elem, n3 = (size_t)ctx->n3;
  const bool uij = ctx->p.gw_mode == AXG_GW_UIJ;
  // snapshot of everything a fused step modifies
  struct Buf { void *src; size_t bytes; void *copy; };
  std::vector<Buf> bufs = {{ctx->phi[ctx->cur], n3 * 2 * rs, nullptr}, {ctx->phid, n3 * 2 * rs, nullptr}};
  if (ctx->cphi) bufs.push_back({ctx->cphi, n3 * 2 * rs, nullptr});
  if (uij) {
    bufs.push_back({ctx->u[ctx->cur], n3 * 6 * rs, nullptr});
    bufs.push_back({ctx->ud, n3 * 6 * rs, nullptr});
    if (ctx->cu) bufs.push_back({ctx->cu, n3 * 6 * rs, nullptr});
  }
  int rc = AXG_OK;
  for (auto &b : bufs) {
    if ((rc = axg_alloc(ctx, &b.copy, b.bytes, "autotune snapshot"))) break;
    cudaMemcpyAsync(b.copy, b.src, b.bytes, cudaMemcpyDeviceToDevice, ctx->stream);
  }
  const int cur0 = ctx->cur, saved_cfg = ctx->tile_cfg;
  const bool saved_kt = ctx->ktiming;
  ctx->ktiming = false;
  int best = -1;
  double best_t = 1e300;
  const double t0 = 10.0, dt = 1e-3;
  for (int cfg = 0; rc == AXG_OK && cfg < axg_evo_tile_count(); ++cfg) {
    if (!axg_evo_tile_supported(ctx, cfg)) continue;
    ctx->tile_cfg = cfg;
    rc = axg_evo_kick_drift(ctx, t0, dt, dt);  // warm-up (and TMA descriptors)
    if (rc) break;
    cudaEventRecord(ctx->user_ev[6], ctx->stream);
    for (int s = 0; s < steps && rc == AXG_OK; ++s) rc = axg_evo_kick_drift(ctx, t0, dt, dt);
    cudaEventRecord(ctx->user_ev[7], ctx->stream);
    cudaEventSynchronize(ctx->user_ev[7]);
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->user_ev[6], ctx->user_ev[7]);
    if (rc == AXG_OK) rc = axg_evo_check_error(ctx);
    if (rc == AXG_OK && ms / steps < best_t) {
      best_t = ms / steps;
      best = cfg;
    }
    // restore the state
    ctx->cur = cur0;
    for (auto &b : bufs) cudaMemcpyAsync(b.src, b.copy, b.bytes, cudaMemcpyDeviceToDevice, ctx->stream);
  }
  cudaStreamSynchronize(ctx->stream);
  for (auto &b : bufs) axg_free(ctx, &b.copy);
  ctx->ktiming = saved_kt;
  ctx->tile_cfg = (rc == AXG_OK && best >= 0) ? best : saved_cfg;
  if (rc != AXG_OK) return rc;
  if (best < 0) return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "no supported tile for this lattice");
  if (best_cfg) *best_cfg = best;
  if (best_ms) *best_ms = best_t;
  return AXG_OK;
}

}  // extern "C"
