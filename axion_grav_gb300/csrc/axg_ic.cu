// axg_ic.cu -- initial conditions (initial.f90) and FP64 volume moments.
#include <cmath>

#include "axg_detmath.h"
#include "axg_internal.h"

namespace {

constexpr double kRefPi = 3.14159265359;
constexpr double kRefTwoPi = 2 * kRefPi;
constexpr double kThrmSigma = 2.449489742783178;

__device__ __forceinline__ int64_t kint(int64_t j, int64_t n) { return (j + n / 2) % n - n / 2; }

__device__ __forceinline__ void gauss_pair(uint64_t seed, uint32_t stream, uint32_t real,
                                           uint64_t index, double *g0, double *g1) {
  axd_u32x4 r = axd_draw(seed, stream, real, index);
  const double u1 = axd_u01_open0(r.v[0], r.v[1]);
  const double u2 = axd_u01(r.v[2], r.v[3]);
  const double rad = sqrt(-2.0 * log(u1));
  double s, c;
  sincos(6.283185307179586 * u2, &s, &c);
  *g0 = rad * c;
  *g1 = rad * s;
}

// Seeded flat spectrum: complex normal on |k| <= kcut (Fourier index order).
__global__ void k_ic_flat_modes(double2 *out, int n, double dwav, double kcut, uint64_t seed,
                                uint32_t real) {
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    const int64_t qx = kint(s % n, n), qy = kint((s / n) % n, n), qz = kint(s / n2, n);
    const double q = sqrt((double)(qx * qx + qy * qy + qz * qz)) * dwav;
    double g0 = 0.0, g1 = 0.0;
    if (q <= kcut) gauss_pair(seed, 0u, real, (uint64_t)s, &g0, &g1);
    out[s] = make_double2(g0, g1);
  }
}

// initial_phi_phidot (initial.f90:372-390) applied to Philox normals.
__global__ void k_ic_thermal_modes(double2 *out, int n, double dwav, double dv_wav,
                                   double tau_ini, double sigma_cr, int ip, uint64_t seed,
                                   uint32_t real) {
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    double g0, g1;
    gauss_pair(seed, (uint32_t)ip, real, (uint64_t)s, &g0, &g1);
    const double xr = g0 * dv_wav, xi = g1 * dv_wav;
    const int64_t qx = kint(s % n, n), qy = kint((s / n) % n, n), qz = kint(s / n2, n);
    double wav2 = sqrt((double)(qx * qx + qy * qy + qz * qz)) * dwav;
    wav2 = wav2 / tau_ini / sigma_cr;
    wav2 = wav2 * wav2;
    const double thrm = kThrmSigma / tau_ini;
    const double m2 = (thrm * thrm - kThrmSigma * kThrmSigma) / 3;
    const double osc = sqrt(m2 + wav2);
    double fbe = exp(-osc / thrm);
    fbe = fbe / (1 - fbe);
    const double var = fbe * osc / dv_wav / sigma_cr;
    double f = sqrt(var / 2);
    if (ip == 1) f = f / (osc * sigma_cr);
    out[s] = make_double2(xr * f, xi * f);
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__global__ void k_sum_abs2(const double2 *a, int64_t n3, double *out) {
  double acc = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    const double2 v = a[s];
    acc += v.x * v.x + v.y * v.y;
  }
  acc = warp_sum(acc);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) atomicAdd(out, v);
  }
}

__global__ void k_scale_c128(double2 *a, int64_t n3, double f) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    double2 v = a[s];
    v.x *= f;
    v.y *= f;
    a[s] = v;
  }
}

__global__ void k_c128_to_f32_comp(const double2 *src, float2 *dst, float2 *comp, int64_t n3) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    const double2 v = src[s];
    const float2 f = make_float2((float)v.x, (float)v.y);
    dst[s] = f;
    if (comp) comp[s] = make_float2((float)((double)f.x - v.x), (float)((double)f.y - v.y));
  }
}

// Volume moments: <|phi|^2>, <|phi'|^2>, <|grad phi|^2> (forward differences), <V>
template <typename V>
__global__ void k_moments(const V *phi, const V *phid, int n, double idx2, double A, double B,
                          double C, double D, double *out) {
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    const int64_t ix = s % n, iy = (s / n) % n, iz = s / n2;
    const V c = phi[s], d = phid[s];
    const double a = (double)c.x, b = (double)c.y;
    const double m = a * a + b * b;
    a0 += m;
    a1 += (double)d.x * (double)d.x + (double)d.y * (double)d.y;
    const int64_t nb[3] = {iz * n2 + iy * n + (ix + 1 == n ? 0 : ix + 1),
                           iz * n2 + (iy + 1 == n ? 0 : iy + 1) * n + ix,
                           (iz + 1 == n ? 0 : iz + 1) * n2 + iy * n + ix};
    double g = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const V e = phi[nb[k]];
      const double dr = (double)e.x - a, di = (double)e.y - b;
      g += dr * dr + di * di;
    }
    a2 += g * idx2;
    a3 += 0.5 * A * m * m + B * m + 2 * C * a + D * (a * a - b * b);
  }
  __shared__ double sh[4][32];
  double v[4] = {warp_sum(a0), warp_sum(a1), warp_sum(a2), warp_sum(a3)};
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 4; ++k) sh[k][threadIdx.x >> 5] = v[k];
  __syncthreads();
  if (threadIdx.x < 32) {
    for (int k = 0; k < 4; ++k) {
      double x = threadIdx.x < (blockDim.x >> 5) ? sh[k][threadIdx.x] : 0.0;
      x = warp_sum(x);
      if (threadIdx.x == 0) atomicAdd(&out[k], x);
    }
  }
}

int grid_for(int64_t count) {
  int64_t b = (count + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

// Zero every evolved quantity except phi (and phidot when keep_phid).
int zero_state(axg_ctx *ctx, bool keep_phid) {
  const size_t n3 = (size_t)ctx->n3, rs = ctx->elem;
  if (!keep_phid) AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->phid, 0, n3 * 2 * rs, ctx->stream));
  if (ctx->cphi) AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->cphi, 0, n3 * 2 * rs, ctx->stream));
  for (void *q : {ctx->u[0], ctx->u[1], ctx->ud, ctx->cu})
    if (q) AXG_CUDA_TRY(ctx, cudaMemsetAsync(q, 0, n3 * 6 * rs, ctx->stream));
  if (ctx->acc) AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->acc, 0, (size_t)ctx->acc_stride * 64, ctx->stream));
  return AXG_OK;
}

// Store a complex128 device field into phi (or phidot) of the context.
int store_field(axg_ctx *ctx, const double2 *src, bool is_phid) {
  const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
  void *dst = is_phid ? ctx->phid : ctx->phi[ctx->cur];
  if (fp32) {
    AXG_LAUNCH(ctx, "ic_to_fp32", k_c128_to_f32_comp, grid_for(ctx->n3), 256, 0, src,
               (float2 *)dst, is_phid ? nullptr : (float2 *)ctx->cphi, ctx->n3);
  } else if ((const void *)src != dst) {
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(dst, src, (size_t)ctx->n3 * 16, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return AXG_OK;
}

}  // namespace

int axg_ic_gauss(axg_ctx *ctx, double kcut, uint32_t realisation) {
  const int n = (int)ctx->n;
  const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
  double2 *buf = nullptr;
  if (fp32) AXG_TRY(axg_alloc(ctx, (void **)&buf, (size_t)ctx->n3 * 16, "ic buffer"));
  else buf = (double2 *)ctx->phi[ctx->cur];
  int rc = AXG_OK;
  cufftHandle plan = 0;
  bool planned = false;
  do {
    const double dwav = kRefTwoPi / ctx->p.dspa / n;
    AXG_LAUNCH(ctx, "ic_flat_modes", k_ic_flat_modes, grid_for(ctx->n3), 256, 0, buf, n, dwav,
               kcut, (uint64_t)ctx->p.seed, realisation);
    if (cufftPlan3d(&plan, n, n, n, CUFFT_Z2Z) != CUFFT_SUCCESS) {
      rc = axg_set_error(ctx, AXG_ERR_CUDA, "cufftPlan3d (ic)");
      break;
    }
    planned = true;
    cufftSetStream(plan, ctx->stream);
    if (cufftExecZ2Z(plan, (cufftDoubleComplex *)buf, (cufftDoubleComplex *)buf, CUFFT_INVERSE) !=
        CUFFT_SUCCESS) {
      rc = axg_set_error(ctx, AXG_ERR_CUDA, "cufftExecZ2Z (ic)");
      break;
    }
    cudaMemsetAsync(ctx->d_red, 0, 8, ctx->stream);
    AXG_LAUNCH(ctx, "ic_sum_abs2", k_sum_abs2, 152 * 4, 256, 0, buf, ctx->n3, ctx->d_red);
    double sum = 0.0;
    cudaMemcpyAsync(&sum, ctx->d_red, 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
      rc = axg_set_error(ctx, AXG_ERR_CUDA, "ic sync");
      break;
    }
    const double mean = sum / (double)ctx->n3;
    const double scale = mean > 0 ? ctx->p.vev / std::sqrt(mean) : 0.0;
    AXG_LAUNCH(ctx, "ic_scale", k_scale_c128, grid_for(ctx->n3), 256, 0, buf, ctx->n3, scale);
    rc = store_field(ctx, buf, false);
    if (rc == AXG_OK) rc = zero_state(ctx, false);
  } while (0);
  if (planned) cufftDestroy(plan);
  if (fp32) {
    cudaStreamSynchronize(ctx->stream);
    axg_free(ctx, (void **)&buf);
  }
  ctx->flags_valid = false;
  if (rc == AXG_OK) AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return rc;
}

int axg_ic_therm(axg_ctx *ctx, double tau_ini, uint32_t realisation) {
  const int n = (int)ctx->n;
  double2 *buf = nullptr;
  AXG_TRY(axg_alloc(ctx, (void **)&buf, (size_t)ctx->n3 * 16, "ic buffer"));
  int rc = AXG_OK;
  cufftHandle plan = 0;
  bool planned = false;
  do {
    if (cufftPlan3d(&plan, n, n, n, CUFFT_Z2Z) != CUFFT_SUCCESS) {
      rc = axg_set_error(ctx, AXG_ERR_CUDA, "cufftPlan3d (ic)");
      break;
    }
    planned = true;
    cufftSetStream(plan, ctx->stream);
    const double dwav = kRefTwoPi / ctx->p.dspa / n;
    const double dv_wav = std::pow(dwav / kRefTwoPi, 3);
    for (int ip = 1; ip <= 2 && rc == AXG_OK; ++ip) {
      AXG_LAUNCH(ctx, "ic_thermal_modes", k_ic_thermal_modes, grid_for(ctx->n3), 256, 0, buf, n,
                 dwav, dv_wav, tau_ini, ctx->p.sigma_cr, ip, (uint64_t)ctx->p.seed, realisation);
      if (cufftExecZ2Z(plan, (cufftDoubleComplex *)buf, (cufftDoubleComplex *)buf,
                       CUFFT_FORWARD) != CUFFT_SUCCESS) {
        rc = axg_set_error(ctx, AXG_ERR_CUDA, "cufftExecZ2Z (ic)");
        break;
      }
      rc = store_field(ctx, buf, ip == 2);
    }
    if (rc == AXG_OK) rc = zero_state(ctx, true);
  } while (0);
  if (planned) cufftDestroy(plan);
  cudaStreamSynchronize(ctx->stream);
  axg_free(ctx, (void **)&buf);
  ctx->flags_valid = false;
  return rc;
}

int axg_moments(axg_ctx *ctx, double tau, double out[4]) {
  double f[4], pot[4];
  axg_kick_coeffs(&ctx->p, tau, 0.0, f, pot);
  AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_red, 0, 4 * 8, ctx->stream));
  const double idx2 = 1.0 / (ctx->p.dspa * ctx->p.dspa);
  if (ctx->p.precision == AXG_PREC_FP32_MIXED) {
    AXG_LAUNCH(ctx, "moments_fp32", k_moments<float2>, 152 * 8, 256, 0,
               (const float2 *)ctx->phi[ctx->cur], (const float2 *)ctx->phid, (int)ctx->n, idx2,
               pot[0], pot[1], pot[2], pot[3], ctx->d_red);
  } else {
    AXG_LAUNCH(ctx, "moments_fp64", k_moments<double2>, 152 * 8, 256, 0,
               (const double2 *)ctx->phi[ctx->cur], (const double2 *)ctx->phid, (int)ctx->n, idx2,
               pot[0], pot[1], pot[2], pot[3], ctx->d_red);
  }
  double h[4];
  AXG_CUDA_TRY(ctx, cudaMemcpyAsync(h, ctx->d_red, 32, cudaMemcpyDeviceToHost, ctx->stream));
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < 4; ++k) out[k] = h[k] / (double)ctx->n3;
  return AXG_OK;
}

extern "C" {
int axg_ic_gaussian_flat(axg_ctx *ctx, double kcut, uint32_t realisation) {
  if (!ctx || !(kcut > 0)) return AXG_ERR_ARG;
  return axg_ic_gauss(ctx, kcut, realisation);
}
int axg_ic_thermal(axg_ctx *ctx, double tau_ini, uint32_t realisation) {
  if (!ctx || !(tau_ini > 0)) return AXG_ERR_ARG;
  return axg_ic_therm(ctx, tau_ini, realisation);
}
int axg_field_moments(axg_ctx *ctx, double tau, double out[4]) {
  if (!ctx || !out || !(tau > 0)) return AXG_ERR_ARG;
  return axg_moments(ctx, tau, out);
}
}
