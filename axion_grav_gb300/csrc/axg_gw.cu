// axg_gw.cu -- gravitational waves (grav_waves.f90) on the GPU.
//
// Green's-function mode (AXG_GW_GREEN), per kick (grav_waves.f90:193-255):
//   1. k_gw_source : the six real sources S_ij = d_i phi d_j phi* + c.c. with
//                    d_i phi = (phi(x+e_i) - phi(x-e_i)) / (2 dx), one pass
//                    over phi writing 6 x N^3 reals (the reference's arr_dphi
//                    is never materialised);
//   2. cuFFT D2Z batched x6: the reference's backward C2C of a real field is
//                    the conjugate of the forward half spectrum;
//   3. k_gw_accumulate: one pass over the full spectrum applying, in the
//                    reference's (i, j) order, the four accumulator updates of
//                    all six components (grav_waves.f90:239-242), with the
//                    polarisation tensor of get_comwav_grav (157-191) computed
//                    in registers.  compat = REF reproduces the cross-wired
//                    (2,1)/(1,2) updates literally.
// Spectra: shell histograms in FP64 (grav_waves.f90:257-321), 25 linear bins
// or log bins; the u_ij path (AXG_GW_UIJ) FFTs w = tau u and w' = u + tau u'
// (R2C, FP32 for the FP32-mixed path), TT-projects per k and accumulates
// 1/2 sum_ij (|W'_TT|^2 + k^2 |W_TT|^2), the continuum-equivalent of the
// Green's-function numerator.
#include <cmath>
#include <vector>

#include "axg_detmath.h"
#include "axg_internal.h"

namespace {

constexpr double kRefPi = 3.14159265359;
constexpr double kRefTwoPi = 2 * kRefPi;
// potential.f90:13-23
constexpr double kBigHInMstar = 2.1332e-42 / 2.435e18;

__device__ __forceinline__ int kint(int j, int n) { return (j + n / 2) % n - n / 2; }

template <typename V>
__global__ void k_gw_source(const V *__restrict__ phi, int n, double d, double *__restrict__ src) {
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    const int ix = (int)(s % n), iy = (int)((s / n) % n), iz = (int)(s / n2);
    const int64_t base = iz * n2 + (int64_t)iy * n;
    const int64_t sx2 = base + (ix + 1 == n ? 0 : ix + 1), sx1 = base + (ix == 0 ? n - 1 : ix - 1);
    const int64_t sy2 = iz * n2 + (int64_t)(iy + 1 == n ? 0 : iy + 1) * n + ix;
    const int64_t sy1 = iz * n2 + (int64_t)(iy == 0 ? n - 1 : iy - 1) * n + ix;
    const int64_t sz2 = (int64_t)(iz + 1 == n ? 0 : iz + 1) * n2 + (int64_t)iy * n + ix;
    const int64_t sz1 = (int64_t)(iz == 0 ? n - 1 : iz - 1) * n2 + (int64_t)iy * n + ix;
    const int64_t a[3] = {sx2, sy2, sz2}, b[3] = {sx1, sy1, sz1};
    double dr[3], di[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const V pa = phi[a[k]], pb = phi[b[k]];
      dr[k] = AXD_DIV(AXD_SUB((double)pa.x, (double)pb.x), d);
      di[k] = AXD_DIV(AXD_SUB((double)pa.y, (double)pb.y), d);
    }
    int c = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j <= i; ++j, ++c) {
        const double r1 = AXD_ADD(AXD_MUL(dr[i], dr[j]), AXD_MUL(di[i], di[j]));
        src[c * n3 + s] = AXD_ADD(r1, r1);
      }
  }
}

// complex helpers in the reference's evaluation order
struct C2 {
  double r, i;
};
__device__ __forceinline__ C2 cmul(C2 a, C2 b) {
  return {AXD_SUB(AXD_MUL(a.r, b.r), AXD_MUL(a.i, b.i)), AXD_ADD(AXD_MUL(a.r, b.i), AXD_MUL(a.i, b.r))};
}
__device__ __forceinline__ C2 cadd(C2 a, C2 b) { return {AXD_ADD(a.r, b.r), AXD_ADD(a.i, b.i)}; }
__device__ __forceinline__ C2 rmul(double s, C2 a) { return {AXD_MUL(s, a.r), AXD_MUL(s, a.i)}; }

__global__ void k_gw_accumulate(const double2 *__restrict__ srcF, int n, double dwav, double tau,
                                double dw, int ref_compat, double2 *__restrict__ acc) {
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  const int nh = n / 2 + 1;
  const int64_t nhalf = (int64_t)n * n * nh;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    const int ix = (int)(s % n), iy = (int)((s / n) % n), iz = (int)(s / n2);
    // backward transform of a real field = conj(forward); forward half spectrum
    // holds kx <= n/2, the rest by Hermitian symmetry F(-k) = conj F(k)
    int64_t hidx;
    bool conj_back;
    if (ix < nh) {
      hidx = ((int64_t)iz * n + iy) * nh + ix;
      conj_back = true;
    } else {
      const int jx = n - ix, jy = iy == 0 ? 0 : n - iy, jz = iz == 0 ? 0 : n - iz;
      hidx = ((int64_t)jz * n + jy) * nh + jx;
      conj_back = false;
    }
    // get_comwav_grav (grav_waves.f90:157-191)
    double qh[3] = {(double)kint(ix, n), (double)kint(iy, n), (double)kint(iz, n)};
    double qq = AXD_ADD(AXD_MUL(qh[0], qh[0]), AXD_MUL(qh[1], qh[1]));
    qq = AXD_ADD(qq, AXD_MUL(qh[2], qh[2]));
    qq = AXD_SQRT(qq);
    C2 p[3] = {{0, 0}, {0, 0}, {0, 0}};
    const bool nonzero = qq > 0.0;
    if (nonzero) {
      for (int k = 0; k < 3; ++k) qh[k] = AXD_DIV(qh[k], qq);
      const double r = AXD_SQRT(AXD_ADD(AXD_MUL(qh[0], qh[0]), AXD_MUL(qh[1], qh[1])));
      double c, sn;
      if (r > 0.0) {
        c = AXD_DIV(qh[0], r);
        sn = AXD_DIV(qh[1], r);
      } else {
        c = 1.0;
        sn = 0.0;
      }
      p[0] = {AXD_MUL(qh[2], c), -sn};
      p[1] = {AXD_MUL(qh[2], sn), c};
      p[2] = {-r, 0.0};
    }
    const double q = AXD_MUL(AXD_MUL(qq, dwav), tau);
    double sq, cq;
    sincos(q, &sq, &cq);
    C2 a11 = {acc[s].x, acc[s].y}, a21 = {acc[n3 + s].x, acc[n3 + s].y},
       a12 = {acc[2 * n3 + s].x, acc[2 * n3 + s].y}, a22 = {acc[3 * n3 + s].x, acc[3 * n3 + s].y};
    int comp = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int j = 0; j <= i; ++j, ++comp) {
        C2 pol = {0.0, 0.0};
        if (nonzero) {
          pol = cmul(p[i], p[j]);
          if (i == j) pol = {AXD_DIV(pol.r, 2.0), AXD_DIV(pol.i, 2.0)};
        }
        const double2 f = srcF[comp * nhalf + hidx];
        const C2 S = {f.x, conj_back ? -f.y : f.y};
        const C2 pp = rmul(dw, pol);
        const C2 pn = {pp.r, -pp.i};
        a11 = cadd(a11, cmul(rmul(cq, pp), S));
        const C2 t21 = cmul(rmul(sq, pp), S);
        const C2 t12 = cmul(rmul(cq, pn), S);
        if (ref_compat) {
          a21 = cadd(a12, t21);
          a12 = cadd(a21, t12);
        } else {
          a21 = cadd(a21, t21);
          a12 = cadd(a12, t12);
        }
        a22 = cadd(a22, cmul(rmul(sq, pn), S));
      }
    }
    acc[s] = make_double2(a11.r, a11.i);
    acc[n3 + s] = make_double2(a21.r, a21.i);
    acc[2 * n3 + s] = make_double2(a12.r, a12.i);
    acc[3 * n3 + s] = make_double2(a22.r, a22.i);
  }
}

// ---------------- shell histograms ----------------
constexpr int kMaxBins = 256;

__device__ __forceinline__ int lin_bin(double q, double dq, int nb) {
  if (!(q > 0.0)) return -1;
  const double id = round(AXD_ADD(AXD_DIV(q, dq), 0.5));
  if (id >= 1 && id <= nb) return (int)id - 1;
  return -1;
}
__device__ __forceinline__ int log_bin(double q, double e0, double ln_ratio, int nb, const double *edges) {
  if (!(q > 0.0) || q < edges[0] || q > edges[nb]) return -1;
  int b = (int)floor(log(q / e0) / ln_ratio * nb);
  if (b >= nb) b = nb - 1;
  if (b < 0) b = 0;
  while (b > 0 && q < edges[b]) --b;
  while (b < nb - 1 && q >= edges[b + 1]) ++b;
  return b;
}

// Green accumulators -> numer / denom per bin
__global__ void k_gw_bin_green(const double2 *__restrict__ acc, int n, double dwav, double dq, int nb,
                               int logmode, const double *__restrict__ edges, double *__restrict__ numer,
                               double *__restrict__ denom) {
  __shared__ double sn[kMaxBins], sd[kMaxBins];
  __shared__ double se[kMaxBins + 1];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) sn[b] = sd[b] = 0.0;
  if (logmode)
    for (int b = threadIdx.x; b <= nb; b += blockDim.x) se[b] = edges[b];
  __syncthreads();
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  const double ln_ratio = logmode ? log(se[nb] / se[0]) : 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    const int ix = (int)(s % n), iy = (int)((s / n) % n), iz = (int)(s / n2);
    const double kx = kint(ix, n), ky = kint(iy, n), kz = kint(iz, n);
    double qq = AXD_ADD(AXD_MUL(kx, kx), AXD_MUL(ky, ky));
    qq = AXD_ADD(qq, AXD_MUL(kz, kz));
    const double q = AXD_MUL(AXD_SQRT(qq), dwav);
    const int b = logmode ? log_bin(q, se[0], ln_ratio, nb, se) : lin_bin(q, dq, nb);
    if (b < 0) continue;
    double v = 0.0;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const double2 z = acc[a * n3 + s];
      v += z.x * z.x + z.y * z.y;
    }
    atomicAdd(&sn[b], v);
    atomicAdd(&sd[b], 1.0);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    if (sd[b] != 0.0) {
      atomicAdd(&numer[b], sn[b]);
      atomicAdd(&denom[b], sd[b]);
    }
  }
}

// u_ij: 12 real fields (tau u_c, u_c + tau u'_c), scaled by dx^3 at use
template <typename V, typename R>
__global__ void k_uij_prepare(const R *__restrict__ u, const R *__restrict__ ud, const R *__restrict__ cu,
                              int64_t n3, double tau, R *__restrict__ w) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      double uv = (double)u[c * n3 + s];
      if (cu) uv -= (double)cu[c * n3 + s];
      const double udv = (double)ud[c * n3 + s];
      w[c * n3 + s] = (R)(tau * uv);
      w[(6 + c) * n3 + s] = (R)(uv + tau * udv);
    }
  }
}

// TT power of a complex symmetric 3x3 (components 11,21,22,31,32,33)
__device__ double tt_power(const double Ur[6], const double Ui[6], const double kh[3]) {
  const int idx[3][3] = {{0, 1, 3}, {1, 2, 4}, {3, 4, 5}};
  double P[3][3], Tr[3][3], Ti[3][3], Rr[3][3], Ri[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) P[a][b] = (a == b ? 1.0 : 0.0) - kh[a] * kh[b];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double sr = 0, si = 0;
      for (int c = 0; c < 3; ++c) {
        sr += P[a][c] * Ur[idx[c][b]];
        si += P[a][c] * Ui[idx[c][b]];
      }
      Tr[a][b] = sr;
      Ti[a][b] = si;
    }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double sr = 0, si = 0;
      for (int c = 0; c < 3; ++c) {
        sr += Tr[a][c] * P[c][b];
        si += Ti[a][c] * P[c][b];
      }
      Rr[a][b] = sr;
      Ri[a][b] = si;
    }
  const double trr = Rr[0][0] + Rr[1][1] + Rr[2][2], tri = Ri[0][0] + Ri[1][1] + Ri[2][2];
  double s = 0;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      const double vr = Rr[a][b] - 0.5 * P[a][b] * trr, vi = Ri[a][b] - 0.5 * P[a][b] * tri;
      s += vr * vr + vi * vi;
    }
  return s;
}

template <typename CV>
__global__ void k_uij_bin(const CV *__restrict__ F, int n, double dwav, double dv, double dq, int nb,
                          int logmode, const double *__restrict__ edges, double *__restrict__ numer,
                          double *__restrict__ denom) {
  __shared__ double sn[kMaxBins], sd[kMaxBins];
  __shared__ double se[kMaxBins + 1];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) sn[b] = sd[b] = 0.0;
  if (logmode)
    for (int b = threadIdx.x; b <= nb; b += blockDim.x) se[b] = edges[b];
  __syncthreads();
  const int nh = n / 2 + 1;
  const int64_t nhalf = (int64_t)n * n * nh;
  const double ln_ratio = logmode ? log(se[nb] / se[0]) : 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nhalf; h += stride) {
    const int ix = (int)(h % nh), iy = (int)((h / nh) % n), iz = (int)(h / ((int64_t)nh * n));
    const double kx = kint(ix, n), ky = kint(iy, n), kz = kint(iz, n);
    const double qq = sqrt(kx * kx + ky * ky + kz * kz);
    const double q = qq * dwav;
    const int b = logmode ? log_bin(q, se[0], ln_ratio, nb, se) : lin_bin(q, dq, nb);
    if (b < 0) continue;
    const double kh[3] = {kx / qq, ky / qq, kz / qq};
    double Ur[6], Ui[6], Dr[6], Di[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const CV a = F[c * nhalf + h], d = F[(6 + c) * nhalf + h];
      Ur[c] = (double)a.x * dv;
      Ui[c] = (double)a.y * dv;
      Dr[c] = (double)d.x * dv;
      Di[c] = (double)d.y * dv;
    }
    const double e0 = tt_power(Dr, Di, kh), e1 = tt_power(Ur, Ui, kh);
    const double wgt = (ix == 0 || 2 * ix == n) ? 1.0 : 2.0;  // Hermitian partner of the half spectrum
    atomicAdd(&sn[b], wgt * 0.5 * (e0 + q * q * e1));
    atomicAdd(&sd[b], wgt);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    if (sd[b] != 0.0) {
      atomicAdd(&numer[b], sn[b]);
      atomicAdd(&denom[b], sd[b]);
    }
  }
}

double gw_fact(const axg_params &p) {
  // grav_waves.f90:265-267
  const double dwav = kRefTwoPi / p.dspa / p.ngrid;
  const double dv_wav = std::pow(dwav / kRefTwoPi, 3);
  const double tc = p.tau_cr;
  const double tc6 = tc * tc * tc * tc * tc * tc;
  const double a4 = p.a_now * p.a_now * p.a_now * p.a_now;
  return 1 / tc6 / (kBigHInMstar * kBigHInMstar) / a4 / 3 / (kRefTwoPi * kRefTwoPi) * dv_wav;
}

int grid_for(int64_t count) {
  int64_t b = (count + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

int ensure_uij_fft(axg_ctx *ctx) {
  if (ctx->plan_u_ok) return AXG_OK;
  const int n = (int)ctx->n;
  const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
  const size_t rs = fp32 ? 4 : 8;
  const int64_t nhalf = (int64_t)n * n * (n / 2 + 1);
  // real input 12 x N^3 followed by complex output 12 x nhalf
  AXG_TRY(axg_alloc(ctx, &ctx->ubuf, (size_t)12 * ctx->n3 * rs + (size_t)12 * nhalf * 2 * rs, "u_ij FFT"));
  int dims[3] = {n, n, n};
  AXG_CUFFT_TRY(ctx, cufftPlanMany(&ctx->plan_u, 3, dims, nullptr, 1, (int)ctx->n3, nullptr, 1,
                                   (int)nhalf, fp32 ? CUFFT_R2C : CUFFT_D2Z, 12));
  AXG_CUFFT_TRY(ctx, cufftSetStream(ctx->plan_u, ctx->stream));
  ctx->plan_u_ok = true;
  return AXG_OK;
}

}  // namespace

int axg_gw_init(axg_ctx *ctx) {
  const int n = (int)ctx->n;
  const int64_t nhalf = (int64_t)n * n * (n / 2 + 1);
  AXG_TRY(axg_alloc(ctx, (void **)&ctx->acc, (size_t)ctx->n3 * 64, "GW accumulators"));
  AXG_TRY(axg_alloc(ctx, (void **)&ctx->gsrc, (size_t)ctx->n3 * 6 * 8, "GW sources"));
  AXG_TRY(axg_alloc(ctx, (void **)&ctx->gsrcF, (size_t)nhalf * 6 * 16, "GW source spectra"));
  AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->acc, 0, (size_t)ctx->n3 * 64, ctx->stream));
  int dims[3] = {n, n, n};
  AXG_CUFFT_TRY(ctx, cufftPlanMany(&ctx->plan_gsrc, 3, dims, nullptr, 1, (int)ctx->n3, nullptr, 1,
                                   (int)nhalf, CUFFT_D2Z, 6));
  ctx->plan_gsrc_ok = true;
  AXG_CUFFT_TRY(ctx, cufftSetStream(ctx->plan_gsrc, ctx->stream));
  return AXG_OK;
}

// grav_wave_integration (grav_waves.f90:193-255) on the current phi
int axg_gw_integration(axg_ctx *ctx, double tau, double dtau) {
  if (!ctx->acc) return axg_set_error(ctx, AXG_ERR_STATE, "gw_mode is not GREEN");
  const int n = (int)ctx->n;
  const double d = ctx->p.dspa * 2;
  if (ctx->p.precision == AXG_PREC_FP32_MIXED)
    AXG_LAUNCH(ctx, "gw_source_fp32", k_gw_source<float2>, grid_for(ctx->n3), 256, 0,
               (const float2 *)ctx->phi[ctx->cur], n, d, ctx->gsrc);
  else
    AXG_LAUNCH(ctx, "gw_source_fp64", k_gw_source<double2>, grid_for(ctx->n3), 256, 0,
               (const double2 *)ctx->phi[ctx->cur], n, d, ctx->gsrc);
  AXG_CUFFT_TRY(ctx, cufftExecD2Z(ctx->plan_gsrc, ctx->gsrc, (cufftDoubleComplex *)ctx->gsrcF));
  const double dv = ctx->p.dspa * ctx->p.dspa * ctx->p.dspa;
  const double dw = tau * dtau * dv * (ctx->p.sigma_cr * ctx->p.sigma_cr);
  const double dwav = kRefTwoPi / ctx->p.dspa / n;
  AXG_LAUNCH(ctx, "gw_accumulate", k_gw_accumulate, grid_for(ctx->n3), 256, 0, ctx->gsrcF, n, dwav,
             tau, dw, ctx->p.compat == AXG_COMPAT_REF ? 1 : 0, ctx->acc);
  return AXG_OK;
}

int axg_gw_spec(axg_ctx *ctx, double tau, int log_bins, double *wave, double *power, double *numer,
                double *denom) {
  const int n = (int)ctx->n;
  const int nb = log_bins ? ctx->p.gw_log_bins : ctx->p.num_bin_grav;
  if (nb < 1 || nb > kMaxBins) return axg_set_error(ctx, AXG_ERR_ARG, "GW bin count out of range (1..256)");
  const double dwav = kRefTwoPi / ctx->p.dspa / n;
  // bins: linear (grav_waves.f90:62-71) or log on [2 pi/(N dx), pi/dx]
  std::vector<double> edges(nb + 1);
  const double qmax = kRefPi / ctx->p.dspa;
  const double dq = qmax / nb;
  if (log_bins) {
    const double kmin = kRefTwoPi / ctx->p.dspa / n;
    for (int k = 0; k <= nb; ++k) edges[k] = kmin * std::pow(qmax / kmin, (double)k / nb);
  } else {
    edges[0] = 0.0;
    for (int k = 1; k <= nb; ++k) edges[k] = edges[k - 1] + dq;
  }
  // device scratch: numer[nb] denom[nb] edges[nb+1]
  if ((size_t)(3 * nb + 1) > ctx->red_cap) return axg_set_error(ctx, AXG_ERR_ARG, "too many bins");
  double *d_num = ctx->d_red, *d_den = ctx->d_red + nb, *d_edge = ctx->d_red + 2 * nb;
  AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_red, 0, sizeof(double) * 2 * nb, ctx->stream));
  AXG_CUDA_TRY(ctx, cudaMemcpyAsync(d_edge, edges.data(), sizeof(double) * (nb + 1), cudaMemcpyHostToDevice,
                                    ctx->stream));
  if (ctx->p.gw_mode == AXG_GW_GREEN) {
    AXG_LAUNCH(ctx, "gw_bin_green", k_gw_bin_green, 152 * 4, 256, 0, ctx->acc, n, dwav, dq, nb, log_bins,
               d_edge, d_num, d_den);
  } else if (ctx->p.gw_mode == AXG_GW_UIJ) {
    AXG_TRY(ensure_uij_fft(ctx));
    const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
    const int64_t nhalf = (int64_t)n * n * (n / 2 + 1);
    const double dv = ctx->p.dspa * ctx->p.dspa * ctx->p.dspa;
    if (fp32) {
      float *w = (float *)ctx->ubuf;
      float2 *F = (float2 *)(w + 12 * ctx->n3);
      AXG_LAUNCH(ctx, "uij_prepare_fp32", (k_uij_prepare<float2, float>), grid_for(ctx->n3), 256, 0,
                 (const float *)ctx->u[ctx->cur], (const float *)ctx->ud, (const float *)ctx->cu, ctx->n3,
                 tau, w);
      AXG_CUFFT_TRY(ctx, cufftExecR2C(ctx->plan_u, w, (cufftComplex *)F));
      AXG_LAUNCH(ctx, "uij_bin_fp32", k_uij_bin<float2>, 152 * 4, 256, 0, F, n, dwav, dv, dq, nb, log_bins,
                 d_edge, d_num, d_den);
    } else {
      double *w = (double *)ctx->ubuf;
      double2 *F = (double2 *)(w + 12 * ctx->n3);
      AXG_LAUNCH(ctx, "uij_prepare_fp64", (k_uij_prepare<double2, double>), grid_for(ctx->n3), 256, 0,
                 (const double *)ctx->u[ctx->cur], (const double *)ctx->ud, (const double *)nullptr, ctx->n3,
                 tau, w);
      AXG_CUFFT_TRY(ctx, cufftExecD2Z(ctx->plan_u, w, (cufftDoubleComplex *)F));
      AXG_LAUNCH(ctx, "uij_bin_fp64", k_uij_bin<double2>, 152 * 4, 256, 0, F, n, dwav, dv, dq, nb, log_bins,
                 d_edge, d_num, d_den);
    }
    (void)nhalf;
  } else {
    return axg_set_error(ctx, AXG_ERR_STATE, "gw_mode is NONE");
  }
  std::vector<double> h(2 * nb);
  AXG_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), ctx->d_red, sizeof(double) * 2 * nb, cudaMemcpyDeviceToHost,
                                    ctx->stream));
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  const double fact = gw_fact(ctx->p);
  for (int k = 0; k < nb; ++k) {
    const double qc = log_bins ? std::sqrt(edges[k] * edges[k + 1]) : (edges[k + 1] + edges[k]) / 2;
    numer[k] = h[k];
    denom[k] = h[nb + k];
    power[k] = denom[k] > 0 ? numer[k] / denom[k] * (qc * qc * qc) * fact : 0.0;
    if (wave) {
      if (log_bins) {
        wave[k] = edges[k];
        if (k == nb - 1) wave[nb] = edges[nb];
      } else {
        wave[k] = qc;
      }
    }
  }
  return AXG_OK;
}

extern "C" {
int axg_grav_spec_estimation(axg_ctx *ctx, double tau, double *wave, double *power, double *numer,
                             double *denom) {
  if (!ctx || !power || !numer || !denom) return AXG_ERR_ARG;
  return axg_gw_spec(ctx, tau, 0, wave, power, numer, denom);
}
int axg_grav_spec_log(axg_ctx *ctx, double tau, double *edges, double *power, double *numer, double *denom) {
  if (!ctx || !power || !numer || !denom) return AXG_ERR_ARG;
  if (ctx->p.gw_log_bins < 1) return axg_set_error(ctx, AXG_ERR_ARG, "gw_log_bins < 1");
  return axg_gw_spec(ctx, tau, 1, edges, power, numer, denom);
}
}
