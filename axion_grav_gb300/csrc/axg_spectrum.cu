// axg_spectrum.cu -- masked field spectrum with window deconvolution
// (spectrum.f90:23-171, 242-567, 736-954) on the GPU.
//
//   init (host, once): mode-coupling table mat_spec(0:500, num_cov) by the
//        reference's 200-point quadrature (spectrum.f90:74-98, 117-171);
//   conv spectrum: k_spec_degrade box-averages phidot over deg^3 and zeroes
//        coarse cells that hold a masked cell (flag bit 4 of the last
//        classification, the device-resident form of the reference's mask
//        files), cuFFT Z2Z backward, k_spec_bin bins |F dx^3|^2 dk^3;
//   window matrix: the reference sums |W(k)|^2 interp_ij(|k|) over all k for
//        each of the num_cov = nb(nb+1)/2 bin pairs (O(num_cov N^3),
//        spectrum.f90:385-428).  Here |W|^2 and the mode count are first
//        histogrammed by integer |k|^2 (k_spec_w2_hist), an exact regrouping,
//        and k_spec_mat sums the histogram against the interpolation table
//        (O(num_cov * 3(N/2)^2));
//   packed Cholesky inverse (dpptrf/dpptri) and dspmv on the host (nb x nb).
#include <cmath>
#include <vector>

#include "axg_binning.h"
#include "axg_detmath.h"
#include "axg_internal.h"

namespace {

constexpr double kRefPi = 3.14159265359;
constexpr double kRefTwoPi = 2 * kRefPi;
constexpr int kNumLargeq = 500;
constexpr int kNumInt = 200;

__device__ __forceinline__ int kint(int j, int n) { return (j + n / 2) % n - n / 2; }

template <typename V>
__global__ void k_spec_degrade(const V *__restrict__ phid, const int8_t *__restrict__ flags, int n, int deg,
                               double inv_deg3, int window, double dv_spa, double2 *__restrict__ out) {
  // inv_deg3 = 1 / deg^3
  const int m = n / deg;
  const int64_t m3 = (int64_t)m * m * m, n2 = (int64_t)n * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < m3; c += stride) {
    const int ix = (int)(c % m), iy = (int)((c / m) % m), iz = (int)(c / ((int64_t)m * m));
    double sr = 0.0, si = 0.0;
    bool masked = false;
    for (int z0 = iz * deg; z0 < (iz + 1) * deg; ++z0)
      for (int y0 = iy * deg; y0 < (iy + 1) * deg; ++y0)
        for (int x0 = ix * deg; x0 < (ix + 1) * deg; ++x0) {
          const int64_t f = z0 * n2 + (int64_t)y0 * n + x0;
          if (flags && (flags[f] & 4)) masked = true;
          if (!window) {
            const V v = phid[f];
            sr = sr + (double)v.x;
            si = si + (double)v.y;
          }
        }
    if (window)
      out[c] = make_double2(masked ? 0.0 : dv_spa, 0.0);
    else
      // deg^3 is a power of two: multiplying by its reciprocal is the same
      // single rounding as the reference's division
      out[c] = masked ? make_double2(0.0, 0.0) : make_double2(sr * inv_deg3, si * inv_deg3);
  }
}

// |F dv_spa|^2 dv_wav per k-site into the bins of |k|^2: the two scalings
// are one factor, scale = dv_spa^2 dv_wav (three FP64 operations per site
// instead of six)
__global__ void k_spec_bin(const double2 *__restrict__ F, int m, const int16_t *__restrict__ tab, double scale,
                           int nb, double *__restrict__ conv, double *__restrict__ count) {
  extern __shared__ double sh[];
  double *sc = sh, *sn = sh + nb;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) sc[b] = sn[b] = 0.0;
  __syncthreads();
  const int64_t m3 = (int64_t)m * m * m;
  BinRun run;
  for (int64_t s0 = run_start(); s0 < m3; s0 += run_stride()) {
    for (int64_t s = s0; s < s0 + kRun && s < m3; ++s) {
      const int kx = kint(s % m, m), ky = kint((s / m) % m, m), kz = kint(s / ((int64_t)m * m), m);
      const int b = tab[kx * kx + ky * ky + kz * kz];
      double v = 0.0;
      if (b >= 0) {
        const double2 f = F[s];
        v = (f.x * f.x + f.y * f.y) * scale;
      }
      run.add(sc, sn, b, v, 1u);
    }
  }
  run.flush(sc, sn);
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    if (sn[b] != 0.0) {
      atomicAdd(&conv[b], sc[b]);
      atomicAdd(&count[b], sn[b]);
    }
  }
}

// the real window of compute_matrix_deconv: dx^3 on unmasked coarse cells
__global__ void k_spec_window(const int8_t *__restrict__ flags, int n, int deg, double dv_spa,
                              double *__restrict__ out) {
  const int m = n / deg;
  const int64_t m3 = (int64_t)m * m * m, n2 = (int64_t)n * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < m3; c += stride) {
    const int ix = (int)(c % m), iy = (int)((c / m) % m), iz = (int)(c / ((int64_t)m * m));
    bool masked = false;
    if (flags)
      for (int z0 = iz * deg; z0 < (iz + 1) * deg && !masked; ++z0)
        for (int y0 = iy * deg; y0 < (iy + 1) * deg && !masked; ++y0)
          for (int x0 = ix * deg; x0 < (ix + 1) * deg; ++x0)
            if (flags[z0 * n2 + (int64_t)y0 * n + x0] & 4) {
              masked = true;
              break;
            }
    out[c] = masked ? 0.0 : dv_spa;
  }
}

// |W|^2 and mode counts per integer |k|^2 from the half spectrum of the real
// window (|W(-k)| = |W(k)|: interior kx planes count twice)
__global__ void k_spec_w2_hist(const double2 *__restrict__ W, int m, double *__restrict__ h,
                               double *__restrict__ cnt) {
  const int mh = m / 2 + 1;
  const int64_t nhalf = (int64_t)m * m * mh;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nhalf; s += stride) {
    const int ix = (int)(s % mh), iy = (int)((s / mh) % m), iz = (int)(s / ((int64_t)mh * m));
    const int kx = kint(ix, m), ky = kint(iy, m), kz = kint(iz, m);
    const int iq2 = kx * kx + ky * ky + kz * kz;
    const double wgt = (ix == 0 || 2 * ix == m) ? 1.0 : 2.0;
    const double2 w = W[s];
    atomicAdd(&h[iq2], wgt * (w.x * w.x + w.y * w.y));
    atomicAdd(&cnt[iq2], wgt);
  }
}

// one block per bin pair ij (spectrum.f90:385-428 regrouped by |k|^2)
// |k| = sqrt(iq2) dwav for every integer |k|^2 up to iq2max, formed once and
// shared by all the (i, j) pairs of k_spec_mat instead of an FP64 square
// root per pair and |k|^2 (FP64 runs at 1/64 of the FP32 rate on GB300)
__global__ void k_spec_qtab(int64_t iq2max, double dwav, double *__restrict__ q) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= iq2max; i += (int64_t)gridDim.x * blockDim.x)
    q[i] = sqrt((double)i) * dwav;
}

__global__ void k_spec_mat(const double *__restrict__ h, const double *__restrict__ cnt,
                           const double *__restrict__ mat_spec, const double *__restrict__ largeq0,
                           const double *__restrict__ dq_spec, const long long *__restrict__ range,
                           const double *__restrict__ qtab, double *__restrict__ mat0, double *__restrict__ tat0) {
  const int ij = blockIdx.x;
  const long long lo = range[2 * ij], hi = range[2 * ij + 1];
  const double *tab = mat_spec + (int64_t)ij * (kNumLargeq + 1);
  const double lq0 = largeq0[ij], idq = 1.0 / dq_spec[ij];  // one division per pair
  double a = 0.0, b = 0.0;
  for (long long iq2 = lo + threadIdx.x; iq2 <= hi; iq2 += blockDim.x) {
    const double c = cnt[iq2];
    if (c == 0.0) continue;
    const double q = qtab[iq2];
    double d = (q - lq0) * idq;
    const double fl = floor(d);
    double u = 0.0;
    if (fl < kNumLargeq && fl >= 0) {
      const int iq = (int)fl;
      d = d - iq;
      u = (1 - d) * tab[iq] + d * tab[iq + 1];
    }
    a += h[iq2] * u;
    b += c * u;
  }
  __shared__ double sa[256], sb[256];
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      sa[threadIdx.x] += sa[threadIdx.x + o];
      sb[threadIdx.x] += sb[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    mat0[ij] = sa[0];
    tat0[ij] = sb[0];
  }
}

// spectrum.f90:117-171
double integrate_p_check(int num, double li, double si, double lj, double sj, double q) {
  double maxp = lj < q + li ? lj : q + li;
  double a = q - li, b = si - q;
  double minp = a > b ? a : b;
  minp = minp > sj ? minp : sj;
  double dp = (maxp - minp) / num;
  double x = 0.0;
  if (dp > 0) {
    for (int ip = 1; ip <= num; ++ip) {
      double p = dp * (ip - 0.5) + minp;
      double maxmu, minmu;
      if (q == 0.0) {
        maxmu = 1.0;
        minmu = -1.0;
      } else {
        maxmu = (li * li - p * p - q * q) / 2 / p / q;
        minmu = (si * si - p * p - q * q) / 2 / p / q;
        maxmu = maxmu < 1.0 ? maxmu : 1.0;
        minmu = minmu > -1.0 ? minmu : -1.0;
      }
      x = x + p * p * dp * (maxmu - minmu);
    }
  }
  return x * kRefTwoPi;
}

// reference LAPACK dpptrf + dpptri ('U'), packed upper
int pp_inverse(int n, double *ap) {
  int jj = 0;
  for (int j = 1; j <= n; ++j) {
    int jc = jj + 1;
    jj = jj + j;
    if (j > 1) {
      double *x = ap + (jc - 1);
      int kk = 1;
      for (int jx = 1; jx <= j - 1; ++jx) {
        double temp = x[jx - 1];
        int k = kk;
        for (int i = 1; i <= jx - 1; ++i) {
          temp = temp - ap[k - 1] * x[i - 1];
          ++k;
        }
        temp = temp / ap[kk + jx - 2];
        x[jx - 1] = temp;
        kk = kk + jx;
      }
    }
    double dot = 0.0;
    for (int i = 0; i < j - 1; ++i) dot = dot + ap[jc - 1 + i] * ap[jc - 1 + i];
    double ajj = ap[jj - 1] - dot;
    if (ajj <= 0.0) {
      ap[jj - 1] = ajj;
      return j;
    }
    ap[jj - 1] = std::sqrt(ajj);
  }
  int jc = 1;
  for (int j = 1; j <= n; ++j) {
    ap[jc + j - 2] = 1.0 / ap[jc + j - 2];
    double ajj = -ap[jc + j - 2];
    double *x = ap + (jc - 1);
    int kk = 1;
    for (int jx = 1; jx <= j - 1; ++jx) {
      if (x[jx - 1] != 0.0) {
        double temp = x[jx - 1];
        int k = kk;
        for (int i = 1; i <= jx - 1; ++i) {
          x[i - 1] = x[i - 1] + temp * ap[k - 1];
          ++k;
        }
        x[jx - 1] = x[jx - 1] * ap[kk + jx - 2];
      }
      kk = kk + jx;
    }
    for (int i = 0; i < j - 1; ++i) x[i] = ajj * x[i];
    jc = jc + j;
  }
  jj = 0;
  for (int j = 1; j <= n; ++j) {
    int jc2 = jj + 1;
    jj = jj + j;
    if (j > 1) {
      const double *xv = ap + (jc2 - 1);
      int kk = 0;
      for (int jx = 0; jx < j - 1; ++jx) {
        if (xv[jx] != 0.0) {
          double temp = 1.0 * xv[jx];
          int k = kk;
          for (int i = 0; i <= jx; ++i) {
            ap[k] = ap[k] + xv[i] * temp;
            ++k;
          }
        }
        kk += jx + 1;
      }
    }
    double ajj = ap[jj - 1];
    for (int i = 0; i < j; ++i) ap[jc2 - 1 + i] = ajj * ap[jc2 - 1 + i];
  }
  return 0;
}

// estimate_covmat (spectrum.f90:593-641): Gaussian modes with the measured
// spectrum (Philox stream 16 + iter), sigma per bin of nint(q/dq + 0.5)
__global__ void k_mc_fill(double2 *F, int m, const int16_t *__restrict__ tab, const double *sigma, uint64_t seed,
                          uint32_t iter) {
  const int64_t m3 = (int64_t)m * m * m;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m3; s += stride) {
    const int kx = kint(s % m, m), ky = kint((s / m) % m, m), kz = kint(s / ((int64_t)m * m), m);
    const int b = tab[kx * kx + ky * ky + kz * kz];
    if (b >= 0) {
      const axd_u32x4 r = axd_draw(seed, 16u + iter, 0u, (uint64_t)s);
      const double u1 = axd_u01_open0(r.v[0], r.v[1]), u2 = axd_u01(r.v[2], r.v[3]);
      const double rad = sqrt(-2.0 * log(u1));
      double sn, cs;
      sincos(6.283185307179586 * u2, &sn, &cs);
      const double sg = sigma[b];
      F[s] = make_double2(rad * cs * sg, rad * sn * sg);
    } else {
      F[s] = make_double2(0.0, 0.0);
    }
  }
}

// masking (spectrum.f90:648): zero coarse cells holding a masked fine cell
__global__ void k_mc_mask(double2 *F, const int8_t *__restrict__ flags, int n, int deg) {
  const int m = n / deg;
  const int64_t m3 = (int64_t)m * m * m, n2 = (int64_t)n * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < m3; c += stride) {
    const int ix = (int)(c % m), iy = (int)((c / m) % m), iz = (int)(c / ((int64_t)m * m));
    bool masked = false;
    for (int z0 = iz * deg; z0 < (iz + 1) * deg && !masked; ++z0)
      for (int y0 = iy * deg; y0 < (iy + 1) * deg && !masked; ++y0)
        for (int x0 = ix * deg; x0 < (ix + 1) * deg; ++x0)
          if (flags[z0 * n2 + (int64_t)y0 * n + x0] & 4) {
            masked = true;
            break;
          }
    if (masked) F[c] = make_double2(0.0, 0.0);
  }
}

int grid_for(int64_t count) {
  int64_t b = (count + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace

// init_spectrum (spectrum.f90:23-103): tables on the host, copied to the device
int axg_spec_init(axg_ctx *ctx) {
  if (ctx->spec_mat) return AXG_OK;
  const int nb = ctx->p.num_bin;
  const int num_cov = nb * (nb + 1) / 2;
  const int deg = 1 << ctx->p.degrade_spec;
  const int m = (int)(ctx->n / deg);
  const double dspa_spec = ctx->p.dspa * deg;
  std::vector<double> &wav = ctx->h_wav;
  wav.assign(nb + 1, 0.0);
  const double qmax = kRefPi / dspa_spec;
  const double dq = qmax / nb;
  for (int iq = 1; iq <= nb; ++iq) wav[iq] = wav[iq - 1] + dq;
  ctx->h_mat_spec.assign((size_t)num_cov * 501, 0.0);
  ctx->h_largeq.assign((size_t)num_cov * 501, 0.0);
  ctx->h_dq.assign(num_cov, 0.0);
  for (int ij = 1; ij <= num_cov; ++ij) {
    int i = (int)std::lround(std::sqrt(2.0 * ij));
    int j = ij - i * (i - 1) / 2;
    double lj = wav[j], sj = wav[j - 1], li = wav[i], si = wav[i - 1];
    double maxq = li + lj;
    double minq = (si > sj ? si : sj) - (li < lj ? li : lj);
    if (minq < 0) minq = 0.0;
    double d = maxq - minq;
    d = d / kNumLargeq;
    ctx->h_dq[ij - 1] = d;
    for (int iq = 0; iq <= kNumLargeq; ++iq) {
      double q = minq + d * iq;
      ctx->h_largeq[(size_t)(ij - 1) * 501 + iq] = q;
      ctx->h_mat_spec[(size_t)(ij - 1) * 501 + iq] = integrate_p_check(kNumInt, li, si, lj, sj, q);
    }
  }
  std::vector<double> l0(num_cov);
  for (int ij = 0; ij < num_cov; ++ij) l0[ij] = ctx->h_largeq[(size_t)ij * 501];
  AXG_TRY(axg_alloc(ctx, (void **)&ctx->spec_mat, ctx->h_mat_spec.size() * 8, "mat_spec"));
  AXG_TRY(axg_alloc(ctx, (void **)&ctx->spec_largeq0, (size_t)num_cov * 8, "largeq"));
  AXG_TRY(axg_alloc(ctx, (void **)&ctx->spec_dq, (size_t)num_cov * 8, "dq_spec"));
  AXG_CUDA_TRY(ctx, cudaMemcpy(ctx->spec_mat, ctx->h_mat_spec.data(), ctx->h_mat_spec.size() * 8, cudaMemcpyHostToDevice));
  AXG_CUDA_TRY(ctx, cudaMemcpy(ctx->spec_largeq0, l0.data(), (size_t)num_cov * 8, cudaMemcpyHostToDevice));
  AXG_CUDA_TRY(ctx, cudaMemcpy(ctx->spec_dq, ctx->h_dq.data(), (size_t)num_cov * 8, cudaMemcpyHostToDevice));
  ctx->ns_spec = m;
  // m^3 complex; the window pass uses it as m^3 reals followed by the D2Z
  // half spectrum m^2 (m/2 + 1), which needs 16 m^2 bytes more
  AXG_TRY(axg_alloc(ctx, (void **)&ctx->spec_buf, (size_t)m * m * m * 16 + (size_t)m * m * 16 + 256,
                    "spectrum buffer"));
  AXG_CUFFT_TRY(ctx, cufftPlan3d(&ctx->plan_spec, m, m, m, CUFFT_Z2Z));
  ctx->plan_spec_ok = true;
  AXG_CUFFT_TRY(ctx, cufftSetStream(ctx->plan_spec, ctx->stream));
  AXG_CUFFT_TRY(ctx, cufftPlan3d(&ctx->plan_window, m, m, m, CUFFT_D2Z));
  ctx->plan_window_ok = true;
  AXG_CUFFT_TRY(ctx, cufftSetStream(ctx->plan_window, ctx->stream));
  return AXG_OK;
}

int axg_spec_estimation(axg_ctx *ctx, double tau, double *wave, double *power, double *conv,
                        double *count) {
  AXG_TRY(axg_spec_init(ctx));
  if (!ctx->flags_valid) {
    int64_t c[3];
    AXG_TRY(axg_def_classify(ctx, (ctx->p.flags & 7) | AXG_F_SPEC_EST, c));
  }
  const int nb = ctx->p.num_bin;
  const int num_cov = nb * (nb + 1) / 2;
  const int deg = 1 << ctx->p.degrade_spec;
  const int n = (int)ctx->n, m = n / deg;
  const int64_t m3 = (int64_t)m * m * m;
  const double dspa_spec = ctx->p.dspa * deg;
  const double dwav = kRefTwoPi / dspa_spec / m;
  const double dv_spa = dspa_spec * dspa_spec * dspa_spec;
  const double dv_wav = std::pow(dwav / kRefTwoPi, 3);
  const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
  const int64_t iq2max = 3LL * (m / 2) * (m / 2);
  // scratch: histogram + counts + mat0/tat0 + bin sums + pair ranges
  double *scratch = nullptr;
  long long *range = nullptr;
  const size_t nscr = (size_t)(3 * (iq2max + 1) + 2 * num_cov + 2 * nb);
  AXG_TRY(axg_alloc(ctx, (void **)&scratch, nscr * 8, "spectrum scratch"));
  int rc = AXG_OK;
  do {
    if ((rc = axg_alloc(ctx, (void **)&range, (size_t)num_cov * 16, "pair ranges"))) break;
    double *h = scratch, *cnt = scratch + iq2max + 1, *mat0 = cnt + iq2max + 1, *tat0 = mat0 + num_cov,
           *d_conv = tat0 + num_cov, *d_cnt = d_conv + nb, *qtab = d_cnt + nb;
    AXG_CUDA_TRY(ctx, cudaMemsetAsync(scratch, 0, nscr * 8, ctx->stream));
    // ---- compute_matrix_deconv (spectrum.f90:344-444) ----
    // the window is real: D2Z half spectrum (|W|^2 is the same for either sign)
    double *wreal = (double *)ctx->spec_buf;
    double2 *whalf = (double2 *)(((uintptr_t)(wreal + m3) + 255) & ~(uintptr_t)255);
    AXG_LAUNCH(ctx, "spec_window", k_spec_window, grid_for(m3), 256, 0, ctx->flags, n, deg, dv_spa, wreal);
    if (axg_ff_use(m))
      AXG_TRY(axg_ff_d2z(ctx, wreal, whalf, m, 1));
    else
      AXG_CUFFT_TRY(ctx, cufftExecD2Z(ctx->plan_window, wreal, (cufftDoubleComplex *)whalf));
    AXG_LAUNCH(ctx, "spec_w2_hist", k_spec_w2_hist, grid_for((int64_t)m * m * (m / 2 + 1)), 256, 0, whalf, m, h,
               cnt);
    std::vector<long long> hr(2 * (size_t)num_cov);
    for (int ij = 0; ij < num_cov; ++ij) {
      double e = ctx->h_largeq[(size_t)ij * 501 + kNumLargeq] / dwav;
      long long imax2 = (long long)std::ceil(e * e) - 1;
      e = ctx->h_largeq[(size_t)ij * 501] / dwav;
      long long imin2 = (long long)std::ceil(e * e);
      hr[2 * ij] = std::max(imin2, 0LL);
      hr[2 * ij + 1] = std::min(imax2, (long long)iq2max);
    }
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(range, hr.data(), hr.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    AXG_LAUNCH(ctx, "spec_qtab", k_spec_qtab, grid_for(iq2max + 1), 256, 0, iq2max, dwav, qtab);
    AXG_LAUNCH(ctx, "spec_mat", k_spec_mat, num_cov, 256, 0, h, cnt, ctx->spec_mat, ctx->spec_largeq0,
               ctx->spec_dq, range, qtab, mat0, tat0);
    // ---- compute_conv_spec (spectrum.f90:466-567) ----
    if (fp32)
      AXG_LAUNCH(ctx, "spec_degrade", k_spec_degrade<float2>, grid_for(m3), 256, 0, (const float2 *)ctx->phid,
                 ctx->flags, n, deg, 1.0 / ((double)deg * deg * deg), 0, dv_spa, ctx->spec_buf);
    else
      AXG_LAUNCH(ctx, "spec_degrade", k_spec_degrade<double2>, grid_for(m3), 256, 0, (const double2 *)ctx->phid,
                 ctx->flags, n, deg, 1.0 / ((double)deg * deg * deg), 0, dv_spa, ctx->spec_buf);
    if (axg_ff_use(m))
      AXG_TRY(axg_ff_z2z(ctx, (double2 *)ctx->spec_buf, m, 1));
    else
      AXG_CUFFT_TRY(ctx, cufftExecZ2Z(ctx->plan_spec, (cufftDoubleComplex *)ctx->spec_buf,
                                      (cufftDoubleComplex *)ctx->spec_buf, CUFFT_INVERSE));
    const double dq = ctx->h_wav[1] - ctx->h_wav[0];
    const int16_t *tab = nullptr;
    AXG_TRY(axg_bin_table(ctx, AXG_BIN_SPECTRUM, m, dwav, dq, nb, 0, nullptr, &tab));
    AXG_LAUNCH(ctx, "spec_bin", k_spec_bin, 152 * 4, 256, 2 * nb * sizeof(double), ctx->spec_buf, m, tab,
               dv_spa * dv_spa * dv_wav, nb, d_conv, d_cnt);
    std::vector<double> hm(2 * num_cov), hb(2 * nb);
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(hm.data(), mat0, hm.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(hb.data(), d_conv, hb.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
    AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<double> mat(num_cov);
    for (int ij = 0; ij < num_cov; ++ij) mat[ij] = hm[ij] / hm[num_cov + ij] * dv_wav * dv_wav;
    if (pp_inverse(nb, mat.data()) != 0) {
      rc = axg_set_error(ctx, AXG_ERR_NUMERIC, "deconvolution matrix not positive definite");
      break;
    }
    // ---- spectrum_estimation (spectrum.f90:267-285) ----
    const double t2 = tau * tau;
    std::vector<double> cv(nb), ct(nb), pw(nb, 0.0);
    for (int i = 1; i <= nb; ++i) {
      cv[i - 1] = hb[i - 1] * t2;
      ct[i - 1] = hb[nb + i - 1];
      for (int j = 1; j <= i; ++j) {
        int ij = i * (i - 1) / 2 + j;
        mat[ij - 1] = mat[ij - 1] / hb[nb + i - 1] / hb[nb + j - 1];
      }
    }
    // dspmv ('U')
    int kk = 1;
    for (int j = 1; j <= nb; ++j) {
      double temp1 = cv[j - 1], temp2 = 0.0;
      int k = kk;
      for (int i = 1; i <= j - 1; ++i) {
        pw[i - 1] = pw[i - 1] + temp1 * mat[k - 1];
        temp2 = temp2 + mat[k - 1] * cv[i - 1];
        ++k;
      }
      pw[j - 1] = pw[j - 1] + temp1 * mat[kk + j - 2] + 1.0 * temp2;
      kk = kk + j;
    }
    ctx->last_power = pw;
    ctx->last_mat_div = mat;
    ctx->last_cov.clear();
    for (int i = 0; i < nb; ++i) {
      if (wave) wave[i] = (ctx->h_wav[i + 1] + ctx->h_wav[i]) / 2;
      power[i] = pw[i];
      if (conv) conv[i] = cv[i] / ct[i];
      if (count) count[i] = ct[i];
    }
  } while (0);
  cudaStreamSynchronize(ctx->stream);
  axg_free(ctx, (void **)&scratch);
  axg_free(ctx, (void **)&range);
  return rc;
}

extern "C" {
int axg_spectrum_estimation(axg_ctx *ctx, double tau, double *wave, double *power, double *conv,
                            double *count) {
  if (!ctx || !power) return AXG_ERR_ARG;
  return axg_spec_estimation(ctx, tau, wave, power, conv, count);
}

// compute_crho (spectrum.f90:316-342) without the covariance term
int axg_compute_crho(axg_ctx *ctx, double *rho) {
  if (!ctx || !rho) return AXG_ERR_ARG;
  if (ctx->last_power.empty()) return axg_set_error(ctx, AXG_ERR_STATE, "no spectrum estimated yet");
  const int nb = ctx->p.num_bin;
  double r = 0.0;
  for (int i = 1; i <= nb; ++i) {
    const double q = (ctx->h_wav[i] + ctx->h_wav[i - 1]) / 2;
    const double dq = ctx->h_wav[i] - ctx->h_wav[i - 1];
    const double q2dq = q * q * dq / kRefTwoPi / kRefPi;
    r = r + ctx->last_power[i - 1] * q2dq;
  }
  *rho = r;
  return AXG_OK;
}
}

// estimate_covmat (spectrum.f90:569-734) on the last spectrum estimate
int axg_spec_covariance(axg_ctx *ctx, int min_mc, int max_mc, double tol, double *cov_out, int *iterations) {
  if (ctx->last_power.empty() || ctx->last_mat_div.empty())
    return axg_set_error(ctx, AXG_ERR_STATE, "no spectrum estimated yet");
  if (!ctx->flags_valid) return axg_set_error(ctx, AXG_ERR_STATE, "mask of the last classification is stale");
  const int nb = ctx->p.num_bin;
  const int num_cov = nb * (nb + 1) / 2;
  const int deg = 1 << ctx->p.degrade_spec;
  const int n = (int)ctx->n, m = n / deg;
  const int64_t m3 = (int64_t)m * m * m;
  const double dspa_spec = ctx->p.dspa * deg;
  const double dwav = kRefTwoPi / dspa_spec / m;
  const double dq = ctx->h_wav[1] - ctx->h_wav[0];
  std::vector<double> sigma(nb), cov(num_cov, 0.0), tmp((size_t)num_cov * max_mc, 0.0), pw0(nb), pw(nb);
  for (int i = 0; i < nb; ++i) {
    const double pwr = ctx->last_power[i];
    sigma[i] = std::sqrt(pwr > 0 ? pwr / 2 : 0.0) / (double)m3;
  }
  double *scr = nullptr;
  auto cleanup = axg_on_exit([&] {
    cudaStreamSynchronize(ctx->stream);
    axg_free(ctx, (void **)&scr);
  });
  AXG_TRY(axg_alloc(ctx, (void **)&scr, sizeof(double) * (size_t)(3 * nb), "covariance scratch"));
  int rc = AXG_OK, iter;
  double *d_sigma = scr, *d_pow = scr + nb, *d_cnt = scr + 2 * nb;
  const int16_t *tab = nullptr;
  AXG_TRY(axg_bin_table(ctx, AXG_BIN_SPECTRUM, m, dwav, dq, nb, 0, nullptr, &tab));
  const bool ff = axg_ff_use(m);  // float-float transforms (FP64 accuracy on the FP32 pipes)
  for (iter = 1; iter <= max_mc && rc == AXG_OK; ++iter) {
    if (iter == 1) AXG_CUDA_TRY(ctx, cudaMemcpyAsync(d_sigma, sigma.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, ctx->stream));
    AXG_CUDA_TRY(ctx, cudaMemsetAsync(d_pow, 0, sizeof(double) * 2 * nb, ctx->stream));
    AXG_LAUNCH(ctx, "mc_fill", k_mc_fill, grid_for(m3), 256, 0, ctx->spec_buf, m, tab, d_sigma, (uint64_t)ctx->p.seed,
               (uint32_t)iter);
    if (ff)
      AXG_TRY(axg_ff_z2z(ctx, (double2 *)ctx->spec_buf, m, 0));
    else
      AXG_CUFFT_TRY(ctx, cufftExecZ2Z(ctx->plan_spec, (cufftDoubleComplex *)ctx->spec_buf,
                                      (cufftDoubleComplex *)ctx->spec_buf, CUFFT_FORWARD));
    AXG_LAUNCH(ctx, "mc_mask", k_mc_mask, grid_for(m3), 256, 0, ctx->spec_buf, ctx->flags, n, deg);
    if (ff)
      AXG_TRY(axg_ff_z2z(ctx, (double2 *)ctx->spec_buf, m, 1));
    else
      AXG_CUFFT_TRY(ctx, cufftExecZ2Z(ctx->plan_spec, (cufftDoubleComplex *)ctx->spec_buf,
                                      (cufftDoubleComplex *)ctx->spec_buf, CUFFT_INVERSE));
    AXG_LAUNCH(ctx, "mc_bin", k_spec_bin, 152 * 4, 256, 2 * nb * sizeof(double), ctx->spec_buf, m, tab, 1.0, nb,
               d_pow, d_cnt);
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(pw0.data(), d_pow, sizeof(double) * nb, cudaMemcpyDeviceToHost, ctx->stream));
    AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    // pow = mat_deconv pow0 - power (dspmv, beta = 1)
    const std::vector<double> &M = ctx->last_mat_div;
    for (int i = 0; i < nb; ++i) pw[i] = -ctx->last_power[i];
    int kk = 1;
    for (int j = 1; j <= nb; ++j) {
      double temp1 = pw0[j - 1], temp2 = 0.0;
      int k = kk;
      for (int i = 1; i <= j - 1; ++i) {
        pw[i - 1] = pw[i - 1] + temp1 * M[k - 1];
        temp2 = temp2 + M[k - 1] * pw0[i - 1];
        ++k;
      }
      pw[j - 1] = pw[j - 1] + temp1 * M[kk + j - 2] + temp2;
      kk = kk + j;
    }
    for (int i = 1; i <= nb; ++i)
      for (int j = 1; j <= i; ++j) {
        const int ij = i * (i - 1) / 2 + j;
        const double u = pw[i - 1] * pw[j - 1];
        tmp[(size_t)(iter - 1) * num_cov + ij - 1] = cov[ij - 1];
        for (int k = 1; k <= iter - 1; ++k) tmp[(size_t)(k - 1) * num_cov + ij - 1] += u;
        cov[ij - 1] = cov[ij - 1] + u;
      }
    if (iter < min_mc) continue;
    // jackknife convergence on the diagonal (spectrum.f90:696-718)
    double diff = 0.0;
    for (int i = 1; i <= nb; ++i) {
      const int ij = i * (i + 1) / 2;
      double u = 0.0, v = 0.0;
      for (int k = 1; k <= iter; ++k) {
        const double x = tmp[(size_t)(k - 1) * num_cov + ij - 1] / (iter - 1);
        u = u + x;
        v = v + x * x;
      }
      u = u / iter;
      v = v / iter;
      v = std::sqrt(v - u * u);
      const double x = cov[ij - 1] / iter;
      const double r = v / x;
      diff = diff > r ? diff : r;
    }
    if (diff < tol) break;
  }
  if (rc != AXG_OK) return rc;
  if (iter > max_mc) iter = max_mc + 1;
  for (int ij = 0; ij < num_cov; ++ij) cov[ij] = cov[ij] / iter;
  ctx->last_cov = cov;
  if (cov_out) std::copy(cov.begin(), cov.end(), cov_out);
  if (iterations) *iterations = iter;
  return AXG_OK;
}

extern "C" {
int axg_spectrum_covariance(axg_ctx *ctx, int min_mc, int max_mc, double tol, double *cov, int *iterations) {
  if (!ctx || min_mc < 2 || max_mc < min_mc || !(tol > 0)) return AXG_ERR_ARG;
  return axg_spec_covariance(ctx, min_mc, max_mc, tol, cov, iterations);
}

// compute_crho (spectrum.f90:316-342) with the covariance term of the last MC run
int axg_compute_crho_cov(axg_ctx *ctx, double *rho, double *drho) {
  if (!ctx || !rho || !drho) return AXG_ERR_ARG;
  if (ctx->last_power.empty() || ctx->last_cov.empty())
    return axg_set_error(ctx, AXG_ERR_STATE, "needs axg_spectrum_estimation and axg_spectrum_covariance first");
  const int nb = ctx->p.num_bin;
  const std::vector<double> &w = ctx->h_wav;
  double r = 0.0, d = 0.0;
  for (int i = 1; i <= nb; ++i) {
    double dd = 0.0;
    for (int j = 1; j <= i; ++j) {
      const int ij = i * (i - 1) / 2 + j;
      const double q = (w[j] + w[j - 1]) / 2, dq = w[j] - w[j - 1];
      double q2dq = q * q * dq / kRefPi / kRefPi;
      if (j == i) q2dq = q2dq / 2;
      dd = dd + ctx->last_cov[ij - 1] * q2dq;
    }
    const double q = (w[i] + w[i - 1]) / 2, dq = w[i] - w[i - 1];
    const double q2dq = q * q * dq / kRefTwoPi / kRefPi;
    d = d + dd * q2dq;
    r = r + ctx->last_power[i - 1] * q2dq;
  }
  *rho = r;
  *drho = std::sqrt(d);
  return AXG_OK;
}

// get_epsilon (spectrum.f90:1002-1036) for one pair of output times
int axg_epsilon(int32_t nb, const double *wav, const double *p1, const double *p2, const double *c1,
                const double *c2, double tau1, double tau2, double *eps, double *deps) {
  if (nb < 1 || !wav || !p1 || !p2 || !c1 || !c2 || !eps || !deps) return AXG_ERR_ARG;
  const double tau = (tau2 + tau1) / 2;
  const double f = tau / 2 / kRefTwoPi;
  double num = 0.0, den = 0.0;
  for (int i = 1; i <= nb; ++i) {
    const double d = p2[i - 1] - p1[i - 1];
    const double q = (wav[i - 1] + wav[i]) / 2;
    num = num + d * q * q;
    den = den + d * q;
  }
  const double e = num / den * f;
  double de = 0.0;
  for (int i = 1; i <= nb; ++i) {
    const double d1 = (wav[i - 1] + wav[i]) / 2;
    for (int j = 1; j <= i; ++j) {
      const int ij = i * (i - 1) / 2 + j;
      const double d2 = (wav[j - 1] + wav[j]) / 2;
      double d = (1 - e / d1 / f) * (1 - e / d2 / f) * (c2[ij - 1] + c1[ij - 1]) * d1 * d1 * d2 * d2;
      if (j != i) d = d * 2;
      de = de + d;
    }
  }
  *eps = e;
  *deps = std::sqrt(de / den / den) * f;
  return AXG_OK;
}
}
