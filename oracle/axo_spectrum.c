/*
 * axo_spectrum.c -- oracle restatement of spectrum.f90 (mode-coupling table,
 * degraded and masked phidot spectrum, deconvolution matrix, packed
 * symmetric solve, conformal energy, Monte-Carlo covariance, epsilon).
 * TEST INFRASTRUCTURE ONLY (see axo.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "axo.h"
#include "axg_detmath.h"

#define REF_PI 3.14159265359
#define REF_TWOPI (2 * REF_PI)
#define NUM_LARGEQ 500
#define NUM_INT 200

static inline int64_t kint(int64_t j, int64_t n) { return (j + n / 2) % n - n / 2; }

/* spectrum.f90:117-171 (DIM==3) */
static double integrate_p_check(int num, double li, double si, double lj, double sj, double q) {
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
  return x * REF_TWOPI;
}

/* spectrum.f90:23-103; mat_spec and largeq are [num_cov][501] */
void axo_init_spectrum(const axg_params *p, double *mat_spec, double *largeq, double *dq_spec,
                       double *wav) {
  const int nb = p->num_bin;
  const int num_cov = nb * (nb + 1) / 2;
  const int deg = 1 << p->degrade_spec;
  const double dspa_spec = p->dspa * deg;
  double q = REF_PI / dspa_spec;
  double dq = q / nb;
  wav[0] = 0.0;
  for (int iq = 1; iq <= nb; ++iq) wav[iq] = wav[iq - 1] + dq;
#pragma omp parallel for schedule(dynamic, 1)
  for (int ij = 1; ij <= num_cov; ++ij) {
    int i = (int)lround(sqrt(2.0 * ij));
    int j = ij - i * (i - 1) / 2;
    double lj = wav[j], sj = wav[j - 1], li = wav[i], si = wav[i - 1];
    double maxq = li + lj;
    double minq = (si > sj ? si : sj) - (li < lj ? li : lj);
    if (minq < 0) minq = 0.0;
    double d = maxq - minq;
    d = d / NUM_LARGEQ;
    dq_spec[ij - 1] = d;
    for (int iq = 0; iq <= NUM_LARGEQ; ++iq) {
      double qq = minq + d * iq;
      largeq[(size_t)(ij - 1) * 501 + iq] = qq;
      mat_spec[(size_t)(ij - 1) * 501 + iq] = integrate_p_check(NUM_INT, li, si, lj, sj, qq);
    }
  }
}

/* spectrum.f90:446-464 */
static double get_mat_spec(const double *mat_spec, const double *largeq, const double *dq_spec,
                           int ij, double q) {
  double d = (q - largeq[(size_t)ij * 501]) / dq_spec[ij];
  double fl = floor(d);
  if (fl < NUM_LARGEQ && fl >= 0) {
    int iq = (int)fl;
    d = d - iq;
    return (1 - d) * mat_spec[(size_t)ij * 501 + iq] + d * mat_spec[(size_t)ij * 501 + iq + 1];
  }
  return 0.0;
}

/* reference BLAS dspmv ('U', alpha=1, beta=0) */
static void dspmv_u(int n, const double *ap, const double *x, double *y) {
  for (int i = 0; i < n; ++i) y[i] = 0.0;
  int kk = 1;
  for (int j = 1; j <= n; ++j) {
    double temp1 = 1.0 * x[j - 1], temp2 = 0.0;
    int k = kk;
    for (int i = 1; i <= j - 1; ++i) {
      y[i - 1] = y[i - 1] + temp1 * ap[k - 1];
      temp2 = temp2 + ap[k - 1] * x[i - 1];
      ++k;
    }
    y[j - 1] = y[j - 1] + temp1 * ap[kk + j - 2] + 1.0 * temp2;
    kk = kk + j;
  }
}

/* coarse cell masked when any fine cell in it carries flag_mask
 * (masking, spectrum.f90:900-954, fed by defects_3d.f90:265-273) */
static void build_mask(const axg_params *p, const int8_t *flags, unsigned char *mask) {
  const int64_t n = p->ngrid, n2 = n * n, deg = 1 << p->degrade_spec, m = n / deg;
  memset(mask, 0, (size_t)(m * m * m));
  if (!flags) return;
  for (int64_t s = 0; s < n * n2; ++s)
    if (flags[s] & 4) {
      int64_t ix = s % n, iy = (s / n) % n, iz = s / n2;
      mask[(iz / deg) * m * m + (iy / deg) * m + ix / deg] = 1;
    }
}

void axo_spectrum_estimation(const axg_params *p, const double *phidot, const int8_t *flags,
                             double tau, double *wave, double *power, double *conv,
                             double *count, double *mat_deconv_out) {
  const int nb = p->num_bin;
  const int num_cov = nb * (nb + 1) / 2;
  const int64_t n = p->ngrid, n2 = n * n, deg = 1 << p->degrade_spec, m = n / deg, m3 = m * m * m;
  const double dspa_spec = p->dspa * deg;
  const double dwav_spec = REF_TWOPI / dspa_spec / m;
  const double dv_spa = dspa_spec * dspa_spec * dspa_spec;
  const double dv_wav = pow(dwav_spec / REF_TWOPI, 3);
  double *mat_spec = (double *)malloc(sizeof(double) * num_cov * 501);
  double *largeq = (double *)malloc(sizeof(double) * num_cov * 501);
  double *dq_spec = (double *)malloc(sizeof(double) * num_cov);
  double *wav = (double *)malloc(sizeof(double) * (nb + 1));
  axo_init_spectrum(p, mat_spec, largeq, dq_spec, wav);
  unsigned char *mask = (unsigned char *)malloc((size_t)m3);
  build_mask(p, flags, mask);
  double *buf = (double *)malloc(sizeof(double) * 2 * m3);

  /* ---- compute_matrix_deconv (spectrum.f90:344-444) ---- */
  for (int64_t s = 0; s < m3; ++s) {
    buf[2 * s] = mask[s] ? 0.0 : dv_spa;
    buf[2 * s + 1] = 0.0;
  }
  axo_fft3d(m, buf, +1);
  double *mat0 = (double *)calloc(num_cov, sizeof(double));
  double *tat0 = (double *)calloc(num_cov, sizeof(double));
#pragma omp parallel for schedule(dynamic, 1)
  for (int ij = 0; ij < num_cov; ++ij) {
    double e = largeq[(size_t)ij * 501 + NUM_LARGEQ] / dwav_spec;
    int64_t imax2 = (int64_t)ceil(e * e) - 1;
    e = largeq[(size_t)ij * 501] / dwav_spec;
    int64_t imin2 = (int64_t)ceil(e * e);
    double a = 0.0, b = 0.0;
    for (int64_t s = 0; s < m3; ++s) {
      int64_t qx = kint(s % m, m), qy = kint((s / m) % m, m), qz = kint(s / (m * m), m);
      int64_t iq2 = qx * qx + qy * qy + qz * qz;
      if (!(iq2 <= imax2 && iq2 >= imin2)) continue;
      double q = sqrt((double)iq2) * dwav_spec;
      double u = get_mat_spec(mat_spec, largeq, dq_spec, ij, q);
      double v = buf[2 * s] * buf[2 * s] + buf[2 * s + 1] * buf[2 * s + 1];
      a = a + v * u;
      b = b + u;
    }
    mat0[ij] = a;
    tat0[ij] = b;
  }
  double *mat = (double *)malloc(sizeof(double) * num_cov);
  for (int ij = 0; ij < num_cov; ++ij) mat[ij] = mat0[ij] / tat0[ij] * dv_wav * dv_wav;
  axo_pp_inverse(nb, mat);
  if (mat_deconv_out) memcpy(mat_deconv_out, mat, sizeof(double) * num_cov);

  /* ---- compute_conv_spec (spectrum.f90:466-567) ---- */
  double dq = wav[1] - wav[0];
  const double inv = (double)(deg * deg * deg);
  for (int64_t iz = 0; iz < m; ++iz)
    for (int64_t iy = 0; iy < m; ++iy)
      for (int64_t ix = 0; ix < m; ++ix) {
        double sr = 0.0, si = 0.0;
        for (int64_t z0 = iz * deg; z0 < (iz + 1) * deg; ++z0)
          for (int64_t y0 = iy * deg; y0 < (iy + 1) * deg; ++y0)
            for (int64_t x0 = ix * deg; x0 < (ix + 1) * deg; ++x0) {
              int64_t f = z0 * n2 + y0 * n + x0;
              sr = sr + phidot[2 * f];
              si = si + phidot[2 * f + 1];
            }
        int64_t c = iz * m * m + iy * m + ix;
        buf[2 * c] = mask[c] ? 0.0 : sr / inv;
        buf[2 * c + 1] = mask[c] ? 0.0 : si / inv;
      }
  axo_fft3d(m, buf, +1);
  for (int k = 0; k < nb; ++k) conv[k] = count[k] = 0.0;
  for (int64_t s = 0; s < m3; ++s) {
    double re = buf[2 * s] * dv_spa, im = buf[2 * s + 1] * dv_spa;
    int64_t qx = kint(s % m, m), qy = kint((s / m) % m, m), qz = kint(s / (m * m), m);
    double q = sqrt((double)(qx * qx + qy * qy + qz * qz)) * dwav_spec;
    double id = round(q / dq + 0.5);
    if (id >= 1 && id <= nb) {
      int i = (int)id;
      conv[i - 1] += (re * re + im * im) * dv_wav;
      count[i - 1] += 1.0;
    }
  }
  /* ---- spectrum_estimation (spectrum.f90:267-275) ---- */
  const double t2 = tau * tau;
  for (int i = 1; i <= nb; ++i) {
    conv[i - 1] = conv[i - 1] * t2;
    for (int j = 1; j <= i; ++j) {
      int ij = i * (i - 1) / 2 + j;
      mat[ij - 1] = mat[ij - 1] / count[i - 1] / count[j - 1];
    }
  }
  dspmv_u(nb, mat, conv, power);
  for (int i = 0; i < nb; ++i) {
    wave[i] = (wav[i + 1] + wav[i]) / 2;
    conv[i] = conv[i] / count[i];
  }
  free(mat_spec); free(largeq); free(dq_spec); free(wav); free(mask); free(buf);
  free(mat0); free(tat0); free(mat);
}

/* spectrum.f90:316-342 without the covariance term */
void axo_compute_crho(const axg_params *p, const double *wav, const double *power, double *rho) {
  const int nb = p->num_bin;
  double r = 0.0;
  for (int i = 1; i <= nb; ++i) {
    double q = (wav[i] + wav[i - 1]) / 2;
    double dq = wav[i] - wav[i - 1];
    double q2dq = q * q * dq / REF_TWOPI / REF_PI;
    r = r + power[i - 1] * q2dq;
  }
  *rho = r;
}

/* estimate_covmat (spectrum.f90:569-734): Gaussian fields with the measured
 * spectrum, masked like the data, re-estimated through the deconvolution
 * matrix; covariance of the estimates with a jackknife convergence test.
 * mat_deconv is the matrix after the division by the mode counts
 * (spectrum.f90:271).  Gaussian draws: Philox stream 16 + iter (the
 * reference uses MKL VSL streams).  A negative deconvolved power gives
 * sigma = 0 for that bin (the reference would take sqrt of a negative). */
void axo_estimate_covmat(const axg_params *p, const int8_t *flags, const double *power,
                         const double *mat_deconv, int min_mc, int max_mc, double tol, double *cov,
                         int *iterations) {
  const int nb = p->num_bin;
  const int num_cov = nb * (nb + 1) / 2;
  const int64_t n = p->ngrid, deg = 1 << p->degrade_spec, m = n / deg, m3 = m * m * m;
  const double dspa_spec = p->dspa * deg;
  const double dwav = REF_TWOPI / dspa_spec / m;
  const double dq = REF_PI / dspa_spec / nb;
  unsigned char *mask = (unsigned char *)malloc((size_t)m3);
  build_mask(p, flags, mask);
  double *buf = (double *)malloc(sizeof(double) * 2 * m3);
  double *sigma = (double *)malloc(sizeof(double) * nb);
  double *tmp = (double *)calloc((size_t)num_cov * max_mc, sizeof(double));
  double *pw0 = (double *)malloc(sizeof(double) * nb), *pw = (double *)malloc(sizeof(double) * nb);
  for (int i = 0; i < nb; ++i) sigma[i] = sqrt(power[i] > 0 ? power[i] / 2 : 0.0) / (double)m3;
  for (int ij = 0; ij < num_cov; ++ij) cov[ij] = 0.0;
  int iter;
  for (iter = 1; iter <= max_mc; ++iter) {
    for (int64_t s = 0; s < m3; ++s) {
      int64_t qx = kint(s % m, m), qy = kint((s / m) % m, m), qz = kint(s / (m * m), m);
      double q = sqrt((double)(qx * qx + qy * qy + qz * qz)) * dwav;
      double id = round(q / dq + 0.5);
      if (id <= nb) {
        axd_u32x4 r = axd_draw(p->seed, 16u + (uint32_t)iter, 0u, (uint64_t)s);
        double u1 = axd_u01_open0(r.v[0], r.v[1]), u2 = axd_u01(r.v[2], r.v[3]);
        double rad = sqrt(-2.0 * log(u1)), th = 6.283185307179586 * u2;
        buf[2 * s] = rad * cos(th) * sigma[(int)id - 1];
        buf[2 * s + 1] = rad * sin(th) * sigma[(int)id - 1];
      } else {
        buf[2 * s] = buf[2 * s + 1] = 0.0;
      }
    }
    axo_fft3d(m, buf, -1);
    for (int64_t s = 0; s < m3; ++s)
      if (mask[s]) buf[2 * s] = buf[2 * s + 1] = 0.0;
    axo_fft3d(m, buf, +1);
    for (int i = 0; i < nb; ++i) pw0[i] = 0.0;
    for (int64_t s = 0; s < m3; ++s) {
      int64_t qx = kint(s % m, m), qy = kint((s / m) % m, m), qz = kint(s / (m * m), m);
      double q = sqrt((double)(qx * qx + qy * qy + qz * qz)) * dwav;
      double id = round(q / dq + 0.5);
      if (id <= nb) pw0[(int)id - 1] += buf[2 * s] * buf[2 * s] + buf[2 * s + 1] * buf[2 * s + 1];
    }
    /* pow = mat_deconv pow0 - power (dspmv with beta = 1) */
    for (int i = 0; i < nb; ++i) pw[i] = -power[i];
    int kk = 1;
    for (int j = 1; j <= nb; ++j) {
      double temp1 = pw0[j - 1], temp2 = 0.0;
      int k = kk;
      for (int i = 1; i <= j - 1; ++i) {
        pw[i - 1] = pw[i - 1] + temp1 * mat_deconv[k - 1];
        temp2 = temp2 + mat_deconv[k - 1] * pw0[i - 1];
        ++k;
      }
      pw[j - 1] = pw[j - 1] + temp1 * mat_deconv[kk + j - 2] + temp2;
      kk = kk + j;
    }
    for (int i = 1; i <= nb; ++i)
      for (int j = 1; j <= i; ++j) {
        int ij = i * (i - 1) / 2 + j;
        double u = pw[i - 1] * pw[j - 1];
        tmp[(size_t)(iter - 1) * num_cov + ij - 1] = cov[ij - 1];
        for (int k = 1; k <= iter - 1; ++k) tmp[(size_t)(k - 1) * num_cov + ij - 1] += u;
        cov[ij - 1] = cov[ij - 1] + u;
      }
    if (iter < min_mc) continue;
    double diff = 0.0;
    for (int i = 1; i <= nb; ++i) {
      int ij = i * (i + 1) / 2;
      double u = 0.0, v = 0.0;
      for (int k = 1; k <= iter; ++k) {
        double x = tmp[(size_t)(k - 1) * num_cov + ij - 1] / (iter - 1);
        u = u + x;
        v = v + x * x;
      }
      u = u / iter;
      v = v / iter;
      v = sqrt(v - u * u);
      double x = cov[ij - 1] / iter;
      double r = v / x;
      diff = diff > r ? diff : r;
    }
    if (diff < tol) break;
  }
  if (iter > max_mc) iter = max_mc + 1; /* not converged: the reference divides by max_mc + 1 */
  for (int ij = 0; ij < num_cov; ++ij) cov[ij] = cov[ij] / iter;
  *iterations = iter;
  free(mask); free(buf); free(sigma); free(tmp); free(pw0); free(pw);
}

/* compute_crho (spectrum.f90:316-342) with the covariance term */
void axo_compute_crho_cov(const axg_params *p, const double *wav, const double *power, const double *cov,
                          double *rho, double *drho) {
  const int nb = p->num_bin;
  double r = 0.0, d = 0.0;
  for (int i = 1; i <= nb; ++i) {
    double dd = 0.0;
    for (int j = 1; j <= i; ++j) {
      int ij = i * (i - 1) / 2 + j;
      double q = (wav[j] + wav[j - 1]) / 2;
      double dq = wav[j] - wav[j - 1];
      double q2dq = q * q * dq / REF_PI / REF_PI;
      if (j == i) q2dq = q2dq / 2;
      dd = dd + cov[ij - 1] * q2dq;
    }
    double q = (wav[i] + wav[i - 1]) / 2;
    double dq = wav[i] - wav[i - 1];
    double q2dq = q * q * dq / REF_TWOPI / REF_PI;
    d = d + dd * q2dq;
    r = r + power[i - 1] * q2dq;
  }
  *rho = r;
  *drho = sqrt(d);
}

/* get_epsilon (spectrum.f90:1002-1036) for one pair of output times */
void axo_epsilon(int nb, const double *wav, const double *p1, const double *p2, const double *c1,
                 const double *c2, double tau1, double tau2, double *eps, double *deps) {
  double tau = (tau2 + tau1) / 2;
  double f = tau / 2 / REF_TWOPI;
  double num = 0.0, den = 0.0;
  for (int i = 1; i <= nb; ++i) {
    double d = p2[i - 1] - p1[i - 1];
    double q = (wav[i - 1] + wav[i]) / 2;
    num = num + d * q * q;
    den = den + d * q;
  }
  double e = num / den * f;
  double de = 0.0;
  for (int i = 1; i <= nb; ++i) {
    double d1 = (wav[i - 1] + wav[i]) / 2;
    for (int j = 1; j <= i; ++j) {
      int ij = i * (i - 1) / 2 + j;
      double d2 = (wav[j - 1] + wav[j]) / 2;
      double d = (1 - e / d1 / f) * (1 - e / d2 / f) * (c2[ij - 1] + c1[ij - 1]) * d1 * d1 * d2 * d2;
      if (j != i) d = d * 2;
      de = de + d;
    }
  }
  *eps = e;
  *deps = sqrt(de / den / den) * f;
}
