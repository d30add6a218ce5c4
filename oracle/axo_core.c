/*
 * axo_core.c -- oracle restatement of potential.f90, evolve.f90 and the
 * initial conditions.  TEST INFRASTRUCTURE ONLY (see axo.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "axo.h"
#include "axg_detmath.h"

/* potential.f90:8 -- pi truncated as in the reference */
#define REF_PI 3.14159265359
#define REF_TWOPI (2 * REF_PI)
/* potential.f90:30 */
#define THRM_SIGMA 2.449489742783178
/* potential.f90:26-27 */
#define N_AXION_IILM 6.68
#define CT_AXION_IILM 6.26
#define C0_AXION 1.0

int axo_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

double axo_det_atan2(double y, double x) { return axd_atan2(y, x); }
void axo_det_sincos(double x, double *s, double *c) { axd_sincos(x, s, c); }
void axo_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  axd_u32x4 c;
  memcpy(c.v, ctr, sizeof(c.v));
  axd_u32x4 o = axd_philox4x32_10(c, key[0], key[1]);
  memcpy(out, o.v, sizeof(o.v));
}

/* potential.f90:34-41 */
double axo_msquared(double thrm) { return (thrm * thrm - THRM_SIGMA * THRM_SIGMA) / 3; }

/* potential.f90:62-79 */
double axo_maxion2(double thrm, double kappa) {
  double thrm12 = kappa * pow(CT_AXION_IILM / C0_AXION, 1.0 / N_AXION_IILM);
  double m;
  if (thrm > thrm12)
    m = CT_AXION_IILM * pow(kappa / thrm, N_AXION_IILM);
  else
    m = C0_AXION;
  double k2 = kappa * kappa;
  return m * (k2 * k2);
}

/* evolve.f90:291-305 (+ the quartic model of the extension) */
void axo_kick_coeffs(const axg_params *p, double t, double dt, double f[4], double pot[4]) {
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
    double thrm = (p->flags & AXG_F_INITIAL_LOOP) ? 0.0 : THRM_SIGMA / t;
    double m2 = axo_msquared(thrm);
    double ma2 = axo_maxion2(thrm, p->kappa);
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
      double ma2 = p->ma2_0 * pow(t / p->tau_axion_on, p->ma2_power);
      if (p->n_dw == 2) {
        pot[1] += ma2 / 4;
        pot[3] = -(ma2 / 4);
      } else {
        pot[2] = -(ma2 * p->vev / 2);
      }
    }
  }
}

/* evolve.f90:10-24 */
void axo_get_dtau(const axg_params *p, double tau1, double tau2, double eps_dtau, double *dtau,
                  int64_t *n) {
  double dwav = REF_TWOPI / p->dspa / p->ngrid; /* settings.f90:295 */
  double mass = (p->potential == AXG_POT_REFERENCE) ? THRM_SIGMA
                                                     : sqrt(2 * p->lambda) * p->vev;
  double omega = mass * tau2 * p->sigma_cr;
  double kmax = dwav * p->ngrid;
  omega = sqrt(kmax * kmax + omega * omega);
  double dt = eps_dtau / omega;
  int64_t nt = (int64_t)ceil((tau2 - tau1) / dt);
  if (nt < 1) nt = 1;
  *dtau = (tau2 - tau1) / nt;
  *n = nt;
}

/* evolve.f90:259-281: data1 = data1 + dt*data2 over the interior */
void axo_evolve_phi(const axg_params *p, double *phi, const double *phidot, double *u,
                    const double *udot, double dt) {
  int64_t n3 = (int64_t)p->ngrid * p->ngrid * p->ngrid;
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < n3; ++s) {
    phi[2 * s] = phi[2 * s] + dt * phidot[2 * s];
    phi[2 * s + 1] = phi[2 * s + 1] + dt * phidot[2 * s + 1];
  }
  if (u) {
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < 6 * n3; ++s) u[s] = u[s] + dt * udot[s];
  }
}

static inline int64_t wrap(int64_t i, int64_t n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

/* evolve.f90:283-339 (kick of phi, 7-point Laplacian with periodic wrap in
 * x, y and, on one rank, z) and the u_ij kick of the extension:
 *   u' <- fact1 u' + fact2 lap(u) + fact_s * S_ij,
 *   S_ij = d_i phi d_j phi* + c.c. = 2 (Re d_i Re d_j + Im d_i Im d_j),
 *   d_i phi = (phi(x+e_i) - phi(x-e_i)) / (2 dspa)  (grav_waves.f90:343-346). */
void axo_evolve_phidot(const axg_params *p, const double *phi, double *phidot, const double *u,
                       double *udot, double t, double dt) {
  const int64_t n = p->ngrid, n2 = n * n, n3 = n2 * n;
  double f[4], pot[4];
  axo_kick_coeffs(p, t, dt, f, pot);
  const double fact1 = f[0], fact2 = f[1], fact3 = f[2], facts = f[3];
  const double A = pot[0], B = pot[1], C = pot[2], D = pot[3];
  const double d = p->dspa * 2;
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t iz = 0; iz < n; ++iz) {
    for (int64_t iy = 0; iy < n; ++iy) {
      int64_t iz1 = wrap(iz - 1, n), iz2 = wrap(iz + 1, n);
      int64_t iy1 = wrap(iy - 1, n), iy2 = wrap(iy + 1, n);
      for (int64_t ix = 0; ix < n; ++ix) {
        int64_t ix1 = wrap(ix - 1, n), ix2 = wrap(ix + 1, n);
        int64_t c = iz * n2 + iy * n + ix;
        int64_t sx1 = iz * n2 + iy * n + ix1, sx2 = iz * n2 + iy * n + ix2;
        int64_t sy1 = iz * n2 + iy1 * n + ix, sy2 = iz * n2 + iy2 * n + ix;
        int64_t sz1 = iz1 * n2 + iy * n + ix, sz2 = iz2 * n2 + iy * n + ix;
        double lr = phi[2 * sx1] + phi[2 * sx2];
        lr = lr + phi[2 * sy1];
        lr = lr + phi[2 * sy2];
        lr = lr + phi[2 * sz1];
        lr = lr + phi[2 * sz2];
        lr = lr - 6 * phi[2 * c];
        double li = phi[2 * sx1 + 1] + phi[2 * sx2 + 1];
        li = li + phi[2 * sy1 + 1];
        li = li + phi[2 * sy2 + 1];
        li = li + phi[2 * sz1 + 1];
        li = li + phi[2 * sz2 + 1];
        li = li - 6 * phi[2 * c + 1];
        /* potential.f90:43-60 dVdphi, generalised to (A s2 + B) phi + C + D conj(phi) */
        double a = phi[2 * c], b = phi[2 * c + 1];
        double s2 = a * a + b * b;
        double g = A * s2 + B;
        double vr = g * a, vi = g * b;
        if (D != 0.0) {
          vr = vr + D * a;
          vi = vi - D * b;
        }
        vr = vr + C;
        double pr = fact1 * phidot[2 * c] + fact2 * lr;
        pr = pr + fact3 * vr;
        double pi_ = fact1 * phidot[2 * c + 1] + fact2 * li;
        pi_ = pi_ + fact3 * vi;
        phidot[2 * c] = pr;
        phidot[2 * c + 1] = pi_;
        if (u) {
          double dr[3], di[3];
          dr[0] = (phi[2 * sx2] - phi[2 * sx1]) / d;
          di[0] = (phi[2 * sx2 + 1] - phi[2 * sx1 + 1]) / d;
          dr[1] = (phi[2 * sy2] - phi[2 * sy1]) / d;
          di[1] = (phi[2 * sy2 + 1] - phi[2 * sy1 + 1]) / d;
          dr[2] = (phi[2 * sz2] - phi[2 * sz1]) / d;
          di[2] = (phi[2 * sz2 + 1] - phi[2 * sz1 + 1]) / d;
          int comp = 0;
          for (int i = 0; i < 3; ++i) {
            for (int j = 0; j <= i; ++j, ++comp) {
              const double *uc = u + comp * n3;
              double src = dr[i] * dr[j] + di[i] * di[j];
              src = 2 * src;
              double lu = uc[sx1] + uc[sx2];
              lu = lu + uc[sy1];
              lu = lu + uc[sy2];
              lu = lu + uc[sz1];
              lu = lu + uc[sz2];
              lu = lu - 6 * uc[c];
              double v = fact1 * udot[comp * n3 + c] + fact2 * lu;
              v = v + facts * src;
              udot[comp * n3 + c] = v;
            }
          }
        }
      }
    }
  }
}

/* evolve.f90:238-257 drift-kick-drift */
int64_t axo_symplectic_integration(const axg_params *p, double *phi, double *phidot, double *u,
                                   double *udot, double *acc, double t1, double t2,
                                   double eps_dtau) {
  double dt;
  int64_t nt;
  axo_get_dtau(p, t1, t2, eps_dtau, &dt, &nt);
  double t = t1;
  int uij = (p->gw_mode == AXG_GW_UIJ) && u;
  for (int64_t it = 1; it <= nt; ++it) {
    if (it == 1) {
      axo_evolve_phi(p, phi, phidot, uij ? u : NULL, udot, dt / 2);
      t = t + dt / 2;
    }
    axo_evolve_phidot(p, phi, phidot, uij ? u : NULL, udot, t, dt);
    if (p->gw_mode == AXG_GW_GREEN && acc) axo_grav_wave_integration(p, phi, acc, t, dt);
    double h = (it == nt) ? dt / 2 : dt;
    axo_evolve_phi(p, phi, phidot, uij ? u : NULL, udot, h);
    t = t + h;
  }
  return nt;
}

/* ---------------------------------------------------------------------- */
/* FFT: iterative radix-2 for powers of two, direct DFT otherwise.         */
/* ---------------------------------------------------------------------- */
static void fft1d_pow2(int64_t n, double *re, double *im, const double *wr, const double *wi) {
  for (int64_t i = 1, j = 0; i < n; ++i) {
    int64_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      double t = re[i]; re[i] = re[j]; re[j] = t;
      t = im[i]; im[i] = im[j]; im[j] = t;
    }
  }
  for (int64_t len = 2; len <= n; len <<= 1) {
    int64_t half = len >> 1, step = n / len;
    for (int64_t i = 0; i < n; i += len) {
      for (int64_t k = 0; k < half; ++k) {
        double twr = wr[k * step], twi = wi[k * step];
        double xr = re[i + k + half], xi = im[i + k + half];
        double tr = xr * twr - xi * twi;
        double ti = xr * twi + xi * twr;
        re[i + k + half] = re[i + k] - tr;
        im[i + k + half] = im[i + k] - ti;
        re[i + k] = re[i + k] + tr;
        im[i + k] = im[i + k] + ti;
      }
    }
  }
}

static void dft1d(int64_t n, double *re, double *im, const double *wr, const double *wi,
                  double *tr, double *ti) {
  for (int64_t k = 0; k < n; ++k) {
    double sr = 0, si = 0;
    for (int64_t j = 0; j < n; ++j) {
      int64_t m = (j * k) % n;
      sr += re[j] * wr[m] - im[j] * wi[m];
      si += re[j] * wi[m] + im[j] * wr[m];
    }
    tr[k] = sr;
    ti[k] = si;
  }
  memcpy(re, tr, n * sizeof(double));
  memcpy(im, ti, n * sizeof(double));
}

void axo_fft3d(int64_t n, double *data, int sign) {
  int pow2 = (n & (n - 1)) == 0;
  double *wr = (double *)malloc(n * sizeof(double));
  double *wi = (double *)malloc(n * sizeof(double));
  const double tp = 6.283185307179586476925286766559;
  for (int64_t k = 0; k < n; ++k) {
    wr[k] = cos(tp * (double)k / (double)n);
    wi[k] = sign * sin(tp * (double)k / (double)n);
  }
  const int64_t n2 = n * n;
  for (int axis = 0; axis < 3; ++axis) {
    int64_t stride = axis == 0 ? 1 : (axis == 1 ? n : n2);
#pragma omp parallel
    {
      double *re = (double *)malloc(n * sizeof(double));
      double *im = (double *)malloc(n * sizeof(double));
      double *tr = (double *)malloc(n * sizeof(double));
      double *ti = (double *)malloc(n * sizeof(double));
#pragma omp for schedule(static)
      for (int64_t line = 0; line < n2; ++line) {
        int64_t base;
        if (axis == 0) base = line * n;
        else if (axis == 1) base = (line / n) * n2 + (line % n);
        else base = line;
        for (int64_t k = 0; k < n; ++k) {
          re[k] = data[2 * (base + k * stride)];
          im[k] = data[2 * (base + k * stride) + 1];
        }
        if (pow2) fft1d_pow2(n, re, im, wr, wi);
        else dft1d(n, re, im, wr, wi, tr, ti);
        for (int64_t k = 0; k < n; ++k) {
          data[2 * (base + k * stride)] = re[k];
          data[2 * (base + k * stride) + 1] = im[k];
        }
      }
      free(re); free(im); free(tr); free(ti);
    }
  }
  free(wr);
  free(wi);
}

/* integer wave-vector component of 0-based FFT index j:
 * mod(j+1 + N/2 - 1, N) - N/2 (grav_waves.f90:165, spectrum.f90:237) */
static inline int64_t kint(int64_t j, int64_t n) { return (j + n / 2) % n - n / 2; }

/* Box-Muller pair from one Philox draw (axd_draw layout). */
static void gauss_pair(uint64_t seed, uint32_t stream, uint32_t real, uint64_t index, double *g0,
                       double *g1) {
  axd_u32x4 r = axd_draw(seed, stream, real, index);
  double u1 = axd_u01_open0(r.v[0], r.v[1]);
  double u2 = axd_u01(r.v[2], r.v[3]);
  double rad = sqrt(-2.0 * log(u1));
  double th = 6.283185307179586 * u2;
  *g0 = rad * cos(th);
  *g1 = rad * sin(th);
}

void axo_ic_gaussian_flat(const axg_params *p, double kcut, uint32_t realisation, double *phi,
                          double *phidot) {
  const int64_t n = p->ngrid, n2 = n * n, n3 = n2 * n;
  const double dwav = REF_TWOPI / p->dspa / n;
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < n3; ++s) {
    int64_t ix = s % n, iy = (s / n) % n, iz = s / n2;
    int64_t qx = kint(ix, n), qy = kint(iy, n), qz = kint(iz, n);
    double q = sqrt((double)(qx * qx + qy * qy + qz * qz)) * dwav;
    double g0 = 0.0, g1 = 0.0;
    if (q <= kcut) gauss_pair(p->seed, 0u, realisation, (uint64_t)s, &g0, &g1);
    phi[2 * s] = g0;
    phi[2 * s + 1] = g1;
  }
  axo_fft3d(n, phi, +1);
  double sum = 0.0;
#pragma omp parallel for reduction(+ : sum) schedule(static)
  for (int64_t s = 0; s < n3; ++s) sum += phi[2 * s] * phi[2 * s] + phi[2 * s + 1] * phi[2 * s + 1];
  double mean = sum / (double)n3;
  double scale = mean > 0 ? p->vev / sqrt(mean) : 0.0;
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < n3; ++s) {
    phi[2 * s] *= scale;
    phi[2 * s + 1] *= scale;
    phidot[2 * s] = 0.0;
    phidot[2 * s + 1] = 0.0;
  }
}

/* initial.f90:80-238 with initial_phi_phidot (initial.f90:363-390) */
void axo_ic_thermal(const axg_params *p, double tau_ini, uint32_t realisation, double *phi,
                    double *phidot) {
  const int64_t n = p->ngrid, n2 = n * n, n3 = n2 * n;
  const double dwav = REF_TWOPI / p->dspa / n;
  const double dv_wav = pow(dwav / REF_TWOPI, 3);
  for (int ip = 1; ip <= 2; ++ip) {
    double *dst = (ip == 1) ? phi : phidot;
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < n3; ++s) {
      int64_t ix = s % n, iy = (s / n) % n, iz = s / n2;
      double g0, g1;
      gauss_pair(p->seed, (uint32_t)ip, realisation, (uint64_t)s, &g0, &g1);
      double xr = g0 * dv_wav, xi = g1 * dv_wav;
      int64_t qx = kint(ix, n), qy = kint(iy, n), qz = kint(iz, n);
      double wav2 = sqrt((double)(qx * qx + qy * qy + qz * qz)) * dwav;
      wav2 = (wav2 / tau_ini / p->sigma_cr);
      wav2 = wav2 * wav2;
      double thrm = THRM_SIGMA / tau_ini;
      double osc = sqrt(axo_msquared(thrm) + wav2);
      double fbe = exp(-osc / thrm);
      fbe = fbe / (1 - fbe);
      double var = fbe * osc / dv_wav / p->sigma_cr;
      double f = sqrt(var / 2);
      if (ip == 1) f = f / (osc * p->sigma_cr);
      dst[2 * s] = xr * f;
      dst[2 * s + 1] = xi * f;
    }
    axo_fft3d(n, dst, -1);
  }
}

void axo_field_moments(const axg_params *p, const double *phi, const double *phidot, double tau,
                       double out[4]) {
  const int64_t n = p->ngrid, n2 = n * n, n3 = n2 * n;
  double f[4], pot[4];
  axo_kick_coeffs(p, tau, 0.0, f, pot);
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  const double idx2 = 1.0 / (p->dspa * p->dspa);
#pragma omp parallel for collapse(2) reduction(+ : s0, s1, s2, s3) schedule(static)
  for (int64_t iz = 0; iz < n; ++iz)
    for (int64_t iy = 0; iy < n; ++iy)
      for (int64_t ix = 0; ix < n; ++ix) {
        int64_t c = iz * n2 + iy * n + ix;
        double a = phi[2 * c], b = phi[2 * c + 1];
        double m = a * a + b * b;
        s0 += m;
        s1 += phidot[2 * c] * phidot[2 * c] + phidot[2 * c + 1] * phidot[2 * c + 1];
        int64_t nb[3] = {iz * n2 + iy * n + wrap(ix + 1, n), iz * n2 + wrap(iy + 1, n) * n + ix,
                         wrap(iz + 1, n) * n2 + iy * n + ix};
        double g = 0;
        for (int k = 0; k < 3; ++k) {
          double dr = phi[2 * nb[k]] - a, di = phi[2 * nb[k] + 1] - b;
          g += dr * dr + di * di;
        }
        s2 += g * idx2;
        /* V with dV/dphi* = (A|phi|^2+B) phi + C + D conj(phi) */
        s3 += 0.5 * pot[0] * m * m + pot[1] * m + 2 * pot[2] * a + pot[3] * (a * a - b * b);
      }
  out[0] = s0 / n3;
  out[1] = s1 / n3;
  out[2] = s2 / n3;
  out[3] = s3 / n3;
}
