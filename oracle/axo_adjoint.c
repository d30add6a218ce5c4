/*
 * axo_adjoint.c -- FP64 tangent-linear reference of the leapfrog of phi and
 * six u_ij, and of the band-integrated GW energy J.  TEST INFRASTRUCTURE
 * ONLY (see axo.h).  The GPU adjoint (reverse sweep) is checked against it
 * with the dot-product identity <grad J, dx0> + dJ/dlambda dlambda = dJ_TL.
 *
 * Model (the step of evolve.f90:283-339 and 259-281 with the u_ij kick):
 *   pi+  = f1 pi + f2 L phi + f3 g(phi),  g = (A|phi|^2 + B) phi + C + D conj(phi)
 *   w+_c = f1 w_c + f2 L u_c + fs S_c(phi),  S_c = 2 (Re D_i phi Re D_j phi + Im .. Im ..)
 *   phi+ = phi + h pi+,   u+ = u + h w+
 * with A = lambda/2, B = -lambda v^2/2 in the quartic model (dA/dlambda = 1/2,
 * dB/dlambda = -v^2/2; the reference potential does not depend on lambda).
 * J = sum over |k| in [kmin, kmax] of 1/2 sum_ij (|W'_TT|^2 + k^2 |W_TT|^2),
 * W = dx^3 FFT(tau u), W' = dx^3 FFT(u + tau w) -- the numerator of the u_ij
 * GW spectrum summed over the band.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "axo.h"

#define REF_PI 3.14159265359
#define REF_TWOPI (2 * REF_PI)

static inline int64_t wrap(int64_t i, int64_t n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
static inline int64_t kint(int64_t j, int64_t n) { return (j + n / 2) % n - n / 2; }

static void lambda_derivs(const axg_params *p, double *dA, double *dB) {
  if (p->potential == AXG_POT_QUARTIC) {
    *dA = 0.5;
    *dB = -(p->vev * p->vev) / 2;
  } else {
    *dA = 0.0;
    *dB = 0.0;
  }
}

/* one TL kick: (pi, w) and their perturbations, using phi, u at kick time */
static void tl_kick(const axg_params *p, const double *phi, double *pi, const double *u, double *w,
                    const double *dphi, double *dpi, const double *du, double *dw, double dlam,
                    double t, double dt) {
  const int64_t n = p->ngrid, n2 = n * n, n3 = n2 * n;
  double f[4], pot[4], dA, dB;
  axo_kick_coeffs(p, t, dt, f, pot);
  lambda_derivs(p, &dA, &dB);
  const double A = pot[0], B = pot[1], C = pot[2], D = pot[3];
  const double d = 2 * p->dspa;
  double *npi = (double *)malloc(sizeof(double) * 2 * n3), *ndpi = (double *)malloc(sizeof(double) * 2 * n3);
  double *nw = (double *)malloc(sizeof(double) * 6 * n3), *ndw = (double *)malloc(sizeof(double) * 6 * n3);
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t iz = 0; iz < n; ++iz)
    for (int64_t iy = 0; iy < n; ++iy)
      for (int64_t ix = 0; ix < n; ++ix) {
        int64_t c = iz * n2 + iy * n + ix;
        int64_t nb[6] = {iz * n2 + iy * n + wrap(ix - 1, n), iz * n2 + iy * n + wrap(ix + 1, n),
                         iz * n2 + wrap(iy - 1, n) * n + ix, iz * n2 + wrap(iy + 1, n) * n + ix,
                         wrap(iz - 1, n) * n2 + iy * n + ix, wrap(iz + 1, n) * n2 + iy * n + ix};
        double lap[2] = {0, 0}, dlap[2] = {0, 0};
        for (int q = 0; q < 2; ++q) {
          for (int k = 0; k < 6; ++k) {
            lap[q] += phi[2 * nb[k] + q];
            dlap[q] += dphi[2 * nb[k] + q];
          }
          lap[q] -= 6 * phi[2 * c + q];
          dlap[q] -= 6 * dphi[2 * c + q];
        }
        double a = phi[2 * c], b = phi[2 * c + 1], da = dphi[2 * c], db = dphi[2 * c + 1];
        double s = a * a + b * b, g0 = A * s + B;
        double gr = g0 * a + D * a + C, gi = g0 * b - D * b;
        double pd = a * da + b * db;
        double dgr = g0 * da + 2 * A * a * pd + D * da + dlam * (dA * s + dB) * a;
        double dgi = g0 * db + 2 * A * b * pd - D * db + dlam * (dA * s + dB) * b;
        npi[2 * c] = f[0] * pi[2 * c] + f[1] * lap[0] + f[2] * gr;
        npi[2 * c + 1] = f[0] * pi[2 * c + 1] + f[1] * lap[1] + f[2] * gi;
        ndpi[2 * c] = f[0] * dpi[2 * c] + f[1] * dlap[0] + f[2] * dgr;
        ndpi[2 * c + 1] = f[0] * dpi[2 * c + 1] + f[1] * dlap[1] + f[2] * dgi;
        if (u) {
          double Dr[3], Di[3], dDr[3], dDi[3];
          for (int k = 0; k < 3; ++k) {
            Dr[k] = (phi[2 * nb[2 * k + 1]] - phi[2 * nb[2 * k]]) / d;
            Di[k] = (phi[2 * nb[2 * k + 1] + 1] - phi[2 * nb[2 * k] + 1]) / d;
            dDr[k] = (dphi[2 * nb[2 * k + 1]] - dphi[2 * nb[2 * k]]) / d;
            dDi[k] = (dphi[2 * nb[2 * k + 1] + 1] - dphi[2 * nb[2 * k] + 1]) / d;
          }
          int comp = 0;
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j <= i; ++j, ++comp) {
              const double *uc = u + comp * n3, *duc = du + comp * n3;
              double lu = -6 * uc[c], dlu = -6 * duc[c];
              for (int k = 0; k < 6; ++k) {
                lu += uc[nb[k]];
                dlu += duc[nb[k]];
              }
              double S = 2 * (Dr[i] * Dr[j] + Di[i] * Di[j]);
              double dS = 2 * (dDr[i] * Dr[j] + Dr[i] * dDr[j] + dDi[i] * Di[j] + Di[i] * dDi[j]);
              nw[comp * n3 + c] = f[0] * w[comp * n3 + c] + f[1] * lu + f[3] * S;
              ndw[comp * n3 + c] = f[0] * dw[comp * n3 + c] + f[1] * dlu + f[3] * dS;
            }
        }
      }
  memcpy(pi, npi, sizeof(double) * 2 * n3);
  memcpy(dpi, ndpi, sizeof(double) * 2 * n3);
  if (u) {
    memcpy(w, nw, sizeof(double) * 6 * n3);
    memcpy(dw, ndw, sizeof(double) * 6 * n3);
  }
  free(npi); free(ndpi); free(nw); free(ndw);
}

static void tl_drift(int64_t n3, double *x, const double *v, double *dx, const double *dv, int64_t m, double h) {
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < m * n3; ++s) {
    x[s] = x[s] + h * v[s];
    dx[s] = dx[s] + h * dv[s];
  }
}

/* J and its linearisation dJ for state (u, w) and perturbation (du, dw) */
static void band_energy(const axg_params *p, const double *u, const double *w, const double *du, const double *dw,
                        double tau, double kmin, double kmax, double *J, double *dJ) {
  const int64_t n = p->ngrid, n2 = n * n, n3 = n2 * n;
  const double dv = p->dspa * p->dspa * p->dspa, dwav = REF_TWOPI / p->dspa / n;
  /* 24 complex fields: a, b, da, db for 6 components */
  double *F = (double *)malloc(sizeof(double) * 2 * 24 * n3);
  for (int c = 0; c < 6; ++c) {
    double *a = F + 2 * (c * n3), *b = F + 2 * ((6 + c) * n3), *ea = F + 2 * ((12 + c) * n3),
           *eb = F + 2 * ((18 + c) * n3);
    for (int64_t s = 0; s < n3; ++s) {
      a[2 * s] = tau * u[c * n3 + s] * dv;
      b[2 * s] = (u[c * n3 + s] + tau * w[c * n3 + s]) * dv;
      ea[2 * s] = du ? tau * du[c * n3 + s] * dv : 0.0;
      eb[2 * s] = du ? (du[c * n3 + s] + tau * dw[c * n3 + s]) * dv : 0.0;
      a[2 * s + 1] = b[2 * s + 1] = ea[2 * s + 1] = eb[2 * s + 1] = 0.0;
    }
    axo_fft3d(n, a, -1);
    axo_fft3d(n, b, -1);
    if (du) {
      axo_fft3d(n, ea, -1);
      axo_fft3d(n, eb, -1);
    }
  }
  double sJ = 0.0, sdJ = 0.0;
  const int idx[3][3] = {{0, 1, 3}, {1, 2, 4}, {3, 4, 5}};
#pragma omp parallel for reduction(+ : sJ, sdJ) schedule(static)
  for (int64_t s = 0; s < n3; ++s) {
    double q[3] = {(double)kint(s % n, n), (double)kint((s / n) % n, n), (double)kint(s / n2, n)};
    double qq = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    double k = qq * dwav;
    if (!(qq > 0) || k < kmin || k > kmax) continue;
    double kh[3] = {q[0] / qq, q[1] / qq, q[2] / qq}, P[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) P[i][j] = (i == j) - kh[i] * kh[j];
    /* Lambda applied to each of the four tensors */
    double TT[4][3][3][2];
    for (int f = 0; f < 4; ++f) {
      double M[3][3][2], R[3][3][2];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          const double *z = F + 2 * ((f * 6 + idx[i][j]) * n3 + s);
          M[i][j][0] = z[0];
          M[i][j][1] = z[1];
        }
      double tr[2] = {0, 0};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          for (int r = 0; r < 2; ++r) {
            double acc = 0;
            for (int a = 0; a < 3; ++a)
              for (int b = 0; b < 3; ++b) acc += P[i][a] * M[a][b][r] * P[b][j];
            R[i][j][r] = acc;
          }
      for (int r = 0; r < 2; ++r) tr[r] = R[0][0][r] + R[1][1][r] + R[2][2][r];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          for (int r = 0; r < 2; ++r) TT[f][i][j][r] = R[i][j][r] - 0.5 * P[i][j] * tr[r];
    }
    double ea = 0, eb = 0, dea = 0, deb = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        ea += TT[0][i][j][0] * TT[0][i][j][0] + TT[0][i][j][1] * TT[0][i][j][1];
        eb += TT[1][i][j][0] * TT[1][i][j][0] + TT[1][i][j][1] * TT[1][i][j][1];
        dea += TT[0][i][j][0] * TT[2][i][j][0] + TT[0][i][j][1] * TT[2][i][j][1];
        deb += TT[1][i][j][0] * TT[3][i][j][0] + TT[1][i][j][1] * TT[3][i][j][1];
      }
    sJ += 0.5 * (eb + k * k * ea);
    sdJ += deb + k * k * dea;
  }
  free(F);
  *J = sJ;
  if (dJ) *dJ = sdJ;
}

double axo_gw_band_energy(const axg_params *p, const double *u, const double *w, double tau, double kmin,
                          double kmax) {
  double J;
  band_energy(p, u, w, NULL, NULL, tau, kmin, kmax, &J, NULL);
  return J;
}

/* Forward state + tangent-linear perturbation through the step sequence of
 * axg_leapfrog; returns J(tau_end) in *J and its linearisation in *dJ. */
void axo_tl_run(const axg_params *p, double *phi, double *phid, double *u, double *ud, double *dphi,
                double *dphid, double *du, double *dud, double dlambda, double t1, double dt, int64_t nsteps,
                int first_half, int last_half, double kmin, double kmax, double *J, double *dJ) {
  const int64_t n3 = (int64_t)p->ngrid * p->ngrid * p->ngrid;
  double t = t1;
  if (first_half) {
    tl_drift(n3, phi, phid, dphi, dphid, 2, dt / 2);
    tl_drift(n3, u, ud, du, dud, 6, dt / 2);
    t = t + dt / 2;
  }
  for (int64_t it = 1; it <= nsteps; ++it) {
    tl_kick(p, phi, phid, u, ud, dphi, dphid, du, dud, dlambda, t, dt);
    double h = (it == nsteps && last_half) ? dt / 2 : dt;
    tl_drift(n3, phi, phid, dphi, dphid, 2, h);
    tl_drift(n3, u, ud, du, dud, 6, h);
    t = t + h;
  }
  band_energy(p, u, ud, du, dud, t, kmin, kmax, J, dJ);
}
