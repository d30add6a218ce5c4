/*
 * axo_gw.c -- oracle restatement of grav_waves.f90 (Green's-function GW
 * integration and spectrum) and of the u_ij TT spectrum of the extension.
 * TEST INFRASTRUCTURE ONLY (see axo.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "axo.h"

#define REF_PI 3.14159265359
#define REF_TWOPI (2 * REF_PI)
/* potential.f90:13-23 */
#define GEV_IN_HZ 1.5192488833521e24
#define BIGH 2.1332e-42
#define MSTAR_IN_GEV 2.435e18
#define BIGH_IN_MSTAR (BIGH / MSTAR_IN_GEV)

static inline int64_t wrap(int64_t i, int64_t n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
static inline int64_t kint(int64_t j, int64_t n) { return (j + n / 2) % n - n / 2; }

/* init_grav (grav_waves.f90:37-45): the Green's-function grid is the lattice
 * coarse-grained by deg = 2^degrade_spec: ngrid_grav = ngrid / deg,
 * dspa_grav = dspa * deg. */
void axo_gw_grid(const axg_params *p, int64_t *ng, double *dspa_g) {
  const int64_t deg = (int64_t)1 << p->degrade_spec;
  *ng = p->ngrid / deg;
  *dspa_g = p->dspa * (double)deg;
}

/* grav_waves.f90:323-356 (no degradation) */
void axo_data1_to_arr_dphi(const axg_params *p, const double *phi, double *dphi) {
  const int64_t n = p->ngrid, n2 = n * n, n3 = n2 * n;
  const double d = p->dspa * 2;
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t iz = 0; iz < n; ++iz)
    for (int64_t iy = 0; iy < n; ++iy)
      for (int64_t ix = 0; ix < n; ++ix) {
        int64_t c = iz * n2 + iy * n + ix;
        int64_t sx2 = iz * n2 + iy * n + wrap(ix + 1, n), sx1 = iz * n2 + iy * n + wrap(ix - 1, n);
        int64_t sy2 = iz * n2 + wrap(iy + 1, n) * n + ix, sy1 = iz * n2 + wrap(iy - 1, n) * n + ix;
        int64_t sz2 = wrap(iz + 1, n) * n2 + iy * n + ix, sz1 = wrap(iz - 1, n) * n2 + iy * n + ix;
        int64_t a[3] = {sx2, sy2, sz2}, b[3] = {sx1, sy1, sz1};
        for (int k = 0; k < 3; ++k) {
          dphi[2 * (k * n3 + c)] = (phi[2 * a[k]] - phi[2 * b[k]]) / d;
          dphi[2 * (k * n3 + c) + 1] = (phi[2 * a[k] + 1] - phi[2 * b[k] + 1]) / d;
        }
      }
}

/* grav_waves.f90:358-415 data1_to_arr_dphi_degrade on one rank: per coarse
 * cell the central differences of the deg^3 fine sites it covers are summed
 * (z outer, then y, then x, each step (sum + phi(x+e)) - phi(x-e)), then
 * divided by d = deg^3 dspa 2.  dphi[3][ng^3][2]. */
void axo_data1_to_arr_dphi_degrade(const axg_params *p, const double *phi, double *dphi) {
  const int64_t n = p->ngrid, n2 = n * n, deg = (int64_t)1 << p->degrade_spec, m = n / deg, m3 = m * m * m;
  const double d = (double)(deg * deg * deg) * p->dspa * 2;
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t cz = 0; cz < m; ++cz)
    for (int64_t cy = 0; cy < m; ++cy)
      for (int64_t cx = 0; cx < m; ++cx) {
        double sr[3] = {0.0, 0.0, 0.0}, si[3] = {0.0, 0.0, 0.0};
        for (int64_t iz = cz * deg; iz < (cz + 1) * deg; ++iz)
          for (int64_t iy = cy * deg; iy < (cy + 1) * deg; ++iy)
            for (int64_t ix = cx * deg; ix < (cx + 1) * deg; ++ix) {
              const int64_t a[3] = {iz * n2 + iy * n + wrap(ix + 1, n), iz * n2 + wrap(iy + 1, n) * n + ix,
                                    wrap(iz + 1, n) * n2 + iy * n + ix};
              const int64_t b[3] = {iz * n2 + iy * n + wrap(ix - 1, n), iz * n2 + wrap(iy - 1, n) * n + ix,
                                    wrap(iz - 1, n) * n2 + iy * n + ix};
              for (int k = 0; k < 3; ++k) {
                sr[k] = (sr[k] + phi[2 * a[k]]) - phi[2 * b[k]];
                si[k] = (si[k] + phi[2 * a[k] + 1]) - phi[2 * b[k] + 1];
              }
            }
        const int64_t c = (cz * m + cy) * m + cx;
        for (int k = 0; k < 3; ++k) {
          dphi[2 * (k * m3 + c)] = sr[k] / d;
          dphi[2 * (k * m3 + c) + 1] = si[k] / d;
        }
      }
}

/* grav_waves.f90:157-191, 0-based FFT indices in ixyz */
void axo_get_comwav_grav(const axg_params *p, const int64_t ixyz[3], double *q, double pol[2],
                         int i, int j) {
  int64_t n;
  double dspa_g;
  axo_gw_grid(p, &n, &dspa_g);
  double qh[3];
  for (int k = 0; k < 3; ++k) qh[k] = (double)kint(ixyz[k], n);
  double qq = qh[0] * qh[0] + qh[1] * qh[1];
  qq = qq + qh[2] * qh[2];
  qq = sqrt(qq);
  if (pol) {
    if (qq > 0.0) {
      for (int k = 0; k < 3; ++k) qh[k] = qh[k] / qq;
      double r = sqrt(qh[0] * qh[0] + qh[1] * qh[1]);
      double c, s;
      if (r > 0.0) {
        c = qh[0] / r;
        s = qh[1] / r;
      } else {
        c = 1.0;
        s = 0.0;
      }
      double pr[3] = {qh[2] * c, qh[2] * s, -r};
      double pim[3] = {-s, c, 0.0};
      double a = pr[i - 1], b = pim[i - 1], cc = pr[j - 1], dd = pim[j - 1];
      pol[0] = a * cc - b * dd;
      pol[1] = a * dd + b * cc;
      if (i == j) {
        pol[0] = pol[0] / 2;
        pol[1] = pol[1] / 2;
      }
    } else {
      pol[0] = 0.0;
      pol[1] = 0.0;
    }
  }
  const double dwav = REF_TWOPI / dspa_g / n; /* dwav_grav, grav_waves.f90:43 */
  *q = qq * dwav;
}

/* grav_waves.f90:193-255 */
void axo_grav_wave_integration(const axg_params *p, const double *phi, double *acc, double tau,
                               double dtau) {
  int64_t n;
  double dspa_g;
  axo_gw_grid(p, &n, &dspa_g);
  const int64_t n2 = n * n, n3 = n2 * n;
  double *dphi = (double *)malloc(sizeof(double) * 2 * 3 * n3);
  double *buf = (double *)malloc(sizeof(double) * 2 * n3);
  /* grav_waves.f90:203-207: the degraded differences unless degrade_spec = 0 */
  if (p->degrade_spec > 0)
    axo_data1_to_arr_dphi_degrade(p, phi, dphi);
  else
    axo_data1_to_arr_dphi(p, phi, dphi);
  const double dv = dspa_g * dspa_g * dspa_g; /* dv_spa_grav, grav_waves.f90:44 */
  const double dw = tau * dtau * dv * (p->sigma_cr * p->sigma_cr);
  const int ref = p->compat == AXG_COMPAT_REF;
  double *a11 = acc, *a21 = acc + 2 * n3, *a12 = acc + 4 * n3, *a22 = acc + 6 * n3;
  for (int i = 1; i <= 3; ++i) {
    for (int j = 1; j <= i; ++j) {
      const double *di = dphi + 2 * (i - 1) * n3, *dj = dphi + 2 * (j - 1) * n3;
#pragma omp parallel for schedule(static)
      for (int64_t s = 0; s < n3; ++s) {
        double ar = di[2 * s], ai = di[2 * s + 1], br = dj[2 * s], bi = dj[2 * s + 1];
        /* a*conj(b) + conj(a)*b */
        double r1 = ar * br + ai * bi, i1 = ai * br - ar * bi;
        double r2 = ar * br + ai * bi, i2 = ar * bi - ai * br;
        buf[2 * s] = r1 + r2;
        buf[2 * s + 1] = i1 + i2;
      }
      axo_fft3d(n, buf, +1);
#pragma omp parallel for schedule(static)
      for (int64_t s = 0; s < n3; ++s) {
        int64_t ixyz[3] = {s % n, (s / n) % n, s / n2};
        double q, pol[2];
        axo_get_comwav_grav(p, ixyz, &q, pol, i, j);
        q = q * tau;
        double c = cos(q), sn = sin(q);
        double ppr = pol[0] * dw, ppi = pol[1] * dw;
        double pnr = ppr, pni = -ppi;
        double Sr = buf[2 * s], Si = buf[2 * s + 1];
        double xr, xi, tr, ti;
        /* arr_grav(1,1) += c*polp*S */
        tr = c * ppr; ti = c * ppi;
        xr = tr * Sr - ti * Si; xi = tr * Si + ti * Sr;
        a11[2 * s] = a11[2 * s] + xr;
        a11[2 * s + 1] = a11[2 * s + 1] + xi;
        /* arr_grav(2,1) = arr_grav(1,2 | 2,1) + s*polp*S */
        tr = sn * ppr; ti = sn * ppi;
        xr = tr * Sr - ti * Si; xi = tr * Si + ti * Sr;
        double o12r = a12[2 * s], o12i = a12[2 * s + 1];
        if (ref) {
          a21[2 * s] = o12r + xr;
          a21[2 * s + 1] = o12i + xi;
        } else {
          a21[2 * s] = a21[2 * s] + xr;
          a21[2 * s + 1] = a21[2 * s + 1] + xi;
        }
        /* arr_grav(1,2) = arr_grav(2,1 new | 1,2) + c*poln*S */
        tr = c * pnr; ti = c * pni;
        xr = tr * Sr - ti * Si; xi = tr * Si + ti * Sr;
        if (ref) {
          a12[2 * s] = a21[2 * s] + xr;
          a12[2 * s + 1] = a21[2 * s + 1] + xi;
        } else {
          a12[2 * s] = o12r + xr;
          a12[2 * s + 1] = o12i + xi;
        }
        /* arr_grav(2,2) += s*poln*S */
        tr = sn * pnr; ti = sn * pni;
        xr = tr * Sr - ti * Si; xi = tr * Si + ti * Sr;
        a22[2 * s] = a22[2 * s] + xr;
        a22[2 * s + 1] = a22[2 * s + 1] + xi;
      }
    }
  }
  free(dphi);
  free(buf);
}

/* grav_waves.f90:265-267 normalisation on an n^3 grid of spacing dspa */
static double gw_fact(const axg_params *p, int64_t n, double dspa) {
  double dwav = REF_TWOPI / dspa / n;
  double dv_wav = pow(dwav / REF_TWOPI, 3);
  double tc = p->tau_cr;
  double tc6 = tc * tc * tc * tc * tc * tc;
  double a4 = p->a_now * p->a_now * p->a_now * p->a_now;
  return 1 / tc6 / (BIGH_IN_MSTAR * BIGH_IN_MSTAR) / a4 / 3 / (REF_TWOPI * REF_TWOPI) * dv_wav;
}

/* grav_waves.f90:62-71 bins on (0, pi / dspa] */
static void lin_edges(double dspa, int nb, double *wave, double *dq_out) {
  double qmax = REF_PI / dspa;
  double dq = qmax / nb;
  double prev = 0.0;
  for (int k = 1; k <= nb; ++k) {
    double cur = prev + dq;
    wave[k - 1] = (cur + prev) / 2; /* bin centre */
    prev = cur;
  }
  *dq_out = dq;
}

/* grav_waves.f90:257-321 */
void axo_grav_spec_estimation(const axg_params *p, const double *acc, double *wave,
                              double *power, double *numer, double *denom) {
  int64_t n;
  double dspa_g;
  axo_gw_grid(p, &n, &dspa_g);
  const int64_t n2 = n * n, n3 = n2 * n;
  const int nb = p->num_bin_grav;
  double dq;
  lin_edges(dspa_g, nb, wave, &dq);
  double fact = gw_fact(p, n, dspa_g);
  for (int k = 0; k < nb; ++k) numer[k] = denom[k] = 0.0;
  for (int64_t s = 0; s < n3; ++s) {
    int64_t ixyz[3] = {s % n, (s / n) % n, s / n2};
    double q;
    axo_get_comwav_grav(p, ixyz, &q, NULL, 0, 0);
    double iqd = round(q / dq + 0.5);
    if (q > 0.0 && iqd >= 1 && iqd <= nb) {
      int iq = (int)iqd;
      double v = 0.0;
      for (int a = 0; a < 4; ++a) {
        double re = acc[2 * (a * n3 + s)], im = acc[2 * (a * n3 + s) + 1];
        v += re * re + im * im;
      }
      denom[iq - 1] += 1;
      numer[iq - 1] += v;
    }
  }
  for (int k = 0; k < nb; ++k) {
    double q = wave[k];
    power[k] = denom[k] > 0 ? numer[k] / denom[k] * (q * q * q) * fact : 0.0;
  }
}

static void log_edges(int64_t n, double dspa, int nlog, double *edges) {
  double kmin = REF_TWOPI / dspa / n, kmax = REF_PI / dspa;
  for (int k = 0; k <= nlog; ++k) edges[k] = kmin * pow(kmax / kmin, (double)k / nlog);
}

/* index of the log bin holding q (q in [edges[0], edges[nlog]]), -1 outside */
static int log_bin(double q, const double *edges, int nlog) {
  if (!(q >= edges[0]) || q > edges[nlog]) return -1;
  double x = log(q / edges[0]) / log(edges[nlog] / edges[0]) * nlog;
  int b = (int)floor(x);
  if (b >= nlog) b = nlog - 1;
  if (b < 0) b = 0;
  /* guard the rounding of log() near an edge */
  while (b > 0 && q < edges[b]) --b;
  while (b < nlog - 1 && q >= edges[b + 1]) ++b;
  return b;
}

void axo_grav_spec_log_green(const axg_params *p, const double *acc, double *edges,
                             double *power, double *numer, double *denom) {
  int64_t n;
  double dspa_g;
  axo_gw_grid(p, &n, &dspa_g);
  const int64_t n2 = n * n, n3 = n2 * n;
  const int nl = p->gw_log_bins;
  log_edges(n, dspa_g, nl, edges);
  double fact = gw_fact(p, n, dspa_g);
  for (int k = 0; k < nl; ++k) numer[k] = denom[k] = 0.0;
  for (int64_t s = 0; s < n3; ++s) {
    int64_t ixyz[3] = {s % n, (s / n) % n, s / n2};
    double q;
    axo_get_comwav_grav(p, ixyz, &q, NULL, 0, 0);
    if (!(q > 0.0)) continue;
    int b = log_bin(q, edges, nl);
    if (b < 0) continue;
    double v = 0.0;
    for (int a = 0; a < 4; ++a) {
      double re = acc[2 * (a * n3 + s)], im = acc[2 * (a * n3 + s) + 1];
      v += re * re + im * im;
    }
    denom[b] += 1;
    numer[b] += v;
  }
  for (int k = 0; k < nl; ++k) {
    double q = sqrt(edges[k] * edges[k + 1]);
    power[k] = denom[k] > 0 ? numer[k] / denom[k] * (q * q * q) * fact : 0.0;
  }
}

/*
 * u_ij spectrum.  w = tau u, w' = u + tau u' (w = a u with a ~ tau obeys
 * w'' - lap w = tau sigma_cr^2 S_ij).  With W = dx^3 FFT(w):
 *   numer(k) = sum_ij ( |W'^TT_ij|^2 + k^2 |W^TT_ij|^2 ).
 * Summed over a k-shell it is the Green's-function numerator
 * sum_pol (|A_c|^2 + |A_s|^2) of grav_waves.f90:283-284 in the continuum
 * limit: with the polarisation p = e1 + i e2 of get_comwav_grav (157-191),
 * |X+|^2 + |X-|^2 = sum_ij |(Lambda S)_ij|^2, and over a shell holding k and
 * -k both reduce to sum_k |int e^{i k tau} tau sigma_cr^2 (Lambda S)(k) dtau|^2
 * (dw carries the dx^3 of W).  The lattice wave equation of u_ij differs
 * from the Green's function e^{i k tau} at O((k dx)^2).  TT:
 * Lambda = P u P - P tr(P u)/2, P = 1 - khat khat, khat from the integer
 * wave vector.
 */
static void tt_accumulate(const double *Ur, const double *Ui, const double kh[3], double *out) {
  /* U symmetric 3x3 complex from 6 comps (11,21,22,31,32,33) */
  double Mr[3][3], Mi[3][3], P[3][3];
  int idx[3][3] = {{0, 1, 3}, {1, 2, 4}, {3, 4, 5}};
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      P[a][b] = (a == b ? 1.0 : 0.0) - kh[a] * kh[b];
      Mr[a][b] = Ur[idx[a][b]];
      Mi[a][b] = Ui[idx[a][b]];
    }
  double Tr[3][3], Ti[3][3], Rr[3][3], Ri[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double sr = 0, si = 0;
      for (int c = 0; c < 3; ++c) {
        sr += P[a][c] * Mr[c][b];
        si += P[a][c] * Mi[c][b];
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
  double trr = Rr[0][0] + Rr[1][1] + Rr[2][2], tri = Ri[0][0] + Ri[1][1] + Ri[2][2];
  double s = 0;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double vr = Rr[a][b] - 0.5 * P[a][b] * trr, vi = Ri[a][b] - 0.5 * P[a][b] * tri;
      s += vr * vr + vi * vi;
    }
  *out = s;
}

static void uij_numer(const axg_params *p, const double *u, const double *udot, double tau,
                      double *qarr, double *varr) {
  const int64_t n = p->ngrid, n2 = n * n, n3 = n2 * n;
  const double dv = p->dspa * p->dspa * p->dspa;
  double *W = (double *)malloc(sizeof(double) * 2 * 12 * n3);
  for (int c = 0; c < 6; ++c) {
    double *w = W + 2 * c * n3, *wd = W + 2 * (6 + c) * n3;
    for (int64_t s = 0; s < n3; ++s) {
      w[2 * s] = tau * u[c * n3 + s] * dv;
      w[2 * s + 1] = 0.0;
      wd[2 * s] = (u[c * n3 + s] + tau * udot[c * n3 + s]) * dv;
      wd[2 * s + 1] = 0.0;
    }
    axo_fft3d(n, w, +1);
    axo_fft3d(n, wd, +1);
  }
  const double dwav = REF_TWOPI / p->dspa / n;
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < n3; ++s) {
    int64_t ixyz[3] = {s % n, (s / n) % n, s / n2};
    double qi[3];
    for (int k = 0; k < 3; ++k) qi[k] = (double)kint(ixyz[k], n);
    double qq = sqrt(qi[0] * qi[0] + qi[1] * qi[1] + qi[2] * qi[2]);
    qarr[s] = qq * dwav;
    if (!(qq > 0)) {
      varr[s] = 0.0;
      continue;
    }
    double kh[3] = {qi[0] / qq, qi[1] / qq, qi[2] / qq};
    double Ur[6], Ui[6], Dr[6], Di[6];
    for (int c = 0; c < 6; ++c) {
      Ur[c] = W[2 * (c * n3 + s)];
      Ui[c] = W[2 * (c * n3 + s) + 1];
      Dr[c] = W[2 * ((6 + c) * n3 + s)];
      Di[c] = W[2 * ((6 + c) * n3 + s) + 1];
    }
    double e0, e1;
    tt_accumulate(Dr, Di, kh, &e0);
    tt_accumulate(Ur, Ui, kh, &e1);
    double k = qarr[s];
    varr[s] = e0 + k * k * e1;
  }
  free(W);
}

void axo_uij_grav_spec(const axg_params *p, const double *u, const double *udot, double tau,
                       double *wave, double *power, double *numer, double *denom) {
  const int64_t n3 = (int64_t)p->ngrid * p->ngrid * p->ngrid;
  const int nb = p->num_bin_grav;
  double *qa = (double *)malloc(sizeof(double) * n3), *va = (double *)malloc(sizeof(double) * n3);
  uij_numer(p, u, udot, tau, qa, va);
  double dq;
  lin_edges(p->dspa, nb, wave, &dq);
  double fact = gw_fact(p, p->ngrid, p->dspa);
  for (int k = 0; k < nb; ++k) numer[k] = denom[k] = 0.0;
  for (int64_t s = 0; s < n3; ++s) {
    double q = qa[s];
    double iqd = round(q / dq + 0.5);
    if (q > 0.0 && iqd >= 1 && iqd <= nb) {
      denom[(int)iqd - 1] += 1;
      numer[(int)iqd - 1] += va[s];
    }
  }
  for (int k = 0; k < nb; ++k) {
    double q = wave[k];
    power[k] = denom[k] > 0 ? numer[k] / denom[k] * (q * q * q) * fact : 0.0;
  }
  free(qa);
  free(va);
}

void axo_uij_grav_spec_log(const axg_params *p, const double *u, const double *udot, double tau,
                           double *edges, double *power, double *numer, double *denom) {
  const int64_t n3 = (int64_t)p->ngrid * p->ngrid * p->ngrid;
  const int nl = p->gw_log_bins;
  double *qa = (double *)malloc(sizeof(double) * n3), *va = (double *)malloc(sizeof(double) * n3);
  uij_numer(p, u, udot, tau, qa, va);
  log_edges(p->ngrid, p->dspa, nl, edges);
  double fact = gw_fact(p, p->ngrid, p->dspa);
  for (int k = 0; k < nl; ++k) numer[k] = denom[k] = 0.0;
  for (int64_t s = 0; s < n3; ++s) {
    double q = qa[s];
    if (!(q > 0.0)) continue;
    int b = log_bin(q, edges, nl);
    if (b < 0) continue;
    denom[b] += 1;
    numer[b] += va[s];
  }
  for (int k = 0; k < nl; ++k) {
    double q = sqrt(edges[k] * edges[k + 1]);
    power[k] = denom[k] > 0 ? numer[k] / denom[k] * (q * q * q) * fact : 0.0;
  }
  free(qa);
  free(va);
}
