/*
 * axo_defects.c -- oracle restatement of defects_3d.f90 (cell classification,
 * per-cell string / wall fits, string velocity, global sums) plus the
 * plaquette-winding string counter of the extension.
 * TEST INFRASTRUCTURE ONLY (see axo.h).
 *
 * Random starts of the string fit come from Philox (stream 3, counter
 * (cell, j/2)) in place of the reference's MKL VSL MCG59 streams
 * (defects_3d.f90:465); atan2 / sin / cos are the project's deterministic
 * versions (axg_detmath.h) so the GPU kernels reproduce every fit bit for bit.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "axo.h"
#include "axg_detmath.h"
#include "axg_ffchi2.h"

#define REF_PI 3.14159265359
#define REF_TWOPI (2 * REF_PI)
/* defects_3d.f90:6 */
#define STRING_PHDIFF REF_PI
#define REMOVAL_PHDIFF (7 * REF_PI / 4)
/* defects_3d.f90:26-27 */
#define MAX_ITER_STRING_POS 1000
#define NUM_SIMP 4
#define MULT_STRING_POS (NUM_SIMP * (MAX_ITER_STRING_POS + 1))

static inline double phase_of(const double *phi, int64_t s, int mode) {
  return mode ? atan2(phi[2 * s + 1], phi[2 * s]) : axd_atan2(phi[2 * s + 1], phi[2 * s]);
}

/* corners of cell (ix, iy, iz): i = (dz*2+dy)*2+dx (defects_3d.f90:37-40, 411) */
static void corner_sites(int64_t n, int64_t ix, int64_t iy, int64_t iz, int64_t s[8]) {
  const int64_t n2 = n * n;
  for (int c = 0; c < 8; ++c) {
    int dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
    s[c] = ((iz + dz) % n) * n2 + ((iy + dy) % n) * n + (ix + dx) % n;
  }
}

/* defects_3d.f90:309-349 */
static int8_t id_with_phase(const double ph[8], int which, int64_t *ns, int64_t *nw, int64_t *nm) {
  double pht[8];
  memcpy(pht, ph, sizeof(pht));
  for (int i = 7; i >= 1; --i)
    for (int j = 1; j <= i; ++j)
      if (pht[j - 1] > pht[j]) {
        double t = pht[j - 1];
        pht[j - 1] = pht[j];
        pht[j] = t;
      }
  int8_t flag = 0;
  double t = pht[0] - pht[7] + REF_TWOPI;
  double tmax = pht[1] - pht[0];
  for (int k = 1; k < 7; ++k) {
    double g = pht[k + 1] - pht[k];
    if (g > tmax) tmax = g;
  }
  if ((which & AXG_F_ID_WALLS) && tmax > t) {
    flag += 2;
    ++*nw;
  } else {
    tmax = t > tmax ? t : tmax;
  }
  if ((which & AXG_F_ID_STRINGS) && tmax < STRING_PHDIFF) {
    flag += 1;
    ++*ns;
  }
  if ((which & AXG_F_SPEC_EST) && tmax < REMOVAL_PHDIFF) {
    flag += 4;
    ++*nm;
  }
  return flag;
}

void axo_classify_cells(const axg_params *p, const double *phi, int which, int phase_mode,
                        int8_t *flags, int64_t counts[3]) {
  const int64_t n = p->ngrid, n2 = n * n, n3 = n2 * n;
  double *ph = (double *)malloc(sizeof(double) * n3);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < n3; ++s) ph[s] = phase_of(phi, s, phase_mode);
  int64_t ns = 0, nw = 0, nm = 0;
#pragma omp parallel for schedule(static) reduction(+ : ns, nw, nm)
  for (int64_t iz = 0; iz < n; ++iz)
    for (int64_t iy = 0; iy < n; ++iy)
      for (int64_t ix = 0; ix < n; ++ix) {
        int64_t cs[8];
        double cp[8];
        corner_sites(n, ix, iy, iz, cs);
        for (int c = 0; c < 8; ++c) cp[c] = ph[cs[c]];
        flags[iz * n2 + iy * n + ix] = id_with_phase(cp, which, &ns, &nw, &nm);
      }
  counts[0] = ns;
  counts[1] = nw;
  counts[2] = nm;
  free(ph);
}

/* Plaquette winding: sum of the wrapped phase differences around each
 * elementary plaquette is 0 or +-2 pi; a nonzero winding marks a plaquette
 * pierced by a string.  counts = plaquettes with normal x, y, z. */
static inline double wrapd(double d) {
  const double pi = AXD_PI_HI, tp = 2 * AXD_PI_HI;
  if (d > pi) return d - tp;
  if (d <= -pi) return d + tp;
  return d;
}
static inline int pierced(double a, double b, double c, double d) {
  double w = wrapd(b - a);
  w = w + wrapd(c - b);
  w = w + wrapd(d - c);
  w = w + wrapd(a - d);
  return w > AXD_PI_HI || w < -AXD_PI_HI;
}
void axo_string_winding(const axg_params *p, const double *phi, int64_t counts[3]) {
  const int64_t n = p->ngrid, n2 = n * n, n3 = n2 * n;
  double *ph = (double *)malloc(sizeof(double) * n3);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < n3; ++s) ph[s] = axd_atan2(phi[2 * s + 1], phi[2 * s]);
  int64_t cx = 0, cy = 0, cz = 0;
#pragma omp parallel for schedule(static) reduction(+ : cx, cy, cz)
  for (int64_t iz = 0; iz < n; ++iz)
    for (int64_t iy = 0; iy < n; ++iy)
      for (int64_t ix = 0; ix < n; ++ix) {
        int64_t x1 = (ix + 1) % n, y1 = (iy + 1) % n, z1 = (iz + 1) % n;
#define PH(x, y, z) ph[(z) * n2 + (y) * n + (x)]
        cz += pierced(PH(ix, iy, iz), PH(x1, iy, iz), PH(x1, y1, iz), PH(ix, y1, iz));
        cx += pierced(PH(ix, iy, iz), PH(ix, y1, iz), PH(ix, y1, z1), PH(ix, iy, z1));
        cy += pierced(PH(ix, iy, iz), PH(ix, iy, z1), PH(x1, iy, z1), PH(x1, iy, iz));
#undef PH
      }
  counts[0] = cx;
  counts[1] = cy;
  counts[2] = cz;
  free(ph);
}

/* defects_3d.f90:385-433 in FP64, kept as the yardstick of the float-float
 * chi2 the fits use (a CPU test compares the two) */
double axo_chi2_string_fp64(const double ph[8], const double pr[4]) {
  double mu = pr[0], phi = pr[1];
  double s4, c4, sp, cp;
  axd_sincos(pr[3], &s4, &c4);
  double u0 = pr[2] * c4;
  double v0 = pr[2] * s4;
  double cm = mu;
  double sm = sqrt(1.0 - mu * mu);
  axd_sincos(phi, &sp, &cp);
  double a = 0.0, b = 0.0;
  for (int iz = 0; iz <= 1; ++iz) {
    double z = iz - 0.5;
    for (int iy = 0; iy <= 1; ++iy) {
      double y = iy - 0.5;
      for (int ix = 0; ix <= 1; ++ix) {
        double x = ix - 0.5;
        int i = (iz * 2 + iy) * 2 + ix;
        double du = -u0 + cm * (x * cp + y * sp) - z * sm;
        double dv = -v0 - x * sp + y * cp;
        double d = ph[i] - axd_atan2(dv, du);
        if (d >= REF_PI)
          d = d - REF_TWOPI;
        else if (d < -REF_PI)
          d = d + REF_TWOPI;
        a = a + d * d;
        b = b + d;
      }
    }
  }
  a = a / 8;
  b = b / 8;
  return a - b * b;
}

/* defects_3d.f90:385-433 as the fits evaluate it: float-float arithmetic
 * (axg_ffchi2.h), the corner phases split into float-float pairs */
double axo_chi2_string_ff(const double ph[8], const double pr[4]) {
  axd_ff f[8];
  for (int i = 0; i < 8; ++i) f[i] = axd_ff_from(ph[i]);
  return axd_chi2_string_ff(f, pr);
}
#define calc_chi2_string axo_chi2_string_ff

/* defects_3d.f90:1027-1056 */
double axo_string_length(const double pos[3], const double dir[3]) {
  const double atmax = 0.867, atmax0 = 0.86602540378378444;
  double tp = atmax, tn = -atmax;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j <= 1; ++j) {
      double w = j - 0.5;
      w = w - pos[i];
      if (fabs(w) > atmax * fabs(dir[i])) continue;
      double t = w / dir[i];
      if (t > 0) {
        if (t < tp) tp = t;
      } else {
        if (t > tn) tn = t;
      }
    }
  if (tp < atmax0 && tn > -atmax0) return tp - tn;
  return 0.0;
}

static int out_of_box(const double t[4]) {
  const double mx[4] = {1.0, REF_PI, sqrt(3.0) / 2, REF_PI};
  const double mn[4] = {-1.0, -REF_PI, 0.0, -REF_PI};
  for (int k = 0; k < 4; ++k)
    if (t[k] > mx[k] || t[k] < mn[k]) return 1;
  return 0;
}

/* defects_3d.f90:435-603 */
void axo_position_string(const double ph[8], uint64_t seed, uint64_t cell, double pos[3],
                         double dir[3], double *gof, double *sl) {
  const double chi2max = 8 * REF_PI * REF_PI, tol = 0.05;
  const double max_s[4] = {1.0, REF_PI, sqrt(3.0) / 2, REF_PI};
  const double min_s[4] = {-1.0, -REF_PI, 0.0, -REF_PI};
  double p_s[5][4], chi2_s[5], c_s[4], t_s[4], s_s[4], chi2, chi2s;
  memset(p_s, 0, sizeof(p_s));
  memset(chi2_s, 0, sizeof(chi2_s));
  int n0 = -1;
  for (int i = 0; i <= MAX_ITER_STRING_POS; ++i) {
    double x[4];
    for (int k = 0; k < 4; ++k) {
      int j = i * 4 + k;
      axd_u32x4 r = axd_draw(seed, 3u, (uint32_t)(j >> 1), cell);
      x[k] = (j & 1) ? axd_u01(r.v[2], r.v[3]) : axd_u01(r.v[0], r.v[1]);
    }
    for (int k = 0; k < 4; ++k) t_s[k] = max_s[k] * x[k] + min_s[k] * (1 - x[k]);
    chi2 = calc_chi2_string(ph, t_s);
    if (n0 <= 0) {
      n0 = n0 + 1;
      chi2_s[n0] = chi2;
      memcpy(p_s[n0], t_s, sizeof(t_s));
      continue;
    }
    if (n0 < NUM_SIMP || chi2 <= chi2_s[n0]) {
      n0 = n0 + 1 < NUM_SIMP ? n0 + 1 : NUM_SIMP;
      int i0 = n0;
      while (chi2 <= chi2_s[i0 - 1]) {
        if (i0 <= NUM_SIMP) {
          chi2_s[i0] = chi2_s[i0 - 1];
          memcpy(p_s[i0], p_s[i0 - 1], sizeof(t_s));
        }
        i0 = i0 - 1;
        if (i0 == 0) break;
      }
      chi2_s[i0] = chi2;
      memcpy(p_s[i0], t_s, sizeof(t_s));
    }
  }
  int it = 0;
  while (chi2_s[0] > tol && it < MAX_ITER_STRING_POS) {
    it = it + 1;
    for (int k = 0; k < 4; ++k) c_s[k] = 0.0;
    for (int i0 = 0; i0 < NUM_SIMP; ++i0)
      for (int k = 0; k < 4; ++k) c_s[k] = c_s[k] + p_s[i0][k];
    for (int k = 0; k < 4; ++k) c_s[k] = c_s[k] / NUM_SIMP;
    /* reflection */
    for (int k = 0; k < 4; ++k) t_s[k] = 2 * c_s[k] - p_s[NUM_SIMP][k];
    chi2 = out_of_box(t_s) ? chi2max : calc_chi2_string(ph, t_s);
    if (chi2 < chi2_s[NUM_SIMP]) {
      /* expansion (defects_3d.f90:525) */
      for (int k = 0; k < 4; ++k) s_s[k] = 3 * c_s[k] - 4 * p_s[NUM_SIMP][k];
      chi2s = out_of_box(s_s) ? chi2max : calc_chi2_string(ph, s_s);
      if (chi2 <= chi2s) {
        chi2_s[NUM_SIMP] = chi2;
        memcpy(p_s[NUM_SIMP], t_s, sizeof(t_s));
      } else {
        chi2_s[NUM_SIMP] = chi2s;
        memcpy(p_s[NUM_SIMP], s_s, sizeof(s_s));
      }
    } else {
      for (int k = 0; k < 4; ++k) s_s[k] = 1.5 * c_s[k] - 0.5 * p_s[NUM_SIMP][k];
      chi2s = out_of_box(s_s) ? chi2max : calc_chi2_string(ph, s_s);
      if (chi2s <= chi2_s[NUM_SIMP]) {
        chi2_s[NUM_SIMP] = chi2s;
        memcpy(p_s[NUM_SIMP], s_s, sizeof(s_s));
      } else {
        for (int i0 = 1; i0 <= NUM_SIMP; ++i0) {
          for (int k = 0; k < 4; ++k) p_s[i0][k] = 0.5 * (p_s[i0][k] + p_s[0][k]);
          chi2_s[i0] = calc_chi2_string(ph, p_s[i0]);
        }
      }
    }
    for (int i0 = NUM_SIMP - 1; i0 >= 0; --i0)
      for (int m = 0; m <= i0; ++m)
        if (chi2_s[m] > chi2_s[m + 1]) {
          double tt[4];
          memcpy(tt, p_s[m], sizeof(tt));
          memcpy(p_s[m], p_s[m + 1], sizeof(tt));
          memcpy(p_s[m + 1], tt, sizeof(tt));
          double c = chi2_s[m];
          chi2_s[m] = chi2_s[m + 1];
          chi2_s[m + 1] = c;
        }
  }
  double mu = p_s[0][0], phi = p_s[0][1];
  double s4, c4, sp, cp;
  axd_sincos(p_s[0][3], &s4, &c4);
  double u0 = p_s[0][2] * c4, v0 = p_s[0][2] * s4;
  chi2 = chi2_s[0];
  axd_sincos(phi, &sp, &cp);
  double sq = sqrt(1.0 - mu * mu);
  dir[0] = sq * cp;
  dir[1] = sq * sp;
  dir[2] = mu;
  pos[0] = u0 * mu * cp - v0 * sp;
  pos[1] = u0 * mu * sp + v0 * cp;
  pos[2] = -(u0 * sqrt(1 - mu * mu));
  *gof = exp(-chi2 / 2);
  *sl = axo_string_length(pos, dir);
}

/* reference BLAS dspr ('U'): ap += alpha x x^T, upper packed */
static void dspr_u(int n, double alpha, const double *x, double *ap) {
  int kk = 0;
  for (int j = 0; j < n; ++j) {
    if (x[j] != 0.0) {
      double temp = alpha * x[j];
      int k = kk;
      for (int i = 0; i <= j; ++i) {
        ap[k] = ap[k] + x[i] * temp;
        ++k;
      }
    }
    kk += j + 1;
  }
}

/* reference LAPACK dpptrf ('U') + dpptri ('U') (with dtpsv, dtptri, dtpmv,
 * dspr, dscal of reference BLAS); returns info */
int axo_pp_inverse(int n, double *ap) {
  /* dpptrf */
  int jj = 0;
  for (int j = 1; j <= n; ++j) {
    int jc = jj + 1;
    jj = jj + j;
    if (j > 1) {
      /* dtpsv('U','T','N', j-1, ap, ap(jc)) */
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
    ap[jj - 1] = sqrt(ajj);
  }
  /* dtptri('U','N') */
  int jc = 1;
  for (int j = 1; j <= n; ++j) {
    ap[jc + j - 2] = 1.0 / ap[jc + j - 2];
    double ajj = -ap[jc + j - 2];
    /* dtpmv('U','N','N', j-1, ap, ap(jc)) */
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
  /* inv(U) * inv(U)^T */
  jj = 0;
  for (int j = 1; j <= n; ++j) {
    jc = jj + 1;
    jj = jj + j;
    if (j > 1) dspr_u(j - 1, 1.0, ap + (jc - 1), ap);
    double ajj = ap[jj - 1];
    for (int i = 0; i < j; ++i) ap[jc - 1 + i] = ajj * ap[jc - 1 + i];
  }
  return 0;
}

/* defects_3d.f90:605-692 (VEL=0) */
static void velocity_string(const axg_params *p, const double *phi, const double *phid,
                            int64_t ix, int64_t iy, int64_t iz, const double pos[3],
                            double vel[3]) {
  const int64_t n = p->ngrid, n2 = n * n;
  double wr[4] = {0}, wi[4] = {0}, dr[4] = {0}, di[4] = {0}, mat[10] = {0}, mat0[10];
  double d[4];
  d[0] = 1.0;
  for (int k = 0; k <= 1; ++k) {
    int64_t zz = (iz + k) % n;
    d[3] = k - pos[2] - 0.5;
    for (int j = 0; j <= 1; ++j) {
      int64_t yy = (iy + j) % n;
      d[2] = j - pos[1] - 0.5;
      for (int i = 0; i <= 1; ++i) {
        int64_t xx = (ix + i) % n;
        d[1] = i - pos[0] - 0.5;
        int64_t s = zz * n2 + yy * n + xx;
        for (int l = 0; l < 4; ++l) {
          wr[l] = wr[l] + d[l] * phi[2 * s];
          wi[l] = wi[l] + d[l] * phi[2 * s + 1];
          dr[l] = dr[l] + d[l] * phid[2 * s];
          di[l] = di[l] + d[l] * phid[2 * s + 1];
        }
        dspr_u(4, 1.0, d, mat);
      }
    }
  }
  for (int l = 0; l < 4; ++l) {
    wr[l] /= 8;
    wi[l] /= 8;
    dr[l] /= 8;
    di[l] /= 8;
  }
  for (int l = 0; l < 10; ++l) mat[l] /= 8;
  memcpy(mat0, mat, sizeof(mat));
  axo_pp_inverse(4, mat0);
  double w0r[4] = {0}, w0i[4] = {0}, d0r[4] = {0}, d0i[4] = {0};
  for (int ii = 1; ii <= 4; ++ii)
    for (int jj = 1; jj <= 4; ++jj) {
      int kk = ii > jj ? ii : jj;
      kk = kk * (kk - 1) / 2 + (ii < jj ? ii : jj);
      double m = mat0[kk - 1];
      w0r[ii - 1] = w0r[ii - 1] + m * wr[jj - 1];
      w0i[ii - 1] = w0i[ii - 1] + m * wi[jj - 1];
      d0r[ii - 1] = d0r[ii - 1] + m * dr[jj - 1];
      d0i[ii - 1] = d0i[ii - 1] + m * di[jj - 1];
    }
  double x = d0r[0], y = d0i[0];
  double a = 0, b = 0, c = 0;
  for (int l = 1; l < 4; ++l) {
    a = a + w0r[l] * w0r[l];
    b = b + w0r[l] * w0i[l];
    c = c + w0i[l] * w0i[l];
  }
  double det = a * c - b * b;
  for (int l = 1; l < 4; ++l) {
    double v = (x * c - y * b) * w0r[l] + (-(x * b) + y * a) * w0i[l];
    vel[l - 1] = -v / det * p->dspa;
  }
}

/* defects_3d.f90:1058-1233; returns the number of edge crossings m */
static int position_wall_m(const double ph[8], double pos[3], double dir[3], double *gof,
                           double *wa) {
  double pp[12][3], th[12], uv[12][2], sn[8], cs[8];
  for (int i = 0; i < 8; ++i) axd_sincos(ph[i], &sn[i], &cs[i]);
  int m = 0;
  for (int iz = 0; iz <= 1; ++iz)
    for (int iy = 0; iy <= 1; ++iy) {
      double u = sn[(iz * 2 + iy) * 2 + 0], v = sn[(iz * 2 + iy) * 2 + 1];
      if (u * v < 0.0) {
        pp[m][0] = (u + v) / (u - v) / 2;
        pp[m][1] = iy - 0.5;
        pp[m][2] = iz - 0.5;
        ++m;
      }
    }
  for (int iy = 0; iy <= 1; ++iy)
    for (int ix = 0; ix <= 1; ++ix) {
      double u = sn[(0 * 2 + iy) * 2 + ix], v = sn[(1 * 2 + iy) * 2 + ix];
      if (u * v < 0.0) {
        pp[m][0] = ix - 0.5;
        pp[m][1] = iy - 0.5;
        pp[m][2] = (u + v) / (u - v) / 2;
        ++m;
      }
    }
  for (int iz = 0; iz <= 1; ++iz)
    for (int ix = 0; ix <= 1; ++ix) {
      double u = sn[(iz * 2 + 0) * 2 + ix], v = sn[(iz * 2 + 1) * 2 + ix];
      if (u * v < 0.0) {
        pp[m][0] = ix - 0.5;
        pp[m][1] = (u + v) / (u - v) / 2;
        pp[m][2] = iz - 0.5;
        ++m;
      }
    }
  if (m < 3) {
    /* the reference aborts here (defects_3d.f90:1121-1132); record an empty wall */
    pos[0] = pos[1] = pos[2] = 0.0;
    dir[0] = dir[1] = dir[2] = 0.0;
    *gof = 0.0;
    *wa = 0.0;
    return m;
  }
  double chi2min = 6.0, mut = 0.0, phit = 0.0, wt = 0.0;
  for (int imu = 1; imu <= 20; ++imu) {
    double mu = ((double)(-20 + 2 * imu) - 1.0) / 20;
    for (int iphi = 1; iphi <= 20; ++iphi) {
      double phi = REF_PI * ((2 * iphi - 1.0) - 20) / 20;
      double sp, cp;
      axd_sincos(phi, &sp, &cp);
      double sq = sqrt(1 - mu * mu);
      double d0[3] = {sq * cp, sq * sp, mu};
      double w = 0.0, chi2 = 0.0;
      for (int i = 0; i < m; ++i) {
        double d = pp[i][0] * d0[0] + pp[i][1] * d0[1];
        d = d + pp[i][2] * d0[2];
        w = w + d;
        chi2 = chi2 + d * d;
      }
      if (w < 0.0)
        w = 0.0;
      else
        w = w / m;
      chi2 = chi2 - m * w * w;
      if (chi2 < chi2min) {
        chi2min = chi2;
        mut = mu;
        phit = phi;
        wt = w;
      }
    }
  }
  double spt, cpt;
  axd_sincos(phit, &spt, &cpt);
  double sqt = sqrt(1 - mut * mut);
  double d0[3] = {sqt * cpt, sqt * spt, mut};
  int num = 0;
  for (int iz = 0; iz <= 1; ++iz)
    for (int iy = 0; iy <= 1; ++iy)
      for (int ix = 0; ix <= 1; ++ix) {
        double disp[3] = {ix - 0.5, iy - 0.5, iz - 0.5};
        double d = disp[0] * d0[0] + disp[1] * d0[1];
        d = d + disp[2] * d0[2];
        d = d - wt;
        if (d * cs[(iz * 2 + iy) * 2 + ix] > 0.0) ++num;
      }
  if (num <= 4) {
    for (int k = 0; k < 3; ++k) d0[k] = -d0[k];
    wt = -wt;
  }
  for (int k = 0; k < 3; ++k) {
    dir[k] = d0[k];
    pos[k] = wt * d0[k];
  }
  *gof = exp(-chi2min / 2);
  double dir1[3] = {mut * cpt, mut * spt, -sqrt(1 - mut * mut)};
  double dir2[3] = {-spt, cpt, 0.0};
  for (int i = 0; i < m; ++i) {
    for (int k = 0; k < 3; ++k) pp[i][k] = pp[i][k] - pos[k];
    double u = dir1[0] * pp[i][0] + dir1[1] * pp[i][1];
    u = u + dir1[2] * pp[i][2];
    double v = dir2[0] * pp[i][0] + dir2[1] * pp[i][1];
    v = v + dir2[2] * pp[i][2];
    th[i] = axd_atan2(v, u);
    uv[i][0] = u;
    uv[i][1] = v;
  }
  for (int i = m - 1; i >= 1; --i)
    for (int j = 1; j <= i; ++j)
      if (th[j - 1] > th[j]) {
        double w = th[j - 1];
        th[j - 1] = th[j];
        th[j] = w;
        double a = uv[j - 1][0], b = uv[j - 1][1];
        uv[j - 1][0] = uv[j][0];
        uv[j - 1][1] = uv[j][1];
        uv[j][0] = a;
        uv[j][1] = b;
      }
  double area = 0.0;
  double w = th[m - 1] - REF_TWOPI;
  double u = sqrt(uv[m - 1][0] * uv[m - 1][0] + uv[m - 1][1] * uv[m - 1][1]);
  for (int i = 0; i < m; ++i) {
    double v = sqrt(uv[i][0] * uv[i][0] + uv[i][1] * uv[i][1]);
    w = th[i] - w;
    area = area + 0.5 * u * v * axd_sin(w);
    u = v;
    w = th[i];
  }
  *wa = area;
  return m;
}

void axo_position_wall(const double ph[8], double pos[3], double dir[3], double *gof,
                       double *wa) {
  position_wall_m(ph, pos, dir, gof, wa);
}

/* grouping_strings / grouping_walls (defects_3d.f90:1235-1260, 1735-1760):
 * threshold = max(2, (width^2 hor)^(1/3)) in lattice units */
static double group_threshold(double wid, double hor) {
  double th = pow(wid * wid * hor, 1.0 / 3.0);
  return th > 2.0 ? th : 2.0;
}

/* lat_dist_periodic (defects_3d.f90:1645-1652) */
static double lat_dist_periodic(int64_t n, const double *a, const double *b) {
  double s = 0.0;
  for (int k = 0; k < 3; ++k) {
    double dp = fabs(a[k] - b[k]);
    double e = (double)n - dp;
    double m = dp < e ? dp : e;
    s = s + m * m;
  }
  return sqrt(s);
}

static int64_t uf_find(int64_t *par, int64_t x) {
  while (par[x] != x) x = par[x];
  return x;
}

/* Connected components of the points (rows of `rows` with positions in
 * columns 0..2) under dist <= th: the partition the reference's grouping
 * produces on one rank and one thread.  The group id written into column
 * `gcol` is the smallest row index of the component. */
static void group_points(int64_t n, double *rows, int width, int64_t np, double th, int gcol) {
  int64_t *par = (int64_t *)malloc(sizeof(int64_t) * np);
  for (int64_t i = 0; i < np; ++i) par[i] = i;
  for (int64_t i = 0; i < np; ++i)
    for (int64_t j = i + 1; j < np; ++j) {
      if (lat_dist_periodic(n, rows + width * i, rows + width * j) <= th) {
        int64_t a = uf_find(par, i), b = uf_find(par, j);
        if (a != b) {
          if (a < b) par[b] = a;
          else par[a] = b;
        }
      }
    }
  for (int64_t i = 0; i < np; ++i) rows[width * i + gcol] = (double)uf_find(par, i);
  free(par);
}

/* per-group totals of column vcol; out = (all, groups above t2, groups above t3) */
static void group_sums(const double *rows, int width, int vcol, int gcol, int64_t np, double t2, double t3,
                       double out[3]) {
  double *tot = (double *)calloc(np, sizeof(double));
  for (int64_t i = 0; i < np; ++i) {
    int64_t g = (int64_t)rows[width * i + gcol];
    tot[g] = tot[g] + rows[width * i + vcol];
  }
  out[0] = out[1] = out[2] = 0.0;
  for (int64_t g = 0; g < np; ++g) {
    if ((int64_t)rows[width * g + gcol] != g) continue; /* not a root */
    out[0] = out[0] + tot[g];
    if (tot[g] > t2) out[1] = out[1] + tot[g];
    if (tot[g] > t3) out[2] = out[2] + tot[g];
  }
  free(tot);
}

/* The second pass of id_defects (defects_3d.f90:152-219) for one string
 * cell s: position_string (435-603) on the 8 corner phases, velocity_string
 * (605-692), the row pos(3) dir(3) vel(3) gof sl cell group. */
static void fit_string_cell(const axg_params *p, const double *phi, const double *phidot, int64_t s,
                            double *r) {
  const int64_t n = p->ngrid, n2 = n * n, ix = s % n, iy = (s / n) % n, iz = s / n2;
  int64_t cs[8];
  double ph[8];
  corner_sites(n, ix, iy, iz, cs);
  for (int c = 0; c < 8; ++c) ph[c] = axd_atan2(phi[2 * cs[c] + 1], phi[2 * cs[c]]);
  double pos[3], dir[3], vel[3], gof, l;
  axo_position_string(ph, p->seed, (uint64_t)s, pos, dir, &gof, &l);
  velocity_string(p, phi, phidot, ix, iy, iz, pos, vel);
  r[0] = pos[0] + ix + 0.5;
  r[1] = pos[1] + iy + 0.5;
  r[2] = pos[2] + iz + 0.5;
  r[3] = dir[0]; r[4] = dir[1]; r[5] = dir[2];
  r[6] = vel[0]; r[7] = vel[1]; r[8] = vel[2];
  r[9] = gof;
  r[10] = l;
  r[11] = (double)s;
  r[12] = -1.0;
}

/* The same for one wall cell: position_wall (1058-1233), the row pos(3)
 * dir(3) gof wa cell group. */
static void fit_wall_cell(const axg_params *p, const double *phi, int64_t s, double *r) {
  const int64_t n = p->ngrid, n2 = n * n, ix = s % n, iy = (s / n) % n, iz = s / n2;
  int64_t cs[8];
  double ph[8];
  corner_sites(n, ix, iy, iz, cs);
  for (int c = 0; c < 8; ++c) ph[c] = axd_atan2(phi[2 * cs[c] + 1], phi[2 * cs[c]]);
  double pos[3], dir[3], gof, a;
  position_wall_m(ph, pos, dir, &gof, &a);
  r[0] = pos[0] + ix + 0.5;
  r[1] = pos[1] + iy + 0.5;
  r[2] = pos[2] + iz + 0.5;
  r[3] = dir[0]; r[4] = dir[1]; r[5] = dir[2];
  r[6] = gof;
  r[7] = a;
  r[8] = (double)s;
  r[9] = -1.0;
}

/* The per-cell fits of id_defects for given cells only (a sample of a large
 * lattice's flagged cells): rows as axo_id_defects writes them. */
void axo_fit_cells(const axg_params *p, const double *phi, const double *phidot, const int64_t *scells,
                   int64_t ns, double *sres, const int64_t *wcells, int64_t nw, double *wres) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < ns; ++k) fit_string_cell(p, phi, phidot, scells[k], sres + 13 * k);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < nw; ++k) fit_wall_cell(p, phi, wcells[k], wres + 10 * k);
}

/* defects_3d.f90:31-307 without grouping (group_strings = group_walls = .false.)
 * and the sums of add_string_length (1654-1733) / add_wall_area (2145-2204). */
void axo_id_defects(const axg_params *p, const double *phi, const double *phidot, double tau,
                    double sl[3], double wa[3], double svel[3], int64_t counts[3],
                    double *strings, int64_t max_strings, double *walls, int64_t max_walls,
                    int8_t *flags_out) {
  const int64_t n = p->ngrid, n2 = n * n, n3 = n2 * n;
  const int which = p->flags & (AXG_F_ID_STRINGS | AXG_F_ID_WALLS | AXG_F_SPEC_EST);
  int8_t *flags = flags_out ? flags_out : (int8_t *)malloc(n3);
  axo_classify_cells(p, phi, which, 0, flags, counts);
  /* cell lists in cell order */
  int64_t *scell = (int64_t *)malloc(sizeof(int64_t) * (counts[0] + 1));
  int64_t *wcell = (int64_t *)malloc(sizeof(int64_t) * (counts[1] + 1));
  int64_t ns = 0, nw = 0;
  for (int64_t s = 0; s < n3; ++s) {
    if (flags[s] & 1) scell[ns++] = s;
    if (flags[s] & 2) wcell[nw++] = s;
  }
  double *sres = (double *)calloc((size_t)(ns + 1) * 13, sizeof(double));
  double *wres = (double *)calloc((size_t)(nw + 1) * 10, sizeof(double));
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t k = 0; k < ns; ++k) fit_string_cell(p, phi, phidot, scell[k], sres + 13 * k);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t k = 0; k < nw; ++k) fit_wall_cell(p, phi, wcell[k], wres + 10 * k);
  const double hor = tau / p->dspa;
  /* add_string_length (defects_3d.f90:1654-1733) */
  if ((p->flags & AXG_F_GROUP_STRINGS) && ns > 0) {
    const double wid = p->width_cr / p->dspa / tau;
    const double th = group_threshold(wid, hor);
    group_points(p->ngrid, sres, 13, ns, th, 12);
    group_sums(sres, 13, 10, 12, ns, 2 * hor, REF_TWOPI * hor, sl);
  } else {
    double s1 = 0.0;
    for (int64_t k = 0; k < ns; ++k) s1 = s1 + sres[13 * k + 10];
    sl[0] = sl[1] = sl[2] = s1;
  }
  int64_t nn = 0;
  double v1 = 0, v2s = 0, v3 = 0;
  for (int64_t k = 0; k < ns; ++k) {
    const double *v = sres + 13 * k + 6;
    double v2 = v[0] * v[0] + v[1] * v[1];
    v2 = v2 + v[2] * v[2];
    if (v2 >= 1.0) continue;
    ++nn;
    v1 = v1 + sqrt(v2);
    v2s = v2s + v2;
    v3 = v3 + 1 / sqrt(1 - v2);
  }
  if (nn == 0) {
    svel[0] = svel[1] = svel[2] = 0.0;
  } else {
    svel[0] = v1 / nn;
    svel[1] = v2s / nn;
    svel[2] = v3 / nn;
  }
  /* add_wall_area (defects_3d.f90:2145-2204) */
  if ((p->flags & AXG_F_GROUP_WALLS) && nw > 0) {
    const double wid = p->thickness_cr / p->dspa / tau;
    const double th = group_threshold(wid, hor);
    group_points(p->ngrid, wres, 10, nw, th, 9);
    group_sums(wres, 10, 7, 9, nw, REF_PI * hor * hor, 4 * REF_PI * hor * hor, wa);
  } else {
    double a1 = 0.0;
    for (int64_t k = 0; k < nw; ++k) a1 = a1 + wres[10 * k + 7];
    wa[0] = wa[1] = wa[2] = a1;
  }
  if (strings)
    memcpy(strings, sres, sizeof(double) * 13 * (size_t)(ns < max_strings ? ns : max_strings));
  if (walls)
    memcpy(walls, wres, sizeof(double) * 10 * (size_t)(nw < max_walls ? nw : max_walls));
  free(scell);
  free(wcell);
  free(sres);
  free(wres);
  if (!flags_out) free(flags);
}
