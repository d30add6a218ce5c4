/*
 * axo.h -- CPU restatement of axion_grav's lattice hot path (FP64, OpenMP).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle against which the
 * GB300 kernels of axion_grav_gb300 are checked, and the timed CPU baseline of
 * bench.py.  Nothing in the product links, loads or calls it.
 *
 * Each function restates one routine of the reference Fortran program
 * (toyokazu-sekiguchi/axion_grav) in the same arithmetic order, with the
 * single-rank MPI decomposition collapsed onto periodic index arithmetic; the
 * citation in front of each definition gives the file:line it follows.
 * Parity with the reference binary itself is UNPINNED: the reference needs
 * ifort, Intel MPI, MKL and FFTW3-MPI, none of which exists here, and it ships
 * no tests or golden outputs.  The restatement is pinned instead by
 * known-answer physics tests and an independent numpy restatement
 * (tests/golden/make_golden.py).
 *
 * Layout: complex fields are interleaved (re, im) doubles [N^3][2] with x
 * fastest (Fortran data1(ix, iy, iz) interior planes); u_ij are [6][N^3]
 * reals in component order (1,1),(2,1),(2,2),(3,1),(3,2),(3,3); the Green's
 * function accumulators are four complex arrays [4][N^3][2] in the order
 * (1,1),(2,1),(1,2),(2,2) of arr_grav.
 */
#ifndef AXO_H
#define AXO_H

#include <stdint.h>

#include "axgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* potential.f90 */
double axo_msquared(double thrm);
double axo_maxion2(double thrm, double kappa);
/* evolve.f90:291-305 kick coefficients + dVdphi coefficients:
 * f = (fact1, fact2, fact3, fact_source), pot = (A, B, C, D) with
 * dV/dphi* = (A|phi|^2 + B) phi + C + D conj(phi). */
void axo_kick_coeffs(const axg_params *p, double t, double dt, double f[4], double pot[4]);
/* evolve.f90:10-24 */
void axo_get_dtau(const axg_params *p, double tau1, double tau2, double eps_dtau, double *dtau,
                  int64_t *n);

/* evolve.f90:259-281 (drift of phi) and the same drift of u_ij when u != NULL */
void axo_evolve_phi(const axg_params *p, double *phi, const double *phidot, double *u,
                    const double *udot, double dt);
/* evolve.f90:283-339 (kick of phi) and the u_ij kick when u != NULL */
void axo_evolve_phidot(const axg_params *p, const double *phi, double *phidot, const double *u,
                       double *udot, double t, double dt);
/* evolve.f90:238-257; with gw_mode GREEN also the per-kick accumulation. */
int64_t axo_symplectic_integration(const axg_params *p, double *phi, double *phidot, double *u,
                                   double *udot, double *acc, double t1, double t2,
                                   double eps_dtau);

/* 3-D complex FFT, unnormalised, exp(sign * 2 pi i k.x / N); in place. */
void axo_fft3d(int64_t n, double *data, int sign);
/* 3-D real->half-complex not needed: full complex transforms only. */

/* grav_waves.f90:37-45: the GW grid, ngrid / 2^degrade_spec sites a side of
 * spacing dspa 2^degrade_spec (Green's-function accumulators are [4][ng^3][2]) */
void axo_gw_grid(const axg_params *p, int64_t *ng, double *dspa_g);
/* grav_waves.f90:323-356: dphi[3][N^3][2] */
void axo_data1_to_arr_dphi(const axg_params *p, const double *phi, double *dphi);
/* grav_waves.f90:358-415 (one rank): dphi[3][ng^3][2] */
void axo_data1_to_arr_dphi_degrade(const axg_params *p, const double *phi, double *dphi);
/* grav_waves.f90:157-191 (pol for component (i, j), 1-based) */
void axo_get_comwav_grav(const axg_params *p, const int64_t ixyz[3], double *q, double pol[2],
                         int i, int j);
/* grav_waves.f90:193-255 */
void axo_grav_wave_integration(const axg_params *p, const double *phi, double *acc, double tau,
                               double dtau);
/* grav_waves.f90:257-321 (power and the raw numer/denom; nb = num_bin_grav) */
void axo_grav_spec_estimation(const axg_params *p, const double *acc, double *wave,
                              double *power, double *numer, double *denom);
/* u_ij TT spectrum (GW_UIJ), same bins and normalisation as Green's mode. */
void axo_uij_grav_spec(const axg_params *p, const double *u, const double *udot, double tau,
                       double *wave, double *power, double *numer, double *denom);
/* log-binned variants: edges[nlog+1] */
void axo_grav_spec_log_green(const axg_params *p, const double *acc, double *edges,
                             double *power, double *numer, double *denom);
void axo_uij_grav_spec_log(const axg_params *p, const double *u, const double *udot, double tau,
                           double *edges, double *power, double *numer, double *denom);

/* defects_3d.f90:31-103 + 309-349; phase_mode 0 = project atan2, 1 = libm atan2 */
void axo_classify_cells(const axg_params *p, const double *phi, int which, int phase_mode,
                        int8_t *flags, int64_t counts[3]);
/* plaquette winding counts per orientation */
void axo_string_winding(const axg_params *p, const double *phi, int64_t counts[3]);
/* defects_3d.f90:31-307 incl. fits and sums; strings/walls lists as in
 * axg_download_defect_lists (may be NULL). */
void axo_id_defects(const axg_params *p, const double *phi, const double *phidot, double tau,
                    double sl[3], double wa[3], double svel[3], int64_t counts[3],
                    double *strings, int64_t max_strings, double *walls, int64_t max_walls,
                    int8_t *flags_out);
/* the fits of id_defects for given string / wall cells (rows as axo_id_defects) */
void axo_fit_cells(const axg_params *p, const double *phi, const double *phidot, const int64_t *scells,
                   int64_t ns, double *sres, const int64_t *wcells, int64_t nw, double *wres);
/* the string-fit chi2 (defects_3d.f90:385-433): the float-float form the
 * fits use, and FP64 as its yardstick */
double axo_chi2_string_ff(const double ph[8], const double pr[4]);
double axo_chi2_string_fp64(const double ph[8], const double pr[4]);
/* single-cell pieces for unit tests */
void axo_position_string(const double ph[8], uint64_t seed, uint64_t cell, double pos[3],
                         double dir[3], double *gof, double *sl);
void axo_position_wall(const double ph[8], double pos[3], double dir[3], double *gof,
                       double *wa);
double axo_string_length(const double pos[3], const double dir[3]);

/* spectrum.f90 */
/* init_spectrum tables: mat_spec[num_cov][501], largeq[num_cov][501], dq[num_cov], wav[nb+1] */
void axo_init_spectrum(const axg_params *p, double *mat_spec, double *largeq, double *dq_spec,
                       double *wav);
/* full spectrum_estimation core; flags from axo_classify_cells (mask bit 4) */
void axo_spectrum_estimation(const axg_params *p, const double *phidot, const int8_t *flags,
                             double tau, double *wave, double *power, double *conv,
                             double *count, double *mat_deconv_out);
void axo_compute_crho(const axg_params *p, const double *wav, const double *power, double *rho);
void axo_estimate_covmat(const axg_params *p, const int8_t *flags, const double *power,
                         const double *mat_deconv, int min_mc, int max_mc, double tol, double *cov,
                         int *iterations);
void axo_compute_crho_cov(const axg_params *p, const double *wav, const double *power, const double *cov,
                          double *rho, double *drho);
void axo_epsilon(int nb, const double *wav, const double *p1, const double *p2, const double *c1,
                 const double *c2, double tau1, double tau2, double *eps, double *deps);
/* packed (upper) Cholesky inverse, dpptrf + dpptri; returns info */
int axo_pp_inverse(int n, double *ap);

/* initial conditions */
void axo_ic_gaussian_flat(const axg_params *p, double kcut, uint32_t realisation, double *phi,
                          double *phidot);
void axo_ic_thermal(const axg_params *p, double tau_ini, uint32_t realisation, double *phi,
                    double *phidot);
/* volume averages (<|phi|^2>, <|phi'|^2>, <|grad phi|^2>, <V>) */
void axo_field_moments(const axg_params *p, const double *phi, const double *phidot, double tau,
                       double out[4]);

/* FP64 tangent-linear reference (axo_adjoint.c) */
double axo_gw_band_energy(const axg_params *p, const double *u, const double *w, double tau, double kmin,
                          double kmax);
void axo_tl_run(const axg_params *p, double *phi, double *phid, double *u, double *ud, double *dphi,
                double *dphid, double *du, double *dud, double dlambda, double t1, double dt, int64_t nsteps,
                int first_half, int last_half, double kmin, double kmax, double *J, double *dJ);

/* deterministic math exports for tests */
double axo_det_atan2(double y, double x);
void axo_det_sincos(double x, double *s, double *c);
void axo_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

int axo_num_threads(void);

#ifdef __cplusplus
}
#endif

#endif
