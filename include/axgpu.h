/*
 * axgpu.h -- C-ABI of the GB300 lattice hot path of axion_grav.
 *
 * The reference program (Fortran 90 + MPI + FFTW) keeps its host side
 * (main.f90, settings.f90, inifile.f90) and replaces the bodies of its module
 * routines with calls into this library through iso_c_binding.  Every entry
 * point names the reference routine it replaces (file:line in the reference
 * project).  All scalars are passed by value, all arrays by pointer; complex
 * arrays are interleaved (re, im) complex128, x fastest, i.e. Fortran
 * complex(C_DOUBLE_COMPLEX) data1(ngrid, ngrid, ...).
 *
 * Ownership: the caller owns every host array; the library owns all device
 * memory and copies only inside axg_upload* / axg_download* and the explicit
 * I/O calls.  One host thread per context; all work of a context is ordered
 * on one CUDA stream.  Every function returns AXG_OK (0) or a negative status;
 * axg_last_error() gives the message.  The library never calls exit().
 */
#ifndef AXGPU_H
#define AXGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the Fortran wrapper maps any nonzero status onto
 *      MpiStop(msg), utils.f90:44-73) ---- */
#define AXG_OK 0
#define AXG_ERR_ARG (-1)
#define AXG_ERR_CUDA (-2)
#define AXG_ERR_NOMEM (-3)
#define AXG_ERR_STATE (-4)
#define AXG_ERR_IO (-5)
#define AXG_ERR_TIMEOUT (-6)
#define AXG_ERR_UNSUPPORTED (-7)
#define AXG_ERR_NUMERIC (-8)

/* ---- field storage / arithmetic of the evolution ---- */
#define AXG_PREC_FP64_PLAIN 0 /* reference-structured: separate drift and kick passes, FP64 */
#define AXG_PREC_FP64_FUSED 1 /* one kick+drift pass per step, FP64 */
#define AXG_PREC_FP32_MIXED 2 /* one pass, FP32 fields, Kahan-compensated drifts */

/* ---- gravitational-wave method ---- */
#define AXG_GW_NONE 0
#define AXG_GW_GREEN 1 /* grav_waves.f90:193-255 Green's-function accumulation */
#define AXG_GW_UIJ 2   /* real-space leapfrog of six u_ij, TT projection at output */

/* ---- settings.f90 logical switches ---- */
#define AXG_F_ID_STRINGS 1
#define AXG_F_ID_WALLS 2
#define AXG_F_SPEC_EST 4
#define AXG_F_GRAV_SPEC 8
#define AXG_F_INITIAL_LOOP 16
#define AXG_F_GROUP_STRINGS 32 /* group_strings: connected string groups (defects_3d.f90:1235) */
#define AXG_F_GROUP_WALLS 64   /* group_walls (defects_3d.f90:1735) */

/* ---- potential model ---- */
#define AXG_POT_REFERENCE 0 /* potential.f90:34-79 thermal mass + IILM tilt */
#define AXG_POT_QUARTIC 1   /* lambda/4 (|phi|^2 - v^2)^2 + m_a^2 v^2 (1 - cos N_DW theta)/N_DW^2 */

/* ---- literal reproduction of reference quirks ---- */
#define AXG_COMPAT_INTENDED 0
#define AXG_COMPAT_REF 1 /* grav_waves.f90:240-241 cross-wired accumulators */

typedef struct axg_params {
  int32_t ngrid;        /* N (even); lattice N^3, periodic (settings.f90:148) */
  int32_t precision;    /* AXG_PREC_* */
  int32_t gw_mode;      /* AXG_GW_* */
  int32_t num_bin;      /* field-spectrum bins (settings.f90:158, default 50) */
  int32_t degrade_spec; /* spectra coarse-grained by 2^degrade_spec (settings.f90:202) */
  int32_t flags;        /* AXG_F_* */
  int32_t compat;       /* AXG_COMPAT_* */
  int32_t potential;    /* AXG_POT_* */
  int32_t n_dw;         /* domain-wall number of the quartic model's axion term (1 or 2) */
  int32_t num_bin_grav; /* GW bins (grav_waves.f90:6, 25) */
  int32_t gw_log_bins;  /* >0: additionally bin the GW spectrum in this many log bins */
  int32_t device;       /* CUDA device ordinal of the context */
  double dspa;          /* lattice spacing dx in tau_cr (settings.f90:294) */
  double sigma_cr;      /* sigma * tau_cr (settings.f90:276) */
  double kappa;         /* axion-mass scale (potential.f90:25) */
  double tau_cr;        /* tau_cr in reduced-Planck units (settings.f90:275) */
  double a_now;         /* present scale factor (settings.f90:274) */
  double width_cr;      /* string width (settings.f90:279) */
  double thickness_cr;  /* wall thickness (settings.f90:280) */
  double lambda;        /* quartic model coupling */
  double vev;           /* quartic model v */
  double ma2_0;         /* quartic model: m_a^2 at tau_axion_on */
  double tau_axion_on;  /* quartic model: axion term switched on at this tau */
  double ma2_power;     /* quartic model: m_a^2 ~ (tau/tau_on)^ma2_power */
  uint64_t seed;        /* Philox key of every random draw (IC, fit starts) */
  uint64_t reserved1;
} axg_params;

typedef struct axg_ctx axg_ctx;

/* ------------------------------------------------------------------ */
/* library / context                                                    */
/* ------------------------------------------------------------------ */
int axg_version(void);
/* Fill *p with the defaults of settings.f90 (num_bin 50, 25 GW bins ...). */
int axg_params_default(axg_params *p);
/* init_grav (grav_waves.f90:27-82) + init_spectrum (spectrum.f90:23-103) +
 * allocate_data (initial.f90:240-285): allocates all device state. */
int axg_create(const axg_params *p, axg_ctx **out);
/* fin_grav (grav_waves.f90:84-90) + fin_spectrum + deallocate_data. */
int axg_destroy(axg_ctx *ctx);
/* Message of the last failing call on ctx (NULL ctx: last axg_create error). */
const char *axg_last_error(const axg_ctx *ctx);
/* Device bytes held by the context (memory_check_mkl, settings.f90:392-422). */
int axg_memory_bytes(const axg_ctx *ctx, int64_t *bytes);

/* ------------------------------------------------------------------ */
/* state transfer                                                       */
/* ------------------------------------------------------------------ */
/* Copy the interior N^3 sites of data1 (phi) and data2 (phidot) in.
 * plane_stride = elements between z-planes of the host array (N*N for a dense
 * array); first_plane = index of the first interior plane (1 for the
 * reference's [N,N,local_0+2] arrays with one halo plane, 0 for dense).
 * Either pointer may be NULL to skip that field. */
int axg_upload(axg_ctx *ctx, const double *phi, const double *phidot, int64_t plane_stride,
               int64_t first_plane);
int axg_download(axg_ctx *ctx, double *phi, double *phidot, int64_t plane_stride,
                 int64_t first_plane);
/* Six u_ij and u_ij' as real FP64 [6][N^3], component order
 * (1,1),(2,1),(2,2),(3,1),(3,2),(3,3) (grav_waves.f90:210-211 loop order). */
int axg_upload_uij(axg_ctx *ctx, const double *u, const double *udot);
int axg_download_uij(axg_ctx *ctx, double *u, double *udot);
/* Four Green's-function accumulators arr_grav(2,2,M^3) as complex128
 * [4][M^3] in the order (1,1),(2,1),(1,2),(2,2) (grav_waves.f90:74), on the
 * GW grid of init_grav: M = ngrid / 2^degrade_spec (grav_waves.f90:37-45). */
int axg_upload_gw_green(axg_ctx *ctx, const double *acc);
int axg_download_gw_green(axg_ctx *ctx, double *acc);

/* ------------------------------------------------------------------ */
/* evolution (evolve.f90)                                              */
/* ------------------------------------------------------------------ */
/* get_dtau (evolve.f90:10-24). */
int axg_get_dtau(const axg_params *p, double tau1, double tau2, double eps_dtau, double *dtau,
                 int64_t *nsteps);
/* evolve_phi (evolve.f90:259-281): phi += dt phidot (and u_ij += dt u_ij').
 * *t is advanced by dt like the reference's intent(inout) t. */
int axg_evolve_phi(axg_ctx *ctx, double *t, double dt);
/* evolve_phidot (evolve.f90:283-339): one kick at conformal time t; with
 * AXG_GW_GREEN also grav_wave_integration(t, dt) (grav_waves.f90:193-255);
 * with AXG_GW_UIJ the u_ij kick with the d_i phi d_j phi* source. */
int axg_evolve_phidot(axg_ctx *ctx, double t, double dt);
/* symplectic_integration (evolve.f90:238-257): drift-kick-drift from t1 to t2
 * with dt from get_dtau.  *nsteps_out receives nt (may be NULL). */
int axg_symplectic_integration(axg_ctx *ctx, double t1, double t2, double eps_dtau,
                               int64_t *nsteps_out);
/* nsteps kick+drift steps of size dt starting at kick time t (fused paths:
 * one pass per step); first_half / last_half apply the half drifts of the DKD
 * scheme before the first / instead of the last full drift.  dt < 0 runs the
 * same scheme backwards in time (t1 is then the later time; every time of
 * the run must stay positive): the damped leapfrog is time-reversible, so
 * leapfrog(t1 + n dt, -dt, n) undoes leapfrog(t1, dt, n) up to rounding. */
int axg_leapfrog(axg_ctx *ctx, double t1, double dt, int64_t nsteps, int first_half,
                 int last_half);

/* Tile shapes of the fused kick+drift kernel: a CTA owns a tx x ty column of
 * the lattice and marches through zc z-planes.  The autotuner times every
 * shape the lattice supports for `steps` steps on a snapshot of the state
 * (restored afterwards) and keeps the fastest.  *pointwise_tma (may be NULL)
 * is 1 for shapes that also stage the pointwise fields (phi', u' and the
 * compensations) by TMA, one plane ahead. */
int axg_tile_count(void);
int axg_tile_info(int i, int32_t *tx, int32_t *ty, int32_t *zc, int32_t *pointwise_tma);
int axg_set_tile(axg_ctx *ctx, int cfg);
int axg_autotune(axg_ctx *ctx, int steps, int *best_cfg, double *best_ms_per_step);

/* ------------------------------------------------------------------ */
/* gravitational waves (grav_waves.f90)                                */
/* ------------------------------------------------------------------ */
/* grav_spec_estimation (grav_waves.f90:257-321) for the current state.
 * Outputs are nbins = num_bin_grav long: bin centres (wave), power_grav,
 * numer and denom.  Green's mode bins on its GW grid: with degrade_spec > 0
 * the sources are the deg^3-box-summed differences of
 * data1_to_arr_dphi_degrade (grav_waves.f90:358-415), the grid has
 * ngrid / deg sites of spacing dspa deg and the bins run to pi / (dspa deg)
 * (grav_waves.f90:37-45, 62-71).  With AXG_GW_UIJ the TT-projected spectrum
 * of u_ij on the full lattice. */
int axg_grav_spec_estimation(axg_ctx *ctx, double tau, double *wave, double *power, double *numer,
                             double *denom);
/* Same quantity binned in params.gw_log_bins logarithmic bins on
 * [2 pi/(N dx), pi/dx]; edges has nbins+1 entries. */
int axg_grav_spec_log(axg_ctx *ctx, double tau, double *edges, double *power, double *numer,
                      double *denom);

/* ------------------------------------------------------------------ */
/* defects (defects_3d.f90)                                            */
/* ------------------------------------------------------------------ */
/* Cell classification pass of id_defects (defects_3d.f90:67-103, 309-349):
 * int8 flags per cell (1 string, 2 wall, 4 mask) kept on the device;
 * counts = (ns, nw, nm).  which = AXG_F_ID_STRINGS|AXG_F_ID_WALLS|AXG_F_SPEC_EST. */
int axg_classify_cells(axg_ctx *ctx, int which, int64_t counts[3]);
int axg_download_defect_flags(axg_ctx *ctx, int8_t *flags);
/* Plaquette winding: number of plaquettes pierced by a string, per
 * orientation (normal x, y, z). */
int axg_string_winding(axg_ctx *ctx, int64_t counts[3]);
/* Whole id_defects (defects_3d.f90:31-307): classification, per-cell string
 * and wall fits (position_string, velocity_string, position_wall) and the sums
 * of add_string_length / add_wall_area (defects_3d.f90:1654-1733, 2145-2204).
 * sl, wa, svel as in the reference (lattice units); counts = (ns, nw, nm). */
int axg_id_defects(axg_ctx *ctx, int64_t idx, double tau, double sl[3], double wa[3],
                   double svel[3], int64_t counts[3]);
/* Per-cell fit results of the last axg_id_defects, in cell order (z, y, x).
 * strings: [ns][13] = pos(3) dir(3) vel(3) gof sl cell group; walls: [nw][10] =
 * pos(3) dir(3) gof wa cell group.  group = smallest list index of the
 * connected group when AXG_F_GROUP_STRINGS / AXG_F_GROUP_WALLS is set, else -1. */
int axg_download_defect_lists(axg_ctx *ctx, double *strings, int64_t max_strings, double *walls,
                              int64_t max_walls);

/* ------------------------------------------------------------------ */
/* field spectrum (spectrum.f90)                                       */
/* ------------------------------------------------------------------ */
/* spectrum_estimation core (spectrum.f90:242-287 without the MC covariance):
 * masked, degraded phidot spectrum, deconvolved with the mode-coupling
 * matrix of the mask of the last classification.  Arrays of num_bin:
 * wave (bin centres), power (power_spec), conv (conv_spec/num_conv_spec),
 * count (num_conv_spec).  tau is tau_id(idx). */
int axg_spectrum_estimation(axg_ctx *ctx, double tau, double *wave, double *power, double *conv,
                            double *count);
/* compute_crho (spectrum.f90:316-342) from the last power spectrum (no
 * covariance: drho = 0). */
int axg_compute_crho(axg_ctx *ctx, double *rho);
/* estimate_covmat (spectrum.f90:569-734): Monte-Carlo covariance (num_bin *
 * (num_bin+1)/2, packed) of the last spectrum estimate, Gaussian fields with
 * that spectrum masked like the data (Philox draws in place of VSL streams);
 * stops after the jackknife test of the diagonal falls below tol (reference:
 * min_mc 10, max_mc 100, tol 0.1).  A negative deconvolved power contributes
 * sigma = 0.  *iterations = MC realisations used (max_mc + 1 when the test
 * never passed, as the reference divides by it). */
int axg_spectrum_covariance(axg_ctx *ctx, int min_mc, int max_mc, double tol, double *cov,
                            int *iterations);
/* compute_crho with the covariance term of the last axg_spectrum_covariance. */
int axg_compute_crho_cov(axg_ctx *ctx, double *rho, double *drho);
/* get_epsilon (spectrum.f90:956-1040) for one pair of output times: wav has
 * num_bin+1 bin edges, p1/p2 the power spectra, c1/c2 their covariances. */
int axg_epsilon(int32_t nb, const double *wav, const double *p1, const double *p2, const double *c1,
                const double *c2, double tau1, double tau2, double *eps, double *deps);

/* ------------------------------------------------------------------ */
/* initial conditions (initial.f90) and diagnostics                    */
/* ------------------------------------------------------------------ */
/* Seeded Gaussian random field: every Fourier mode with |k| <= kcut an
 * independent complex normal, others zero; normalised to <|phi|^2> = vev^2;
 * phidot = 0; u = u' = 0. */
int axg_ic_gaussian_flat(axg_ctx *ctx, double kcut, uint32_t realisation);
/* get_initial_thermal (initial.f90:80-238, 363-390) at tau_ini with the
 * project's Philox draws in place of MKL VSL streams. */
int axg_ic_thermal(axg_ctx *ctx, double tau_ini, uint32_t realisation);
/* Volume averages in FP64: out = (<|phi|^2>, <|phi'|^2>, <|grad phi|^2>, <V(phi)>)
 * at conformal time tau. */
int axg_field_moments(axg_ctx *ctx, double tau, double out[4]);

/* ------------------------------------------------------------------ */
/* checkpoint / resume (evolve.f90:401-546)                            */
/* ------------------------------------------------------------------ */
/* io_chk: raw complex128 phi block then phidot block, x fastest, global order
 * (evolve.f90:498-503); plus u_ij blocks when present and a CRC32 sidecar
 * file path+".crc".  FP32-mixed contexts also write path+".fp32", the raw
 * FP32 state with its Kahan compensations, the CRC32 of the checkpoint it
 * belongs to and a CRC32 of its own, and read it back when it belongs to the
 * checkpoint being read, so that a resumed run continues bit for bit (a
 * damaged sidecar is an error; one left by an earlier checkpoint of the path
 * is ignored, and FP64 contexts remove it when they write).  write_chk's
 * param.chk is written by axg_write_param_chk. */
int axg_write_chk(axg_ctx *ctx, const char *path);
int axg_read_chk(axg_ctx *ctx, const char *path);
/* param.chk "idx tau flag" (evolve.f90:407-421, 445-448). */
int axg_write_param_chk(const char *path, int64_t idx, double tau, int flag_defects);
int axg_read_param_chk(const char *path, int64_t *idx, double *tau, int *flag_defects);

/* ------------------------------------------------------------------ */
/* timing / profiling                                                  */
/* ------------------------------------------------------------------ */
int axg_synchronize(axg_ctx *ctx);
/* Record a CUDA event on the context stream (slot 0..7). */
int axg_event_record(axg_ctx *ctx, int slot);
/* Milliseconds between two recorded slots (synchronises on the later one). */
int axg_event_elapsed(axg_ctx *ctx, int slot_a, int slot_b, float *ms);
/* When on, every kernel launch is bracketed by events and its time is
 * accumulated per kernel name (for the roofline). */
int axg_set_kernel_timing(axg_ctx *ctx, int on);
/* Name, launches and total ms of the i-th timed kernel; AXG_ERR_ARG past the end. */
int axg_kernel_timing(axg_ctx *ctx, int i, char *name, int64_t name_len, int64_t *launches,
                      double *total_ms);
/* Number of kernels launched on this context since creation. */
int axg_launch_count(const axg_ctx *ctx, int64_t *launches);
/* Self-test of the failure path of the fused kernels' bounded TMA stage
 * waits (no counterpart in the reference, whose errors end in MpiStop,
 * utils.f90:44-73): one CTA waits on a stage barrier that nothing arrives
 * on and issues no copy, gives up after wait_cycles SM cycles (1e3 .. 4e9)
 * and raises the same device flag as a timed-out stage wait.  Returns
 * AXG_ERR_TIMEOUT with the fused kernel's message; the flag is cleared and
 * the context stays usable. */
int axg_selftest_wait_timeout(axg_ctx *ctx, int64_t wait_cycles);

/* ------------------------------------------------------------------ */
/* adjoint (no counterpart in the reference)                            */
/* ------------------------------------------------------------------ */
/* Gradient of the band-integrated GW energy
 *   J = sum_{kmin <= |k| <= kmax} 1/2 sum_ij (|W'_TT|^2 + k^2 |W_TT|^2)
 * (half the numerator of axg_grav_spec_estimation with gw_mode UIJ, summed
 * over the band, at the end of the run) after the leapfrog of axg_leapfrog(t1, dt,
 * nsteps, first_half, last_half) from the current state.  Forward run with a
 * checkpoint every `stride` steps; reverse sweep steps the state back by
 * time-reversibility (re-anchored on each checkpoint) and applies the
 * hand-written adjoint of each kick and drift.  Returns J, dJ/dlambda
 * (quartic model, A = lambda/2, B = -lambda v^2/2) and, when the pointers are
 * non-NULL, dJ/dphi and dJ/dphi' of the initial state as complex128 host
 * arrays (d/dRe + i d/dIm).  ms_forward / ms_reverse (may be NULL) give the
 * GPU time of the two sweeps.  gw_mode UIJ, any precision: the forward run
 * is the context's own step (FP64-plain, FP64-fused or FP32-mixed) and the
 * adjoint runs in the same arithmetic (FP32 for FP32-mixed; dJ/dlambda is
 * accumulated in FP64).  The context is left at the final state of the
 * forward run. */
int axg_adjoint_gw_band(axg_ctx *ctx, double t1, double dt, int64_t nsteps, int first_half,
                        int last_half, int64_t stride, double kmin, double kmax, double *J,
                        double *dJ_dlambda, double *grad_phi0, double *grad_phidot0,
                        double *ms_forward, double *ms_reverse);

/* ------------------------------------------------------------------ */
/* batched ensembles (no counterpart in the reference, which runs one  */
/* realisation per job)                                                 */
/* ------------------------------------------------------------------ */
typedef struct axg_ensemble axg_ensemble;
/* count member lattices of possibly different ngrid and seed; they must share
 * a fused precision (FP32-mixed or FP64-fused), gw_mode NONE or UIJ, dspa,
 * sigma_cr and the potential, so that one step has the same coefficients for
 * all of them.  Each member is a full context (IC, defects, spectra,
 * transfers through axg_ensemble_member); all work on one stream. */
int axg_ensemble_create(const axg_params *members, int32_t count, axg_ensemble **out);
int axg_ensemble_destroy(axg_ensemble *e);
const char *axg_ensemble_last_error(const axg_ensemble *e);
int axg_ensemble_size(const axg_ensemble *e, int32_t *count);
int axg_ensemble_member(axg_ensemble *e, int32_t i, axg_ctx **member);
/* axg_leapfrog for every member at once: each step is ONE persistent launch
 * over all members' columns.  use_graph: the first interval of a given
 * (nsteps, dt, half-step) shape runs eagerly and is captured into a CUDA
 * graph that later intervals of that shape replay. */
int axg_ensemble_leapfrog(axg_ensemble *e, double t1, double dt, int64_t nsteps, int first_half,
                          int last_half, int use_graph);
/* choose the tile shape shared by all members and the launch mode (state
 * restored) */
int axg_ensemble_autotune(axg_ensemble *e, int steps, int *best_cfg, double *best_ms_per_step);
/* fixes the tile shape (axg_tile_info index) of the batched kernel; it must
 * fit every member */
int axg_ensemble_set_tile(axg_ensemble *e, int cfg);
/* launch mode of the batched kernel: persistent = 1 runs one resident set of
 * CTAs that walk the (member, column, z-chunk) items with a grid stride;
 * persistent = 0 launches one CTA per item.  Results are identical. */
int axg_ensemble_set_launch_mode(axg_ensemble *e, int persistent);
int axg_ensemble_launch_mode(const axg_ensemble *e, int *persistent);
int axg_ensemble_launch_count(const axg_ensemble *e, int64_t *launches);
/* Ensemble means of the per-realisation outputs at conformal time tau, from
 * each member's own call (so every realisation's result is the one its own
 * lattice gives):
 *  - the GW spectrum of grav_spec_estimation (grav_waves.f90:257-321; gw_mode
 *    UIJ): the members share dspa, so their num_bin_grav linear bins on
 *    (0, pi/dx] coincide; power_mean / power_sem = mean and standard error
 *    of power_grav over the members with modes in the bin, denom = modes
 *    summed over the members, wave = bin centres (any output may be NULL
 *    but power_mean);
 *  - the string parameter xi = (tau/dx)^2 sl / N^3 / 4 and the wall
 *    parameter A = (tau/dx) wa / N^3 / 2 of defects_and_spectrum
 *    (evolve.f90:191-192) from each member's id_defects (defects_3d.f90:31-307,
 *    the member's flags select strings / walls / grouping): mean and
 *    standard error per component. */
int axg_ensemble_grav_spec_mean(axg_ensemble *e, double tau, double *wave, double *power_mean, double *power_sem,
                                double *denom);
int axg_ensemble_defect_mean(axg_ensemble *e, int64_t idx, double tau, double xi_mean[3], double xi_sem[3],
                             double area_mean[3], double area_sem[3]);

/* ------------------------------------------------------------------ */
/* allocation-free diagnostics                                          */
/* ------------------------------------------------------------------ */
/* No counterpart in the reference.  The volume moments of axg_field_moments
 * for fields the caller already holds on the device, for callers that cannot
 * allocate device memory at that point (their device memory is owned by their
 * own allocator or pool, or a cudaMalloc there would stall work they have
 * queued).  d_phi and d_phidot are complex128 device arrays of p->ngrid^3
 * sites (x fastest); out (host) receives <|phi|^2>, <|phi'|^2>,
 * <|grad phi|^2>, <V(phi)> at conformal time tau; stream may be NULL.  The
 * call allocates nothing: its scratch is a fixed array inside the library
 * (one partial sum per z-plane, so p->ngrid <= 2048; larger lattices are
 * rejected with AXG_ERR_ARG), held by every GPU that loads the library until
 * the process exits.  The first call on a device looks up that array's device
 * address (once per device, with the device current).  The call synchronises
 * its stream (it returns the moments on the host), so it cannot be part of a
 * captured graph.  A cudaDeviceReset of a device ends the life of everything
 * this library set up on it, that address included: after one, the process
 * makes no further call into the library on that device.  All calls share
 * the array, so calls that overlap on the GPU race; serialise them (one
 * stream, or synchronise).  Errors are reported through axg_last_error(NULL). */
int axg_field_moments_noalloc(const axg_params *p, const double *d_phi, const double *d_phidot,
                              double tau, double out[4], void *stream);

/* ------------------------------------------------------------------ */
/* text outputs in the reference's formats, for C hosts                 */
/* ------------------------------------------------------------------ */
/* A Fortran host keeps the reference's own writers; these write the same
 * files from host arrays, with the reference's edit descriptors (integers
 * I12, reals E20.10e3, ten significant digits correctly rounded).  No GPU
 * work.  AXG_OK, AXG_ERR_ARG or AXG_ERR_IO (axg_last_error(NULL)).
 *  - axg_write_spectrum: <root>_spectrum_<idx>.dat, rows (q, P, conv/count,
 *    count) (spectrum.f90:278-285);
 *  - axg_write_covariance: <root>_covariance_<idx>.dat, rows (i, j, cov_ij)
 *    of the packed upper covariance, i = 1..nb, j = 1..i (spectrum.f90:294-302);
 *  - axg_write_gravspec: <root>_gravspec_<idx>.dat, rows (tau, q, q f_cr, P_GW,
 *    modes), f_cr in Hz from tau_cr and a_now (grav_waves.f90:266,308-316);
 *  - axg_append_string_wall_line: one (idx, tau, tau^2 zeta, xi(3), A(3), v(3))
 *    line of _string_wall_parameters.txt (evolve.f90:90,127,202);
 *  - axg_append_crho_line: one (idx, crho(3)) line of _crho.txt (evolve.f90:128);
 *  - axg_append_eps_line: one line of _eps.txt from two output times
 *    (idx, idx2, tau1, tau2, their mean, eps, deps, delta rho, its error;
 *    crho = (rho, drho) at each time) (spectrum.f90:1034-1035). */
int axg_write_spectrum(const char *root, int32_t idx, const double *wave, const double *power,
                       const double *conv_per_mode, const double *count, int32_t nb);
int axg_write_covariance(const char *root, int32_t idx, const double *cov, int32_t nb);
int axg_write_gravspec(const char *root, int32_t idx, double tau, const double *wave, const double *power,
                       const double *denom, int32_t nb, double tau_cr, double a_now);
int axg_append_string_wall_line(const char *path, int32_t idx, double tau, double zeta_tau2, const double xi[3],
                                const double area[3], const double vel[3]);
int axg_append_crho_line(const char *path, int32_t idx, double crho0, double crho1, double crho2);
int axg_append_eps_line(const char *path, int32_t idx, int32_t idx2, double tau1, double tau2, double eps,
                        double deps, const double crho1[2], const double crho2[2]);

#ifdef __cplusplus
}
#endif

#endif /* AXGPU_H */
