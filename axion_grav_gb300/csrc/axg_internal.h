// axg_internal.h -- context and shared helpers of libaxgpu (GB300, sm_103a).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/axgpu.h"

// Error codes written by kernels into ctx->d_err (first writer wins).
#define AXG_KERR_MBAR_TIMEOUT 1
#define AXG_KERR_BOUNDS 2

// Fused-kernel tile configurations known to the autotuner.
// pw = 1: the pointwise fields (phi', u', compensations) are staged by TMA
// too, one plane ahead, instead of being loaded into registers.
struct axg_tile_cfg {
  int tx, ty, zc, pw;
};

// Device-side descriptor of one ensemble member (tensor maps of both
// ping-pong buffers plus the field pointers); it takes the alignment of its
// tensor maps, as TMA requires.
struct axg_ens_member_dev {
  CUtensorMap tm[2][6];  // [buffer][phi_row, phi_body, phi_halo, u_row, u_body, u_halo]
  CUtensorMap pw[4];     // pointwise planes: phid, cphi, ud, cu
  void *phi[2], *phid, *cphi, *u[2], *ud, *cu;
  int64_t n3;
  int32_t n, ncols;
  long long item_begin;  // first work item (column x z-chunk) of this member
};
static_assert(alignof(axg_ens_member_dev) >= 64, "tensor maps in device memory need 64-byte alignment");

// Per-step coefficients of the batched kick + drift (read by the kernel
// from device memory so a captured step graph can be replayed).
struct axg_ens_coef {
  double f[4], pot[4], dtd, pad[3];
};

struct axg_kernel_stat {
  std::string name;
  int64_t launches = 0;
  double total_ms = 0.0;
};

struct axg_tmaps {
  bool valid = false;
  int cfg = -1;
  CUtensorMap phi_row[2], phi_body[2], phi_halo[2];
  CUtensorMap u_row[2], u_body[2], u_halo[2];
  CUtensorMap pw[4];  // phid, cphi, ud, cu (body boxes; not ping-ponged)
};

struct axg_bin_cache_entry {
  int16_t *tab = nullptr;
  size_t cap = 0;
  int m = 0, nb = 0;
  double dwav = 0, dq = 0;
  std::vector<double> edges;
};

struct axg_ctx {
  axg_params p{};
  axg_bin_cache_entry bin_cache[3];  // GW linear, GW log, field spectrum
  int64_t n = 0, n3 = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  // host<->device transfers: a copy stream and two staging buffers, so the
  // copy of one chunk overlaps the precision conversion of the previous one
  cudaStream_t xstream = nullptr;
  void *xstage[2] = {nullptr, nullptr};
  cudaEvent_t xev_copied[2] = {nullptr, nullptr}, xev_done[2] = {nullptr, nullptr}, xev_start = nullptr;

  // evolution state; phi[cur] / u[cur] are current (fused paths ping-pong)
  void *phi[2] = {nullptr, nullptr};
  void *phid = nullptr;
  void *cphi = nullptr;  // Kahan compensation of the phi drift (FP32 path)
  void *u[2] = {nullptr, nullptr};
  void *ud = nullptr;
  void *cu = nullptr;  // Kahan compensation of the u drift (FP32 path)
  int cur = 0;
  size_t elem = 8;  // bytes of one real of the field storage

  // Green's-function GW state (grav_waves.f90)
  // the GW grid of init_grav (grav_waves.f90:37-45): gw_n = ngrid / 2^degrade_spec
  // sites a side, spacing gw_dspa = dspa 2^degrade_spec
  int gw_n = 0;
  double gw_dspa = 0;
  bool gw_ff_real = false;  // degraded FP64 sources stored, then the float-float D2Z (axg_ff_d2z)
  double2 *acc = nullptr;  // Green accumulators [4][n3]; FP32-mixed: float4 (re hi, re lo, im hi, im lo)  // [4][n3]
  double *gsrc = nullptr;  // [6][n3] real sources S_ij (float for FP32-mixed)
  double2 *gsrcF = nullptr;  // [6][n*n*(n/2+1)] (float2 for FP32-mixed)
  float2 *gw_omega = nullptr;  // [n3] |k| dwav per k-site as float hi + lo (FP32-mixed Green mode)
  double *gw_pol = nullptr;    // FP64 Green mode: [12][n*n*(n/2+1)] float2 e+ (re, im as float-float), then
                               // [n*n*(n/2+1)] double |k| dwav; or null
  bool acc_ff = false;         // Green accumulators are float-float float4 (FP32-mixed, and the FP64 paths
                               // on the float-float transforms), else double2
  int64_t acc_stride = 0;      // Green accumulator entries per component (axg_gw_acc_entries)
  bool gw_own_fft = false;     // Green sources transformed by axg_fft_ff.cu (FP64: float-float D2Z; FP32:
                               // the fused source + R2C), else by cuFFT; fixed when the context is made
  bool uij_own_fft = false;    // u_ij spectrum: fields formed in our own row transforms (no real buffer, no plan)
  int gsrc_pitch = 0;          // kx row pitch of gsrcF (axg_f32_spec_pitch for the FP32 own transforms, else n/2+1)
  int u_pitch = 0;             // kx row pitch of the u_ij spectra in ubuf (likewise)
  float *ff_tw = nullptr;      // float-float FFT twiddles W_n^k, k < n/2 (axg_fft_ff.cu)
  int ff_tw_n = 0;
  cufftHandle plan_gsrc = 0;
  bool plan_gsrc_ok = false;

  // defects
  int8_t *flags = nullptr;  // per cell, bits 1/2/4
  float *phase = nullptr;  // per site FP32 phase (filtered classification)
  double *phase64 = nullptr;  // per site FP64 deterministic phase (the fits of id_defects)
  bool flags_valid = false;
  // fit results of the last id_defects
  double *d_strings = nullptr;
  double *d_walls = nullptr;
  int64_t cap_strings = 0, cap_walls = 0;
  int64_t last_ns = 0, last_nw = 0, last_nm = 0;

  // spectra
  double *spec_mat = nullptr;  // mat_spec [num_cov][501]
  double *spec_largeq0 = nullptr, *spec_dq = nullptr;  // per ij
  std::vector<double> h_mat_spec, h_largeq, h_dq, h_wav;
  std::vector<double> last_power;
  std::vector<double> last_mat_div;  // deconvolution matrix after the division by mode counts
  std::vector<double> last_cov;      // MC covariance of the last spectrum (num_cov)
  double2 *spec_buf = nullptr;  // (N/deg)^3 complex
  cufftHandle plan_spec = 0;
  bool plan_spec_ok = false;
  cufftHandle plan_window = 0;  // D2Z of the real window (its half spectrum follows the real input in spec_buf)
  bool plan_window_ok = false;
  int64_t ns_spec = 0;

  // GW spectra of u_ij (R2C of 12 fields)
  cufftHandle plan_u = 0;
  bool plan_u_ok = false;
  void *ubuf = nullptr;  // real inputs / complex outputs workspace

  // reductions
  double *d_red = nullptr;  // small FP64 reduction buffer
  unsigned long long *d_cnt = nullptr;  // small counter buffer
  int *d_err = nullptr;
  size_t red_cap = 0;

  // tensor maps for the fused kernel
  axg_tmaps tm;
  int tile_cfg = -1;  // chosen tile configuration (-1: default)

  // timing
  cudaEvent_t user_ev[8] = {};
  bool ktiming = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  std::vector<cudaEvent_t> ev_pool;
  std::map<std::string, int> kid;
  std::vector<axg_kernel_stat> kstats;
  int64_t launches = 0;
  int64_t bytes = 0;

  std::string err;
};

// ---------------------------------------------------------------------------
// error helpers (return a status from the enclosing C-ABI function)
// ---------------------------------------------------------------------------
int axg_set_error(axg_ctx *ctx, int code, const std::string &msg);

#define AXG_CUDA_TRY(ctx, call)                                                       \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return axg_set_error((ctx), AXG_ERR_CUDA,                                       \
                           std::string(#call) + ": " + cudaGetErrorString(e_));       \
  } while (0)

#define AXG_CUFFT_TRY(ctx, call)                                                      \
  do {                                                                                \
    cufftResult r_ = (call);                                                          \
    if (r_ != CUFFT_SUCCESS)                                                          \
      return axg_set_error((ctx), AXG_ERR_CUDA,                                       \
                           std::string(#call) + ": cufft error " + std::to_string((int)r_)); \
  } while (0)

#define AXG_TRY(expr)        \
  do {                       \
    int s_ = (expr);         \
    if (s_ != AXG_OK) return s_; \
  } while (0)

#ifdef __CUDACC__
// x * f for f = 2^k, bit-identical to the FP64 multiply but on the integer
// pipe: for a normal x whose product stays normal the product only adds k to
// the exponent field.  Zero, subnormal, infinite or NaN x, and products that
// would leave the normal range, take the FP64 multiply.  (GB300 issues FP64
// at 1/64 of the FP32 rate, so exact power-of-two scalings move off it.)
// The rare FP64 path is a real call, so that it is branched over instead of
// being issued predicated-off on every lane.
static __device__ __noinline__ double axg_mul_pow2_fp64(double x, double f) { return __dmul_rn(x, f); }
__device__ __forceinline__ double axg_mul_pow2(double x, double f) {
  const long long fb = __double_as_longlong(f);
  const int k = (int)((fb >> 52) & 0x7ff) - 1023;
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e > 0 && e < 0x7ff && e + k > 0 && e + k < 0x7ff) return __longlong_as_double(b + ((long long)k << 52));
  return axg_mul_pow2_fp64(x, f);
}
#endif

// Runs its function when the scope ends, also on the early returns of the
// AXG_* macros (scratch buffers, plans and events of multi-step routines).
template <typename F>
struct axg_scope_exit {
  F f;
  ~axg_scope_exit() { f(); }
};
template <typename F>
axg_scope_exit<F> axg_on_exit(F f) {
  return axg_scope_exit<F>{f};
}

// ---------------------------------------------------------------------------
// kernel launch bookkeeping (per-kernel event timing for the roofline)
// ---------------------------------------------------------------------------
void axg_kt_begin(axg_ctx *ctx, const char *name);
void axg_kt_end(axg_ctx *ctx);
int axg_kt_flush(axg_ctx *ctx);

#define AXG_LAUNCH(ctx, name, kern, grid, block, smem, ...)                         \
  do {                                                                              \
    axg_kt_begin((ctx), (name));                                                    \
    kern<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);                  \
    axg_kt_end((ctx));                                                              \
    (ctx)->launches++;                                                              \
    cudaError_t le_ = cudaGetLastError();                                           \
    if (le_ != cudaSuccess)                                                         \
      return axg_set_error((ctx), AXG_ERR_CUDA,                                     \
                           std::string("launch ") + (name) + ": " + cudaGetErrorString(le_)); \
  } while (0)

// ---------------------------------------------------------------------------
// device allocation helper (counts bytes)
// ---------------------------------------------------------------------------
int axg_alloc(axg_ctx *ctx, void **ptr, size_t bytes, const char *what);
void axg_free(axg_ctx *ctx, void **ptr);

// ---------------------------------------------------------------------------
// internal entry points implemented in the kernel files
// ---------------------------------------------------------------------------
// evolution (axg_evolve.cu)
int axg_evo_drift(axg_ctx *ctx, double h);                  // drift of current state
int axg_evo_kick_plain(axg_ctx *ctx, double t, double dt);  // FP64-plain kick (phi, u)
int axg_evo_kick_drift(axg_ctx *ctx, double t, double dt, double dtd);  // fused step
int axg_evo_check_error(axg_ctx *ctx);
// cuTensorMapEncodeTiled (interleave and swizzle none, L2 promotion 256 B)
int axg_encode_tmap(axg_ctx *ctx, CUtensorMap *m, CUtensorMapDataType dt, int rank, void *base,
                    const cuuint64_t *dims, const cuuint64_t *strides, const cuuint32_t *box);
int axg_evo_tile_count();
axg_tile_cfg axg_evo_tile(int i);
int axg_evo_tile_supported(const axg_ctx *ctx, int i);
int axg_evo_default_tile(const axg_ctx *ctx);
int axg_evo_tile_preference(bool fp32, int rank);  // tile index of the rank-th preferred shape
int axg_evo_build_tmaps(axg_ctx *ctx, int cfg);
// one launch over every member's columns (ensemble.cu drives it); persistent
// = resident CTAs walk the items, else one CTA per item
// 3-D batched D2Z at FP64 accuracy in float-float arithmetic (axg_fft_ff.cu):
// cuFFT's layout and convention, n a power of two in [16, 512]
// (axg_ff_use: supported, and not switched off by AXG_FFT_FF=0, which the
// tests use to compare with cuFFT)
bool axg_ff_fft_supported(int n);
bool axg_ff_use(int n);
// keep_ff: the output stays float-float, (re hi, re lo, im hi, im lo) per
// complex value in the same 16 bytes, for a consumer that reads it so
int axg_ff_d2z(axg_ctx *ctx, const double *in, double2 *out, int n, int batch, bool keep_ff = false);
int axg_ff_z2z(axg_ctx *ctx, double2 *data, int n, int inverse);  // in place, one n^3 volume
// The Green accumulators hold the stored half spectrum only: component a of
// the entry h = (hz n + hy) (n/2 + 1) + hx is acc[a acc_stride + h], and the
// site of -k is its conjugate (real sources, and e+(-k) = conj e+(k)).  On
// the Nyquist y and z rows (hy or hz = n/2) the index of -k maps to itself,
// not to -k, so for 0 < hx < n/2 those mirrored sites keep entries of their
// own after the half spectrum: nhalf + gw_nyq_extra(hx, hy, hz, n).
__host__ __device__ inline int64_t axg_gw_acc_entries(int n) {
  return (int64_t)n * n * (n / 2 + 1) + (int64_t)(n / 2 - 1) * (2 * n - 1);
}
__host__ __device__ inline int64_t gw_nyq_extra(int hx, int hy, int hz, int n) {
  return (int64_t)(hx - 1) * (2 * n - 1) + (hy == n / 2 ? hz : n + (hy < n / 2 ? hy : hy - 1));
}

// Row pitch (complex values) of the complex-float half spectra of the own
// transforms: n/2 + 1 rounded up to a multiple of 4, so that every kx row
// starts on a 32-byte sector and the rows' byte stride suits TMA (a multiple
// of 16).  Columns n/2 + 1 .. pitch - 1 are padding that no consumer reads.
inline int axg_f32_spec_pitch(int n) { return (n / 2 + 1 + 3) & ~3; }
// the six FP32-mixed Green sources of phi and their forward transforms, out
// [6][n][n][pitch] complex float (cuFFT's R2C values, rows of
// axg_f32_spec_pitch(n)); n as axg_ff_fft_supported
int axg_gw_source_r2c_f32(axg_ctx *ctx, const float2 *phi, float2 *out, int n, float scale);
// the u_ij spectrum's twelve real fields (tau u_c, u_c + tau u'_c) and their
// forward transforms, out [12][n][n][pitch] complex float (rows of
// axg_f32_spec_pitch(n)); cu: the FP32 Kahan compensation of u, or null
int axg_uij_r2c_f32(axg_ctx *ctx, const float *u, const float *ud, const float *cu, float tau, float2 *out, int n);
int axg_uij_d2z_ff(axg_ctx *ctx, const double *u, const double *ud, double tau, double2 *out, int n);
// the six FP64 Green sources of phi (d = 2 dx; inv_d, d_pow2 as
// gw_sources_fp64) and their float-float D2Z, out as axg_ff_d2z for batch 6
int axg_gw_source_d2z_ff(axg_ctx *ctx, const double2 *phi, double d, double inv_d, int d_pow2, double2 *out, int n,
                         bool keep_ff);
int axg_evo_batch_step(axg_ctx *any, cudaStream_t stream, const axg_ens_member_dev *d_mem, int nmem,
                       long long total_items, int cur, const axg_ens_coef *d_coef, int step, int cfg,
                       int *d_err, bool fp32, bool uij, double dspa, bool persistent);

// kick coefficients (axg_capi.cu) -- evolve.f90:291-305
void axg_kick_coeffs(const axg_params *p, double t, double dt, double f[4], double pot[4]);

// GW (axg_gw.cu)
int axg_gw_init(axg_ctx *ctx);
int axg_gw_integration(axg_ctx *ctx, double tau, double dtau);
int axg_gw_spec(axg_ctx *ctx, double tau, int log_bins, double *wave, double *power,
                double *numer, double *denom);

// defects (axg_defects.cu)
int axg_def_classify(axg_ctx *ctx, int which, int64_t counts[3]);
int axg_def_winding(axg_ctx *ctx, int64_t counts[3]);
int axg_def_id_defects(axg_ctx *ctx, double tau, double sl[3], double wa[3], double svel[3],
                       int64_t counts[3]);

// spectrum (axg_spectrum.cu)
int axg_spec_init(axg_ctx *ctx);
int axg_spec_estimation(axg_ctx *ctx, double tau, double *wave, double *power, double *conv,
                        double *count);

// initial conditions / moments (axg_ic.cu)
int axg_ic_gauss(axg_ctx *ctx, double kcut, uint32_t realisation);
int axg_ic_therm(axg_ctx *ctx, double tau_ini, uint32_t realisation);
int axg_moments(axg_ctx *ctx, double tau, double out[4]);

// conversion helpers (axg_capi.cu)
int axg_phi_to_fp64(axg_ctx *ctx, double2 *dst);   // current phi as complex128 (device)
int axg_phid_to_fp64(axg_ctx *ctx, double2 *dst);  // current phidot as complex128 (device)
