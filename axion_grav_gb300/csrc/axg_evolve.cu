// axg_evolve.cu -- leapfrog kernels of the lattice hot path (evolve.f90:238-339).
//
// Three arithmetic paths:
//  * FP64-plain (drop-in for evolve_phi / evolve_phidot): a pointwise drift
//    kernel and a 7-point stencil kick kernel, FP64, every operation written
//    with non-contractible IEEE intrinsics in the reference's order so the
//    result is bit-identical to the CPU restatement.
//  * FP64-fused and FP32-mixed: one pass per step computing the kick and the
//    following drift.  phi and u_ij ping-pong between two buffers; the stencil
//    fields (phi, u) of each z-plane are staged in shared memory by TMA
//    (cp.async.bulk.tensor) into a ring of mbarrier-tracked stages while the
//    pointwise fields (phi', u', Kahan compensations) stream through registers.
//    A CTA owns a TX x TY column of the lattice and marches through zc planes.
//    Halos: y rows and x columns are separate TMA boxes at wrapped coordinates
//    (periodic lattice), x boxes 16 bytes wide so their x coordinate is always
//    16-byte aligned.
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdlib>

#include "axg_detmath.h"
#include "axg_internal.h"
#include "axg_tma.h"

namespace {

constexpr int kStages = 4;            // TMA ring depth (z-1, z, z+1, prefetch)
constexpr int kPwStages = 2;          // pointwise ring depth (z, prefetch of z+1)

// ------------------------------------------------------------------------
// FP64-plain kernels (evolve.f90:259-281 and 283-339)
// ------------------------------------------------------------------------
struct KickCoeffs {
  double f1, f2, f3, fs;  // fact1, fact2, fact3, source factor
  double A, B, C, D;      // dV/dphi* = (A|phi|^2+B) phi + C + D conj(phi)
  double d;               // 2 dspa (grav_waves.f90:331)
  double inv_d;           // 1/d, used only when d is a power of two (then x/d == x*inv_d exactly)
  int d_pow2;
};

// x / d, replaced by the exact multiplication by 1/d when d is a power of two
__device__ __forceinline__ double div_d(double x, double d, double inv_d, int pow2) {
  return pow2 ? axg_mul_pow2(x, inv_d) : AXD_DIV(x, d);
}

__global__ void k_drift_fp64(double2 *__restrict__ phi, const double2 *__restrict__ phid,
                             double *__restrict__ u, const double *__restrict__ ud, int64_t n3,
                             double h, int uij) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    double2 a = phi[s];
    const double2 b = phid[s];
    a.x = AXD_ADD(a.x, AXD_MUL(h, b.x));
    a.y = AXD_ADD(a.y, AXD_MUL(h, b.y));
    phi[s] = a;
    if (uij) {
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const int64_t i = c * n3 + s;
        u[i] = AXD_ADD(u[i], AXD_MUL(h, ud[i]));
      }
    }
  }
}

__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// UIJ: also kick the six u_ij (a template parameter, so the phi-only kick
// keeps the registers, and the resident warps, of its own work)
template <bool UIJ>
__global__ void __launch_bounds__(256) k_kick_fp64(const double2 *__restrict__ phi,
                                                   double2 *__restrict__ phid,
                                                   const double *__restrict__ u,
                                                   double *__restrict__ ud, int n, KickCoeffs k) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  const int iy = blockIdx.y * blockDim.y + threadIdx.y;
  const int iz = blockIdx.z;
  if (ix >= n || iy >= n) return;
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  const int ix1 = wrapi(ix - 1, n), ix2 = wrapi(ix + 1, n);
  const int iy1 = wrapi(iy - 1, n), iy2 = wrapi(iy + 1, n);
  const int iz1 = wrapi(iz - 1, n), iz2 = wrapi(iz + 1, n);
  const int64_t c = iz * n2 + (int64_t)iy * n + ix;
  const int64_t sx1 = iz * n2 + (int64_t)iy * n + ix1, sx2 = iz * n2 + (int64_t)iy * n + ix2;
  const int64_t sy1 = iz * n2 + (int64_t)iy1 * n + ix, sy2 = iz * n2 + (int64_t)iy2 * n + ix;
  const int64_t sz1 = iz1 * n2 + (int64_t)iy * n + ix, sz2 = iz2 * n2 + (int64_t)iy * n + ix;
  const double2 pc = phi[c], px1 = phi[sx1], px2 = phi[sx2], py1 = phi[sy1], py2 = phi[sy2],
                pz1 = phi[sz1], pz2 = phi[sz2];
  // dlap (evolve.f90:325-328), left to right
  double lr = AXD_ADD(px1.x, px2.x);
  lr = AXD_ADD(lr, py1.x);
  lr = AXD_ADD(lr, py2.x);
  lr = AXD_ADD(lr, pz1.x);
  lr = AXD_ADD(lr, pz2.x);
  lr = AXD_SUB(lr, AXD_MUL(6.0, pc.x));
  double li = AXD_ADD(px1.y, px2.y);
  li = AXD_ADD(li, py1.y);
  li = AXD_ADD(li, py2.y);
  li = AXD_ADD(li, pz1.y);
  li = AXD_ADD(li, pz2.y);
  li = AXD_SUB(li, AXD_MUL(6.0, pc.y));
  // dVdphi (potential.f90:43-60)
  const double s2 = AXD_ADD(AXD_MUL(pc.x, pc.x), AXD_MUL(pc.y, pc.y));
  const double g = AXD_ADD(AXD_MUL(k.A, s2), k.B);
  double vr = AXD_MUL(g, pc.x), vi = AXD_MUL(g, pc.y);
  if (k.D != 0.0) {
    vr = AXD_ADD(vr, AXD_MUL(k.D, pc.x));
    vi = AXD_SUB(vi, AXD_MUL(k.D, pc.y));
  }
  vr = AXD_ADD(vr, k.C);
  // data2 = fact1*data2 + fact2*dlap + fact3*ddv (evolve.f90:330)
  const double2 pd = phid[c];
  double pr = AXD_ADD(AXD_MUL(k.f1, pd.x), AXD_MUL(k.f2, lr));
  pr = AXD_ADD(pr, AXD_MUL(k.f3, vr));
  double pi_ = AXD_ADD(AXD_MUL(k.f1, pd.y), AXD_MUL(k.f2, li));
  pi_ = AXD_ADD(pi_, AXD_MUL(k.f3, vi));
  phid[c] = make_double2(pr, pi_);
  if constexpr (UIJ) {
    double dr[3], di[3];
    dr[0] = div_d(AXD_SUB(px2.x, px1.x), k.d, k.inv_d, k.d_pow2);
    di[0] = div_d(AXD_SUB(px2.y, px1.y), k.d, k.inv_d, k.d_pow2);
    dr[1] = div_d(AXD_SUB(py2.x, py1.x), k.d, k.inv_d, k.d_pow2);
    di[1] = div_d(AXD_SUB(py2.y, py1.y), k.d, k.inv_d, k.d_pow2);
    dr[2] = div_d(AXD_SUB(pz2.x, pz1.x), k.d, k.inv_d, k.d_pow2);
    di[2] = div_d(AXD_SUB(pz2.y, pz1.y), k.d, k.inv_d, k.d_pow2);
    int comp = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int j = 0; j <= i; ++j, ++comp) {
        const double *uc = u + comp * n3;
        double src = AXD_ADD(AXD_MUL(dr[i], dr[j]), AXD_MUL(di[i], di[j]));
        src = axg_mul_pow2(src, 2.0);
        double lu = AXD_ADD(uc[sx1], uc[sx2]);
        lu = AXD_ADD(lu, uc[sy1]);
        lu = AXD_ADD(lu, uc[sy2]);
        lu = AXD_ADD(lu, uc[sz1]);
        lu = AXD_ADD(lu, uc[sz2]);
        lu = AXD_SUB(lu, AXD_MUL(6.0, uc[c]));
        double v = AXD_ADD(AXD_MUL(k.f1, ud[comp * n3 + c]), AXD_MUL(k.f2, lu));
        v = AXD_ADD(v, AXD_MUL(k.fs, src));
        ud[comp * n3 + c] = v;
      }
    }
  }
}

// ------------------------------------------------------------------------
// FP32 Kahan drift (first half drift of the fused scheme)
// ------------------------------------------------------------------------
__device__ __forceinline__ void kahan_add(float &x, float &c, float inc) {
  const float y = inc - c;
  const float t = x + y;
  c = (t - x) - y;
  x = t;
}

__global__ void k_drift_fp32(float2 *__restrict__ phi, const float2 *__restrict__ phid,
                             float2 *__restrict__ cphi, float *__restrict__ u,
                             const float *__restrict__ ud, float *__restrict__ cu, int64_t n3,
                             float h, int uij) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    float2 a = phi[s], c = cphi[s];
    const float2 b = phid[s];
    kahan_add(a.x, c.x, h * b.x);
    kahan_add(a.y, c.y, h * b.y);
    phi[s] = a;
    cphi[s] = c;
    if (uij) {
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const int64_t i = k * n3 + s;
        float x = u[i], cc = cu[i];
        kahan_add(x, cc, h * ud[i]);
        u[i] = x;
        cu[i] = cc;
      }
    }
  }
}

// TMA / mbarrier primitives (inline PTX): axg_tma.h
using namespace axg_tma;

// ------------------------------------------------------------------------
// fused kernel: one stage of shared memory holds one z-plane of the stencil
// fields of a TX x TY column with its halos.
// ------------------------------------------------------------------------
template <typename R>
struct V2;
template <>
struct V2<float> {
  using T = float2;
};
template <>
struct V2<double> {
  using T = double2;
};

constexpr int align128(int b) { return (b + 127) / 128 * 128; }

template <typename R, int TX, int TY, bool UIJ>
struct StageLayout {
  using V = typename V2<R>::T;
  static constexpr int PHW = sizeof(R) == 4 ? 2 : 1;  // phi halo width (16 B rule for FP32)
  static constexpr int UHW = 16 / (int)sizeof(R);     // u halo width (16 B)
  static constexpr int phi_main = 0;
  static constexpr int phi_main_sz = align128((TY + 2) * TX * (int)sizeof(V));
  static constexpr int phi_hl = phi_main + phi_main_sz;
  static constexpr int phi_h_sz = align128(TY * PHW * (int)sizeof(V));
  static constexpr int phi_hr = phi_hl + phi_h_sz;
  static constexpr int u_top = phi_hr + phi_h_sz;
  static constexpr int u_row_sz = UIJ ? align128(6 * TX * (int)sizeof(R)) : 0;
  static constexpr int u_body = u_top + u_row_sz;
  static constexpr int u_body_sz = UIJ ? align128(6 * TY * TX * (int)sizeof(R)) : 0;
  static constexpr int u_bot = u_body + u_body_sz;
  static constexpr int u_hl = u_bot + u_row_sz;
  static constexpr int u_h_sz = UIJ ? align128(6 * TY * UHW * (int)sizeof(R)) : 0;
  static constexpr int u_hr = u_hl + u_h_sz;
  static constexpr int bytes = u_hr + u_h_sz;
  // bytes actually delivered by the TMA boxes of one stage
  static constexpr int tx_bytes =
      (TY + 2) * TX * (int)sizeof(V) + 2 * TY * PHW * (int)sizeof(V) +
      (UIJ ? (2 * 6 * TX + 6 * TY * TX + 2 * 6 * TY * UHW) * (int)sizeof(R) : 0);
};

// One plane of the pointwise fields of a TX x TY column (phid, cphi, ud, cu);
// each is a body box, so the bytes delivered equal the layout's size.
template <typename R, int TX, int TY, bool UIJ>
struct PwLayout {
  using V = typename V2<R>::T;
  static constexpr bool F32 = sizeof(R) == 4;
  static constexpr int phid = 0;
  static constexpr int phid_sz = align128(TX * TY * (int)sizeof(V));
  static constexpr int cphi = phid + phid_sz;
  static constexpr int cphi_sz = F32 ? phid_sz : 0;
  static constexpr int ud = cphi + cphi_sz;
  static constexpr int ud_sz = UIJ ? align128(6 * TX * TY * (int)sizeof(R)) : 0;
  static constexpr int cu = ud + ud_sz;
  static constexpr int cu_sz = (UIJ && F32) ? ud_sz : 0;
  static constexpr int bytes = cu + cu_sz;
  static constexpr int tx_bytes = TX * TY * (int)sizeof(V) * (F32 ? 2 : 1) +
                                  (UIJ ? 6 * TX * TY * (int)sizeof(R) * (F32 ? 2 : 1) : 0);
  static_assert(tx_bytes == bytes, "pointwise boxes must fill the layout exactly");
};

// dynamic shared memory of one fused CTA: stencil ring, pointwise ring,
// mbarriers, alignment slack
template <typename R, int TX, int TY, bool UIJ, bool PW>
constexpr int fused_smem_bytes() {
  return kStages * StageLayout<R, TX, TY, UIJ>::bytes + (PW ? kPwStages * PwLayout<R, TX, TY, UIJ>::bytes : 0) +
         (kStages + kPwStages) * 8 + 128;
}

struct PwMaps {
  CUtensorMap m[4];  // phid, cphi, ud, cu
};

template <typename R>
struct FusedParams {
  typename V2<R>::T *phi_out;
  typename V2<R>::T *phid;
  typename V2<R>::T *cphi;  // FP32 only
  R *u_out;
  R *ud;
  R *cu;  // FP32 only
  int64_t n3;
  int n, zc;
  R f1, f2, f3, fsc, dtd, A, B, C, D;
  double d;  // 2 dspa (FP64 path keeps the reference's division)
  double inv_d;
  int d_pow2;
  int *err;
};

template <typename R>
__device__ __forceinline__ void tma_phi(uint32_t dst, const CUtensorMap *m, int x, int y, int z,
                                        uint32_t bar) {
  if constexpr (sizeof(R) == 4)
    tma_load_3d(dst, m, x, y, z, bar);  // 8-byte elements holding (re, im) float pairs
  else
    tma_load_4d(dst, m, 0, x, y, z, bar);  // (re|im, x, y, z) doubles
}

// ---- per-site arithmetic of the fused step, shared by the TMA kernels and
// the plain stencil kernel so every launch shape gives the same bits.  The
// FP32 forms pin their fused multiply-adds with round-once intrinsics; the
// FP64 forms use the reference's unfused operations in its order.

// phi kick + drift at one site from its 7-point stencil; pd, cp: phi' and
// the compensation of phi at the site (cp unused in FP64)
__device__ __forceinline__ void site_phi(const FusedParams<float> &P, float2 c0, float2 xm, float2 xp, float2 ym,
                                         float2 yp, float2 zm, float2 zp, float2 pd, float2 &cp, float2 &pdn,
                                         float2 &pn) {
  // difference-form Laplacian, Kahan drift
  const float lr = ((xm.x - c0.x) + (xp.x - c0.x)) + ((ym.x - c0.x) + (yp.x - c0.x)) + ((zm.x - c0.x) + (zp.x - c0.x));
  const float li = ((xm.y - c0.y) + (xp.y - c0.y)) + ((ym.y - c0.y) + (yp.y - c0.y)) + ((zm.y - c0.y) + (zp.y - c0.y));
  const float s2 = __fmaf_rn(c0.x, c0.x, __fmul_rn(c0.y, c0.y));
  const float g = __fmaf_rn(P.A, s2, P.B);
  const float vr = __fadd_rn(__fmaf_rn(g, c0.x, __fmul_rn(P.D, c0.x)), P.C);
  const float vi = __fmaf_rn(g, c0.y, -__fmul_rn(P.D, c0.y));
  pdn.x = __fmaf_rn(P.f3, vr, __fmaf_rn(P.f2, lr, __fmul_rn(P.f1, pd.x)));
  pdn.y = __fmaf_rn(P.f3, vi, __fmaf_rn(P.f2, li, __fmul_rn(P.f1, pd.y)));
  pn = c0;
  kahan_add(pn.x, cp.x, __fmul_rn(P.dtd, pdn.x));
  kahan_add(pn.y, cp.y, __fmul_rn(P.dtd, pdn.y));
}

__device__ __forceinline__ void site_phi(const FusedParams<double> &P, double2 c0, double2 xm, double2 xp,
                                         double2 ym, double2 yp, double2 zm, double2 zp, double2 pd, double2 &,
                                         double2 &pdn, double2 &pn) {
  double lr = AXD_ADD(xm.x, xp.x);
  lr = AXD_ADD(lr, ym.x);
  lr = AXD_ADD(lr, yp.x);
  lr = AXD_ADD(lr, zm.x);
  lr = AXD_ADD(lr, zp.x);
  lr = AXD_SUB(lr, AXD_MUL(6.0, c0.x));
  double li = AXD_ADD(xm.y, xp.y);
  li = AXD_ADD(li, ym.y);
  li = AXD_ADD(li, yp.y);
  li = AXD_ADD(li, zm.y);
  li = AXD_ADD(li, zp.y);
  li = AXD_SUB(li, AXD_MUL(6.0, c0.y));
  const double s2 = AXD_ADD(AXD_MUL(c0.x, c0.x), AXD_MUL(c0.y, c0.y));
  const double g = AXD_ADD(AXD_MUL(P.A, s2), P.B);
  double vr = AXD_MUL(g, c0.x), vi = AXD_MUL(g, c0.y);
  if (P.D != 0.0) {
    vr = AXD_ADD(vr, AXD_MUL(P.D, c0.x));
    vi = AXD_SUB(vi, AXD_MUL(P.D, c0.y));
  }
  vr = AXD_ADD(vr, P.C);
  double pr = AXD_ADD(AXD_MUL(P.f1, pd.x), AXD_MUL(P.f2, lr));
  pr = AXD_ADD(pr, AXD_MUL(P.f3, vr));
  double pi_ = AXD_ADD(AXD_MUL(P.f1, pd.y), AXD_MUL(P.f2, li));
  pi_ = AXD_ADD(pi_, AXD_MUL(P.f3, vi));
  pdn = make_double2(pr, pi_);
  pn = make_double2(AXD_ADD(c0.x, AXD_MUL(P.dtd, pr)), AXD_ADD(c0.y, AXD_MUL(P.dtd, pi_)));
}

// the six sources S_c (c = (1,1),(2,1),(2,2),(3,1),(3,2),(3,3)) at one site
// from the phi differences; FP32: raw differences (1 / (2dx)^2 and the
// factor 2 are folded into fsc); FP64: the reference's (d_i phi)(d_j phi)*
// with d = 2 dx and the factor 2
__device__ __forceinline__ void site_sources(const FusedParams<float> &, float2 xm, float2 xp, float2 ym, float2 yp,
                                             float2 zm, float2 zp, float S[6]) {
  const float gxr = xp.x - xm.x, gxi = xp.y - xm.y;
  const float gyr = yp.x - ym.x, gyi = yp.y - ym.y;
  const float gzr = zp.x - zm.x, gzi = zp.y - zm.y;
  S[0] = __fmaf_rn(gxr, gxr, __fmul_rn(gxi, gxi));
  S[1] = __fmaf_rn(gyr, gxr, __fmul_rn(gyi, gxi));
  S[2] = __fmaf_rn(gyr, gyr, __fmul_rn(gyi, gyi));
  S[3] = __fmaf_rn(gzr, gxr, __fmul_rn(gzi, gxi));
  S[4] = __fmaf_rn(gzr, gyr, __fmul_rn(gzi, gyi));
  S[5] = __fmaf_rn(gzr, gzr, __fmul_rn(gzi, gzi));
}

__device__ __forceinline__ void site_sources(const FusedParams<double> &P, double2 xm, double2 xp, double2 ym,
                                             double2 yp, double2 zm, double2 zp, double S[6]) {
  double dr[3], di[3];
  dr[0] = div_d(AXD_SUB(xp.x, xm.x), P.d, P.inv_d, P.d_pow2);
  di[0] = div_d(AXD_SUB(xp.y, xm.y), P.d, P.inv_d, P.d_pow2);
  dr[1] = div_d(AXD_SUB(yp.x, ym.x), P.d, P.inv_d, P.d_pow2);
  di[1] = div_d(AXD_SUB(yp.y, ym.y), P.d, P.inv_d, P.d_pow2);
  dr[2] = div_d(AXD_SUB(zp.x, zm.x), P.d, P.inv_d, P.d_pow2);
  di[2] = div_d(AXD_SUB(zp.y, zm.y), P.d, P.inv_d, P.d_pow2);
  int c = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j, ++c) S[c] = axg_mul_pow2(AXD_ADD(AXD_MUL(dr[i], dr[j]), AXD_MUL(di[i], di[j])), 2.0);
}

// one u_ij component: kick with source S, drift (FP32: Kahan with cc)
__device__ __forceinline__ void site_u(const FusedParams<float> &P, float S, float uc, float uxm, float uxp,
                                       float uym, float uyp, float uzm, float uzp, float udv, float &cc, float &udn,
                                       float &un) {
  const float lu = ((uxm - uc) + (uxp - uc)) + ((uym - uc) + (uyp - uc)) + ((uzm - uc) + (uzp - uc));
  udn = __fmaf_rn(P.fsc, S, __fmaf_rn(P.f2, lu, __fmul_rn(P.f1, udv)));
  un = uc;
  kahan_add(un, cc, __fmul_rn(P.dtd, udn));
}

__device__ __forceinline__ void site_u(const FusedParams<double> &P, double S, double uc, double uxm, double uxp,
                                       double uym, double uyp, double uzm, double uzp, double udv, double &,
                                       double &udn, double &un) {
  double lu = AXD_ADD(uxm, uxp);
  lu = AXD_ADD(lu, uym);
  lu = AXD_ADD(lu, uyp);
  lu = AXD_ADD(lu, uzm);
  lu = AXD_ADD(lu, uzp);
  lu = AXD_SUB(lu, AXD_MUL(6.0, uc));
  double v = AXD_ADD(AXD_MUL(P.f1, udv), AXD_MUL(P.f2, lu));
  udn = AXD_ADD(v, AXD_MUL(P.fsc, S));
  un = AXD_ADD(uc, AXD_MUL(P.dtd, udn));
}

// One TX x TY column of zc planes starting at (x0, y0, z0): stage the
// stencil planes by TMA, compute kick + drift, store.  `gplane` counts the
// planes this CTA has staged so far, so stage indices and mbarrier phases
// continue across the columns a persistent CTA processes.  Returns false
// (after recording the error) when a TMA wait timed out.  With PW the
// pointwise fields of plane k arrive by TMA in a kPwStages ring (`gpw`
// continues across columns like `gplane`); without it they are loaded into
// registers at the top of each plane.
template <typename R, int TX, int TY, bool UIJ, bool PW>
__device__ __forceinline__ bool fused_column(const CUtensorMap *tm_prow, const CUtensorMap *tm_pbody,
                                             const CUtensorMap *tm_phalo, const CUtensorMap *tm_urow,
                                             const CUtensorMap *tm_ubody, const CUtensorMap *tm_uhalo,
                                             const CUtensorMap *tm_pw, const FusedParams<R> &P, int x0, int y0,
                                             int z0, unsigned char *smem, uint64_t *bars, uint32_t &gplane,
                                             unsigned char *pwsmem, uint64_t *pbars, uint32_t &gpw) {
  using L = StageLayout<R, TX, TY, UIJ>;
  using PL = PwLayout<R, TX, TY, UIJ>;
  using V = typename V2<R>::T;
  const int n = P.n, zc = P.zc;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int nplanes = zc + 2;

  auto issue = [&](int p) {
    int z = z0 - 1 + p;
    z = z < 0 ? z + n : (z >= n ? z - n : z);
    const int s = (int)((gplane + (uint32_t)p) % kStages);
    unsigned char *st = smem + s * L::bytes;
    const uint32_t bar = smem_u32(&bars[s]);
    mbar_expect_tx(bar, (uint32_t)L::tx_bytes);
    const int ym = y0 == 0 ? n - 1 : y0 - 1;
    const int yp = y0 + TY == n ? 0 : y0 + TY;
    const int xpl = x0 - L::PHW < 0 ? x0 - L::PHW + n : x0 - L::PHW;
    const int xr = x0 + TX == n ? 0 : x0 + TX;
    tma_phi<R>(smem_u32(st + L::phi_main), tm_prow, x0, ym, z, bar);
    tma_phi<R>(smem_u32(st + L::phi_main + TX * (int)sizeof(V)), tm_pbody, x0, y0, z, bar);
    tma_phi<R>(smem_u32(st + L::phi_main + (TY + 1) * TX * (int)sizeof(V)), tm_prow, x0, yp, z, bar);
    tma_phi<R>(smem_u32(st + L::phi_hl), tm_phalo, xpl, y0, z, bar);
    tma_phi<R>(smem_u32(st + L::phi_hr), tm_phalo, xr, y0, z, bar);
    if constexpr (UIJ) {
      const int xul = x0 - L::UHW < 0 ? x0 - L::UHW + n : x0 - L::UHW;
      tma_load_4d(smem_u32(st + L::u_top), tm_urow, x0, ym, z, 0, bar);
      tma_load_4d(smem_u32(st + L::u_body), tm_ubody, x0, y0, z, 0, bar);
      tma_load_4d(smem_u32(st + L::u_bot), tm_urow, x0, yp, z, 0, bar);
      tma_load_4d(smem_u32(st + L::u_hl), tm_uhalo, xul, y0, z, 0, bar);
      tma_load_4d(smem_u32(st + L::u_hr), tm_uhalo, xr, y0, z, 0, bar);
    }
  };

  auto pslot = [&](int k) { return (int)((gpw + (uint32_t)k) % kPwStages); };
  auto pparity = [&](int k) { return (uint32_t)(((gpw + (uint32_t)k) / kPwStages) & 1); };
  auto issue_pw = [&](int k) {
    const int slot = pslot(k);
    unsigned char *st = pwsmem + slot * PL::bytes;
    const uint32_t bar = smem_u32(&pbars[slot]);
    mbar_expect_tx(bar, (uint32_t)PL::tx_bytes);
    const int z = z0 + k;
    tma_phi<R>(smem_u32(st + PL::phid), &tm_pw[0], x0, y0, z, bar);
    if constexpr (sizeof(R) == 4) tma_phi<R>(smem_u32(st + PL::cphi), &tm_pw[1], x0, y0, z, bar);
    if constexpr (UIJ) {
      tma_load_4d(smem_u32(st + PL::ud), &tm_pw[2], x0, y0, z, 0, bar);
      if constexpr (sizeof(R) == 4) tma_load_4d(smem_u32(st + PL::cu), &tm_pw[3], x0, y0, z, 0, bar);
    }
  };

  if (tid == 0) {
    // a persistent CTA's earlier column read these buffers (generic proxy)
    fence_proxy_async();
    const int first = nplanes < kStages ? nplanes : kStages;
    for (int p = 0; p < first; ++p) issue(p);
    if constexpr (PW) {
      const int pfirst = zc < kPwStages ? zc : kPwStages;
      for (int k = 0; k < pfirst; ++k) issue_pw(k);
    }
  }
  auto stage_of = [&](int p) { return (int)((gplane + (uint32_t)p) % kStages); };
  auto parity_of = [&](int p) { return (uint32_t)(((gplane + (uint32_t)p) / kStages) & 1); };
  bool ok = mbar_wait_bounded(smem_u32(&bars[stage_of(0)]), parity_of(0));
  ok = ok && mbar_wait_bounded(smem_u32(&bars[stage_of(1)]), parity_of(1));
  if (__syncthreads_or(!ok)) {
    if (tid == 0) atomicCAS(P.err, 0, AXG_KERR_MBAR_TIMEOUT);
    return false;
  }

  const int64_t n2 = (int64_t)n * n;
  for (int k = 0; k < zc; ++k) {
    const int p = k + 1;
    const int z = z0 + k;
    const int64_t s = z * n2 + (int64_t)(y0 + ty) * n + (x0 + tx);
    // pointwise fields of this plane: registers (issued before the stage
    // wait) or the TMA ring
    V pd;
    V cp;
    R udv[UIJ ? 6 : 1], cuv[UIJ ? 6 : 1];
    if constexpr (!PW) {
      pd = P.phid[s];
      if constexpr (sizeof(R) == 4) cp = P.cphi[s];
      if constexpr (UIJ) {
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          udv[c] = P.ud[c * P.n3 + s];
          if constexpr (sizeof(R) == 4) cuv[c] = P.cu[c * P.n3 + s];
        }
      }
    }
    const int snext = stage_of(p + 1);
    ok = mbar_wait_bounded(smem_u32(&bars[snext]), parity_of(p + 1));
    if constexpr (PW) {
      ok = ok && mbar_wait_bounded(smem_u32(&pbars[pslot(k)]), pparity(k));
      if (ok) {
        const unsigned char *pws = pwsmem + pslot(k) * PL::bytes;
        pd = reinterpret_cast<const V *>(pws + PL::phid)[ty * TX + tx];
        if constexpr (sizeof(R) == 4) cp = reinterpret_cast<const V *>(pws + PL::cphi)[ty * TX + tx];
        if constexpr (UIJ) {
#pragma unroll
          for (int c = 0; c < 6; ++c) {
            udv[c] = reinterpret_cast<const R *>(pws + PL::ud)[(c * TY + ty) * TX + tx];
            if constexpr (sizeof(R) == 4) cuv[c] = reinterpret_cast<const R *>(pws + PL::cu)[(c * TY + ty) * TX + tx];
          }
        }
      }
    }

    if (ok) {
      const unsigned char *sp = smem + stage_of(p - 1) * L::bytes;
      const unsigned char *sc = smem + stage_of(p) * L::bytes;
      const unsigned char *sn = smem + snext * L::bytes;
      const V *pm = reinterpret_cast<const V *>(sc + L::phi_main);
      const V *phl = reinterpret_cast<const V *>(sc + L::phi_hl);
      const V *phr = reinterpret_cast<const V *>(sc + L::phi_hr);
      const V c0 = pm[(ty + 1) * TX + tx];
      const V xm = tx > 0 ? pm[(ty + 1) * TX + tx - 1] : phl[ty * L::PHW + L::PHW - 1];
      const V xp = tx < TX - 1 ? pm[(ty + 1) * TX + tx + 1] : phr[ty * L::PHW];
      const V ym = pm[ty * TX + tx];
      const V yp = pm[(ty + 2) * TX + tx];
      const V zm = reinterpret_cast<const V *>(sp + L::phi_main)[(ty + 1) * TX + tx];
      const V zp = reinterpret_cast<const V *>(sn + L::phi_main)[(ty + 1) * TX + tx];

      V pdn, pn;
      site_phi(P, c0, xm, xp, ym, yp, zm, zp, pd, cp, pdn, pn);
      P.phid[s] = pdn;
      if constexpr (sizeof(R) == 4) P.cphi[s] = cp;
      P.phi_out[s] = pn;
      if constexpr (UIJ) {
        R S[6];
        site_sources(P, xm, xp, ym, yp, zm, zp, S);
        const R *ub = reinterpret_cast<const R *>(sc + L::u_body);
        const R *ut = reinterpret_cast<const R *>(sc + L::u_top);
        const R *ubt = reinterpret_cast<const R *>(sc + L::u_bot);
        const R *uhl = reinterpret_cast<const R *>(sc + L::u_hl);
        const R *uhr = reinterpret_cast<const R *>(sc + L::u_hr);
        const R *ubp = reinterpret_cast<const R *>(sp + L::u_body);
        const R *ubn = reinterpret_cast<const R *>(sn + L::u_body);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const int o = (c * TY + ty) * TX + tx;
          const R uc = ub[o];
          const R uxm = tx > 0 ? ub[o - 1] : uhl[(c * TY + ty) * L::UHW + L::UHW - 1];
          const R uxp = tx < TX - 1 ? ub[o + 1] : uhr[(c * TY + ty) * L::UHW];
          const R uym = ty > 0 ? ub[o - TX] : ut[c * TX + tx];
          const R uyp = ty < TY - 1 ? ub[o + TX] : ubt[c * TX + tx];
          const R uzm = ubp[o], uzp = ubn[o];
          R cc = sizeof(R) == 4 ? cuv[c] : R(0), udn, un;
          site_u(P, S[c], uc, uxm, uxp, uym, uyp, uzm, uzp, udv[c], cc, udn, un);
          P.ud[c * P.n3 + s] = udn;
          if constexpr (sizeof(R) == 4) P.cu[c * P.n3 + s] = cc;
          P.u_out[c * P.n3 + s] = un;
        }
      }
    }
    // all threads are done with stage (p-1); refill it with plane p-1+kStages
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicCAS(P.err, 0, AXG_KERR_MBAR_TIMEOUT);
      return false;
    }
    if (tid == 0) {
      const bool more = p - 1 + kStages < nplanes;
      const bool pmore = PW && k + kPwStages < zc;
      if (more || pmore) fence_proxy_async();
      if (more) issue(p - 1 + kStages);
      if constexpr (PW)
        if (pmore) issue_pw(k + kPwStages);
    }
  }
  gplane += (uint32_t)nplanes;
  if constexpr (PW) gpw += (uint32_t)zc;
  return true;
}

__device__ __forceinline__ void init_stage_barriers(uint64_t *bars) {
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    for (int s = 0; s < kStages + kPwStages; ++s) mbar_init(smem_u32(&bars[s]), 1);
    fence_barrier_init();
    fence_proxy_async();
  }
  __syncthreads();
}

template <typename R, int TX, int TY, bool UIJ, bool PW>
__global__ void __launch_bounds__(TX *TY, (sizeof(R) == 4 && TX * TY <= 256 ? 2 : 1))
    k_fused(const __grid_constant__ CUtensorMap tm_prow, const __grid_constant__ CUtensorMap tm_pbody,
            const __grid_constant__ CUtensorMap tm_phalo, const __grid_constant__ CUtensorMap tm_urow,
            const __grid_constant__ CUtensorMap tm_ubody, const __grid_constant__ CUtensorMap tm_uhalo,
            const __grid_constant__ PwMaps pwm, const FusedParams<R> P) {
  using L = StageLayout<R, TX, TY, UIJ>;
  using PL = PwLayout<R, TX, TY, UIJ>;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  unsigned char *pwsmem = smem + kStages * L::bytes;
  uint64_t *bars = reinterpret_cast<uint64_t *>(pwsmem + (PW ? kPwStages * PL::bytes : 0));
  init_stage_barriers(bars);
  const int ncx = P.n / TX;
  const int x0 = (blockIdx.x % ncx) * TX, y0 = (blockIdx.x / ncx) * TY, z0 = blockIdx.y * P.zc;
  uint32_t gplane = 0, gpw = 0;
  fused_column<R, TX, TY, UIJ, PW>(&tm_prow, &tm_pbody, &tm_phalo, &tm_urow, &tm_ubody, &tm_uhalo, pwm.m, P, x0,
                                   y0, z0, smem, bars, gplane, pwsmem, bars + kStages, gpw);
}

// ------------------------------------------------------------------------
// batched kernel: ensembles of lattices of uneven sizes in one launch.  Work
// items are (member, column, z-chunk) in member order, columns fastest.  Each
// CTA walks the items with a grid stride, re-using its TMA ring (stage phases
// continue through `gplane`); launched with one CTA per item the loop runs
// once and the hardware scheduler balances the SMs.  Per-step coefficients come
// from device memory so the whole step sequence can be graph-captured once.
// ------------------------------------------------------------------------
template <typename R, int TX, int TY, bool UIJ, bool PW>
__global__ void __launch_bounds__(TX *TY, (sizeof(R) == 4 && TX * TY <= 256 ? 2 : 1))
    k_fused_batch(const axg_ens_member_dev *__restrict__ mem, int nmem, long long total, int cur,
                  const axg_ens_coef *__restrict__ coefs, int step, int zc, double dspa, int *err) {
  using L = StageLayout<R, TX, TY, UIJ>;
  using PL = PwLayout<R, TX, TY, UIJ>;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  unsigned char *pwsmem = smem + kStages * L::bytes;
  uint64_t *bars = reinterpret_cast<uint64_t *>(pwsmem + (PW ? kPwStages * PL::bytes : 0));
  init_stage_barriers(bars);
  const axg_ens_coef &K = coefs[step];
  FusedParams<R> P;
  P.f1 = (R)K.f[0];
  P.f2 = (R)K.f[1];
  P.f3 = (R)K.f[2];
  P.fsc = sizeof(R) == 4 ? (R)(K.f[3] * 2.0 / ((2.0 * dspa) * (2.0 * dspa))) : (R)K.f[3];
  P.dtd = (R)K.dtd;
  P.A = (R)K.pot[0];
  P.B = (R)K.pot[1];
  P.C = (R)K.pot[2];
  P.D = (R)K.pot[3];
  P.d = 2.0 * dspa;
  P.inv_d = 1.0 / P.d;
  int ex;
  P.d_pow2 = sizeof(R) == 8 && frexp(P.d, &ex) == 0.5;
  P.zc = zc;
  P.err = err;
  uint32_t gplane = 0, gpw = 0;
  for (long long w = blockIdx.x; w < total; w += gridDim.x) {
    int lo = 0, hi = nmem - 1;  // last member with item_begin <= w
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (mem[mid].item_begin <= w) lo = mid;
      else hi = mid - 1;
    }
    const axg_ens_member_dev &D = mem[lo];
    const long long local = w - D.item_begin;
    const int col = (int)(local % D.ncols), chunk = (int)(local / D.ncols);
    const int ncx = D.n / TX;
    P.n = D.n;
    P.n3 = D.n3;
    P.phi_out = reinterpret_cast<typename V2<R>::T *>(D.phi[1 - cur]);
    P.phid = reinterpret_cast<typename V2<R>::T *>(D.phid);
    P.cphi = reinterpret_cast<typename V2<R>::T *>(D.cphi);
    P.u_out = reinterpret_cast<R *>(D.u[1 - cur]);
    P.ud = reinterpret_cast<R *>(D.ud);
    P.cu = reinterpret_cast<R *>(D.cu);
    const CUtensorMap *tm = D.tm[cur];
    if (!fused_column<R, TX, TY, UIJ, PW>(&tm[0], &tm[1], &tm[2], &tm[3], &tm[4], &tm[5], D.pw, P,
                                          (col % ncx) * TX, (col / ncx) * TY, chunk * zc, smem, bars, gplane, pwsmem,
                                          bars + kStages, gpw))
      return;
  }
}

// ------------------------------------------------------------------------
// The fused step as a plain stencil kernel: one thread per site, the stencil
// read from global memory (through L1 / L2).  It serves lattices that no TMA
// tile shape fits (N not a multiple of 32) and runs the same per-site
// arithmetic as the tiled kernels, so it gives the same bits.
// ------------------------------------------------------------------------
template <typename R, bool UIJ>
__global__ void __launch_bounds__(256) k_fused_plain(const typename V2<R>::T *__restrict__ phi_in,
                                                     const R *__restrict__ u_in, FusedParams<R> P) {
  using V = typename V2<R>::T;
  const int n = P.n;
  const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y * blockDim.y + threadIdx.y, iz = blockIdx.z;
  if (ix >= n || iy >= n) return;
  const int64_t n2 = (int64_t)n * n;
  const int xm1 = ix == 0 ? n - 1 : ix - 1, xp1 = ix + 1 == n ? 0 : ix + 1;
  const int ym1 = iy == 0 ? n - 1 : iy - 1, yp1 = iy + 1 == n ? 0 : iy + 1;
  const int zm1 = iz == 0 ? n - 1 : iz - 1, zp1 = iz + 1 == n ? 0 : iz + 1;
  const int64_t row = (int64_t)iz * n2 + (int64_t)iy * n;
  const int64_t s = row + ix, sxm = row + xm1, sxp = row + xp1;
  const int64_t sym = (int64_t)iz * n2 + (int64_t)ym1 * n + ix, syp = (int64_t)iz * n2 + (int64_t)yp1 * n + ix;
  const int64_t szm = (int64_t)zm1 * n2 + (int64_t)iy * n + ix, szp = (int64_t)zp1 * n2 + (int64_t)iy * n + ix;
  const V c0 = phi_in[s], xm = phi_in[sxm], xp = phi_in[sxp], ym = phi_in[sym], yp = phi_in[syp], zm = phi_in[szm],
          zp = phi_in[szp];
  const V pd = P.phid[s];
  V cp{};
  if constexpr (sizeof(R) == 4) cp = P.cphi[s];
  V pdn, pn;
  site_phi(P, c0, xm, xp, ym, yp, zm, zp, pd, cp, pdn, pn);
  P.phid[s] = pdn;
  if constexpr (sizeof(R) == 4) P.cphi[s] = cp;
  P.phi_out[s] = pn;
  if constexpr (UIJ) {
    R S[6];
    site_sources(P, xm, xp, ym, yp, zm, zp, S);
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const R *u = u_in + c * P.n3;
      R cc = sizeof(R) == 4 ? P.cu[c * P.n3 + s] : R(0), udn, un;
      site_u(P, S[c], u[s], u[sxm], u[sxp], u[sym], u[syp], u[szm], u[szp], P.ud[c * P.n3 + s], cc, udn, un);
      P.ud[c * P.n3 + s] = udn;
      if constexpr (sizeof(R) == 4) P.cu[c * P.n3 + s] = cc;
      P.u_out[c * P.n3 + s] = un;
    }
  }
}

// ------------------------------------------------------------------------
// tile table (autotuner search space) and host-side launch
// ------------------------------------------------------------------------
const axg_tile_cfg kTiles[] = {
    {32, 16, 32, 0}, {32, 8, 32, 0}, {32, 16, 64, 0}, {32, 8, 64, 0}, {32, 16, 16, 0}, {32, 8, 16, 0},
    {32, 4, 32, 0},  {32, 4, 32, 1}, {32, 8, 32, 1},  {32, 4, 64, 1}, {32, 4, 16, 1}, {32, 8, 64, 1},
};
constexpr int kNumTiles = sizeof(kTiles) / sizeof(kTiles[0]);

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

int encode(axg_ctx *ctx, CUtensorMap *m, CUtensorMapDataType dt, int rank, void *base,
           const cuuint64_t *dims, const cuuint64_t *strides, const cuuint32_t *box) {
  auto fn = encode_fn();
  if (!fn) return axg_set_error(ctx, AXG_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  CUresult r = fn(m, dt, (cuuint32_t)rank, base, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return axg_set_error(ctx, AXG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return AXG_OK;
}

int build_tmaps(axg_ctx *ctx, int cfg) {
  if (ctx->tm.valid && ctx->tm.cfg == cfg) return AXG_OK;
  const axg_tile_cfg t = kTiles[cfg];
  const cuuint64_t n = (cuuint64_t)ctx->n;
  const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
  const bool uij = ctx->p.gw_mode == AXG_GW_UIJ;
  const int rs = fp32 ? 4 : 8;  // bytes of one real
  for (int b = 0; b < 2; ++b) {
    if (fp32) {
      cuuint64_t dims[3] = {n, n, n};
      cuuint64_t str[2] = {n * 8, n * n * 8};
      cuuint32_t row[3] = {(cuuint32_t)t.tx, 1, 1}, body[3] = {(cuuint32_t)t.tx, (cuuint32_t)t.ty, 1},
                 halo[3] = {2, (cuuint32_t)t.ty, 1};
      AXG_TRY(encode(ctx, &ctx->tm.phi_row[b], CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, ctx->phi[b], dims, str, row));
      AXG_TRY(encode(ctx, &ctx->tm.phi_body[b], CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, ctx->phi[b], dims, str, body));
      AXG_TRY(encode(ctx, &ctx->tm.phi_halo[b], CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, ctx->phi[b], dims, str, halo));
    } else {
      cuuint64_t dims[4] = {2, n, n, n};
      cuuint64_t str[3] = {16, n * 16, n * n * 16};
      cuuint32_t row[4] = {2, (cuuint32_t)t.tx, 1, 1}, body[4] = {2, (cuuint32_t)t.tx, (cuuint32_t)t.ty, 1},
                 halo[4] = {2, 1, (cuuint32_t)t.ty, 1};
      AXG_TRY(encode(ctx, &ctx->tm.phi_row[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, ctx->phi[b], dims, str, row));
      AXG_TRY(encode(ctx, &ctx->tm.phi_body[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, ctx->phi[b], dims, str, body));
      AXG_TRY(encode(ctx, &ctx->tm.phi_halo[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, ctx->phi[b], dims, str, halo));
    }
    if (uij) {
      const CUtensorMapDataType dt = fp32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
      cuuint64_t dims[4] = {n, n, n, 6};
      cuuint64_t str[3] = {n * rs, n * n * rs, n * n * n * rs};
      const cuuint32_t uhw = 16 / rs;
      cuuint32_t row[4] = {(cuuint32_t)t.tx, 1, 1, 6}, body[4] = {(cuuint32_t)t.tx, (cuuint32_t)t.ty, 1, 6},
                 halo[4] = {uhw, (cuuint32_t)t.ty, 1, 6};
      AXG_TRY(encode(ctx, &ctx->tm.u_row[b], dt, 4, ctx->u[b], dims, str, row));
      AXG_TRY(encode(ctx, &ctx->tm.u_body[b], dt, 4, ctx->u[b], dims, str, body));
      AXG_TRY(encode(ctx, &ctx->tm.u_halo[b], dt, 4, ctx->u[b], dims, str, halo));
    } else {
      // unused placeholders (kernel never dereferences them without UIJ)
      ctx->tm.u_row[b] = ctx->tm.phi_row[b];
      ctx->tm.u_body[b] = ctx->tm.phi_body[b];
      ctx->tm.u_halo[b] = ctx->tm.phi_halo[b];
    }
  }
  // pointwise planes (body boxes of phid, cphi, ud, cu); unused maps copy a valid one
  if (fp32) {
    cuuint64_t dims[3] = {n, n, n};
    cuuint64_t str[2] = {n * 8, n * n * 8};
    cuuint32_t body[3] = {(cuuint32_t)t.tx, (cuuint32_t)t.ty, 1};
    AXG_TRY(encode(ctx, &ctx->tm.pw[0], CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, ctx->phid, dims, str, body));
    AXG_TRY(encode(ctx, &ctx->tm.pw[1], CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, ctx->cphi, dims, str, body));
  } else {
    cuuint64_t dims[4] = {2, n, n, n};
    cuuint64_t str[3] = {16, n * 16, n * n * 16};
    cuuint32_t body[4] = {2, (cuuint32_t)t.tx, (cuuint32_t)t.ty, 1};
    AXG_TRY(encode(ctx, &ctx->tm.pw[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, ctx->phid, dims, str, body));
    ctx->tm.pw[1] = ctx->tm.pw[0];
  }
  if (uij) {
    const CUtensorMapDataType dt = fp32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    cuuint64_t dims[4] = {n, n, n, 6};
    cuuint64_t str[3] = {n * rs, n * n * rs, n * n * n * rs};
    cuuint32_t body[4] = {(cuuint32_t)t.tx, (cuuint32_t)t.ty, 1, 6};
    AXG_TRY(encode(ctx, &ctx->tm.pw[2], dt, 4, ctx->ud, dims, str, body));
    if (fp32) AXG_TRY(encode(ctx, &ctx->tm.pw[3], dt, 4, ctx->cu, dims, str, body));
    else ctx->tm.pw[3] = ctx->tm.pw[2];
  } else {
    ctx->tm.pw[2] = ctx->tm.pw[3] = ctx->tm.pw[0];
  }
  ctx->tm.valid = true;
  ctx->tm.cfg = cfg;
  return AXG_OK;
}

template <typename R, int TX, int TY, bool UIJ, bool PW>
int launch_fused_t(axg_ctx *ctx, const FusedParams<R> &P, const char *name) {
  constexpr int smem = fused_smem_bytes<R, TX, TY, UIJ, PW>();
  static bool attr_set = false;
  if (!attr_set) {
    AXG_CUDA_TRY(ctx, cudaFuncSetAttribute(k_fused<R, TX, TY, UIJ, PW>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr_set = true;
  }
  const int b = ctx->cur;
  dim3 grid((unsigned)((ctx->n / TX) * (ctx->n / TY)), (unsigned)(ctx->n / P.zc));
  dim3 block(TX, TY);
  PwMaps pwm;
  for (int q = 0; q < 4; ++q) pwm.m[q] = ctx->tm.pw[q];
  AXG_LAUNCH(ctx, name, (k_fused<R, TX, TY, UIJ, PW>), grid, block, smem, ctx->tm.phi_row[b],
             ctx->tm.phi_body[b], ctx->tm.phi_halo[b], ctx->tm.u_row[b], ctx->tm.u_body[b],
             ctx->tm.u_halo[b], pwm, P);
  return AXG_OK;
}

template <typename R, bool UIJ>
int launch_fused_cfg(axg_ctx *ctx, const FusedParams<R> &P, int cfg, const char *name) {
  const axg_tile_cfg t = kTiles[cfg];
  if (t.pw) {
    if (t.tx == 32 && t.ty == 8) return launch_fused_t<R, 32, 8, UIJ, true>(ctx, P, name);
    if (t.tx == 32 && t.ty == 4) return launch_fused_t<R, 32, 4, UIJ, true>(ctx, P, name);
  } else {
    if (t.tx == 32 && t.ty == 16) return launch_fused_t<R, 32, 16, UIJ, false>(ctx, P, name);
    if (t.tx == 32 && t.ty == 8) return launch_fused_t<R, 32, 8, UIJ, false>(ctx, P, name);
    if (t.tx == 32 && t.ty == 4) return launch_fused_t<R, 32, 4, UIJ, false>(ctx, P, name);
  }
  return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "tile configuration");
}

}  // namespace

// --------------------------------------------------------------------------
int axg_evo_build_tmaps(axg_ctx *ctx, int cfg) { return build_tmaps(ctx, cfg); }

int axg_evo_tile_count() { return kNumTiles; }
axg_tile_cfg axg_evo_tile(int i) { return kTiles[i]; }

int axg_evo_tile_supported(const axg_ctx *ctx, int i) {
  if (i < 0 || i >= kNumTiles) return 0;
  const axg_tile_cfg t = kTiles[i];
  const int64_t n = ctx->n;
  if (n % t.tx || n % t.ty || n % t.zc) return 0;
  if (n < 2 * t.ty || n < 4) return 0;
  // shared memory budget per CTA (227 KB)
  const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
  const bool uij = ctx->p.gw_mode == AXG_GW_UIJ;
  const int rs = fp32 ? 4 : 8, vs = 2 * rs;
  const int phw = fp32 ? 2 : 1, uhw = 16 / rs;
  auto a = [](int b) { return (b + 127) / 128 * 128; };
  int st = a((t.ty + 2) * t.tx * vs) + 2 * a(t.ty * phw * vs);
  if (uij) st += 2 * a(6 * t.tx * rs) + a(6 * t.ty * t.tx * rs) + 2 * a(6 * t.ty * uhw * rs);
  int pw = 0;
  if (t.pw) {
    if (t.ty != 4 && t.ty != 8) return 0;  // instantiated pointwise-TMA tiles
    pw = a(t.tx * t.ty * vs) * (fp32 ? 2 : 1) + (uij ? a(6 * t.tx * t.ty * rs) * (fp32 ? 2 : 1) : 0);
  }
  if (kStages * st + kPwStages * pw + (kStages + kPwStages) * 8 + 128 > 227 * 1024) return 0;
  return 1;
}

int axg_evo_default_tile(const axg_ctx *ctx) {
  // the first supported shape in the preference order
  const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
  for (int i = 0; i < kNumTiles; ++i) {
    const int cfg = axg_evo_tile_preference(fp32, i);
    if (axg_evo_tile_supported(ctx, cfg)) return cfg;
  }
  return -1;
}

// Preferred order for a context that was not autotuned.  FP32: the shapes
// with the pointwise fields in the TMA ring first (the autotuner's picks at
// 256^3 to 1024^3); FP64 is bound by the FP64 pipe and nearly indifferent
// to the shape.
int axg_evo_tile_preference(bool fp32, int rank) {
  if (rank < 0 || rank >= kNumTiles) return -1;
  static const int pref_fp32[] = {8, 11, 10, 7, 9, 1, 0, 3, 2, 5, 4, 6};
  static const int pref_fp64[] = {7, 1, 3, 5, 8, 9, 10, 11, 0, 2, 4, 6};
  static_assert(sizeof(pref_fp32) / sizeof(int) == kNumTiles && sizeof(pref_fp64) / sizeof(int) == kNumTiles,
                "one entry per tile shape");
  return fp32 ? pref_fp32[rank] : pref_fp64[rank];
}

int axg_evo_drift(axg_ctx *ctx, double h) {
  const int uij = ctx->p.gw_mode == AXG_GW_UIJ;
  const int64_t n3 = ctx->n3;
  int blocks = (int)((n3 + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  const int b = ctx->cur;
  if (ctx->p.precision == AXG_PREC_FP32_MIXED) {
    AXG_LAUNCH(ctx, "drift_fp32_kahan", k_drift_fp32, blocks, 256, 0, (float2 *)ctx->phi[b],
               (const float2 *)ctx->phid, (float2 *)ctx->cphi, (float *)ctx->u[b],
               (const float *)ctx->ud, (float *)ctx->cu, n3, (float)h, uij);
  } else {
    AXG_LAUNCH(ctx, "drift_fp64", k_drift_fp64, blocks, 256, 0, (double2 *)ctx->phi[b],
               (const double2 *)ctx->phid, (double *)ctx->u[b], (const double *)ctx->ud, n3, h,
               uij);
  }
  return AXG_OK;
}

int axg_evo_kick_plain(axg_ctx *ctx, double t, double dt) {
  if (ctx->p.precision == AXG_PREC_FP32_MIXED)
    return axg_set_error(ctx, AXG_ERR_STATE, "separate kick is the FP64 path; FP32 runs fused");
  double f[4], pot[4];
  axg_kick_coeffs(&ctx->p, t, dt, f, pot);
  const double d = ctx->p.dspa * 2;
  int ex;
  const int pow2 = std::frexp(d, &ex) == 0.5;
  KickCoeffs k{f[0], f[1], f[2], f[3], pot[0], pot[1], pot[2], pot[3], d, 1.0 / d, pow2};
  const int n = (int)ctx->n;
  dim3 block(32, 8);
  dim3 grid((n + 31) / 32, (n + 7) / 8, n);
  const int b = ctx->cur;
  if (ctx->p.gw_mode == AXG_GW_UIJ)
    AXG_LAUNCH(ctx, "kick_fp64_plain", k_kick_fp64<true>, grid, block, 0, (const double2 *)ctx->phi[b],
               (double2 *)ctx->phid, (const double *)ctx->u[b], (double *)ctx->ud, n, k);
  else
    AXG_LAUNCH(ctx, "kick_fp64_plain", k_kick_fp64<false>, grid, block, 0, (const double2 *)ctx->phi[b],
               (double2 *)ctx->phid, (const double *)nullptr, (double *)nullptr, n, k);
  return AXG_OK;
}

int axg_evo_kick_drift(axg_ctx *ctx, double t, double dt, double dtd) {
  if (ctx->p.precision == AXG_PREC_FP64_PLAIN)
    return axg_set_error(ctx, AXG_ERR_STATE, "fused step requested on the FP64-plain path");
  int cfg = ctx->tile_cfg >= 0 ? ctx->tile_cfg : axg_evo_default_tile(ctx);
  // no TMA tile shape fits (N not a multiple of 32): the plain stencil
  // kernel; AXG_FUSED_PLAIN=1 selects it for any N (tests compare the two)
  const char *pe = std::getenv("AXG_FUSED_PLAIN");
  const bool plain = cfg < 0 || !axg_evo_tile_supported(ctx, cfg) || (pe && pe[0] == '1');
  if (!plain) AXG_TRY(build_tmaps(ctx, cfg));
  double f[4], pot[4];
  axg_kick_coeffs(&ctx->p, t, dt, f, pot);
  const bool uij = ctx->p.gw_mode == AXG_GW_UIJ;
  const int b = ctx->cur, o = 1 - b;
  const axg_tile_cfg tc = plain ? axg_tile_cfg{32, 8, 1, 0} : kTiles[cfg];
  const dim3 pblock(32, 8), pgrid((unsigned)((ctx->n + 31) / 32), (unsigned)((ctx->n + 7) / 8), (unsigned)ctx->n);
  if (ctx->p.precision == AXG_PREC_FP32_MIXED) {
    FusedParams<float> P;
    P.phi_out = (float2 *)ctx->phi[o];
    P.phid = (float2 *)ctx->phid;
    P.cphi = (float2 *)ctx->cphi;
    P.u_out = (float *)ctx->u[o];
    P.ud = (float *)ctx->ud;
    P.cu = (float *)ctx->cu;
    P.n3 = ctx->n3;
    P.n = (int)ctx->n;
    P.zc = tc.zc;
    P.f1 = (float)f[0];
    P.f2 = (float)f[1];
    P.f3 = (float)f[2];
    // source with raw differences: fs * 2 * (d_i d_j) / (2 dx)^2
    P.fsc = (float)(f[3] * 2.0 / ((2.0 * ctx->p.dspa) * (2.0 * ctx->p.dspa)));
    P.dtd = (float)dtd;
    P.A = (float)pot[0];
    P.B = (float)pot[1];
    P.C = (float)pot[2];
    P.D = (float)pot[3];
    P.d = 2.0 * ctx->p.dspa;
    P.inv_d = 1.0 / P.d;
    P.d_pow2 = 0;
    P.err = ctx->d_err;
    if (plain && uij)
      AXG_LAUNCH(ctx, "fused_kd_fp32_uij_plain", (k_fused_plain<float, true>), pgrid, pblock, 0,
                 (const float2 *)ctx->phi[b], (const float *)ctx->u[b], P);
    else if (plain)
      AXG_LAUNCH(ctx, "fused_kd_fp32_phi_plain", (k_fused_plain<float, false>), pgrid, pblock, 0,
                 (const float2 *)ctx->phi[b], (const float *)ctx->u[b], P);
    else if (uij) AXG_TRY((launch_fused_cfg<float, true>(ctx, P, cfg, "fused_kd_fp32_uij")));
    else AXG_TRY((launch_fused_cfg<float, false>(ctx, P, cfg, "fused_kd_fp32_phi")));
  } else {
    FusedParams<double> P;
    P.phi_out = (double2 *)ctx->phi[o];
    P.phid = (double2 *)ctx->phid;
    P.cphi = nullptr;
    P.u_out = (double *)ctx->u[o];
    P.ud = (double *)ctx->ud;
    P.cu = nullptr;
    P.n3 = ctx->n3;
    P.n = (int)ctx->n;
    P.zc = tc.zc;
    P.f1 = f[0];
    P.f2 = f[1];
    P.f3 = f[2];
    P.fsc = f[3];
    P.dtd = dtd;
    P.A = pot[0];
    P.B = pot[1];
    P.C = pot[2];
    P.D = pot[3];
    P.d = 2.0 * ctx->p.dspa;
    int ex;
    P.d_pow2 = std::frexp(P.d, &ex) == 0.5;
    P.inv_d = 1.0 / P.d;
    P.err = ctx->d_err;
    if (plain && uij)
      AXG_LAUNCH(ctx, "fused_kd_fp64_uij_plain", (k_fused_plain<double, true>), pgrid, pblock, 0,
                 (const double2 *)ctx->phi[b], (const double *)ctx->u[b], P);
    else if (plain)
      AXG_LAUNCH(ctx, "fused_kd_fp64_phi_plain", (k_fused_plain<double, false>), pgrid, pblock, 0,
                 (const double2 *)ctx->phi[b], (const double *)ctx->u[b], P);
    else if (uij) AXG_TRY((launch_fused_cfg<double, true>(ctx, P, cfg, "fused_kd_fp64_uij")));
    else AXG_TRY((launch_fused_cfg<double, false>(ctx, P, cfg, "fused_kd_fp64_phi")));
  }
  ctx->cur = o;
  return AXG_OK;
}

namespace {
// The give-up path of the bounded stage wait, run on its own: one CTA
// initialises a stage barrier that expects one arrival, issues no copy and
// never arrives, so every thread's bounded wait runs out after `limit`
// cycles; the CTA then raises the timeout flag exactly as the fused kernel
// does (__syncthreads_or, one atomicCAS) and returns.  Nothing is in flight
// when it gives up.
__global__ void k_wait_timeout_selftest(long long limit, int *err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&bar), 1);
    fence_barrier_init();
  }
  __syncthreads();
  const bool ok = mbar_wait_bounded(smem_u32(&bar), 0, limit);
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) atomicCAS(err, 0, AXG_KERR_MBAR_TIMEOUT);
  }
}
}  // namespace

extern "C" int axg_selftest_wait_timeout(axg_ctx *ctx, int64_t wait_cycles) {
  if (!ctx || wait_cycles < 1000 || wait_cycles > axg_tma::kWaitCycles) return AXG_ERR_ARG;
  AXG_LAUNCH(ctx, "wait_timeout_selftest", k_wait_timeout_selftest, 1, 128, 0, (long long)wait_cycles, ctx->d_err);
  return axg_evo_check_error(ctx);
}

int axg_encode_tmap(axg_ctx *ctx, CUtensorMap *m, CUtensorMapDataType dt, int rank, void *base,
                    const cuuint64_t *dims, const cuuint64_t *strides, const cuuint32_t *box) {
  return encode(ctx, m, dt, rank, base, dims, strides, box);
}

int axg_evo_check_error(axg_ctx *ctx) {
  int h = 0;
  AXG_CUDA_TRY(ctx, cudaMemcpyAsync(&h, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (h == AXG_KERR_MBAR_TIMEOUT) {
    int z = 0;
    cudaMemcpy(ctx->d_err, &z, sizeof(int), cudaMemcpyHostToDevice);
    return axg_set_error(ctx, AXG_ERR_TIMEOUT, "TMA stage wait timed out (fused kernel or FFT column pass)");
  }
  if (h != 0) {
    int z = 0;
    cudaMemcpy(ctx->d_err, &z, sizeof(int), cudaMemcpyHostToDevice);
    return axg_set_error(ctx, AXG_ERR_CUDA, "kernel reported error " + std::to_string(h));
  }
  return AXG_OK;
}

namespace {
template <typename R, int TX, int TY, bool UIJ, bool PW>
int launch_batch_t(axg_ctx *ctx, cudaStream_t stream, const axg_ens_member_dev *d_mem, int nmem, long long total,
                   int cur, const axg_ens_coef *d_coef, int step, int zc, double dspa, int *d_err, bool persistent) {
  constexpr int smem = fused_smem_bytes<R, TX, TY, UIJ, PW>();
  static bool attr_set = false;
  if (!attr_set) {
    AXG_CUDA_TRY(ctx, cudaFuncSetAttribute(k_fused_batch<R, TX, TY, UIJ, PW>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr_set = true;
  }
  int per_sm = 0;
  AXG_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fused_batch<R, TX, TY, UIJ, PW>,
                                                                  TX * TY, smem));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  // persistent: resident CTAs walk the items with a grid stride; otherwise
  // one CTA per item and the hardware scheduler balances the SMs
  long long grid = persistent ? (long long)std::max(per_sm, 1) * std::max(sms, 1) : total;
  if (grid > total) grid = total;
  k_fused_batch<R, TX, TY, UIJ, PW><<<(unsigned)grid, dim3(TX, TY), smem, stream>>>(d_mem, nmem, total, cur,
                                                                                   d_coef, step, zc, dspa, d_err);
  ctx->launches++;
  AXG_CUDA_TRY(ctx, cudaGetLastError());
  return AXG_OK;
}
}  // namespace

int axg_evo_batch_step(axg_ctx *any, cudaStream_t stream, const axg_ens_member_dev *d_mem, int nmem,
                       long long total_items, int cur, const axg_ens_coef *d_coef, int step, int cfg,
                       int *d_err, bool fp32, bool uij, double dspa, bool persistent) {
  const axg_tile_cfg t = kTiles[cfg];
#define AXG_BATCH(R, TY_, U, PW_)                                                                         \
  return launch_batch_t<R, 32, TY_, U, PW_>(any, stream, d_mem, nmem, total_items, cur, d_coef, step, t.zc, dspa, \
                                            d_err, persistent)
#define AXG_BATCH_TY(R, U)                        \
  if (t.pw) {                                     \
    if (t.ty == 8) AXG_BATCH(R, 8, U, true);      \
    if (t.ty == 4) AXG_BATCH(R, 4, U, true);      \
  } else {                                        \
    if (t.ty == 16) AXG_BATCH(R, 16, U, false);   \
    if (t.ty == 8) AXG_BATCH(R, 8, U, false);     \
    if (t.ty == 4) AXG_BATCH(R, 4, U, false);     \
  }
  if (fp32) {
    if (uij) { AXG_BATCH_TY(float, true) }
    else { AXG_BATCH_TY(float, false) }
  } else {
    if (uij) { AXG_BATCH_TY(double, true) }
    else { AXG_BATCH_TY(double, false) }
  }
#undef AXG_BATCH_TY
#undef AXG_BATCH
  return axg_set_error(any, AXG_ERR_UNSUPPORTED, "tile configuration");
}
