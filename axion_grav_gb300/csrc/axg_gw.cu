// axg_gw.cu -- gravitational waves (grav_waves.f90) on the GPU.
//
// Green's-function mode (AXG_GW_GREEN), per kick (grav_waves.f90:193-255):
//   1. k_gw_source : the six real sources S_ij = d_i phi d_j phi* + c.c. with
//                    d_i phi = (phi(x+e_i) - phi(x-e_i)) / (2 dx), one pass
//                    over phi writing 6 x N^3 reals (the reference's arr_dphi
//                    is never materialised);
//   2. cuFFT D2Z (R2C for FP32-mixed) batched x6: the reference's backward
//                    C2C of a real field is the conjugate of the forward half
//                    spectrum;
//   3. k_gw_accumulate: one pass over the full spectrum.  Per k the
//                    polarisation tensor of get_comwav_grav (157-191) is
//                    formed in registers, the six sources are contracted into
//                    X+ = sum_ij e+_ij S_ij and X- = sum_ij e-_ij S_ij, and
//                    the four accumulators of grav_waves.f90:239-242 take
//                    dw (cos, sin)(k tau) X+-.  compat = REF reproduces the
//                    cross-wired (2,1)/(1,2) updates through their closed form
//                    over the six components.  FP64 for the FP64 paths; the
//                    FP32-mixed path contracts in FP32 (sources, transforms,
//                    polarisation, sin/cos of the FP64-reduced phase) and
//                    accumulates in FP64.
// Spectra: shell histograms in FP64 (grav_waves.f90:257-321), 25 linear bins
// or log bins; the u_ij path (AXG_GW_UIJ) FFTs w = tau u and w' = u + tau u'
// (R2C, FP32 for the FP32-mixed path), TT-projects per k and accumulates
// sum_ij (|W'_TT|^2 + k^2 |W_TT|^2), which over a k-shell tends to the
// Green's-function numerator as dx -> 0 (second order in k dx).
#include <cmath>
#include <cstdlib>
#include <vector>

#include "axg_binning.h"
#include "axg_detmath.h"
#include "axg_ff.h"
#include "axg_gw_source.h"
#include "axg_internal.h"

namespace {

constexpr double kRefPi = 3.14159265359;
constexpr double kRefTwoPi = 2 * kRefPi;
// potential.f90:13-23
constexpr double kBigHInMstar = 2.1332e-42 / 2.435e18;

__device__ __forceinline__ int kint(int j, int n) { return (j + n / 2) % n - n / 2; }

// FP64 sources in the reference's operation order (gw_sources_fp64)
__global__ void k_gw_source(const double2 *__restrict__ phi, int n, double d, double inv_d, int d_pow2,
                            double *__restrict__ src) {
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    const int ix = (int)(s % n), iy = (int)((s / n) % n), iz = (int)(s / n2);
    const int64_t base = iz * n2 + (int64_t)iy * n;
    const int64_t sx2 = base + (ix + 1 == n ? 0 : ix + 1), sx1 = base + (ix == 0 ? n - 1 : ix - 1);
    const int64_t sy2 = iz * n2 + (int64_t)(iy + 1 == n ? 0 : iy + 1) * n + ix;
    const int64_t sy1 = iz * n2 + (int64_t)(iy == 0 ? n - 1 : iy - 1) * n + ix;
    const int64_t sz2 = (int64_t)(iz + 1 == n ? 0 : iz + 1) * n2 + (int64_t)iy * n + ix;
    const int64_t sz1 = (int64_t)(iz == 0 ? n - 1 : iz - 1) * n2 + (int64_t)iy * n + ix;
    const double2 pa[3] = {phi[sx2], phi[sy2], phi[sz2]}, pb[3] = {phi[sx1], phi[sy1], phi[sz1]};
    double S[6];
    gw_sources_fp64(pa, pb, d, inv_d, d_pow2, S);
#pragma unroll
    for (int c = 0; c < 6; ++c) src[c * n3 + s] = S[c];
  }
}

// FP32 sources from the FP32 field: raw differences, scaled by 2/d^2 once
__global__ void k_gw_source_f32(const float2 *__restrict__ phi, int n, float scale, float *__restrict__ src) {
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    const int ix = (int)(s % n), iy = (int)((s / n) % n), iz = (int)(s / n2);
    const int64_t base = iz * n2 + (int64_t)iy * n;
    const int64_t a[3] = {base + (ix + 1 == n ? 0 : ix + 1), iz * n2 + (int64_t)(iy + 1 == n ? 0 : iy + 1) * n + ix,
                          (int64_t)(iz + 1 == n ? 0 : iz + 1) * n2 + (int64_t)iy * n + ix};
    const int64_t b[3] = {base + (ix == 0 ? n - 1 : ix - 1), iz * n2 + (int64_t)(iy == 0 ? n - 1 : iy - 1) * n + ix,
                          (int64_t)(iz == 0 ? n - 1 : iz - 1) * n2 + (int64_t)iy * n + ix};
    float dr[3], di[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float2 pa = phi[a[k]], pb = phi[b[k]];
      dr[k] = pa.x - pb.x;
      di[k] = pa.y - pb.y;
    }
    int c = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j <= i; ++j, ++c) src[c * n3 + s] = scale * (dr[i] * dr[j] + di[i] * di[j]);
  }
}

// data1_to_arr_dphi_degrade (grav_waves.f90:358-415) fused with the six
// sources, for degrade_spec > 0: one thread per cell of the GW grid
// (m = n / deg a side).  The central differences of the deg^3 fine sites a
// cell covers are summed in the reference's order (z, then y, then x; each
// step (sum + phi(x + e)) - phi(x - e)), divided by d = deg^3 dx 2 and
// multiplied as in gw_sources_fp64.  src: [6][m^3].
__global__ void k_gw_source_degrade(const double2 *__restrict__ phi, int n, int deg, double d, double inv_d,
                                    int d_pow2, double *__restrict__ src) {
  const int m = n / deg;
  const int64_t n2 = (int64_t)n * n, m3 = (int64_t)m * m * m;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < m3; c += stride) {
    const int cx = (int)(c % m), cy = (int)((c / m) % m), cz = (int)(c / ((int64_t)m * m));
    double xr[3] = {0.0, 0.0, 0.0}, xi[3] = {0.0, 0.0, 0.0};
    for (int iz = cz * deg; iz < (cz + 1) * deg; ++iz) {
      const int64_t z0 = iz * n2, zp = (iz + 1 == n ? 0 : iz + 1) * n2, zm = (iz == 0 ? n - 1 : iz - 1) * n2;
      for (int iy = cy * deg; iy < (cy + 1) * deg; ++iy) {
        const int64_t y0 = (int64_t)iy * n, yp = (int64_t)(iy + 1 == n ? 0 : iy + 1) * n,
                      ym = (int64_t)(iy == 0 ? n - 1 : iy - 1) * n;
        for (int ix = cx * deg; ix < (cx + 1) * deg; ++ix) {
          const int xp = ix + 1 == n ? 0 : ix + 1, xm = ix == 0 ? n - 1 : ix - 1;
          const double2 a[3] = {phi[z0 + y0 + xp], phi[z0 + yp + ix], phi[zp + y0 + ix]};
          const double2 b[3] = {phi[z0 + y0 + xm], phi[z0 + ym + ix], phi[zm + y0 + ix]};
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            xr[k] = AXD_SUB(AXD_ADD(xr[k], a[k].x), b[k].x);
            xi[k] = AXD_SUB(AXD_ADD(xi[k], a[k].y), b[k].y);
          }
        }
      }
    }
    double S[6];
    gw_sources_from_diff(xr, xi, d, inv_d, d_pow2, S);
#pragma unroll
    for (int k = 0; k < 6; ++k) src[k * m3 + c] = S[k];
  }
}

// The FP32-mixed form: the differences of the FP32 field are summed as
// differences (sum + (phi(x + e) - phi(x - e))), which keeps the FP32 sum
// accurate for smooth fields, and the products are scaled by 2 / d^2 once.
__global__ void k_gw_source_degrade_f32(const float2 *__restrict__ phi, int n, int deg, float scale,
                                        float *__restrict__ src) {
  const int m = n / deg;
  const int64_t n2 = (int64_t)n * n, m3 = (int64_t)m * m * m;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < m3; c += stride) {
    const int cx = (int)(c % m), cy = (int)((c / m) % m), cz = (int)(c / ((int64_t)m * m));
    float xr[3] = {0.f, 0.f, 0.f}, xi[3] = {0.f, 0.f, 0.f};
    for (int iz = cz * deg; iz < (cz + 1) * deg; ++iz) {
      const int64_t z0 = iz * n2, zp = (iz + 1 == n ? 0 : iz + 1) * n2, zm = (iz == 0 ? n - 1 : iz - 1) * n2;
      for (int iy = cy * deg; iy < (cy + 1) * deg; ++iy) {
        const int64_t y0 = (int64_t)iy * n, yp = (int64_t)(iy + 1 == n ? 0 : iy + 1) * n,
                      ym = (int64_t)(iy == 0 ? n - 1 : iy - 1) * n;
        for (int ix = cx * deg; ix < (cx + 1) * deg; ++ix) {
          const int xp = ix + 1 == n ? 0 : ix + 1, xm = ix == 0 ? n - 1 : ix - 1;
          const float2 a[3] = {phi[z0 + y0 + xp], phi[z0 + yp + ix], phi[zp + y0 + ix]};
          const float2 b[3] = {phi[z0 + y0 + xm], phi[z0 + ym + ix], phi[zm + y0 + ix]};
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            xr[k] += a[k].x - b[k].x;
            xi[k] += a[k].y - b[k].y;
          }
        }
      }
    }
    int k = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j <= i; ++j, ++k) src[k * m3 + c] = scale * (xr[i] * xr[j] + xi[i] * xi[j]);
  }
}

// |k| dwav per stored half-spectrum entry as a float-float pair, the phase
// rate of the FP32 Green accumulation
__global__ void k_gw_omega(int n, double dwav, float2 *__restrict__ om) {
  const int nh = n / 2 + 1;
  const int64_t nhalf = (int64_t)n * n * nh;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nhalf; h += stride) {
    const double kx = kint((int)(h % nh), n), ky = kint((int)((h / nh) % n), n), kz = kint((int)(h / ((int64_t)nh * n)), n);
    const double w = sqrt(kx * kx + ky * ky + kz * kz) * dwav;
    const float hi = (float)w;
    om[h] = make_float2(hi, (float)(w - (double)hi));
  }
}

// get_comwav_grav (grav_waves.f90:157-191): p = (qz c - i s, qz s + i c, -r)
// for the unit vector q of k, (c, s) its azimuth; e+_ij = p_i p_j, halved on
// the diagonal, in the component order (1,1),(2,1),(2,2),(3,1),(3,2),(3,3).
// Divisions are reciprocal multiplies (one rounding more than the reference).
template <typename R>
__device__ __forceinline__ bool gw_polarisation(R kx, R ky, R kz, R qq, R pr[6], R pi[6]) {
  if (!(qq > 0)) return false;
  const R iq = R(1) / qq;
  const R qx = kx * iq, qy = ky * iq, qz = kz * iq;
  const R r = sqrt(qx * qx + qy * qy);
  R c = 1, sn = 0;
  if (r > 0) {
    const R ir = R(1) / r;
    c = qx * ir;
    sn = qy * ir;
  }
  const R ar[3] = {qz * c, qz * sn, -r}, ai[3] = {-sn, c, 0};
  int comp = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j, ++comp) {
      R er = ar[i] * ar[j] - ai[i] * ai[j], ei = ar[i] * ai[j] + ai[i] * ar[j];
      if (i == j) {
        er *= R(0.5);
        ei *= R(0.5);
      }
      pr[comp] = er;
      pi[comp] = ei;
    }
  return true;
}

// X+ = sum e+ S, X- = sum conj(e+) S and the last component's conj(e+) S
template <typename R, typename V>
__device__ __forceinline__ void gw_contract(const V *__restrict__ srcF, int64_t nhalf, int64_t hidx, bool conj_back,
                                            const R pr[6], const R pi[6], R xp[2], R xm[2], R last_m[2]) {
  xp[0] = xp[1] = xm[0] = xm[1] = 0;
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const V f = srcF[c * nhalf + hidx];
    const R sr = f.x, si = conj_back ? -f.y : f.y;
    const R a = pr[c] * sr, b = pi[c] * si, e = pr[c] * si, g = pi[c] * sr;
    xp[0] += a - b;
    xp[1] += e + g;
    xm[0] += a + b;
    xm[1] += e - g;
    if (c == 5) {
      last_m[0] = a + b;
      last_m[1] = e - g;
    }
  }
}

// Component a of entry s is acc[a astride + s].
// a11 += w_c X+, a21 += w_s X+, a12 += w_c X-, a22 += w_s X- (INTENDED);
// REF: per component a21 <- a12 + t21, a12 <- a21 + t12, i.e. after the six
// components a12 = a12 + w_s X+ + w_c X-, a21 = a12(new) - w_c (last X-).
__device__ __forceinline__ void gw_update(double2 *__restrict__ acc, int64_t astride, int64_t s, double wc, double ws,
                                          const double xp[2], const double xm[2], const double lm[2],
                                          int ref_compat) {
  double2 a11 = acc[s], a21 = acc[astride + s], a12 = acc[2 * astride + s], a22 = acc[3 * astride + s];
  a11.x = fma(wc, xp[0], a11.x);
  a11.y = fma(wc, xp[1], a11.y);
  a22.x = fma(ws, xm[0], a22.x);
  a22.y = fma(ws, xm[1], a22.y);
  if (ref_compat) {
    a12.x = fma(wc, xm[0], fma(ws, xp[0], a12.x));
    a12.y = fma(wc, xm[1], fma(ws, xp[1], a12.y));
    a21.x = fma(-wc, lm[0], a12.x);
    a21.y = fma(-wc, lm[1], a12.y);
  } else {
    a21.x = fma(ws, xp[0], a21.x);
    a21.y = fma(ws, xp[1], a21.y);
    a12.x = fma(wc, xm[0], a12.x);
    a12.y = fma(wc, xm[1], a12.y);
  }
  acc[s] = a11;
  acc[astride + s] = a21;
  acc[2 * astride + s] = a12;
  acc[3 * astride + s] = a22;
}

// The polarisation tensor and phase rate |k| dwav of every half-spectrum k:
// e+ real and imaginary parts as float-float pairs, [12][nhalf] float2, then
// the rates, [nhalf] double (104 B per half-spectrum k).  They depend on k
// only; GB300 issues FP64 at 1/64 of the FP32 rate, and forming them took
// about half of the per-k FP64 work of a Green step.  For -k the
// polarisation vector is the conjugate (q and its azimuth change sign), so
// e+(-k) = conj e+(k) exactly: the negations are exact and the products
// keep their operands.
__device__ __forceinline__ float2 f2_pack(double x) {
  const F2 v = f2_from(x);
  return make_float2(v.h, v.l);
}

__global__ void k_gw_pol_table(int n, double dwav, float2 *__restrict__ pol, double *__restrict__ rate) {
  const int nh = n / 2 + 1;
  const int64_t nhalf = (int64_t)n * n * nh;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nhalf; h += stride) {
    const int ix = (int)(h % nh), iy = (int)((h / nh) % n), iz = (int)(h / ((int64_t)nh * n));
    const double kx = kint(ix, n), ky = kint(iy, n), kz = kint(iz, n);
    const double qq = sqrt(kx * kx + ky * ky + kz * kz);
    double pr[6], pi[6];
    if (!gw_polarisation<double>(kx, ky, kz, qq, pr, pi))
      for (int c = 0; c < 6; ++c) pr[c] = pi[c] = 0.0;
    for (int c = 0; c < 6; ++c) {
      pol[c * nhalf + h] = f2_pack(pr[c]);
      pol[(6 + c) * nhalf + h] = f2_pack(pi[c]);
    }
    rate[h] = qq * dwav;
  }
}

// Green accumulation with the polarisation formed per k in FP64 (no table):
// one thread per stored half-spectrum entry, as k_gw_accumulate_tab.  The
// accumulators hold the stored half spectrum (plus the Nyquist-row mirrors);
// the site of -k is the conjugate of its entry.
__global__ void k_gw_accumulate(const double2 *__restrict__ srcF, int n, double dwav, double tau, double dw,
                                int ref_compat, int64_t astride, double2 *__restrict__ acc) {
  const int nh = n / 2 + 1;
  const int64_t nhalf = (int64_t)n * n * nh;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nhalf; h += stride) {
    const int hx = (int)(h % nh), hy = (int)((h / nh) % n), hz = (int)(h / ((int64_t)nh * n));
    const double kx = kint(hx, n), ky = kint(hy, n), kz = kint(hz, n);
    const double qq = sqrt(kx * kx + ky * ky + kz * kz);
    double pr[6], pi[6];
    if (!gw_polarisation<double>(kx, ky, kz, qq, pr, pi)) {
      // k = 0: every e_ij is 0; the cross-wired REF updates still copy a12 into a21
      if (ref_compat) acc[astride + h] = acc[2 * astride + h];
      continue;
    }
    double sq, cq;
    sincos(qq * dwav * tau, &sq, &cq);
    double xp[2], xm[2], lm[2];
    gw_contract<double, double2>(srcF, nhalf, h, true, pr, pi, xp, xm, lm);
    gw_update(acc, astride, h, dw * cq, dw * sq, xp, xm, lm, ref_compat);
    if (hx > 0 && hx < n / 2 && (hy == n / 2 || hz == n / 2)) {
      // the mirrored site on a Nyquist y / z row: its own polarisation; the
      // same |k|, so the same phase
      const double jkx = kint(n - hx, n), jky = kint(hy == 0 ? 0 : n - hy, n), jkz = kint(hz == 0 ? 0 : n - hz, n);
      gw_polarisation<double>(jkx, jky, jkz, sqrt(jkx * jkx + jky * jky + jkz * jkz), pr, pi);
      gw_contract<double, double2>(srcF, nhalf, h, false, pr, pi, xp, xm, lm);
      gw_update(acc, astride, nhalf + gw_nyq_extra(hx, hy, hz, n), dw * cq, dw * sq, xp, xm, lm, ref_compat);
    }
  }
}

// A source spectrum value as float-float: from the float-float transform
// (float4: re hi, re lo, im hi, im lo) or from an FP64 one.
__device__ __forceinline__ void src_ff(float4 v, F2 &r, F2 &i) {
  r = {v.x, v.y};
  i = {v.z, v.w};
}
__device__ __forceinline__ void src_ff(double2 v, F2 &r, F2 &i) {
  r = f2_from(v.x);
  i = f2_from(v.y);
}

// sin and cos of x (|x| < 1e6) as float-float pairs.  x is reduced by pi/2
// in FP64 with the three-part Cody-Waite constant of axd_sincos (6 FP64
// operations), the remainder |r| <= pi/4 is split into float-float, and the
// Taylor series of sin (to r^17) and cos (to r^16) run by Horner in
// float-float on the FP32 pipes; the first omitted terms are below 1e-16.
// The coefficients are (-1)^k / n! as float-float pairs.
__device__ __forceinline__ void ff_sincos(double x, F2 &sn, F2 &cs) {
  const double kf = rint(x * AXD_TWO_OVER_PI);
  double rd = fma(-kf, AXD_CW_P1, x);
  rd = fma(-kf, AXD_CW_P2, rd);
  rd = fma(-kf, AXD_CW_P3, rd);
  const int q = (int)(long long)kf & 3;
  const F2 r = f2_from(rd);
  const F2 r2 = f2_add(f2_mul(r, r), F2{0.f, 0.f});
  constexpr float ks[9][2] = {{1.0f, 0.0f},
                              {-0.1666666716337204f, 4.967053879312289e-09f},
                              {0.008333333767950535f, -4.34617203337595e-10f},
                              {-0.00019841270113829523f, 2.725596874933456e-12f},
                              {2.7557318844628753e-06f, 3.793571224297229e-14f},
                              {-2.5052107943679403e-08f, -4.4176230446483665e-16f},
                              {1.6059044372074283e-10f, -5.352526511562726e-18f},
                              {-7.647163609812713e-13f, -1.2200710471178288e-20f},
                              {2.8114573589663704e-15f, -1.0462084739763658e-22f}};
  constexpr float kc[9][2] = {{1.0f, 0.0f},
                              {-0.5f, 0.0f},
                              {0.0416666679084301f, -1.2417634698280722e-09f},
                              {-0.0013888889225199819f, 3.3631094437103215e-11f},
                              {2.4801587642286904e-05f, -3.40699609366682e-13f},
                              {-2.755731998149713e-07f, 7.575112209051195e-15f},
                              {2.0876755879584152e-09f, 1.1082839147459852e-16f},
                              {-1.147074536050896e-11f, -2.372207689231238e-19f},
                              {4.7794772561329454e-14f, 7.62544404448643e-22f}};
  F2 ps = {ks[8][0], ks[8][1]}, pc = {kc[8][0], kc[8][1]};
#pragma unroll
  for (int k = 7; k >= 0; --k) {
    ps = f2_add(f2_mul(ps, r2), F2{ks[k][0], ks[k][1]});
    pc = f2_add(f2_mul(pc, r2), F2{kc[k][0], kc[k][1]});
  }
  const F2 s0 = f2_add(f2_mul(ps, r), F2{0.f, 0.f});  // sin r
  const F2 c0 = pc;                                   // cos r
  // x = q pi / 2 + r
  sn = (q & 1) ? c0 : s0;
  cs = (q & 1) ? s0 : c0;
  if (q == 2 || q == 3) sn = f2_neg(sn);
  if (q == 1 || q == 2) cs = f2_neg(cs);
}

// acc += w x for float-float complex values (float4: re hi, re lo, im hi, im lo)
__device__ __forceinline__ void ff_axpy(float4 &a, F2 w, F2 xr, F2 xi) {
  const F2 r = f2_add(F2{a.x, a.y}, f2_mul(w, xr)), i = f2_add(F2{a.z, a.w}, f2_mul(w, xi));
  a = make_float4(r.h, r.l, i.h, i.l);
}

// Green accumulation with the polarisation table: the contraction
// X+- = sum e+- S runs in float-float on the FP32 pipes (four f2_dot2 per
// component), the phase sin / cos and the accumulator updates in FP64.
//
// ACCFF: the accumulators are float-float (float4) as in the FP32-mixed path,
// the phase sin / cos are float-float (ff_sincos) and the updates run in
// float-float, so a k-site issues about ten FP64 operations.
// The contraction of one k-site from float-float polarisation parts er, ei
// and the stored source spectrum entry h: p = X+, m = X-, l = the last
// component's X-.  neg_si: the stored entry is S(k)'s conjugate (k in the
// stored half), so its imaginary part changes sign.
template <typename SRC>
__device__ __forceinline__ void ff_contract(const SRC *__restrict__ srcF, int64_t nhalf, int64_t h, const F2 er[6],
                                            const F2 ei[6], bool neg_si, F2 &p0, F2 &p1, F2 &m0, F2 &m1, F2 &l0,
                                            F2 &l1) {
  p0 = p1 = m0 = m1 = l0 = l1 = F2{0.f, 0.f};
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    F2 sr, si;
    src_ff(srcF[c * nhalf + h], sr, si);
    if (neg_si) si = f2_neg(si);
    // a = er sr, b = ei si, e = er si, g = ei sr: X+ += (a - b, e + g), X- += (a + b, e - g)
    const F2 t0 = f2_dot2(er[c], sr, ei[c], si, -1.f), t1 = f2_dot2(er[c], si, ei[c], sr, 1.f);
    const F2 t2 = f2_dot2(er[c], sr, ei[c], si, 1.f), t3 = f2_dot2(er[c], si, ei[c], sr, -1.f);
    p0 = f2_add(p0, t0);
    p1 = f2_add(p1, t1);
    m0 = f2_add(m0, t2);
    m1 = f2_add(m1, t3);
    if (c == 5) {
      l0 = t2;
      l1 = t3;
    }
  }
}

// float-float accumulators at site s: a11 += wc X+, a22 += ws X-, and a12,
// a21 as in gw_update
__device__ __forceinline__ void ff_update(float4 *__restrict__ acc, int64_t astride, int64_t s, F2 wc, F2 ws, F2 p0,
                                          F2 p1, F2 m0, F2 m1, F2 l0, F2 l1, int ref_compat) {
  float4 a11 = acc[s], a21 = acc[astride + s], a12 = acc[2 * astride + s], a22 = acc[3 * astride + s];
  ff_axpy(a11, wc, p0, p1);
  ff_axpy(a22, ws, m0, m1);
  if (ref_compat) {
    // a12 += ws X+ + wc X-, then a21 = a12 - wc (last X-)
    ff_axpy(a12, ws, p0, p1);
    ff_axpy(a12, wc, m0, m1);
    a21 = a12;
    ff_axpy(a21, f2_neg(wc), l0, l1);
  } else {
    ff_axpy(a21, ws, p0, p1);
    ff_axpy(a12, wc, m0, m1);
  }
  acc[s] = a11;
  acc[astride + s] = a21;
  acc[2 * astride + s] = a12;
  acc[3 * astride + s] = a22;
}


// Green accumulation with the polarisation table: the contraction
// X+- = sum e+- S runs in float-float on the FP32 pipes (four f2_dot2 per
// component), the phase sin / cos and the accumulator updates in FP64.
//
// ACCFF: the accumulators are float-float (float4) as in the FP32-mixed path,
// the phase sin / cos are float-float (ff_sincos) and the updates run in
// float-float, so a k-site issues about ten FP64 operations.
//
// One thread per stored half-spectrum entry h = (hx, hy, hz).  The
// accumulators hold that half spectrum only: for 0 < hx < n/2 the site of -k
// in the other half has S(-k) = conj S(k) (real sources) and e+(-k) =
// conj e+(k), so X+-(-k) = conj X+-(k) and its accumulators stay the exact
// conjugates (the negations are exact, so they are the bits an update of
// its own would give).  When hy or hz is the Nyquist index n/2 the mirrored
// site's wave vector index maps to itself (kint(n/2) = -n/2) and is not -k:
// its polarisation is formed directly and it has entries of its own
// (gw_nyq_extra).  |k|, and so the phase, is the same at both sites.
template <typename SRC, bool ACCFF>
__global__ void __launch_bounds__(256, 3) k_gw_accumulate_tab(const SRC *__restrict__ srcF, const float2 *__restrict__ pol,
                                    const double *__restrict__ rates, int n, double dwav, double tau, double dw,
                                    float dw_hi, float dw_lo, int ref_compat, int64_t astride,
                                    void *__restrict__ accp) {
  const int nh = n / 2 + 1;
  const int64_t nhalf = (int64_t)n * n * nh;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nhalf; h += stride) {
    const int hx = (int)(h % nh), hy = (int)((h / nh) % n), hz = (int)(h / ((int64_t)nh * n));
    const double rate = rates[h];
    if (!(rate > 0)) {
      // k = 0 (h = 0): every e_ij is 0; the cross-wired REF updates still
      // copy a12 into a21
      if (ref_compat) {
        if constexpr (ACCFF) {
          float4 *acc = static_cast<float4 *>(accp);
          acc[astride + h] = acc[2 * astride + h];
        } else {
          double2 *acc = static_cast<double2 *>(accp);
          acc[astride + h] = acc[2 * astride + h];
        }
      }
      continue;
    }
    F2 er[6], ei[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const float2 a = pol[c * nhalf + h], b = pol[(6 + c) * nhalf + h];
      er[c] = {a.x, a.y};
      ei[c] = {b.x, b.y};
    }
    F2 p0, p1, m0, m1, l0, l1;
    ff_contract(srcF, nhalf, h, er, ei, true, p0, p1, m0, m1, l0, l1);
    // the mirrored site's own contraction on a Nyquist y or z row
    const bool nyq = hx > 0 && hx < n / 2 && (hy == n / 2 || hz == n / 2);
    F2 q0, q1, r0, r1, v0, v1;
    if (nyq) {
      const int jx = n - hx, jy = hy == 0 ? 0 : n - hy, jz = hz == 0 ? 0 : n - hz;
      const double kx = kint(jx, n), ky = kint(jy, n), kz = kint(jz, n);
      const double qq = sqrt(kx * kx + ky * ky + kz * kz);
      double pr[6], pi[6];
      if (!gw_polarisation<double>(kx, ky, kz, qq, pr, pi))
        for (int c = 0; c < 6; ++c) pr[c] = pi[c] = 0.0;
      for (int c = 0; c < 6; ++c) {
        er[c] = f2_from(pr[c]);
        ei[c] = f2_from(pi[c]);
      }
      ff_contract(srcF, nhalf, h, er, ei, false, q0, q1, r0, r1, v0, v1);
    }
    const int64_t e2 = nyq ? nhalf + gw_nyq_extra(hx, hy, hz, n) : -1;
    if constexpr (ACCFF) {
      F2 sq, cq;
      ff_sincos(rate * tau, sq, cq);
      const F2 dwf = {dw_hi, dw_lo};
      const F2 wc = f2_add(f2_mul(dwf, cq), F2{0.f, 0.f}), ws = f2_add(f2_mul(dwf, sq), F2{0.f, 0.f});
      float4 *acc = static_cast<float4 *>(accp);
      ff_update(acc, astride, h, wc, ws, p0, p1, m0, m1, l0, l1, ref_compat);
      if (nyq) ff_update(acc, astride, e2, wc, ws, q0, q1, r0, r1, v0, v1, ref_compat);
    } else {
      double sq, cq;
      sincos(rate * tau, &sq, &cq);
      double2 *acc = static_cast<double2 *>(accp);
      {
        const double xp[2] = {f2_to(p0), f2_to(p1)}, xm[2] = {f2_to(m0), f2_to(m1)}, lm[2] = {f2_to(l0), f2_to(l1)};
        gw_update(acc, astride, h, dw * cq, dw * sq, xp, xm, lm, ref_compat);
      }
      if (nyq) {
        const double xp[2] = {f2_to(q0), f2_to(q1)}, xm[2] = {f2_to(r0), f2_to(r1)}, lm[2] = {f2_to(v0), f2_to(v1)};
        gw_update(acc, astride, e2, dw * cq, dw * sq, xp, xm, lm, ref_compat);
      }
    }
  }
}

// (hi, lo) += x: TwoSum of hi and x, the error folded into lo, then
// renormalised (Fast2Sum); hi + lo carries about 48 significant bits
__device__ __forceinline__ void ff_add(float &hi, float &lo, float x) {
  const float s = hi + x;
  const float bb = s - hi;
  const float err = (hi - (s - bb)) + (x - bb);
  const float l = lo + err;
  hi = s + l;
  lo = l - (hi - s);
}

// 2 pi = kC1 + kC2 + kC3 with kC1, kC2 of 8 significant bits (Cody-Waite), so
// m kC1 and m kC2 are exact for |m| < 2^16, i.e. phases below 4e5 rad
constexpr float kC1 = 6.28125f;
constexpr float kC2 = 0.0019378662109375f;
constexpr float kC3 = -2.559031372584286e-06f;
constexpr float kInv2Pi = 0.15915493667125702f;

// |k| dk tau reduced to about [-pi, pi] (absolute error ~3e-7): the product
// of the float-float omega and tau keeps its rounding error exactly (fmaf)
__device__ __forceinline__ float gw_phase(float2 om, float th, float tl) {
  const float ph = om.x * th;
  const float pl = fmaf(om.x, th, -ph) + fmaf(om.x, tl, om.y * th);
  const float m = rintf(ph * kInv2Pi);
  float r = fmaf(-m, kC1, ph);
  r = fmaf(-m, kC2, r);
  r = r + pl;
  return fmaf(-m, kC3, r);
}

// float-float accumulators at site s from FP32 X+, X- and the weights
__device__ __forceinline__ void f32_update(float4 *__restrict__ acc, int64_t astride, int64_t s, float wc, float ws,
                                           const float xp[2], const float xm[2], const float lm[2], int ref_compat) {
  float4 a11 = acc[s], a21 = acc[astride + s], a12 = acc[2 * astride + s], a22 = acc[3 * astride + s];
  ff_add(a11.x, a11.y, wc * xp[0]);
  ff_add(a11.z, a11.w, wc * xp[1]);
  ff_add(a22.x, a22.y, ws * xm[0]);
  ff_add(a22.z, a22.w, ws * xm[1]);
  if (ref_compat) {
    ff_add(a12.x, a12.y, fmaf(wc, xm[0], ws * xp[0]));
    ff_add(a12.z, a12.w, fmaf(wc, xm[1], ws * xp[1]));
    a21 = a12;
    ff_add(a21.x, a21.y, -wc * lm[0]);
    ff_add(a21.z, a21.w, -wc * lm[1]);
  } else {
    ff_add(a21.x, a21.y, ws * xp[0]);
    ff_add(a21.z, a21.w, ws * xp[1]);
    ff_add(a12.x, a12.y, wc * xm[0]);
    ff_add(a12.z, a12.w, wc * xm[1]);
  }
  acc[s] = a11;
  acc[astride + s] = a21;
  acc[2 * astride + s] = a12;
  acc[3 * astride + s] = a22;
}

// FP32-mixed Green accumulation: FP32 sources, polarisation, phase and
// contraction; the accumulators are float-float pairs (re hi, re lo, im hi,
// im lo), so no FP64 instruction is issued per k-site.  One thread per stored
// half-spectrum entry; the accumulators hold that half spectrum and the
// Nyquist-row mirrors, as in k_gw_accumulate_tab.  The source spectra have
// kx rows of sp entries (the own transforms pad them), the accumulators and
// phase rates rows of n/2 + 1.
__global__ void __launch_bounds__(256, 4) k_gw_accumulate_f32(const float2 *__restrict__ srcF, int sp,
                                                              const float2 *__restrict__ om, int n, float th,
                                                              float tl, float dw, int ref_compat, int64_t astride,
                                                              float4 *__restrict__ acc) {
  const int nh = n / 2 + 1;
  const int64_t nhalf = (int64_t)n * n * nh, nspec = (int64_t)n * n * sp;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nhalf; h += stride) {
    const int hx = (int)(h % nh), hy = (int)((h / nh) % n), hz = (int)(h / ((int64_t)nh * n));
    const int64_t hs = (h / nh) * sp + hx;  // the entry in the source spectra
    const float kx = (float)kint(hx, n), ky = (float)kint(hy, n), kz = (float)kint(hz, n);
    const float qq = sqrtf(kx * kx + ky * ky + kz * kz);
    float pr[6], pi[6];
    if (!gw_polarisation<float>(kx, ky, kz, qq, pr, pi)) {
      if (ref_compat) acc[astride + h] = acc[2 * astride + h];  // k = 0 (h = 0)
      continue;
    }
    float sq, cq;
    sincosf(gw_phase(om[h], th, tl), &sq, &cq);
    const float wc = dw * cq, ws = dw * sq;
    float xp[2], xm[2], lm[2];
    gw_contract<float, float2>(srcF, nspec, hs, true, pr, pi, xp, xm, lm);
    f32_update(acc, astride, h, wc, ws, xp, xm, lm, ref_compat);
    if (hx > 0 && hx < n / 2 && (hy == n / 2 || hz == n / 2)) {
      const int jx = n - hx, jy = hy == 0 ? 0 : n - hy, jz = hz == 0 ? 0 : n - hz;
      const float jkx = (float)kint(jx, n), jky = (float)kint(jy, n), jkz = (float)kint(jz, n);
      gw_polarisation<float>(jkx, jky, jkz, sqrtf(jkx * jkx + jky * jky + jkz * jkz), pr, pi);
      gw_contract<float, float2>(srcF, nspec, hs, false, pr, pi, xp, xm, lm);
      f32_update(acc, astride, nhalf + gw_nyq_extra(hx, hy, hz, n), wc, ws, xp, xm, lm, ref_compat);
    }
  }
}

// ---------------- shell histograms ----------------
constexpr int kMaxBins = 256;

// |A|^2 of one accumulator entry: FP64, or float-float (FP32-mixed)
__device__ __forceinline__ double acc_norm2(double2 z) { return z.x * z.x + z.y * z.y; }
__device__ __forceinline__ double acc_norm2(float4 z) {
  const double re = (double)z.x + (double)z.y, im = (double)z.z + (double)z.w;
  return re * re + im * im;
}

// Green accumulators -> numer / denom per bin (bin of |k|^2 from the table).
// A stored entry with 0 < hx < n/2 stands for k and -k (the same |k|): its
// |A|^2 counts twice, or once plus the Nyquist-row mirror's own entry.
template <typename A>
__global__ void k_gw_bin_green(const A *__restrict__ acc, int n, int64_t astride, const int16_t *__restrict__ tab,
                               int nb, double *__restrict__ numer, double *__restrict__ denom) {
  __shared__ double sn[kMaxBins], sd[kMaxBins];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) sn[b] = sd[b] = 0.0;
  __syncthreads();
  const int nh = n / 2 + 1;
  const int64_t nhalf = (int64_t)n * n * nh;
  BinRun run;
  for (int64_t h0 = run_start(); h0 < nhalf; h0 += run_stride()) {
    for (int64_t h = h0; h < h0 + kRun && h < nhalf; ++h) {
      const int hx = (int)(h % nh), hy = (int)((h / nh) % n), hz = (int)(h / ((int64_t)nh * n));
      const int kx = kint(hx, n), ky = kint(hy, n), kz = kint(hz, n);
      const int b = tab[kx * kx + ky * ky + kz * kz];
      const bool mirror = hx > 0 && hx < n / 2;
      double v = 0.0;
      if (b >= 0) {
        double v1 = 0.0;
#pragma unroll
        for (int a = 0; a < 4; ++a) v1 += acc_norm2(acc[a * astride + h]);
        v = v1;
        if (mirror) {
          if (hy == n / 2 || hz == n / 2) {
            const int64_t e = nhalf + gw_nyq_extra(hx, hy, hz, n);
            double v2 = 0.0;
#pragma unroll
            for (int a = 0; a < 4; ++a) v2 += acc_norm2(acc[a * astride + e]);
            v += v2;
          } else {
            v += v1;
          }
        }
      }
      run.add(sn, sd, b, v, mirror ? 2u : 1u);
    }
  }
  run.flush(sn, sd);
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    if (sd[b] != 0.0) {
      atomicAdd(&numer[b], sn[b]);
      atomicAdd(&denom[b], sd[b]);
    }
  }
}

// u_ij: one of the 12 real fields (f < 6: tau u_f; else u_c + tau u'_c,
// c = f - 6), scaled by dx^3 at use; the cuFFT path transforms them one at
// a time through one real buffer of n^3
template <typename R>
__global__ void k_uij_prepare(const R *__restrict__ u, const R *__restrict__ ud, const R *__restrict__ cu,
                              int64_t n3, double tau, int f, R *__restrict__ w) {
  const int c = f < 6 ? f : f - 6;
  const R *uc = u + c * n3, *udc = ud + c * n3, *cuc = cu ? cu + c * n3 : nullptr;
  const R t = (R)tau;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    // in the precision of the spectrum: FP32 for FP32-mixed (the Kahan
    // compensation is below FP32 resolution of u; it is applied all the same)
    R uv = uc[s];
    if (cuc) uv -= cuc[s];
    w[s] = f < 6 ? t * uv : uv + t * udc[s];
  }
}

// TT power of a complex symmetric 3x3 (components 11,21,22,31,32,33)
// |Lambda U|^2 of the TT projection; R = float for FP32 spectra (the shell
// sums stay FP64)
template <typename R>
__device__ R tt_power(const R Ur[6], const R Ui[6], const R kh[3]) {
  const int idx[3][3] = {{0, 1, 3}, {1, 2, 4}, {3, 4, 5}};
  R P[3][3], Tr[3][3], Ti[3][3], Rr[3][3], Ri[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) P[a][b] = (a == b ? R(1) : R(0)) - kh[a] * kh[b];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      R sr = 0, si = 0;
      for (int c = 0; c < 3; ++c) {
        sr += P[a][c] * Ur[idx[c][b]];
        si += P[a][c] * Ui[idx[c][b]];
      }
      Tr[a][b] = sr;
      Ti[a][b] = si;
    }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      R sr = 0, si = 0;
      for (int c = 0; c < 3; ++c) {
        sr += Tr[a][c] * P[c][b];
        si += Ti[a][c] * P[c][b];
      }
      Rr[a][b] = sr;
      Ri[a][b] = si;
    }
  const R trr = Rr[0][0] + Rr[1][1] + Rr[2][2], tri = Ri[0][0] + Ri[1][1] + Ri[2][2];
  R s = 0;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      const R vr = Rr[a][b] - R(0.5) * P[a][b] * trr, vi = Ri[a][b] - R(0.5) * P[a][b] * tri;
      s += vr * vr + vi * vi;
    }
  return s;
}

// F: the twelve half spectra, kx rows of sp entries
template <typename CV>
__global__ void k_uij_bin(const CV *__restrict__ F, int sp, int n, double dwav, double dv,
                          const int16_t *__restrict__ tab, int nb, double *__restrict__ numer,
                          double *__restrict__ denom) {
  __shared__ double sn[kMaxBins], sd[kMaxBins];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) sn[b] = sd[b] = 0.0;
  __syncthreads();
  const int nh = n / 2 + 1;
  const int64_t nhalf = (int64_t)n * n * nh, nspec = (int64_t)n * n * sp;
  const double dv2 = dv * dv, dwav2 = dwav * dwav;
  BinRun run;
  for (int64_t h0 = run_start(); h0 < nhalf; h0 += run_stride()) {
    for (int64_t h = h0; h < h0 + kRun && h < nhalf; ++h) {
      const int ix = (int)(h % nh), iy = (int)((h / nh) % n), iz = (int)(h / ((int64_t)nh * n));
      const int kx = kint(ix, n), ky = kint(iy, n), kz = kint(iz, n);
      const int k2 = kx * kx + ky * ky + kz * kz;
      const int b = tab[k2];
      double v = 0.0;
      unsigned wgt = 0;
      if (b >= 0) {
        // the TT projection in the precision of the spectrum (FP32 for FP32-mixed)
        using R = decltype(F[0].x);
        const R iq = R(1) / sqrt((R)k2);
        const R kh[3] = {(R)kx * iq, (R)ky * iq, (R)kz * iq};
        R Ur[6], Ui[6], Dr[6], Di[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const int64_t hs = (h / nh) * sp + ix;
          const CV a = F[c * nspec + hs], d = F[(6 + c) * nspec + hs];
          Ur[c] = a.x;
          Ui[c] = a.y;
          Dr[c] = d.x;
          Di[c] = d.y;
        }
        wgt = (ix == 0 || 2 * ix == n) ? 1u : 2u;  // Hermitian partner of the half spectrum
        if constexpr (sizeof(R) == 4) {
          // FP32 spectra: the entry's energy in FP32, one conversion to the
          // FP64 shell sums (a handful of FP64 operations fewer per entry)
          const float e = tt_power<R>(Dr, Di, kh) + (float)k2 * (float)dwav2 * tt_power<R>(Ur, Ui, kh);
          v = (double)e * (wgt * dv2);
        } else {
          const double e0 = (double)tt_power<R>(Dr, Di, kh) * dv2, e1 = (double)tt_power<R>(Ur, Ui, kh) * dv2;
          v = wgt * (e0 + (double)k2 * dwav2 * e1);
        }
      }
      run.add(sn, sd, b, v, wgt);
    }
  }
  run.flush(sn, sd);
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    if (sd[b] != 0.0) {
      atomicAdd(&numer[b], sn[b]);
      atomicAdd(&denom[b], sd[b]);
    }
  }
}

// grav_waves.f90:265-267 on an n^3 grid of spacing dspa (the GW grid of
// init_grav for Green's mode, the lattice for u_ij)
double gw_fact(const axg_params &p, int n, double dspa) {
  const double dwav = kRefTwoPi / dspa / n;
  const double dv_wav = std::pow(dwav / kRefTwoPi, 3);
  const double tc = p.tau_cr;
  const double tc6 = tc * tc * tc * tc * tc * tc;
  const double a4 = p.a_now * p.a_now * p.a_now * p.a_now;
  return 1 / tc6 / (kBigHInMstar * kBigHInMstar) / a4 / 3 / (kRefTwoPi * kRefTwoPi) * dv_wav;
}

int grid_for(int64_t count) {
  int64_t b = (count + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

int ensure_uij_fft(axg_ctx *ctx) {
  if (ctx->plan_u_ok || ctx->ubuf) return AXG_OK;
  const int n = (int)ctx->n;
  const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
  const size_t rs = fp32 ? 4 : 8;
  const int64_t nhalf = (int64_t)n * n * (n / 2 + 1);
  // our own transforms (power-of-two N up to 512; AXG_FFT_FF=0: cuFFT) form
  // the twelve fields in their row pass: only the 12 half spectra are stored
  ctx->uij_own_fft = axg_ff_use(n);
  ctx->u_pitch = n / 2 + 1;
  if (ctx->uij_own_fft) {
    if (fp32) ctx->u_pitch = axg_f32_spec_pitch(n);
    const size_t bytes = (size_t)12 * n * n * ctx->u_pitch * 2 * rs;
    AXG_TRY(axg_alloc(ctx, &ctx->ubuf, bytes, "u_ij spectra"));
    AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->ubuf, 0, bytes, ctx->stream));  // the padding columns
    return AXG_OK;
  }
  // one real field of N^3 followed by the complex output 12 x nhalf; the
  // twelve fields go through the real buffer one at a time (at 1024^3 a
  // batch of twelve would need 48 GiB of real input and cuFFT rejects it)
  AXG_TRY(axg_alloc(ctx, &ctx->ubuf, (size_t)ctx->n3 * rs + (size_t)12 * nhalf * 2 * rs, "u_ij FFT"));
  AXG_CUFFT_TRY(ctx, cufftPlan3d(&ctx->plan_u, n, n, n, fp32 ? CUFFT_R2C : CUFFT_D2Z));
  AXG_CUFFT_TRY(ctx, cufftSetStream(ctx->plan_u, ctx->stream));
  ctx->plan_u_ok = true;
  return AXG_OK;
}

}  // namespace

int axg_gw_init(axg_ctx *ctx) {
  // init_grav (grav_waves.f90:37-45): everything of Green's mode lives on the
  // GW grid, the lattice coarse-grained by deg = 2^degrade_spec
  const int deg = 1 << ctx->p.degrade_spec;
  const int n = (int)ctx->n / deg;
  ctx->gw_n = n;
  ctx->gw_dspa = ctx->p.dspa * deg;
  const int64_t n3 = (int64_t)n * n * n;
  const int64_t nhalf = (int64_t)n * n * (n / 2 + 1);
  const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
  const size_t rs = fp32 ? 4 : 8;
  // our own transforms for power-of-two N up to 512 (AXG_FFT_FF=0: cuFFT);
  // on the full lattice they form the sources inside their row pass, so the
  // real sources are never stored.  Degraded sources are stored (n^3 is
  // 1/8 of the lattice or less) and transformed by the float-float D2Z
  // (FP64 paths) or cuFFT (FP32-mixed).
  ctx->gw_own_fft = deg == 1 && axg_ff_use(n);
  ctx->gw_ff_real = deg > 1 && !fp32 && axg_ff_use(n);
  ctx->acc_stride = axg_gw_acc_entries(n);
  AXG_TRY(axg_alloc(ctx, (void **)&ctx->acc, (size_t)ctx->acc_stride * 64, "GW accumulators"));
  if (!ctx->gw_own_fft) AXG_TRY(axg_alloc(ctx, (void **)&ctx->gsrc, (size_t)n3 * 6 * rs, "GW sources"));
  ctx->gsrc_pitch = fp32 && ctx->gw_own_fft ? axg_f32_spec_pitch(n) : n / 2 + 1;
  {
    const size_t bytes = (size_t)n * n * ctx->gsrc_pitch * 6 * 2 * rs;
    AXG_TRY(axg_alloc(ctx, (void **)&ctx->gsrcF, bytes, "GW source spectra"));
    AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->gsrcF, 0, bytes, ctx->stream));  // the padding columns
  }
  AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->acc, 0, (size_t)ctx->acc_stride * 64, ctx->stream));
  if (fp32) {
    AXG_TRY(axg_alloc(ctx, (void **)&ctx->gw_omega, (size_t)nhalf * 8, "GW phase rates"));
    AXG_LAUNCH(ctx, "gw_omega", k_gw_omega, grid_for(nhalf), 256, 0, n, kRefTwoPi / ctx->gw_dspa / n, ctx->gw_omega);
  } else {
    // The FP64 polarisation table (13 doubles per half-spectrum k) when it
    // takes at most an eighth of the device memory (512^3: 7 GB); otherwise
    // the accumulation forms the polarisation per step.
    // AXG_GW_POL_TABLE=0 forces the per-step form (tests compare the two).
    size_t freeb = 0, total = 0;
    cudaMemGetInfo(&freeb, &total);
    const size_t tb = (size_t)nhalf * 13 * 8;
    const char *env = std::getenv("AXG_GW_POL_TABLE");
    const bool want = !(env && env[0] == '0');
    if (want && tb <= total / 8) {
      AXG_TRY(axg_alloc(ctx, (void **)&ctx->gw_pol, tb, "GW polarisation table"));
      AXG_LAUNCH(ctx, "gw_pol_table", k_gw_pol_table, grid_for(nhalf), 256, 0, n, kRefTwoPi / ctx->gw_dspa / n,
                 reinterpret_cast<float2 *>(ctx->gw_pol), ctx->gw_pol + 12 * nhalf);
    }
  }
  // float-float accumulators where the transforms are float-float too: the
  // whole Green accumulation then stays on the FP32 pipes but for the phase
  // reduction
  ctx->acc_ff = fp32 || (ctx->gw_pol != nullptr && (ctx->gw_own_fft || ctx->gw_ff_real));
  if (!ctx->gw_own_fft && !ctx->gw_ff_real) {
    int dims[3] = {n, n, n};
    AXG_CUFFT_TRY(ctx, cufftPlanMany(&ctx->plan_gsrc, 3, dims, nullptr, 1, (int)n3, nullptr, 1,
                                     (int)nhalf, fp32 ? CUFFT_R2C : CUFFT_D2Z, 6));
    ctx->plan_gsrc_ok = true;
    AXG_CUFFT_TRY(ctx, cufftSetStream(ctx->plan_gsrc, ctx->stream));
  }
  return AXG_OK;
}

// grav_wave_integration (grav_waves.f90:193-255) on the current phi
int axg_gw_integration(axg_ctx *ctx, double tau, double dtau) {
  if (!ctx->acc) return axg_set_error(ctx, AXG_ERR_STATE, "gw_mode is not GREEN");
  // the GW grid (n = ngrid / deg, spacing dspa deg): grav_waves.f90:37-45
  const int n = ctx->gw_n, nl = (int)ctx->n, deg = nl / n;
  const int64_t n3 = (int64_t)n * n * n;
  // data1_to_arr_dphi: d = 2 dx (grav_waves.f90:337); degraded: deg^3 dx 2 (:383)
  const double d = deg == 1 ? ctx->p.dspa * 2 : (double)(deg * deg * deg) * ctx->p.dspa * 2;
  const double dv = ctx->gw_dspa * ctx->gw_dspa * ctx->gw_dspa;  // dv_spa_grav
  const double dw = tau * dtau * dv * (ctx->p.sigma_cr * ctx->p.sigma_cr);
  const double dwav = kRefTwoPi / ctx->gw_dspa / n;  // dwav_grav
  const int ref = ctx->p.compat == AXG_COMPAT_REF ? 1 : 0;
  const int64_t nhalf = (int64_t)n * n * (n / 2 + 1);
  if (ctx->p.precision == AXG_PREC_FP32_MIXED) {
    if (deg > 1) {
      float *src = (float *)ctx->gsrc;
      AXG_LAUNCH(ctx, "gw_source_degrade_fp32", k_gw_source_degrade_f32, grid_for(n3), 256, 0,
                 (const float2 *)ctx->phi[ctx->cur], nl, deg, (float)(2.0 / (d * d)), src);
      AXG_CUFFT_TRY(ctx, cufftExecR2C(ctx->plan_gsrc, src, (cufftComplex *)ctx->gsrcF));
    } else if (ctx->gw_own_fft) {
      AXG_TRY(axg_gw_source_r2c_f32(ctx, (const float2 *)ctx->phi[ctx->cur], (float2 *)ctx->gsrcF, n,
                                    (float)(2.0 / (d * d))));
    } else {
      float *src = (float *)ctx->gsrc;
      AXG_LAUNCH(ctx, "gw_source_fp32", k_gw_source_f32, grid_for(n3), 256, 0,
                 (const float2 *)ctx->phi[ctx->cur], n, (float)(2.0 / (d * d)), src);
      AXG_CUFFT_TRY(ctx, cufftExecR2C(ctx->plan_gsrc, src, (cufftComplex *)ctx->gsrcF));
    }
    const float th = (float)tau, tl = (float)(tau - (double)th);
    AXG_LAUNCH(ctx, "gw_accumulate_fp32", k_gw_accumulate_f32, grid_for(nhalf), 256, 0,
               (const float2 *)ctx->gsrcF, ctx->gsrc_pitch, ctx->gw_omega, n, th, tl, (float)dw, ref,
               ctx->acc_stride, (float4 *)ctx->acc);
    return AXG_OK;
  }
  int ex;
  const int pow2 = std::frexp(d, &ex) == 0.5;
  // the six source transforms: float-float for power-of-two N (FP64
  // accuracy on the FP32 pipes, the sources formed in the row pass; kept as
  // float-float pairs when the float-float contraction reads them), else
  // the FP64 sources and cuFFT
  const bool ff = ctx->gw_own_fft || ctx->gw_ff_real, tab = ctx->gw_pol != nullptr;
  if (deg > 1) {
    AXG_LAUNCH(ctx, "gw_source_degrade_fp64", k_gw_source_degrade, grid_for(n3), 256, 0,
               (const double2 *)ctx->phi[ctx->cur], nl, deg, d, 1.0 / d, pow2, ctx->gsrc);
    if (ctx->gw_ff_real)
      AXG_TRY(axg_ff_d2z(ctx, ctx->gsrc, ctx->gsrcF, n, 6, tab));
    else
      AXG_CUFFT_TRY(ctx, cufftExecD2Z(ctx->plan_gsrc, ctx->gsrc, (cufftDoubleComplex *)ctx->gsrcF));
  } else if (ctx->gw_own_fft) {
    AXG_TRY(axg_gw_source_d2z_ff(ctx, (const double2 *)ctx->phi[ctx->cur], d, 1.0 / d, pow2, ctx->gsrcF, n, tab));
  } else {
    AXG_LAUNCH(ctx, "gw_source_fp64", k_gw_source, grid_for(n3), 256, 0, (const double2 *)ctx->phi[ctx->cur], n,
               d, 1.0 / d, pow2, ctx->gsrc);
    AXG_CUFFT_TRY(ctx, cufftExecD2Z(ctx->plan_gsrc, ctx->gsrc, (cufftDoubleComplex *)ctx->gsrcF));
  }
  const float dw_hi = (float)dw, dw_lo = (float)(dw - (double)dw_hi);
  const float2 *pol = reinterpret_cast<const float2 *>(ctx->gw_pol);
  const double *rates = ctx->gw_pol + 12 * nhalf;
  if (tab && ff && ctx->acc_ff)
    AXG_LAUNCH(ctx, "gw_accumulate", (k_gw_accumulate_tab<float4, true>), grid_for(nhalf), 256, 0,
               reinterpret_cast<const float4 *>(ctx->gsrcF), pol, rates, n, dwav, tau, dw, dw_hi, dw_lo, ref,
               ctx->acc_stride, (void *)ctx->acc);
  else if (tab && ff)
    AXG_LAUNCH(ctx, "gw_accumulate", (k_gw_accumulate_tab<float4, false>), grid_for(nhalf), 256, 0,
               reinterpret_cast<const float4 *>(ctx->gsrcF), pol, rates, n, dwav, tau, dw, dw_hi, dw_lo, ref,
               ctx->acc_stride, (void *)ctx->acc);
  else if (tab && ctx->acc_ff)
    AXG_LAUNCH(ctx, "gw_accumulate", (k_gw_accumulate_tab<double2, true>), grid_for(nhalf), 256, 0,
               (const double2 *)ctx->gsrcF, pol, rates, n, dwav, tau, dw, dw_hi, dw_lo, ref,
               ctx->acc_stride, (void *)ctx->acc);
  else if (tab)
    AXG_LAUNCH(ctx, "gw_accumulate", (k_gw_accumulate_tab<double2, false>), grid_for(nhalf), 256, 0,
               (const double2 *)ctx->gsrcF, pol, rates, n, dwav, tau, dw, dw_hi, dw_lo, ref,
               ctx->acc_stride, (void *)ctx->acc);
  else
    AXG_LAUNCH(ctx, "gw_accumulate", k_gw_accumulate, grid_for(nhalf), 256, 0, ctx->gsrcF, n, dwav, tau, dw, ref,
               ctx->acc_stride, ctx->acc);
  return AXG_OK;
}

int axg_gw_spec(axg_ctx *ctx, double tau, int log_bins, double *wave, double *power, double *numer,
                double *denom) {
  // Green's mode bins on its GW grid (grav_waves.f90:37-45, coarse when
  // degrade_spec > 0); u_ij on the lattice
  const bool green = ctx->p.gw_mode == AXG_GW_GREEN;
  const int n = green ? ctx->gw_n : (int)ctx->n;
  const double dspa = green ? ctx->gw_dspa : ctx->p.dspa;
  const int nb = log_bins ? ctx->p.gw_log_bins : ctx->p.num_bin_grav;
  if (nb < 1 || nb > kMaxBins) return axg_set_error(ctx, AXG_ERR_ARG, "GW bin count out of range (1..256)");
  const double dwav = kRefTwoPi / dspa / n;
  // bins: linear (grav_waves.f90:62-71) or log on [2 pi/(N dx), pi/dx]
  std::vector<double> edges(nb + 1);
  const double qmax = kRefPi / dspa;
  const double dq = qmax / nb;
  if (log_bins) {
    const double kmin = kRefTwoPi / dspa / n;
    for (int k = 0; k <= nb; ++k) edges[k] = kmin * std::pow(qmax / kmin, (double)k / nb);
  } else {
    edges[0] = 0.0;
    for (int k = 1; k <= nb; ++k) edges[k] = edges[k - 1] + dq;
  }
  // device scratch: numer[nb] denom[nb]
  if ((size_t)(2 * nb) > ctx->red_cap) return axg_set_error(ctx, AXG_ERR_ARG, "too many bins");
  double *d_num = ctx->d_red, *d_den = ctx->d_red + nb;
  AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_red, 0, sizeof(double) * 2 * nb, ctx->stream));
  const int16_t *tab = nullptr;
  AXG_TRY(axg_bin_table(ctx, AXG_BIN_GW, n, dwav, dq, nb, log_bins, edges.data(), &tab));
  if (ctx->p.gw_mode == AXG_GW_GREEN) {
    if (ctx->acc_ff)
      AXG_LAUNCH(ctx, "gw_bin_green", k_gw_bin_green<float4>, 152 * 4, 256, 0, (const float4 *)ctx->acc, n,
                 ctx->acc_stride, tab, nb, d_num, d_den);
    else
      AXG_LAUNCH(ctx, "gw_bin_green", k_gw_bin_green<double2>, 152 * 4, 256, 0, ctx->acc, n, ctx->acc_stride, tab, nb,
                 d_num, d_den);
  } else if (ctx->p.gw_mode == AXG_GW_UIJ) {
    AXG_TRY(ensure_uij_fft(ctx));
    const bool fp32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
    const int64_t nhalf = (int64_t)n * n * (n / 2 + 1);
    const double dv = ctx->p.dspa * ctx->p.dspa * ctx->p.dspa;
    if (fp32) {
      float *w = (float *)ctx->ubuf;
      float2 *F = ctx->uij_own_fft ? (float2 *)ctx->ubuf : (float2 *)(w + ctx->n3);
      if (ctx->uij_own_fft) {
        AXG_TRY(axg_uij_r2c_f32(ctx, (const float *)ctx->u[ctx->cur], (const float *)ctx->ud,
                                (const float *)ctx->cu, (float)tau, F, n));
      } else {
        for (int f = 0; f < 12; ++f) {
          AXG_LAUNCH(ctx, "uij_prepare_fp32", k_uij_prepare<float>, grid_for(ctx->n3), 256, 0,
                     (const float *)ctx->u[ctx->cur], (const float *)ctx->ud, (const float *)ctx->cu, ctx->n3, tau,
                     f, w);
          AXG_CUFFT_TRY(ctx, cufftExecR2C(ctx->plan_u, w, (cufftComplex *)F + f * nhalf));
        }
      }
      AXG_LAUNCH(ctx, "uij_bin_fp32", k_uij_bin<float2>, 152 * 4, 256, 0, F, ctx->u_pitch, n, dwav, dv, tab, nb,
                 d_num, d_den);
    } else {
      double *w = (double *)ctx->ubuf;
      double2 *F = ctx->uij_own_fft ? (double2 *)ctx->ubuf : (double2 *)(w + ctx->n3);
      if (ctx->uij_own_fft) {
        AXG_TRY(axg_uij_d2z_ff(ctx, (const double *)ctx->u[ctx->cur], (const double *)ctx->ud, tau, F, n));
      } else {
        for (int f = 0; f < 12; ++f) {
          AXG_LAUNCH(ctx, "uij_prepare_fp64", k_uij_prepare<double>, grid_for(ctx->n3), 256, 0,
                     (const double *)ctx->u[ctx->cur], (const double *)ctx->ud, (const double *)nullptr, ctx->n3,
                     tau, f, w);
          AXG_CUFFT_TRY(ctx, cufftExecD2Z(ctx->plan_u, w, (cufftDoubleComplex *)F + f * nhalf));
        }
      }
      AXG_LAUNCH(ctx, "uij_bin_fp64", k_uij_bin<double2>, 152 * 4, 256, 0, F, ctx->u_pitch, n, dwav, dv, tab, nb,
                 d_num, d_den);
    }
  } else {
    return axg_set_error(ctx, AXG_ERR_STATE, "gw_mode is NONE");
  }
  std::vector<double> h(2 * nb);
  AXG_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), ctx->d_red, sizeof(double) * 2 * nb, cudaMemcpyDeviceToHost,
                                    ctx->stream));
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  AXG_TRY(axg_evo_check_error(ctx));  // a TMA wait of the z pass that ran out
  const double fact = gw_fact(ctx->p, n, dspa);
  for (int k = 0; k < nb; ++k) {
    const double qc = log_bins ? std::sqrt(edges[k] * edges[k + 1]) : (edges[k + 1] + edges[k]) / 2;
    numer[k] = h[k];
    denom[k] = h[nb + k];
    power[k] = denom[k] > 0 ? numer[k] / denom[k] * (qc * qc * qc) * fact : 0.0;
    if (wave) {
      if (log_bins) {
        wave[k] = edges[k];
        if (k == nb - 1) wave[nb] = edges[nb];
      } else {
        wave[k] = qc;
      }
    }
  }
  return AXG_OK;
}

extern "C" {
int axg_grav_spec_estimation(axg_ctx *ctx, double tau, double *wave, double *power, double *numer,
                             double *denom) {
  if (!ctx || !power || !numer || !denom) return AXG_ERR_ARG;
  return axg_gw_spec(ctx, tau, 0, wave, power, numer, denom);
}
int axg_grav_spec_log(axg_ctx *ctx, double tau, double *edges, double *power, double *numer, double *denom) {
  if (!ctx || !power || !numer || !denom) return AXG_ERR_ARG;
  if (ctx->p.gw_log_bins < 1) return axg_set_error(ctx, AXG_ERR_ARG, "gw_log_bins < 1");
  return axg_gw_spec(ctx, tau, 1, edges, power, numer, denom);
}
}
