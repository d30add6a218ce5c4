// axg_adjoint.cu -- hand-written adjoint of the leapfrog of phi and six u_ij.
//
// Objective: the band-integrated GW energy of the u_ij spectrum at the end
// of the run,
//   J = sum_{kmin <= |k| <= kmax} 1/2 sum_ij (|W'_TT(k)|^2 + k^2 |W_TT(k)|^2),
//   W = dx^3 FFT(tau u), W' = dx^3 FFT(u + tau u'),
// i.e. half the band sum of the numerator of axg_grav_spec_estimation (GW_UIJ).
// Outputs: J, dJ/dlambda (quartic model: A = lambda/2, B = -lambda v^2/2) and
// the gradients with respect to the initial phi and phi' (complex, d/dRe +
// i d/dIm), from which the gradients with respect to Fourier-mode amplitudes
// follow by one FFT.
//
// Scheme, in the precision of the context (R = double for FP64-plain and
// FP64-fused, float for FP32-mixed):
//   forward  : the context's own step (plain drift / kick kernels, or the
//              fused TMA kernel with its ping-pong buffers and Kahan drift),
//              a checkpoint of phi and phi' (and the FP32 compensation of
//              phi) every `stride` steps;
//   terminal : D2Z of tau u and u + tau u' (12 fields, FP64), per k the
//              TT-projected band weights, Z2D back: dJ/du, dJ/du';
//   reverse  : for each step, phi and phi' are stepped BACK using the
//              leapfrog's time-reversibility (phi = phi+ - h pi+; pi = (pi+ -
//              f2 L phi - f3 g(phi)) / f1) and re-anchored on the exact
//              checkpoint every `stride` steps.  u_ij enters the equations
//              linearly and its adjoint never reads u, so u and u' are not
//              stepped back (they stay at the final state).  The adjoint step
//              is two stencil passes (k_adj_step; z-marching when 32
//              divides N, as k_adj_step_roll in FP32, which also fuses the
//              backward re-step of phi, and k_adj_step_tiled in FP64:
//              Laplacians of the adjoint momenta, the transposed potential
//              Jacobian, the source adjoint's
//              Q_i = 2 fs (sum_j wbar_ij D_j phi + wbar_ii D_i phi);
//              k_adj_divq: phibar += sum_i D_i^T Q_i).  Laplacians are summed
//              as differences from the centre (exact for smooth fields in
//              FP32); divisions by f1 and 2 dx are multiplications by
//              reciprocals computed once per step on the host.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "axg_internal.h"

namespace {

constexpr double kRefTwoPi = 2 * 3.14159265359;

__device__ __forceinline__ int64_t site(int x, int y, int z, int n) { return ((int64_t)z * n + y) * n + x; }
__device__ __forceinline__ int wr(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

template <typename R>
struct V2T;
template <>
struct V2T<float> {
  using T = float2;
};
template <>
struct V2T<double> {
  using T = double2;
};

template <typename R>
__device__ __forceinline__ typename V2T<R>::T mk(R x, R y) {
  typename V2T<R>::T v;
  v.x = x;
  v.y = y;
  return v;
}

// per-step coefficients in the arithmetic type of the adjoint
template <typename R>
struct Coef {
  R f1, f2, f3, fs, h, A, B, C, D, dA, dB, inv_f1, inv_d;
};

struct StepCoef {
  double f1, f2, f3, fs, h, A, B, C, D, dA, dB, d, inv_f1, inv_d;
  template <typename R>
  Coef<R> as() const {
    return Coef<R>{(R)f1, (R)f2, (R)f3, (R)fs, (R)h, (R)A, (R)B, (R)C, (R)D, (R)dA, (R)dB, (R)inv_f1, (R)inv_d};
  }
};

// Pinned arithmetic: every operation rounds once, in the order written.  The
// adjoint-step variants below (plain stencil, shared-memory ring, register
// roll, and the roll with the backward re-step fused in) share the point
// formulas that follow, so they give the same bits whatever contractions the
// compiler would otherwise pick in each kernel.
__device__ __forceinline__ float pmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double pmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float padd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double padd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float pfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double pfma(double a, double b, double c) { return __fma_rn(a, b, c); }

// adjoint of the drift: x + h y (pibar + h phibar, wbar + h ubar)
template <typename R>
__device__ __forceinline__ R dcomb(R x, R y, R h) {
  return pfma(h, y, x);
}

template <typename R>
__device__ __forceinline__ R mod2(R a, R b) {
  return pfma(a, a, pmul(b, b));
}

// central difference (a - b) / (2 dx)
template <typename R>
__device__ __forceinline__ R cdiff(R a, R b, R inv_d) {
  return pmul(padd(a, -b), inv_d);
}

__device__ __forceinline__ void kahan_sub(float &x, float &c, float dec) {
  const float y = -dec - c;
  const float t = x + y;
  c = (t - x) - y;
  x = t;
}

// backward drift of one component: phi -= h pi (FP32: Kahan-compensated like
// the forward drift)
__device__ __forceinline__ void rev_drift1(float &x, float &c, float h, float b) { kahan_sub(x, c, pmul(h, b)); }
__device__ __forceinline__ void rev_drift1(double &x, double &, double h, double b) { x = pfma(-h, b, x); }

// backward kick at one site: pi = (pi+ - f2 L phi - f3 g(phi)) / f1
template <typename R>
__device__ __forceinline__ typename V2T<R>::T rev_kick1(typename V2T<R>::T pv, R lr, R li, R p0r, R p0i,
                                                        const Coef<R> &k) {
  const R g0 = pfma(k.A, mod2(p0r, p0i), k.B);
  const R gr = padd(pfma(g0, p0r, pmul(k.D, p0r)), k.C), gi = pfma(g0, p0i, -pmul(k.D, p0i));
  return mk<R>(pmul(pfma(-k.f3, gr, pfma(-k.f2, lr, pv.x)), k.inv_f1),
               pmul(pfma(-k.f3, gi, pfma(-k.f2, li, pv.y)), k.inv_f1));
}

// adjoint of the kick at one site, without the D^T Q part of phibar: from
// itil at the site (i0), its Laplacian (l), phi (p0) and phibar+ (pb):
// phibar, pibar and the site's dJ/dlambda term
template <typename R>
struct AdjOut {
  typename V2T<R>::T pb, ib;
  R lam;
};

template <typename R>
__device__ __forceinline__ AdjOut<R> adj_point(R i0r, R i0i, R lr, R li, R p0r, R p0i, R pbr, R pbi,
                                               const Coef<R> &k) {
  const R s = mod2(p0r, p0i), g0 = pfma(k.A, s, k.B);
  const R pd = pfma(p0r, i0r, pmul(p0i, i0i));
  const R a2 = pmul(R(2), k.A);
  const R jr = pfma(k.D, i0r, pfma(g0, i0r, pmul(pmul(a2, p0r), pd)));
  const R ji = pfma(-k.D, i0i, pfma(g0, i0i, pmul(pmul(a2, p0i), pd)));
  AdjOut<R> o;
  o.pb = mk<R>(pfma(k.f3, jr, pfma(k.f2, lr, pbr)), pfma(k.f3, ji, pfma(k.f2, li, pbi)));
  o.ib = mk<R>(pmul(k.f1, i0r), pmul(k.f1, i0i));
  o.lam = pmul(pmul(k.f3, pfma(k.dA, s, k.dB)), pd);
  return o;
}

// the source adjoint Q_i = 2 fs (sum_j wtil_ij D_j phi + wtil_ii D_i phi)
template <typename R>
__device__ __forceinline__ void adj_q(const R wt[6], const R Dr[3], const R Di[3], R fs, R q[6]) {
  const int idx[3][3] = {{0, 1, 3}, {1, 2, 4}, {3, 4, 5}};
  const R fs2 = pmul(R(2), fs);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    R qr = pmul(wt[idx[i][i]], Dr[i]), qi = pmul(wt[idx[i][i]], Di[i]);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      qr = pfma(wt[idx[i][j]], Dr[j], qr);
      qi = pfma(wt[idx[i][j]], Di[j], qi);
    }
    q[2 * i] = pmul(fs2, qr);
    q[2 * i + 1] = pmul(fs2, qi);
  }
}

// backward drift: phi -= h pi
template <typename R>
__global__ void k_rev_drift(typename V2T<R>::T *phi, typename V2T<R>::T *cphi, const typename V2T<R>::T *pi,
                            int64_t n3, R h) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    auto a = phi[s];
    const auto b = pi[s];
    typename V2T<R>::T c = mk<R>(0, 0);
    if constexpr (sizeof(R) == 4) c = cphi[s];
    rev_drift1(a.x, c.x, h, b.x);
    rev_drift1(a.y, c.y, h, b.y);
    if constexpr (sizeof(R) == 4) cphi[s] = c;
    phi[s] = a;
  }
}

// backward kick: pi = (pi+ - f2 L phi - f3 g(phi)) / f1
template <typename R>
__global__ void k_rev_kick(const typename V2T<R>::T *__restrict__ phi, typename V2T<R>::T *__restrict__ pi, int n,
                           Coef<R> k) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y * blockDim.y + threadIdx.y, iz = blockIdx.z;
  if (ix >= n || iy >= n) return;
  const int64_t c = site(ix, iy, iz, n);
  const int64_t nb[6] = {site(wr(ix - 1, n), iy, iz, n), site(wr(ix + 1, n), iy, iz, n), site(ix, wr(iy - 1, n), iz, n),
                         site(ix, wr(iy + 1, n), iz, n), site(ix, iy, wr(iz - 1, n), n), site(ix, iy, wr(iz + 1, n), n)};
  const auto p0 = phi[c];
  // Laplacian as differences from the centre, summed x-, x+, y-, y+, z-, z+
  R lr = phi[nb[0]].x - p0.x, li = phi[nb[0]].y - p0.y;
  for (int q = 1; q < 6; ++q) {
    const auto v = phi[nb[q]];
    lr = lr + (v.x - p0.x);
    li = li + (v.y - p0.y);
  }
  pi[c] = rev_kick1<R>(pi[c], lr, li, p0.x, p0.y, k);
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Adjoint of one kick+drift at the pre-kick state phi (in: adjoint after the
// step; out: adjoint before it, except the D^T Q part of phibar).  dJ/dlambda
// is summed per site in FP64 here.
template <typename R>
__global__ void k_adj_step(const typename V2T<R>::T *__restrict__ phi, const typename V2T<R>::T *__restrict__ pb_in,
                           const typename V2T<R>::T *__restrict__ ib_in, const R *__restrict__ ub_in,
                           const R *__restrict__ wb_in, typename V2T<R>::T *__restrict__ pb_out,
                           typename V2T<R>::T *__restrict__ ib_out, R *__restrict__ ub_out, R *__restrict__ wb_out,
                           R *__restrict__ Q, int n, Coef<R> k, double *__restrict__ dlam) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y * blockDim.y + threadIdx.y, iz = blockIdx.z;
  double lam_part = 0.0;
  if (ix < n && iy < n) {
    const int64_t n3 = (int64_t)n * n * n;
    const int64_t c = site(ix, iy, iz, n);
    const int64_t nb[6] = {site(wr(ix - 1, n), iy, iz, n), site(wr(ix + 1, n), iy, iz, n),
                           site(ix, wr(iy - 1, n), iz, n), site(ix, wr(iy + 1, n), iz, n),
                           site(ix, iy, wr(iz - 1, n), n), site(ix, iy, wr(iz + 1, n), n)};
    // itil = pibar+ + h phibar+ at the site and its neighbours
    auto it = [&](int64_t q) {
      const auto a = ib_in[q], b = pb_in[q];
      return mk<R>(dcomb(a.x, b.x, k.h), dcomb(a.y, b.y, k.h));
    };
    const auto i0 = it(c);
    const auto v0 = it(nb[0]);
    R lr = v0.x - i0.x, li = v0.y - i0.y;
    for (int q = 1; q < 6; ++q) {
      const auto v = it(nb[q]);
      lr = lr + (v.x - i0.x);
      li = li + (v.y - i0.y);
    }
    const auto p0 = phi[c];
    const auto pbv = pb_in[c];
    const AdjOut<R> o = adj_point<R>(i0.x, i0.y, lr, li, p0.x, p0.y, pbv.x, pbv.y, k);
    pb_out[c] = o.pb;
    ib_out[c] = o.ib;
    const R s = p0.x * p0.x + p0.y * p0.y;
    lam_part = (double)k.f3 * ((double)k.dA * (double)s + (double)k.dB) * ((double)p0.x * i0.x + (double)p0.y * i0.y);
    R Dr[3], Di[3];
    for (int q = 0; q < 3; ++q) {
      const auto a = phi[nb[2 * q + 1]], b = phi[nb[2 * q]];
      Dr[q] = cdiff(a.x, b.x, k.inv_d);
      Di[q] = cdiff(a.y, b.y, k.inv_d);
    }
    R wt[6];
    for (int cc = 0; cc < 6; ++cc) {
      const R *wb = wb_in + cc * n3, *ub = ub_in + cc * n3;
      const R w0 = dcomb(wb[c], ub[c], k.h);
      wt[cc] = w0;
      R lu = dcomb(wb[nb[0]], ub[nb[0]], k.h) - w0;
      for (int q = 1; q < 6; ++q) lu = lu + (dcomb(wb[nb[q]], ub[nb[q]], k.h) - w0);
      ub_out[cc * n3 + c] = pfma(k.f2, lu, ub[c]);
      wb_out[cc * n3 + c] = pmul(k.f1, w0);
    }
    R q[6];
    adj_q(wt, Dr, Di, k.fs, q);
    for (int i = 0; i < 6; ++i) Q[i * n3 + c] = q[i];
  }
  lam_part = warp_sum(lam_part);
  if ((threadIdx.x & 31) == 0 && lam_part != 0.0) atomicAdd(dlam, lam_part);
}

// The same adjoint step, shared-memory tiled and z-marching: a block owns a
// TX x TY column of zc planes and keeps a 3-plane ring of (TX+2) x (TY+2)
// tiles of itil = pibar + h phibar (complex), wtil = wbar + h ubar (six
// reals) and phi (complex).  Tiles are filled with coalesced loads that form
// the combinations once per element, so a site costs about 24 scalar loads
// instead of about 100 scattered ones; the z neighbours come from the ring.
// The lambda contribution is summed per thread and per warp in R and added
// with one FP64 atomic per warp.
template <typename R, int TX, int TY>
__global__ void __launch_bounds__(TX *TY) k_adj_step_tiled(
    const typename V2T<R>::T *__restrict__ phi, const typename V2T<R>::T *__restrict__ pb_in,
    const typename V2T<R>::T *__restrict__ ib_in, const R *__restrict__ ub_in, const R *__restrict__ wb_in,
    typename V2T<R>::T *__restrict__ pb_out, typename V2T<R>::T *__restrict__ ib_out, R *__restrict__ ub_out,
    R *__restrict__ wb_out, R *__restrict__ Q, int n, int zc, Coef<R> k, double *__restrict__ dlam) {
  constexpr int W = TX + 2, H = TY + 2, PLANE = W * H, SLOT = 10 * PLANE;
  extern __shared__ unsigned char adj_smem[];
  R *sm = reinterpret_cast<R *>(adj_smem);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int ncx = n / TX;
  const int x0 = (blockIdx.x % ncx) * TX, y0 = (blockIdx.x / ncx) * TY, z0 = blockIdx.y * zc;
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  auto load_plane = [&](int z, int slot) {
    z = wr(z, n);
    R *t = sm + slot * SLOT;
    for (int e = tid; e < PLANE; e += TX * TY) {
      const int gx = wr(x0 + e % W - 1, n), gy = wr(y0 + e / W - 1, n);
      const int64_t g = (int64_t)z * n2 + (int64_t)gy * n + gx;
      const auto a = ib_in[g], b = pb_in[g];
      t[e] = dcomb(a.x, b.x, k.h);
      t[PLANE + e] = dcomb(a.y, b.y, k.h);
#pragma unroll
      for (int c = 0; c < 6; ++c) t[(2 + c) * PLANE + e] = dcomb(wb_in[c * n3 + g], ub_in[c * n3 + g], k.h);
      const auto p = phi[g];
      t[8 * PLANE + e] = p.x;
      t[9 * PLANE + e] = p.y;
    }
  };
  load_plane(z0 - 1, 0);
  load_plane(z0, 1);
  R lam = 0;
  const int ci = (ty + 1) * W + (tx + 1);
  for (int kk = 0; kk < zc; ++kk) {
    const int z = z0 + kk;
    load_plane(z + 1, (kk + 2) % 3);
    __syncthreads();
    const R *tm = sm + (kk % 3) * SLOT, *tc = sm + ((kk + 1) % 3) * SLOT, *tp = sm + ((kk + 2) % 3) * SLOT;
    const int64_t c = (int64_t)z * n2 + (int64_t)(y0 + ty) * n + (x0 + tx);
    // Laplacian of itil (differences from the centre)
    const R i0r = tc[ci], i0i = tc[PLANE + ci];
    const R lr = (tc[ci - 1] - i0r) + (tc[ci + 1] - i0r) + (tc[ci - W] - i0r) + (tc[ci + W] - i0r) +
                 (tm[ci] - i0r) + (tp[ci] - i0r);
    const R li = (tc[PLANE + ci - 1] - i0i) + (tc[PLANE + ci + 1] - i0i) + (tc[PLANE + ci - W] - i0i) +
                 (tc[PLANE + ci + W] - i0i) + (tm[PLANE + ci] - i0i) + (tp[PLANE + ci] - i0i);
    const R p0r = tc[8 * PLANE + ci], p0i = tc[9 * PLANE + ci];
    const auto pbv = pb_in[c];
    const AdjOut<R> o = adj_point<R>(i0r, i0i, lr, li, p0r, p0i, pbv.x, pbv.y, k);
    pb_out[c] = o.pb;
    ib_out[c] = o.ib;
    lam = padd(lam, o.lam);
    // central differences of phi
    const R Dr[3] = {cdiff(tc[8 * PLANE + ci + 1], tc[8 * PLANE + ci - 1], k.inv_d),
                     cdiff(tc[8 * PLANE + ci + W], tc[8 * PLANE + ci - W], k.inv_d),
                     cdiff(tp[8 * PLANE + ci], tm[8 * PLANE + ci], k.inv_d)};
    const R Di[3] = {cdiff(tc[9 * PLANE + ci + 1], tc[9 * PLANE + ci - 1], k.inv_d),
                     cdiff(tc[9 * PLANE + ci + W], tc[9 * PLANE + ci - W], k.inv_d),
                     cdiff(tp[9 * PLANE + ci], tm[9 * PLANE + ci], k.inv_d)};
    R wt[6];
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) {
      const R *w = tc + (2 + cc) * PLANE;
      const R w0 = w[ci];
      wt[cc] = w0;
      const R lu = (w[ci - 1] - w0) + (w[ci + 1] - w0) + (w[ci - W] - w0) + (w[ci + W] - w0) +
                   (tm[(2 + cc) * PLANE + ci] - w0) + (tp[(2 + cc) * PLANE + ci] - w0);
      ub_out[cc * n3 + c] = pfma(k.f2, lu, ub_in[cc * n3 + c]);
      wb_out[cc * n3 + c] = pmul(k.f1, w0);
    }
    R q[6];
    adj_q(wt, Dr, Di, k.fs, q);
#pragma unroll
    for (int i = 0; i < 6; ++i) Q[i * n3 + c] = q[i];
    __syncthreads();  // the ring slot of plane z - 1 is refilled next
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lam += __shfl_down_sync(0xffffffffu, lam, o);
  if ((tid & 31) == 0 && lam != R(0)) atomicAdd(dlam, (double)lam);
}

template <typename R, int TX, int TY>
constexpr int adj_tiled_smem() {
  return 3 * 10 * (TX + 2) * (TY + 2) * (int)sizeof(R);
}

// The adjoint step with the z neighbours in registers: each thread owns one
// (x, y) column of a TX x TY tile and walks zc planes, holding the
// combinations (itil, wtil, phi) at z - 1, z and z + 1 in registers.  Only
// the current plane, with its x and y halo, goes through shared memory, in
// two slots, so one barrier per plane suffices.  The raw fields of plane
// z + 2 are loaded into registers before plane z is computed, so their
// latency overlaps the arithmetic, and the raw centre values double as the
// additive terms of the outputs (no second load).
//
// REV fuses the backward re-step of phi into the same pass: the kernel reads
// the state after the step (phi+, its FP32 compensation, pi+), drifts phi
// back at every stencil point, kicks pi back at the centre, and writes phi,
// its compensation and pi to the other buffers; the adjoint step then uses
// that phi.  Per site this saves the write and two re-reads of phi, and two
// launches.  The point formulas are those of k_rev_drift, k_rev_kick and
// k_adj_step, so every variant gives the same bits.
template <typename R, bool REV>
struct AdjRaw {
  typename V2T<R>::T ib, pb, ph;
  R wb[6], ub[6];
  typename V2T<R>::T cph, pv;  // REV: compensation of phi+ (FP32) and pi+
};

template <typename R>
struct AdjCmb {
  R ir, ii, w[6], pr, pi;
};

// centre values a plane carries to its outputs
template <typename R>
struct AdjCentre {
  R pb[2], ub[6];
  R pv[2], c[2];  // REV: pi+ and the updated compensation of phi
};

template <typename R, int TX, int TY, bool REV>
__global__ void __launch_bounds__(TX *TY, sizeof(R) == 4 ? 2 : 1) k_adj_step_roll(
    const typename V2T<R>::T *__restrict__ phi, const typename V2T<R>::T *__restrict__ pb_in,
    const typename V2T<R>::T *__restrict__ ib_in, const R *__restrict__ ub_in, const R *__restrict__ wb_in,
    typename V2T<R>::T *__restrict__ pb_out, typename V2T<R>::T *__restrict__ ib_out, R *__restrict__ ub_out,
    R *__restrict__ wb_out, R *__restrict__ Q, int n, int zc, Coef<R> k, double *__restrict__ dlam,
    const typename V2T<R>::T *__restrict__ cphi_in, const typename V2T<R>::T *__restrict__ pi_in,
    typename V2T<R>::T *__restrict__ phi_out, typename V2T<R>::T *__restrict__ cphi_out,
    typename V2T<R>::T *__restrict__ pi_out) {
  static_assert(TX == 32, "one warp per tile row");
  static_assert(2 * TY <= 32 && TY >= 3, "halo duties of warps 0-2");
  constexpr bool F32 = sizeof(R) == 4;
  constexpr int W = TX + 2, H = TY + 2, PLANE = W * H, SLOT = 10 * PLANE;
  extern __shared__ unsigned char adj_smem[];
  R *sm = reinterpret_cast<R *>(adj_smem);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int ncx = n / TX;
  const int x0 = (blockIdx.x % ncx) * TX, y0 = (blockIdx.x / ncx) * TY, z0 = blockIdx.y * zc;
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  const int64_t own = (int64_t)(y0 + ty) * n + (x0 + tx);
  // halo duty: warp 0 the row y0 - 1, warp 1 the row y0 + TY, warp 2 (lanes
  // below 2 TY) the columns x0 - 1 and x0 + TX; the corners are never read
  int64_t hoff = -1;
  int hsi = 0;
  if (ty == 0) {
    hoff = (int64_t)wr(y0 - 1, n) * n + x0 + tx;
    hsi = tx + 1;
  } else if (ty == 1) {
    hoff = (int64_t)wr(y0 + TY, n) * n + x0 + tx;
    hsi = (TY + 1) * W + tx + 1;
  } else if (ty == 2 && tx < 2 * TY) {
    const int r = tx % TY;
    const bool lo = tx < TY;
    hoff = (int64_t)(y0 + r) * n + wr(lo ? x0 - 1 : x0 + TX, n);
    hsi = (r + 1) * W + (lo ? 0 : TX + 1);
  }
  const bool halo = hoff >= 0;
  auto load = [&](int z, int64_t off, AdjRaw<R, REV> &r) {
    const int64_t g = (int64_t)wr(z, n) * n2 + off;
    r.ib = ib_in[g];
    r.pb = pb_in[g];
    r.ph = phi[g];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      r.wb[c] = wb_in[c * n3 + g];
      r.ub[c] = ub_in[c * n3 + g];
    }
    if constexpr (REV) {
      if constexpr (F32) r.cph = cphi_in[g];
      r.pv = pi_in[g];
    }
  };
  // combined values of a point; REV drifts phi back first (cnew receives the
  // updated compensation)
  auto combine = [&](const AdjRaw<R, REV> &r, R *cnew) {
    AdjCmb<R> m;
    m.ir = dcomb(r.ib.x, r.pb.x, k.h);
    m.ii = dcomb(r.ib.y, r.pb.y, k.h);
#pragma unroll
    for (int c = 0; c < 6; ++c) m.w[c] = dcomb(r.wb[c], r.ub[c], k.h);
    m.pr = r.ph.x;
    m.pi = r.ph.y;
    if constexpr (REV) {
      R cx = 0, cy = 0;
      if constexpr (F32) {
        cx = r.cph.x;
        cy = r.cph.y;
      }
      rev_drift1(m.pr, cx, k.h, r.pv.x);
      rev_drift1(m.pi, cy, k.h, r.pv.y);
      cnew[0] = cx;
      cnew[1] = cy;
    }
    return m;
  };
  auto centre = [&](const AdjRaw<R, REV> &r, AdjCentre<R> &o) {
    o.pb[0] = r.pb.x;
    o.pb[1] = r.pb.y;
#pragma unroll
    for (int c = 0; c < 6; ++c) o.ub[c] = r.ub[c];
    if constexpr (REV) {
      o.pv[0] = r.pv.x;
      o.pv[1] = r.pv.y;
    }
  };
  auto store = [&](R *slot, int si, const AdjCmb<R> &m) {
    slot[si] = m.ir;
    slot[PLANE + si] = m.ii;
#pragma unroll
    for (int c = 0; c < 6; ++c) slot[(2 + c) * PLANE + si] = m.w[c];
    slot[8 * PLANE + si] = m.pr;
    slot[9 * PLANE + si] = m.pi;
  };
  const int ci = (ty + 1) * W + (tx + 1);
  AdjRaw<R, REV> rn, rh;
  R cdummy[2];
  AdjCentre<R> oc, on;
  load(z0 - 1, own, rn);
  AdjCmb<R> prev = combine(rn, cdummy);
  load(z0, own, rn);
  AdjCmb<R> cur = combine(rn, oc.c);
  centre(rn, oc);
  store(sm, ci, cur);
  if (halo) {
    load(z0, hoff, rh);
    store(sm, hsi, combine(rh, cdummy));
  }
  load(z0 + 1, own, rn);
  if (halo && zc > 1) load(z0 + 1, hoff, rh);
  R lam = 0;
  for (int kk = 0; kk < zc; ++kk) {
    const int z = z0 + kk;
    __syncthreads();  // plane z is complete in slot kk & 1; the other slot is free
    const AdjCmb<R> next = combine(rn, on.c);
    centre(rn, on);
    if (kk + 1 < zc) {
      R *tn = sm + ((kk + 1) & 1) * SLOT;
      store(tn, ci, next);
      if (halo) store(tn, hsi, combine(rh, cdummy));
      load(z + 2, own, rn);  // prefetch: `next` of plane z + 1
      if (halo && kk + 2 < zc) load(z + 2, hoff, rh);
    }
    const R *tc = sm + (kk & 1) * SLOT;
    const int64_t c = (int64_t)z * n2 + own;
    const R p0r = cur.pr, p0i = cur.pi;
    if constexpr (REV) {
      const R lpr = (tc[8 * PLANE + ci - 1] - p0r) + (tc[8 * PLANE + ci + 1] - p0r) + (tc[8 * PLANE + ci - W] - p0r) +
                    (tc[8 * PLANE + ci + W] - p0r) + (prev.pr - p0r) + (next.pr - p0r);
      const R lpi = (tc[9 * PLANE + ci - 1] - p0i) + (tc[9 * PLANE + ci + 1] - p0i) + (tc[9 * PLANE + ci - W] - p0i) +
                    (tc[9 * PLANE + ci + W] - p0i) + (prev.pi - p0i) + (next.pi - p0i);
      pi_out[c] = rev_kick1<R>(mk<R>(oc.pv[0], oc.pv[1]), lpr, lpi, p0r, p0i, k);
      phi_out[c] = mk<R>(p0r, p0i);
      if constexpr (F32) cphi_out[c] = mk<R>(oc.c[0], oc.c[1]);
    }
    const R i0r = cur.ir, i0i = cur.ii;
    const R lr = (tc[ci - 1] - i0r) + (tc[ci + 1] - i0r) + (tc[ci - W] - i0r) + (tc[ci + W] - i0r) +
                 (prev.ir - i0r) + (next.ir - i0r);
    const R li = (tc[PLANE + ci - 1] - i0i) + (tc[PLANE + ci + 1] - i0i) + (tc[PLANE + ci - W] - i0i) +
                 (tc[PLANE + ci + W] - i0i) + (prev.ii - i0i) + (next.ii - i0i);
    const AdjOut<R> o = adj_point<R>(i0r, i0i, lr, li, p0r, p0i, oc.pb[0], oc.pb[1], k);
    pb_out[c] = o.pb;
    ib_out[c] = o.ib;
    lam = padd(lam, o.lam);
    const R Dr[3] = {cdiff(tc[8 * PLANE + ci + 1], tc[8 * PLANE + ci - 1], k.inv_d),
                     cdiff(tc[8 * PLANE + ci + W], tc[8 * PLANE + ci - W], k.inv_d), cdiff(next.pr, prev.pr, k.inv_d)};
    const R Di[3] = {cdiff(tc[9 * PLANE + ci + 1], tc[9 * PLANE + ci - 1], k.inv_d),
                     cdiff(tc[9 * PLANE + ci + W], tc[9 * PLANE + ci - W], k.inv_d), cdiff(next.pi, prev.pi, k.inv_d)};
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) {
      const R *w = tc + (2 + cc) * PLANE;
      const R w0 = cur.w[cc];
      const R lu = (w[ci - 1] - w0) + (w[ci + 1] - w0) + (w[ci - W] - w0) + (w[ci + W] - w0) + (prev.w[cc] - w0) +
                   (next.w[cc] - w0);
      ub_out[cc * n3 + c] = pfma(k.f2, lu, oc.ub[cc]);
      wb_out[cc * n3 + c] = pmul(k.f1, w0);
    }
    R q[6];
    adj_q(cur.w, Dr, Di, k.fs, q);
#pragma unroll
    for (int i = 0; i < 6; ++i) Q[i * n3 + c] = q[i];
    prev = cur;
    cur = next;
    oc = on;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lam += __shfl_down_sync(0xffffffffu, lam, o);
  if (((ty * TX + tx) & 31) == 0 && lam != R(0)) atomicAdd(dlam, (double)lam);
}

template <typename R, int TX, int TY>
constexpr int adj_roll_smem() {
  return 2 * 10 * (TX + 2) * (TY + 2) * (int)sizeof(R);
}

// phibar += sum_i D_i^T Q_i,  D_i^T Q(x) = (Q(x - e_i) - Q(x + e_i)) / d
template <typename R>
__global__ void k_adj_divq(typename V2T<R>::T *__restrict__ pb, const R *__restrict__ Q, int n, R inv_d) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y * blockDim.y + threadIdx.y, iz = blockIdx.z;
  if (ix >= n || iy >= n) return;
  const int64_t n3 = (int64_t)n * n * n;
  const int64_t c = site(ix, iy, iz, n);
  const int64_t m[3] = {site(wr(ix - 1, n), iy, iz, n), site(ix, wr(iy - 1, n), iz, n), site(ix, iy, wr(iz - 1, n), n)};
  const int64_t p[3] = {site(wr(ix + 1, n), iy, iz, n), site(ix, wr(iy + 1, n), iz, n), site(ix, iy, wr(iz + 1, n), n)};
  auto v = pb[c];
  for (int i = 0; i < 3; ++i) {
    v.x += (Q[(2 * i) * n3 + m[i]] - Q[(2 * i) * n3 + p[i]]) * inv_d;
    v.y += (Q[(2 * i + 1) * n3 + m[i]] - Q[(2 * i + 1) * n3 + p[i]]) * inv_d;
  }
  pb[c] = v;
}

// adjoint of the first half drift phi += h pi: pibar += h phibar (u likewise)
template <typename R>
__global__ void k_adj_half_drift(const typename V2T<R>::T *pb, typename V2T<R>::T *ib, const R *ub, R *wb, int64_t n3,
                                 R h) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    auto a = ib[s];
    const auto b = pb[s];
    a.x += h * b.x;
    a.y += h * b.y;
    ib[s] = a;
    for (int c = 0; c < 6; ++c) wb[c * n3 + s] += h * ub[c * n3 + s];
  }
}

// 12 real FP64 inputs of the terminal spectrum: a = tau u, b = u + tau w
// (the FP32 state carries u as u - cu)
template <typename R>
__global__ void k_adj_terminal_in(const R *u, const R *cu, const R *w, int64_t n3, double tau, double *out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride)
    for (int c = 0; c < 6; ++c) {
      double uv = (double)u[c * n3 + s];
      if (cu) uv -= (double)cu[c * n3 + s];
      out[c * n3 + s] = tau * uv;
      out[(6 + c) * n3 + s] = uv + tau * (double)w[c * n3 + s];
    }
}

// per half-spectrum k: J contribution and the band weights M k^2 dx^6 Lambda(Xa), M dx^6 Lambda(Xb)
__global__ void k_adj_terminal_k(double2 *F, int n, double dwav, double dx6, double kmin, double kmax, double *J) {
  const int nh = n / 2 + 1;
  const int64_t nhalf = (int64_t)n * n * nh;
  const int idx[3][3] = {{0, 1, 3}, {1, 2, 4}, {3, 4, 5}};
  double jpart = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nhalf; h += stride) {
    const int ix = (int)(h % nh), iy = (int)((h / nh) % n), iz = (int)(h / ((int64_t)nh * n));
    const double q[3] = {(double)((ix + n / 2) % n - n / 2), (double)((iy + n / 2) % n - n / 2),
                         (double)((iz + n / 2) % n - n / 2)};
    const double qq = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    const double kk = qq * dwav;
    const bool in = qq > 0 && kk >= kmin && kk <= kmax;
    for (int f = 0; f < 2; ++f) {
      double2 X[6];
      for (int c = 0; c < 6; ++c) X[c] = F[(f * 6 + c) * nhalf + h];
      double2 Y[6];
      if (in) {
        double P[3][3];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) P[i][j] = (i == j) - q[i] * q[j] / (qq * qq);
        double Rr[3][3], Ri[3][3];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            double ar = 0, ai = 0;
            for (int a = 0; a < 3; ++a)
              for (int b = 0; b < 3; ++b) {
                ar += P[i][a] * X[idx[a][b]].x * P[b][j];
                ai += P[i][a] * X[idx[a][b]].y * P[b][j];
              }
            Rr[i][j] = ar;
            Ri[i][j] = ai;
          }
        const double tr = Rr[0][0] + Rr[1][1] + Rr[2][2], ti = Ri[0][0] + Ri[1][1] + Ri[2][2];
        double e = 0;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            Rr[i][j] -= 0.5 * P[i][j] * tr;
            Ri[i][j] -= 0.5 * P[i][j] * ti;
            e += Rr[i][j] * Rr[i][j] + Ri[i][j] * Ri[i][j];
          }
        const double wgt = (f == 0 ? kk * kk : 1.0) * dx6;
        const double herm = (ix == 0 || 2 * ix == n) ? 1.0 : 2.0;
        jpart += herm * 0.5 * wgt * e;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j <= i; ++j) Y[idx[i][j]] = make_double2(wgt * Rr[i][j], wgt * Ri[i][j]);
      } else {
        for (int c = 0; c < 6; ++c) Y[c] = make_double2(0.0, 0.0);
      }
      for (int c = 0; c < 6; ++c) F[(f * 6 + c) * nhalf + h] = Y[c];
    }
  }
  jpart = warp_sum(jpart);
  if ((threadIdx.x & 31) == 0 && jpart != 0.0) atomicAdd(J, jpart);
}

// ubar = mult (tau ga + gb), wbar = mult tau gb from the Z2D outputs
template <typename R>
__global__ void k_adj_terminal_out(const double *g, int64_t n3, double tau, R *ub, R *wb) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const double mult[6] = {1, 2, 1, 2, 2, 1};
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride)
    for (int c = 0; c < 6; ++c) {
      const double ga = g[c * n3 + s], gb = g[(6 + c) * n3 + s];
      ub[c * n3 + s] = (R)(mult[c] * (tau * ga + gb));
      wb[c * n3 + s] = (R)(mult[c] * tau * gb);
    }
}

// FP32 adjoint fields to complex128 for the caller
__global__ void k_adj_to_c128(const float2 *src, double2 *dst, int64_t n3) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride)
    dst[s] = make_double2((double)src[s].x, (double)src[s].y);
}

int grid_for(int64_t count) {
  int64_t b = (count + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

StepCoef coef_at(const axg_params &p, double t, double dt, double h) {
  double f[4], pot[4];
  axg_kick_coeffs(&p, t, dt, f, pot);
  StepCoef k;
  k.f1 = f[0];
  k.f2 = f[1];
  k.f3 = f[2];
  k.fs = f[3];
  k.h = h;
  k.A = pot[0];
  k.B = pot[1];
  k.C = pot[2];
  k.D = pot[3];
  if (p.potential == AXG_POT_QUARTIC) {
    k.dA = 0.5;
    k.dB = -(p.vev * p.vev) / 2;
  } else {
    k.dA = k.dB = 0.0;
  }
  k.d = 2 * p.dspa;
  k.inv_f1 = 1.0 / k.f1;
  k.inv_d = 1.0 / k.d;
  return k;
}

// Which adjoint-step kernel runs.  All three give bit-identical adjoint
// fields (the lambda sum differs in its last bits: the plain kernel sums in
// FP64 per site).  AXG_ADJOINT_STEP_KERNEL = plain | ring | roll overrides
// the choice, for the tests that compare them.
enum class AdjKernel { plain, ring, roll };

AdjKernel adj_kernel_choice(int n, bool f32) {
  const bool tiled = n % 32 == 0;
  AdjKernel k = !tiled ? AdjKernel::plain : (f32 ? AdjKernel::roll : AdjKernel::ring);
  if (const char *v = std::getenv("AXG_ADJOINT_STEP_KERNEL")) {
    if (!std::strcmp(v, "plain")) k = AdjKernel::plain;
    else if (tiled && !std::strcmp(v, "ring")) k = AdjKernel::ring;
    else if (tiled && !std::strcmp(v, "roll")) k = AdjKernel::roll;
  }
  return k;
}

template <typename R>
int adjoint_run(axg_ctx *ctx, double t1, double dt, int64_t nsteps, int first_half, int last_half, int64_t stride,
                double kmin, double kmax, double *J_out, double *dJ_dlambda, double *grad_phi0, double *grad_phidot0,
                double *ms_forward, double *ms_reverse) {
  using V = typename V2T<R>::T;
  constexpr bool F32 = sizeof(R) == 4;
  const bool plain = ctx->p.precision == AXG_PREC_FP64_PLAIN;
  const int n = (int)ctx->n;
  const int64_t n3 = ctx->n3, nhalf = (int64_t)n * n * (n / 2 + 1);
  const size_t adj_b = (size_t)n3 * (2 * sizeof(V) + 12 * sizeof(R));  // one adjoint state
  const size_t ck_b = (size_t)n3 * sizeof(V) * (F32 ? 3 : 2);           // phi (+ its compensation), phi'
  const int64_t nck = nsteps / stride + 1;
  char *ck = nullptr, *adj = nullptr, *spare = nullptr;
  R *Q = nullptr;
  double *fbuf = nullptr;
  int rc = AXG_OK;
  cufftHandle pf = 0, pb = 0;
  bool pfo = false, pbo = false;
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  auto cleanup = axg_on_exit([&] {
    cudaStreamSynchronize(ctx->stream);
    if (pfo) cufftDestroy(pf);
    if (pbo) cufftDestroy(pb);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    axg_free(ctx, (void **)&ck);
    axg_free(ctx, (void **)&adj);
    axg_free(ctx, (void **)&Q);
    axg_free(ctx, (void **)&fbuf);
    axg_free(ctx, (void **)&spare);
    ctx->flags_valid = false;
  });
  do {
    // nck checkpoints plus the final phi, phi' (restored after the reverse sweep)
    if ((rc = axg_alloc(ctx, (void **)&ck, ck_b * (nck + 1), "adjoint checkpoints"))) break;
    if ((rc = axg_alloc(ctx, (void **)&adj, adj_b * 2, "adjoint state"))) break;
    if ((rc = axg_alloc(ctx, (void **)&Q, (size_t)n3 * 6 * sizeof(R), "adjoint Q"))) break;
    if ((rc = axg_alloc(ctx, (void **)&fbuf, (size_t)12 * n3 * 8 + (size_t)12 * nhalf * 16, "adjoint FFT"))) break;
    int dims[3] = {n, n, n};
    if (cufftPlanMany(&pf, 3, dims, nullptr, 1, (int)n3, nullptr, 1, (int)nhalf, CUFFT_D2Z, 12) != CUFFT_SUCCESS ||
        cufftPlanMany(&pb, 3, dims, nullptr, 1, (int)nhalf, nullptr, 1, (int)n3, CUFFT_Z2D, 12) != CUFFT_SUCCESS) {
      rc = axg_set_error(ctx, AXG_ERR_CUDA, "adjoint cuFFT plans");
      break;
    }
    pfo = pbo = true;
    cufftSetStream(pf, ctx->stream);
    cufftSetStream(pb, ctx->stream);
    // the fused paths ping-pong phi and u: always address the current buffers
    auto cur_phi = [&]() { return (V *)ctx->phi[ctx->cur]; };
    V *pi = (V *)ctx->phid, *cphi = F32 ? (V *)ctx->cphi : nullptr;
    auto save = [&](int64_t k) {
      char *dst = ck + ck_b * k;
      const size_t fb = (size_t)n3 * sizeof(V);
      cudaMemcpyAsync(dst, cur_phi(), fb, cudaMemcpyDeviceToDevice, ctx->stream);
      cudaMemcpyAsync(dst + fb, pi, fb, cudaMemcpyDeviceToDevice, ctx->stream);
      if (F32) cudaMemcpyAsync(dst + 2 * fb, cphi, fb, cudaMemcpyDeviceToDevice, ctx->stream);
    };
    auto load_to = [&](int64_t k, V *dphi, V *dpi, V *dcphi) {
      const char *src = ck + ck_b * k;
      const size_t fb = (size_t)n3 * sizeof(V);
      cudaMemcpyAsync(dphi, src, fb, cudaMemcpyDeviceToDevice, ctx->stream);
      cudaMemcpyAsync(dpi, src + fb, fb, cudaMemcpyDeviceToDevice, ctx->stream);
      if (F32) cudaMemcpyAsync(dcphi, src + 2 * fb, fb, cudaMemcpyDeviceToDevice, ctx->stream);
    };
    auto load = [&](int64_t k) { load_to(k, cur_phi(), pi, cphi); };
    // ---------------- forward with checkpoints ----------------
    cudaEventRecord(e0, ctx->stream);
    double t = t1;
    if (first_half) {
      if ((rc = axg_evo_drift(ctx, dt / 2))) break;
      t = t + dt / 2;
    }
    save(0);
    std::vector<double> kt(nsteps + 1), kh(nsteps + 1);
    for (int64_t it = 1; it <= nsteps && rc == AXG_OK; ++it) {
      const double h = (it == nsteps && last_half) ? dt / 2 : dt;
      kt[it] = t;
      kh[it] = h;
      if (plain) {
        if ((rc = axg_evo_kick_plain(ctx, t, dt))) break;
        if ((rc = axg_evo_drift(ctx, h))) break;
      } else if ((rc = axg_evo_kick_drift(ctx, t, dt, h))) {
        break;
      }
      t = t + h;
      if (it % stride == 0) save(it / stride);
    }
    if (rc) break;
    save(nck);  // final phi, phi'
    const double tau_end = t;
    cudaEventRecord(e1, ctx->stream);
    // ---------------- terminal adjoint ----------------
    V *pb_a = (V *)adj, *ib_a = pb_a + n3;
    R *ub_a = (R *)(ib_a + n3), *wb_a = ub_a + 6 * n3;
    V *pb_b = (V *)(adj + adj_b), *ib_b = pb_b + n3;
    R *ub_b = (R *)(ib_b + n3), *wb_b = ub_b + 6 * n3;
    double *fin = fbuf;
    double2 *F = (double2 *)(fbuf + 12 * n3);
    AXG_LAUNCH(ctx, "adj_terminal_in", k_adj_terminal_in<R>, grid_for(n3), 256, 0, (const R *)ctx->u[ctx->cur],
               F32 ? (const R *)ctx->cu : nullptr, (const R *)ctx->ud, n3, tau_end, fin);
    if (cufftExecD2Z(pf, fin, (cufftDoubleComplex *)F) != CUFFT_SUCCESS) {
      rc = axg_set_error(ctx, AXG_ERR_CUDA, "adjoint D2Z");
      break;
    }
    AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_red, 0, 16, ctx->stream));
    const double dx = ctx->p.dspa, dx6 = dx * dx * dx * dx * dx * dx;
    const double dwav = kRefTwoPi / ctx->p.dspa / n;
    AXG_LAUNCH(ctx, "adj_terminal_k", k_adj_terminal_k, grid_for(nhalf), 256, 0, F, n, dwav, dx6, kmin, kmax,
               ctx->d_red);
    if (cufftExecZ2D(pb, (cufftDoubleComplex *)F, fin) != CUFFT_SUCCESS) {
      rc = axg_set_error(ctx, AXG_ERR_CUDA, "adjoint Z2D");
      break;
    }
    AXG_CUDA_TRY(ctx, cudaMemsetAsync(adj, 0, (size_t)n3 * 2 * sizeof(V), ctx->stream));  // phibar, pibar = 0
    AXG_LAUNCH(ctx, "adj_terminal_out", k_adj_terminal_out<R>, grid_for(n3), 256, 0, fin, n3, tau_end, ub_a, wb_a);
    // ---------------- reverse sweep ----------------
    double *dlam = ctx->d_red + 1;
    dim3 blk(32, 8), grd((n + 31) / 32, (n + 7) / 8, n);
    // the tiled steps need N divisible by the 32 x 8 column and the z chunk;
    // FP32 rolls the z neighbours through registers, FP64 (twice the
    // registers per value) keeps the 3-plane ring
    const int tzc = 32;
    const AdjKernel kind = adj_kernel_choice(n, F32);
    constexpr int tsmem = adj_tiled_smem<R, 32, 8>(), rsmem = adj_roll_smem<R, 32, 8>();
    const dim3 tgrid((unsigned)((n / 32) * (n / 8)), (unsigned)(kind != AdjKernel::plain ? n / tzc : 1));
    {
      static bool attr = false;
      if (!attr) {
        AXG_CUDA_TRY(ctx, cudaFuncSetAttribute(k_adj_step_tiled<R, 32, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               tsmem));
        AXG_CUDA_TRY(ctx, cudaFuncSetAttribute(k_adj_step_roll<R, 32, 8, false>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, rsmem));
        AXG_CUDA_TRY(ctx, cudaFuncSetAttribute(k_adj_step_roll<R, 32, 8, true>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, rsmem));
        attr = true;
      }
    }
    // The roll kernel steps phi back inside the adjoint step and so cannot
    // work in place: phi, its compensation and pi ping-pong between the
    // context's buffers (slot 0) and spares.
    V *rphi[2] = {cur_phi(), nullptr}, *rcphi[2] = {cphi, nullptr}, *rpi[2] = {pi, nullptr};
    int rs = 0;
    if (kind == AdjKernel::roll) {
      if ((rc = axg_alloc(ctx, (void **)&spare, (size_t)n3 * sizeof(V) * 3, "adjoint re-step buffers"))) break;
      rphi[1] = (V *)spare;
      rpi[1] = rphi[1] + n3;
      rcphi[1] = F32 ? rpi[1] + n3 : nullptr;
    }
    bool a_is_in = true;
    V *phi = cur_phi();  // the plain and ring paths step phi back in place in the final buffer
    for (int64_t it = nsteps; it >= 1 && rc == AXG_OK; --it) {
      const StepCoef kc = coef_at(ctx->p, kt[it], dt, kh[it]);
      const Coef<R> kr = kc.template as<R>();
      // state after step it -> state before step it (pre-kick); the
      // checkpoints re-anchor it every `stride` steps
      const bool anchor = (it - 1) % stride == 0;
      if (kind == AdjKernel::roll) {
        if (anchor) load_to((it - 1) / stride, rphi[rs], rpi[rs], rcphi[rs]);
      } else if (anchor) {
        load((it - 1) / stride);
      } else {
        AXG_LAUNCH(ctx, "adj_rev_drift", k_rev_drift<R>, grid_for(n3), 256, 0, phi, cphi, pi, n3, (R)kh[it]);
        AXG_LAUNCH(ctx, "adj_rev_kick", k_rev_kick<R>, grd, blk, 0, phi, pi, n, kr);
      }
      V *pbi = a_is_in ? pb_a : pb_b, *ibi = a_is_in ? ib_a : ib_b, *pbo_ = a_is_in ? pb_b : pb_a,
        *ibo = a_is_in ? ib_b : ib_a;
      R *ubi = a_is_in ? ub_a : ub_b, *wbi = a_is_in ? wb_a : wb_b, *ubo = a_is_in ? ub_b : ub_a,
        *wbo = a_is_in ? wb_b : wb_a;
      if (kind == AdjKernel::roll) {
        if (anchor) {
          AXG_LAUNCH(ctx, "adj_step", (k_adj_step_roll<R, 32, 8, false>), tgrid, dim3(32, 8), rsmem, rphi[rs], pbi,
                     ibi, ubi, wbi, pbo_, ibo, ubo, wbo, Q, n, tzc, kr, dlam, nullptr, nullptr, nullptr, nullptr,
                     nullptr);
        } else {
          AXG_LAUNCH(ctx, "adj_step_rev", (k_adj_step_roll<R, 32, 8, true>), tgrid, dim3(32, 8), rsmem, rphi[rs], pbi,
                     ibi, ubi, wbi, pbo_, ibo, ubo, wbo, Q, n, tzc, kr, dlam, rcphi[rs], rpi[rs], rphi[1 - rs],
                     rcphi[1 - rs], rpi[1 - rs]);
          rs = 1 - rs;
        }
      } else if (kind == AdjKernel::ring) {
        AXG_LAUNCH(ctx, "adj_step", (k_adj_step_tiled<R, 32, 8>), tgrid, dim3(32, 8), tsmem, phi, pbi, ibi, ubi, wbi,
                   pbo_, ibo, ubo, wbo, Q, n, tzc, kr, dlam);
      } else {
        AXG_LAUNCH(ctx, "adj_step", k_adj_step<R>, grd, blk, 0, phi, pbi, ibi, ubi, wbi, pbo_, ibo, ubo, wbo, Q, n, kr,
                   dlam);
      }
      AXG_LAUNCH(ctx, "adj_divq", k_adj_divq<R>, grd, blk, 0, pbo_, Q, n, kr.inv_d);
      a_is_in = !a_is_in;
    }
    if (rc) break;
    V *pbf = a_is_in ? pb_a : pb_b, *ibf = a_is_in ? ib_a : ib_b;
    R *ubf = a_is_in ? ub_a : ub_b, *wbf = a_is_in ? wb_a : wb_b;
    if (first_half)
      AXG_LAUNCH(ctx, "adj_half_drift", k_adj_half_drift<R>, grid_for(n3), 256, 0, pbf, ibf, ubf, wbf, n3, (R)(dt / 2));
    cudaEventRecord(e2, ctx->stream);
    double h2[2];
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(h2, ctx->d_red, 16, cudaMemcpyDeviceToHost, ctx->stream));
    double *outs[2] = {grad_phi0, grad_phidot0};
    V *srcs[2] = {pbf, ibf};
    for (int q = 0; q < 2; ++q) {
      if (!outs[q]) continue;
      const void *src = srcs[q];
      if constexpr (F32) {
        k_adj_to_c128<<<grid_for(n3), 256, 0, ctx->stream>>>((const float2 *)srcs[q], (double2 *)fbuf, n3);
        ctx->launches++;
        src = fbuf;
      }
      AXG_CUDA_TRY(ctx, cudaMemcpyAsync(outs[q], src, (size_t)n3 * 16, cudaMemcpyDeviceToHost, ctx->stream));
      if (F32) AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // fbuf is reused
    }
    AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    *J_out = h2[0];
    if (dJ_dlambda) *dJ_dlambda = h2[1];
    float f1 = 0, f2 = 0;
    cudaEventElapsedTime(&f1, e0, e1);
    cudaEventElapsedTime(&f2, e1, e2);
    if (ms_forward) *ms_forward = f1;
    if (ms_reverse) *ms_reverse = f2;
    // the context state is left at the end of the forward run, as after
    // axg_leapfrog: u, u' were never stepped back; phi, phi' come back from
    // the final slot
    load(nck);
    AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  } while (0);
  return rc;
}

}  // namespace

extern "C" int axg_adjoint_gw_band(axg_ctx *ctx, double t1, double dt, int64_t nsteps, int first_half,
                                   int last_half, int64_t stride, double kmin, double kmax, double *J_out,
                                   double *dJ_dlambda, double *grad_phi0, double *grad_phidot0, double *ms_forward,
                                   double *ms_reverse) {
  if (!ctx || nsteps < 1 || stride < 1 || !(dt > 0) || !(t1 > 0) || !J_out) return AXG_ERR_ARG;
  if (ctx->p.gw_mode != AXG_GW_UIJ)
    return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "the adjoint needs gw_mode UIJ (J is the u_ij band energy)");
  if (ctx->p.precision == AXG_PREC_FP32_MIXED)
    return adjoint_run<float>(ctx, t1, dt, nsteps, first_half, last_half, stride, kmin, kmax, J_out, dJ_dlambda,
                              grad_phi0, grad_phidot0, ms_forward, ms_reverse);
  return adjoint_run<double>(ctx, t1, dt, nsteps, first_half, last_half, stride, kmin, kmax, J_out, dJ_dlambda,
                             grad_phi0, grad_phidot0, ms_forward, ms_reverse);
}
