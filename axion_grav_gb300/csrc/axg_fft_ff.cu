// axg_fft_ff.cu -- 3-D FFTs at FP64 accuracy in float-float arithmetic, and
// the FP32 transform of the Green's-function sources.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, and an FP64 FFT is bound by
// it: cuFFT's 512^3 D2Z takes about 15.5 ms, while moving its bytes takes
// about 1 ms.  Here every value is a float-float pair (axg_ff.h) and the
// butterflies run on the FP32 pipes; complex twiddle products are two f2_dot2
// terms.  The input doubles are split into float-float on load and the
// output is hi + lo in double (or stays float-float for a consumer that
// reads it so), so the transform agrees with an FP64 FFT to about 1e-13 of
// the spectrum's largest value.
//
// Layout and convention are cuFFT's: batched D2Z, in [batch][n][n][n] reals,
// out [batch][n][n][n/2+1] complex, forward (exp(-2 pi i k x / n)),
// unnormalised; and in-place Z2Z of one [n][n][n] volume in either
// direction (the complex row pass replaces the real one).  Three passes,
// each one read and one write of the spectrum (the output buffer holds the
// float-float intermediate):
//   rows    : per x-row, the n reals as n/2 complex points z[m] = x[2m] +
//             i x[2m+1], an n/2-point FFT, and the split of Z into the n/2+1
//             outputs X[k] = E[k] + W_n^k O[k];
//   y, z    : n-point FFTs along y and along z, a few adjacent kx columns per
//             CTA so every row of the tile is one 64-byte segment.
// The complex-float transforms (FP32-mixed Green sources and u_ij fields)
// store their half spectra with kx rows padded to a multiple of 4 complex
// values (axg_f32_spec_pitch): their y pass reads 32-byte rows on sector
// boundaries, and their z pass moves its tiles by TMA (k_cols_z_tma).
// Each line is a Stockham radix-8 FFT in registers (f_stockham): a 512-point
// line takes two shared-memory exchanges, the first pass reads its inputs
// from global memory and the column passes' last pass writes there.
// Twiddles W_n^k come from a float-float table made on the host in FP64.
// Powers of two from 16 to 512.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "axg_ff.h"
#include "axg_gw_source.h"
#include "axg_internal.h"
#include "axg_tma.h"

namespace {

// complex float-float in a float4: (re.h, re.l, im.h, im.l)
__device__ __forceinline__ F2 re(float4 v) { return {v.x, v.y}; }
__device__ __forceinline__ F2 im(float4 v) { return {v.z, v.w}; }
__device__ __forceinline__ float4 cx(F2 r, F2 i) { return make_float4(r.h, r.l, i.h, i.l); }

// Complex arithmetic of the two value types the transforms run in: complex
// float (float2) and complex float-float (float4).
__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 c_conj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 c_half(float2 a) { return make_float2(0.5f * a.x, 0.5f * a.y); }
__device__ __forceinline__ float2 c_div_2i(float2 d) { return make_float2(0.5f * d.y, -0.5f * d.x); }  // d / 2i

__device__ __forceinline__ float4 c_add(float4 a, float4 b) { return cx(f2_add(re(a), re(b)), f2_add(im(a), im(b))); }
__device__ __forceinline__ float4 c_sub(float4 a, float4 b) { return cx(f2_sub(re(a), re(b)), f2_sub(im(a), im(b))); }
__device__ __forceinline__ float4 c_mul(float4 a, float4 b) {
  return cx(f2_dot2(re(a), re(b), im(a), im(b), -1.f), f2_dot2(re(a), im(b), im(a), re(b), 1.f));
}
__device__ __forceinline__ float4 c_conj(float4 a) { return make_float4(a.x, a.y, -a.z, -a.w); }
__device__ __forceinline__ float4 c_neg(float4 a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }
__device__ __forceinline__ float4 c_half(float4 a) { return cx(f2_half(re(a)), f2_half(im(a))); }  // exact
__device__ __forceinline__ float4 c_div_2i(float4 d) { return cx(f2_half(im(d)), f2_neg(f2_half(re(d)))); }

// a W_4 = a (-i), inverse a (+i): exact
template <bool INV>
__device__ __forceinline__ float2 c_w4(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
template <bool INV>
__device__ __forceinline__ float4 c_w4(float4 a) {
  return INV ? make_float4(-a.z, -a.w, a.x, a.y) : make_float4(a.z, a.w, -a.x, -a.y);
}

// a W_8 = a (1 -+ i) / sqrt 2 and a W_8^3 = a (-1 -+ i) / sqrt 2 (the upper
// sign forward); 1 / sqrt 2 as a float and as a float-float pair
constexpr float kRs2 = 0.70710678118654752440f;
constexpr float kRs2Hi = 0.70710676908493041992f, kRs2Lo = 1.2101617485882343e-08f;
template <bool INV>
__device__ __forceinline__ float2 c_w8(float2 a) {
  return INV ? make_float2((a.x - a.y) * kRs2, (a.x + a.y) * kRs2) : make_float2((a.x + a.y) * kRs2, (a.y - a.x) * kRs2);
}
template <bool INV>
__device__ __forceinline__ float2 c_w8_3(float2 a) {
  return INV ? make_float2((-a.x - a.y) * kRs2, (a.x - a.y) * kRs2)
             : make_float2((a.y - a.x) * kRs2, (-a.x - a.y) * kRs2);
}
template <bool INV>
__device__ __forceinline__ float4 c_w8(float4 a) {
  const F2 r = re(a), i = im(a), s = {kRs2Hi, kRs2Lo};
  return INV ? cx(f2_mul(f2_sub(r, i), s), f2_mul(f2_add(r, i), s)) : cx(f2_mul(f2_add(r, i), s), f2_mul(f2_sub(i, r), s));
}
template <bool INV>
__device__ __forceinline__ float4 c_w8_3(float4 a) {
  const F2 r = re(a), i = im(a), s = {kRs2Hi, kRs2Lo};
  return INV ? cx(f2_neg(f2_mul(f2_add(r, i), s)), f2_mul(f2_sub(r, i), s))
             : cx(f2_mul(f2_sub(i, r), s), f2_neg(f2_mul(f2_add(r, i), s)));
}

template <typename T>
__device__ __forceinline__ T c_zero() {
  T z;
  if constexpr (sizeof(T) == 8) z = make_float2(0.f, 0.f);
  else z = make_float4(0.f, 0.f, 0.f, 0.f);
  return z;
}

// a complex float-float from two doubles (re, im)
__device__ __forceinline__ float4 c_from(double2 x) { return cx(f2_from(x.x), f2_from(x.y)); }

// In-register DFTs of 2, 4 and 8 points, natural order in and out; INV uses
// exp(+2 pi i / R).  The 8-point one is two 4-point DFTs of the even and odd
// inputs joined with W_8^k.
template <bool INV, typename T>
__device__ __forceinline__ void c_dft4(T &x0, T &x1, T &x2, T &x3) {
  const T a = c_add(x0, x2), b = c_sub(x0, x2), c = c_add(x1, x3), d = c_w4<INV>(c_sub(x1, x3));
  x0 = c_add(a, c);
  x1 = c_add(b, d);
  x2 = c_sub(a, c);
  x3 = c_sub(b, d);
}
template <int R, bool INV, typename T>
__device__ __forceinline__ void c_dft(T *v) {
  if constexpr (R == 2) {
    const T t = v[0];
    v[0] = c_add(t, v[1]);
    v[1] = c_sub(t, v[1]);
  } else if constexpr (R == 4) {
    c_dft4<INV>(v[0], v[1], v[2], v[3]);
  } else {
    T e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    c_dft4<INV>(e0, e1, e2, e3);
    c_dft4<INV>(o0, o1, o2, o3);
    o1 = c_w8<INV>(o1);
    o2 = c_w4<INV>(o2);
    o3 = c_w8_3<INV>(o3);
    v[0] = c_add(e0, o0);
    v[4] = c_sub(e0, o0);
    v[1] = c_add(e1, o1);
    v[5] = c_sub(e1, o1);
    v[2] = c_add(e2, o2);
    v[6] = c_sub(e2, o2);
    v[3] = c_add(e3, o3);
    v[7] = c_sub(e3, o3);
  }
}

// Stockham autosort FFT of L points, L / 8 threads per line, 8 values per
// thread in registers.  Pass (R, NS), NS the product of the earlier radices:
// iteration jj < L / R reads x[jj + r L / R], multiplies input r by
// W_(NS R)^(r (jj mod NS)), takes the R-point DFT and writes output r to
// (jj / NS) NS R + jj mod NS + r NS.  Radix 8 while 8 divides what is left,
// then one radix-4 or radix-2 pass; a thread runs 8 / R iterations per pass.
// Input and output are in natural order.  Between passes the values go
// through shared memory, element i of the line at line[pad(i) * ls]
// (pad(i) = i + i / 8 keeps the radix-8 strides off a single bank); the last
// pass hands its outputs to `store`.  tw[k] = W_(L ts)^k, k < L ts.
__device__ __forceinline__ int fpad(int i) { return i + (i >> 3); }

// Unpadded lines of 8-byte (complex float) elements, element i at fswz(i):
// the low four bits, the element's bank pair within 128 bytes, XORed with
// bits 3..6.  Aligned runs of 16 elements (a half warp's 8-byte request) keep
// 16 distinct bank pairs, and so do the passes' stride-8 and stride-64
// writes.  With 8-byte elements the i + i / 8 padding made every consecutive
// read and write two-way conflicted; with 16-byte elements (float-float,
// 8 lanes per request) it is conflict-free and stays.
__device__ __forceinline__ int fswz(int i) { return i ^ ((i >> 3) & 15); }
template <bool SW>
__device__ __forceinline__ int fidx(int i) {
  if constexpr (SW) return fswz(i);
  else return fpad(i);
}

template <int L, int NS, bool INV, bool REC = false, bool SW = false, typename T, typename Store>
__device__ __forceinline__ void f_stockham(T v[8], int j, T *line, int ls, const T *tw, int ts, Store store) {
  constexpr int REM = L / NS, R = REM >= 8 ? 8 : REM, NI = 8 / R, TH = L / 8;
#pragma unroll
  for (int q = 0; q < NI; ++q) {
    const int jj = j + q * TH;
    if constexpr (NS > 1) {
      const int k = jj & (NS - 1);
      if constexpr (REC) {
        // one table read; the powers by complex multiplication (REC is for
        // the FP32 transforms).  SW: tw is the per-pass table of
        // load_twc, tw[NS + k] = W_(NS R)^k, read at consecutive k.
        T w1 = SW ? tw[NS + k] : tw[k * (L / (NS * R)) * ts];
        if (INV) w1 = c_conj(w1);
        T w = w1;
#pragma unroll
        for (int r = 1; r < R; ++r) {
          v[q * R + r] = c_mul(v[q * R + r], w);
          w = c_mul(w, w1);
        }
      } else {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          T w = tw[r * k * (L / (NS * R)) * ts];
          if (INV) w = c_conj(w);
          v[q * R + r] = c_mul(v[q * R + r], w);
        }
      }
    }
    c_dft<R, INV>(&v[q * R]);
  }
  if constexpr (NS * R == L) {
#pragma unroll
    for (int q = 0; q < NI; ++q) {
      const int jj = j + q * TH;
#pragma unroll
      for (int r = 0; r < R; ++r) store(jj + r * NS, v[q * R + r]);  // last pass: NS = L / R, jj < NS
    }
  } else {
#pragma unroll
    for (int q = 0; q < NI; ++q) {
      const int jj = j + q * TH, d = (jj / NS) * NS * R + (jj & (NS - 1));
#pragma unroll
      for (int r = 0; r < R; ++r) line[fidx<SW>(d + r * NS) * ls] = v[q * R + r];
    }
    __syncthreads();
    constexpr int NS2 = NS * R, R2 = L / NS2 >= 8 ? 8 : L / NS2;
#pragma unroll
    for (int q = 0; q < 8 / R2; ++q)
#pragma unroll
      for (int r = 0; r < R2; ++r) v[q * R2 + r] = line[fidx<SW>(j + q * TH + r * (L / R2)) * ls];
    __syncthreads();
    f_stockham<L, NS2, INV, REC, SW>(v, j, line, ls, tw, ts, store);
  }
}

// the twiddle table W_L^k, k < L, in shared memory from the first L / 2
// entries of the float-float table (W^(k + L/2) = -W^k)
__device__ __forceinline__ void load_tw(float4 *tw, const float4 *__restrict__ twff, int half) {
  for (int k = threadIdx.x; k < half; k += blockDim.x) {
    const float4 w = twff[k];
    tw[k] = w;
    tw[k + half] = c_neg(w);
  }
}
__device__ __forceinline__ void load_tw(float2 *tw, const float4 *__restrict__ twff, int half) {
  for (int k = threadIdx.x; k < half; k += blockDim.x) {
    const float4 w = twff[k];
    tw[k] = make_float2(w.x, w.z);
    tw[k + half] = make_float2(-w.x, -w.z);
  }
}

// The split of an M-point FFT Z of packed reals into X[k], k <= M:
// X[k] = E[k] + W_N^k O[k], E = (Z[k] + conj Z[M-k]) / 2,
// O = (Z[k] - conj Z[M-k]) / 2i (W_N^M = -1).
template <int M, typename T>
__device__ __forceinline__ T real_split(const T *line, int k, const T *tw) {
  const T zk = line[fpad(k % M)], zc = c_conj(line[fpad((M - k) % M)]);
  const T E = c_half(c_add(zk, zc)), O = c_div_2i(c_sub(zk, zc));
  return k == M ? c_sub(E, O) : c_add(E, k == 0 ? O : c_mul(tw[k], O));
}

// The twiddles of the FP32 row transforms in shared memory, from the
// float-float W_N^k table (N = 2M, high parts): tws[k] = W_N^k for k <= M / 2
// (the split) and twc[NS + k] = W_(NS R)^k, k < NS, for each pass NS > 1 of
// the M-point transform (NS a power of 8, R = min(8, M / NS); the ranges
// [NS, 2 NS) are disjoint).
template <int M>
__device__ __forceinline__ void load_tw_rows(float2 *tws, float2 *twc, const float4 *__restrict__ twff) {
  for (int e = threadIdx.x; e < M + M / 2 + 1; e += blockDim.x) {
    if (e <= M / 2) {
      const float4 w = twff[e];
      tws[e] = make_float2(w.x, w.z);
      continue;
    }
    const int c = e - (M / 2 + 1);
    int ns = 1;
    while (ns * 8 <= c) ns *= 8;
    const int k = c - ns;
    if (ns == 1 || k >= ns) continue;  // unused entries
    const int R = M / ns >= 8 ? 8 : M / ns;
    const float4 w = twff[k * (2 * M / (ns * R))];
    twc[c] = make_float2(w.x, w.z);
  }
}

// The split of the FP32 row transforms, two outputs per read pair: with
// E = (Z[k] + conj Z[M-k]) / 2, O = (Z[k] - conj Z[M-k]) / 2i and
// P = W_N^k O, X[k] = E + P and X[M - k] = conj(E - P) (E and O of M - k are
// the conjugates of those of k, W_N^(M-k) = -conj W_N^k); k = 0 gives X[0]
// and X[M], and its thread adds X[M/2].  Line b at s + b rowline_pitch<M>(),
// element i at fswz(i); task t of line b for t < M / 2, consecutive t on
// consecutive threads.
//
// Line pitch: M elements where a half warp's 16 threads lie in one line
// (M >= 128); shorter lines are M + M / 8 apart, so that the two or more
// lines of a half warp start on different banks.
template <int M>
constexpr int rowline_pitch() {
  return M >= 128 ? M : M + M / 8;
}
//
// The row kernels run 12 lines of M / 8 threads, i.e. 3 M / 2 threads:
// thread x takes t = x mod (M / 2) in lines x / (M / 2) + 3 i, so its two
// read addresses within a line and its twiddle serve all of its lines.
template <int M, int NL, typename Out>
__device__ __forceinline__ void split_pairs(const float2 *s, const float2 *tws, Out out) {
  constexpr int H = M / 2, LP = rowline_pitch<M>(), BS = 3;  // blockDim.x = BS H
  static_assert(NL % BS == 0, "split_pairs: lines in groups of three");
  const int t = threadIdx.x % H, b0 = threadIdx.x / H;
  const int ik = fswz(t), im = fswz((M - t) & (M - 1));
  const float2 w = tws[t];
#pragma unroll
  for (int i = 0; i < NL / BS; ++i) {
    const int b = b0 + BS * i;
    const float2 *line = s + b * LP;
    const float2 zk = line[ik], zm = c_conj(line[im]);
    const float2 E = c_half(c_add(zk, zm)), O = c_div_2i(c_sub(zk, zm));
    const float2 P = c_mul(w, O);
    out(b, t, c_add(E, P));
    out(b, M - t, c_conj(c_sub(E, P)));
    if (t == 0) {
      const float2 zh = line[fswz(H)], zhc = c_conj(zh);
      out(b, H, c_add(c_half(c_add(zh, zhc)), c_mul(tws[H], c_div_2i(c_sub(zh, zhc)))));
    }
  }
}

constexpr int kFfRows = 8;   // rows per CTA of the float-float real row pass
constexpr int kFfCRows = 4;  // rows per CTA of the float-float complex row pass
constexpr int kFfCols = 4;   // kx columns per CTA of the float-float column passes (64 bytes)

// Row pass: kFfRows rows of N = 2M reals -> M + 1 complex each (float-float).
template <int M>
__global__ void __launch_bounds__(kFfRows * M / 8) k_ff_rows(const double *__restrict__ in, float4 *__restrict__ out,
                                                             int64_t rows, const float4 *__restrict__ twff) {
  constexpr int N = 2 * M, NH = M + 1, TH = M / 8, LP = M + M / 8;
  __shared__ float4 s[kFfRows * LP];
  __shared__ float4 tw[N];  // W_N^k, k < N
  load_tw(tw, twff, M);
  const int64_t r0 = (int64_t)blockIdx.x * kFfRows;
  const int ln = threadIdx.x / TH, j = threadIdx.x % TH;
  const bool ok = r0 + ln < rows;
  const double2 *x = reinterpret_cast<const double2 *>(in + (r0 + ln) * N);
  float4 v[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = ok ? c_from(x[j + r * TH]) : c_zero<float4>();
  __syncthreads();  // twiddles
  float4 *line = s + ln * LP;
  f_stockham<M, 1, false>(v, j, line, 1, tw, 2, [&](int i, float4 z) { line[fpad(i)] = z; });  // W_M = W_N^2
  __syncthreads();
  for (int idx = threadIdx.x; idx < kFfRows * NH; idx += blockDim.x) {
    const int b = idx / NH, k = idx % NH;
    if (r0 + b < rows) out[(r0 + b) * NH + k] = real_split<M>(s + b * LP, k, tw);
  }
}

// Complex row pass: kFfCRows contiguous rows of L complex doubles -> L
// float-float points each, transformed in place of the input (each CTA
// reads all of its rows before it writes).
template <int L, bool INV>
__global__ void __launch_bounds__(kFfCRows * L / 8) k_ff_rows_c2c(double2 *__restrict__ data, int64_t rows,
                                                                  const float4 *__restrict__ twff) {
  constexpr int TH = L / 8, LP = L + L / 8;
  __shared__ float4 s[kFfCRows * LP];
  __shared__ float4 tw[L];
  load_tw(tw, twff, L / 2);
  const int64_t r0 = (int64_t)blockIdx.x * kFfCRows;
  const int ln = threadIdx.x / TH, j = threadIdx.x % TH;
  const bool ok = r0 + ln < rows;
  float4 v[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = ok ? c_from(data[(r0 + ln) * L + j + r * TH]) : c_zero<float4>();
  __syncthreads();
  float4 *out = reinterpret_cast<float4 *>(data) + (r0 + ln) * L;
  f_stockham<L, 1, INV>(v, j, s + ln * LP, 1, tw, 1, [&](int i, float4 z) {
    if (ok) out[i] = z;
  });
}

// Column pass: L-point FFTs along an axis of the half spectrum for NC
// adjacent kx.  Line (o, kx): element j at (o / ninner) shi + (o % ninner)
// slo + j sj + kx.  Thread (j, c) of column c loads its first-pass inputs
// from global memory and the last pass stores there; with `last` (float-
// float only) the result goes out as double2 in place.
template <typename T, int L, int NC>
constexpr size_t cols_smem() {
  return ((size_t)(L + L / 8) * NC + L) * sizeof(T);
}

template <typename T, int L, int NC, bool INV>
__global__ void __launch_bounds__(NC * L / 8) k_cols(T *__restrict__ data, int nh, int ninner, int64_t shi,
                                                     int64_t slo, int64_t sj, const float4 *__restrict__ twff,
                                                     int last) {
  constexpr int TH = L / 8, LP = L + L / 8;
  extern __shared__ __align__(16) unsigned char cols_sm[];
  T *s = reinterpret_cast<T *>(cols_sm);
  T *tw = s + LP * NC;  // W_L^k, k < L
  load_tw(tw, twff, L / 2);
  const int nkb = (nh + NC - 1) / NC;
  const int o = blockIdx.x / nkb, kx0 = (blockIdx.x % nkb) * NC;
  const int64_t base = (int64_t)(o / ninner) * shi + (int64_t)(o % ninner) * slo + kx0;
  const int c = threadIdx.x % NC, j = threadIdx.x / NC;
  const bool ok = kx0 + c < nh;
  T v[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = ok ? data[base + (int64_t)(j + r * TH) * sj + c] : c_zero<T>();
  __syncthreads();  // twiddles
  f_stockham<L, 1, INV>(v, j, s + c, NC, tw, 1, [&](int i, T z) {
    if (!ok) return;
    const int64_t a = base + (int64_t)i * sj + c;
    if constexpr (sizeof(T) == 16) {
      if (last) {
        reinterpret_cast<double2 *>(data)[a] = make_double2(f2_to(re(z)), f2_to(im(z)));
        return;
      }
    }
    data[a] = z;
  });
}

// launch k_cols<T, L, NC, INV> (its shared memory may exceed the 48 KB default)
template <typename T, int L, int NC, bool INV>
int launch_cols(axg_ctx *ctx, const char *name, int64_t blocks, T *data, int nh, int ninner, int64_t shi, int64_t slo,
                int64_t sj, const float4 *tw, int last) {
  static bool attr = false;
  constexpr size_t sm = cols_smem<T, L, NC>();
  if (!attr && sm > 48 * 1024) {
    AXG_CUDA_TRY(ctx, cudaFuncSetAttribute(k_cols<T, L, NC, INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    attr = true;
  }
  AXG_LAUNCH(ctx, name, (k_cols<T, L, NC, INV>), (unsigned)blocks, NC * L / 8, sm, data, nh, ninner, shi, slo, sj, tw,
             last);
  return AXG_OK;
}

template <int L, bool INV>
int z2z_t(axg_ctx *ctx, double2 *data, const float4 *tw) {
  constexpr int n = L;
  const int64_t rows = (int64_t)n * n, plane = (int64_t)n * n, vol = plane * n;
  float4 *f = reinterpret_cast<float4 *>(data);
  AXG_LAUNCH(ctx, "fft_ff_rows_c2c", (k_ff_rows_c2c<L, INV>), (unsigned)((rows + kFfCRows - 1) / kFfCRows),
             kFfCRows * L / 8, 0, data, rows, tw);
  const int nkb = n / kFfCols;
  AXG_TRY((launch_cols<float4, L, kFfCols, INV>(ctx, "fft_ff_y", (int64_t)n * nkb, f, n, n, vol, plane, (int64_t)n,
                                                 tw, 0)));
  AXG_TRY((launch_cols<float4, L, kFfCols, INV>(ctx, "fft_ff_z", (int64_t)n * nkb, f, n, n, vol, (int64_t)n, plane,
                                                 tw, 1)));
  return AXG_OK;
}

// the y and z passes of a batched float-float D2Z whose row pass is done
template <int L>
int d2z_cols_t(axg_ctx *ctx, float4 *f, int batch, const float4 *tw, bool keep_ff) {
  constexpr int n = L, nh = L / 2 + 1;
  const int nkb = (nh + kFfCols - 1) / kFfCols;
  const int64_t plane = (int64_t)n * nh, vol = plane * n;
  // y: lines (field, z); z: lines (field, y)
  AXG_TRY((launch_cols<float4, L, kFfCols, false>(ctx, "fft_ff_y", (int64_t)batch * n * nkb, f, nh, n, vol, plane,
                                                   (int64_t)nh, tw, 0)));
  AXG_TRY((launch_cols<float4, L, kFfCols, false>(ctx, "fft_ff_z", (int64_t)batch * n * nkb, f, nh, n, vol,
                                                   (int64_t)nh, plane, tw, keep_ff ? 0 : 1)));
  return AXG_OK;
}

template <int L>
int d2z_t(axg_ctx *ctx, const double *in, double2 *out, int batch, const float4 *tw, bool keep_ff) {
  constexpr int n = L;
  const int64_t rows = (int64_t)batch * n * n;
  float4 *f = reinterpret_cast<float4 *>(out);
  AXG_LAUNCH(ctx, "fft_ff_rows", k_ff_rows<L / 2>, (unsigned)((rows + kFfRows - 1) / kFfRows), kFfRows * L / 16, 0,
             in, f, rows, tw);
  return d2z_cols_t<L>(ctx, f, batch, tw, keep_ff);
}

// FP64-plain Green step: the six FP64 sources (gw_sources_fp64, the
// reference's operations) formed inside the float-float row pass, so they
// never reach HBM.  One CTA per x-row (y, z): six lines, one per source, of
// M = N / 2 packed points z[m] = S(2m) + i S(2m + 1).  The FP64 pipe does
// the sources' arithmetic only; their float-float split runs on the integer
// pipes (f2_from_bits).  Output as k_ff_rows for batch 6.
// One thread per packed point m in the source phase (M threads, one round).
template <int M>
__global__ void __launch_bounds__(M) k_ff_gws_rows(const double2 *__restrict__ phi, double d, double inv_d,
                                                           int d_pow2, float4 *__restrict__ out,
                                                           const float4 *__restrict__ twff) {
  constexpr int N = 2 * M, NH = M + 1, TH = M / 8, LP = M + M / 8;
  __shared__ float4 s[8 * LP];
  __shared__ float4 tw[N];  // W_N^k, k < N
  load_tw(tw, twff, M);
  const int64_t row = blockIdx.x, nhalf = (int64_t)N * N * NH;
  const int y = (int)(row % N), z = (int)(row / N);
  const double2 *prow = phi + row * N;
  const double2 *pym = phi + ((int64_t)z * N + (y == 0 ? N - 1 : y - 1)) * N;
  const double2 *pyp = phi + ((int64_t)z * N + (y + 1 == N ? 0 : y + 1)) * N;
  const double2 *pzm = phi + ((int64_t)(z == 0 ? N - 1 : z - 1) * N + y) * N;
  const double2 *pzp = phi + ((int64_t)(z + 1 == N ? 0 : z + 1) * N + y) * N;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const int x0 = 2 * m;
    const double2 p0 = prow[x0], p1 = prow[x0 + 1];
    const double2 xm = prow[x0 == 0 ? N - 1 : x0 - 1], xp = prow[x0 + 2 == N ? 0 : x0 + 2];
    double S0[6], S1[6];
    {
      const double2 pa[3] = {p1, pyp[x0], pzp[x0]}, pb[3] = {xm, pym[x0], pzm[x0]};
      gw_sources_fp64(pa, pb, d, inv_d, d_pow2, S0);
    }
    {
      const double2 pa[3] = {xp, pyp[x0 + 1], pzp[x0 + 1]}, pb[3] = {p0, pym[x0 + 1], pzm[x0 + 1]};
      gw_sources_fp64(pa, pb, d, inv_d, d_pow2, S1);
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) s[c * LP + fpad(m)] = cx(f2_from_bits(S0[c]), f2_from_bits(S1[c]));
    s[6 * LP + fpad(m)] = s[7 * LP + fpad(m)] = c_zero<float4>();
  }
  __syncthreads();
  {
    // M threads = 8 lines of M / 8: lines 6 and 7 are scratch, transformed
    // so that every thread reaches the same barriers, and never read
    const int ln = threadIdx.x / TH, j = threadIdx.x % TH;
    float4 *line = s + ln * LP;
    float4 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = line[fpad(j + r * TH)];
    __syncthreads();
    f_stockham<M, 1, false>(v, j, line, 1, tw, 2, [&](int i, float4 x) { line[fpad(i)] = x; });  // W_M = W_N^2
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < 6 * NH; idx += blockDim.x) {
    const int b = idx / NH, k = idx % NH;
    out[b * nhalf + row * NH + k] = real_split<M>(s + b * LP, k, tw);
  }
}

template <int L>
int ff_gws_d2z_t(axg_ctx *ctx, const double2 *phi, double d, double inv_d, int d_pow2, double2 *out,
                 const float4 *tw, bool keep_ff) {
  constexpr int n = L, M = L / 2;
  float4 *f = reinterpret_cast<float4 *>(out);
  AXG_LAUNCH(ctx, "gw_source_rows_fp64", k_ff_gws_rows<M>, (unsigned)((int64_t)n * n), M, 0, phi, d, inv_d, d_pow2,
             f, tw);
  return d2z_cols_t<L>(ctx, f, 6, tw, keep_ff);
}

// ---------------------------------------------------------------------------
// FP32 transform of the six Green's-function sources, the source computation
// fused into the row pass.  The FP32-mixed Green step needs the forward
// transforms of S_ij = (2 / d^2) (dr_i dr_j + di_i di_j), d_i the raw
// central differences of phi: the row kernel forms S_ij for its rows from
// phi (the stencil rows come through L1 / L2) and runs the real-to-half x
// transform of all six at once, so the real sources never reach HBM; the y
// and z passes are the column passes in complex float.  Output as cuFFT's
// R2C: [6][n][n][n/2+1] complex float.  Twiddles are the high parts of the
// float-float table, i.e. W_n^k rounded to float.

constexpr int kSrcRows = 2;  // x-rows per CTA of the source row pass (6 x 2 lines)

// Opts a kernel into `smem` bytes of dynamic shared memory above the 48 KB
// default on the current device (a host-side call, repeated per launch so
// that every device a context runs on gets it)
template <typename K>
int allow_smem(axg_ctx *ctx, K kern, size_t smem) {
  if (smem > 48 * 1024)
    AXG_CUDA_TRY(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  return AXG_OK;
}

// Dynamic shared memory of the FP32 row kernels: nl lines, then the split
// and per-pass twiddles
template <int M>
constexpr size_t rows_f32_smem(int nl) {
  return ((size_t)nl * rowline_pitch<M>() + (M / 2 + 1) + M) * sizeof(float2);
}

// Row pass with the sources, for rows (y, z) = row0 .. row0 + kSrcRows - 1
// of the N = 2M lattice.  Line c kSrcRows + r holds source c of row r
// packed as M complex points z[m] = S(2m) + i S(2m + 1); an M-point FFT per
// line (M / 8 threads each), then the split into X[k], k <= M.
template <int M>
__global__ void __launch_bounds__(6 * kSrcRows * M / 8) k_gws_rows(const float2 *__restrict__ phi, float scale,
                                                                   float2 *__restrict__ out, int sp,
                                                                   const float4 *__restrict__ twff) {
  constexpr int N = 2 * M, NL = 6 * kSrcRows, TH = M / 8, LP = rowline_pitch<M>();
  extern __shared__ __align__(16) unsigned char rows_sm[];
  float2 *s = reinterpret_cast<float2 *>(rows_sm);
  float2 *tws = s + NL * LP, *twc = tws + (M / 2 + 1);
  load_tw_rows<M>(tws, twc, twff);
  const int64_t row0 = (int64_t)blockIdx.x * kSrcRows, nspec = (int64_t)N * N * sp;
  // Sources: thread m < M forms both rows' six sources at x = 2m, 2m + 1.
  // The rows are y0 and y0 + 1 of one z plane (y0 even), so their
  // y-neighbours are the rows y0 - 1 .. y0 + 2, two of them the rows
  // themselves: 12 loads for the pair instead of 14.
  static_assert(kSrcRows == 2, "the source phase pairs rows y0 and y0 + 1");
  const int y0 = (int)(row0 % N), z = (int)(row0 / N);
  const int64_t zr = (int64_t)z * N, zmr = (int64_t)(z == 0 ? N - 1 : z - 1) * N,
                zpr = (int64_t)(z + 1 == N ? 0 : z + 1) * N;
  const float2 *r0 = phi + (zr + y0) * N, *r1 = r0 + N;
  const float2 *rym = phi + (zr + (y0 == 0 ? N - 1 : y0 - 1)) * N;
  const float2 *ryp = phi + (zr + (y0 + 2 == N ? 0 : y0 + 2)) * N;
  const float2 *rzm0 = phi + (zmr + y0) * N, *rzm1 = rzm0 + N;
  const float2 *rzp0 = phi + (zpr + y0) * N, *rzp1 = rzp0 + N;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const int x0 = 2 * m, xl = x0 == 0 ? N - 1 : x0 - 1, xr = x0 + 2 == N ? 0 : x0 + 2;
    auto ld4 = [&](const float2 *row) { return *reinterpret_cast<const float4 *>(row + x0); };
    const float4 a_m = ld4(rym), a_0 = ld4(r0), a_1 = ld4(r1), a_p = ld4(ryp);
    const float4 zm0 = ld4(rzm0), zm1 = ld4(rzm1), zp0 = ld4(rzp0), zp1 = ld4(rzp1);
    const float2 xm0 = r0[xl], xp0 = r0[xr], xm1 = r1[xl], xp1 = r1[xr];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const float4 c01 = r ? a_1 : a_0, pym = r ? a_0 : a_m, pyp = r ? a_p : a_1;  // phi(x0), phi(x0 + 1)
      const float4 pzm = r ? zm1 : zm0, pzp = r ? zp1 : zp0;
      const float2 xm = r ? xm1 : xm0, xp = r ? xp1 : xp0;
      float S[2][6];
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        float dr[3], di[3];
        dr[0] = t == 0 ? c01.z - xm.x : xp.x - c01.x;
        di[0] = t == 0 ? c01.w - xm.y : xp.y - c01.y;
        dr[1] = t == 0 ? pyp.x - pym.x : pyp.z - pym.z;
        di[1] = t == 0 ? pyp.y - pym.y : pyp.w - pym.w;
        dr[2] = t == 0 ? pzp.x - pzm.x : pzp.z - pzm.z;
        di[2] = t == 0 ? pzp.y - pzm.y : pzp.w - pzm.w;
        int c = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j <= i; ++j, ++c) S[t][c] = scale * (dr[i] * dr[j] + di[i] * di[j]);
      }
#pragma unroll
      for (int c = 0; c < 6; ++c) s[(c * kSrcRows + r) * LP + fswz(m)] = make_float2(S[0][c], S[1][c]);
    }
  }
  __syncthreads();
  {
    const int ln = threadIdx.x / TH, j = threadIdx.x % TH;
    float2 *line = s + ln * LP;
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = line[fswz(j + r * TH)];
    __syncthreads();
    f_stockham<M, 1, false, true, true>(v, j, line, 1, twc, 1, [&](int i, float2 x) { line[fswz(i)] = x; });
  }
  __syncthreads();
  split_pairs<M, NL>(s, tws, [&](int b, int k, float2 x) {
    out[(b / kSrcRows) * nspec + (row0 + b % kSrcRows) * sp + k] = x;
  });
}

// The u_ij spectrum's twelve real fields, tau u_c and u_c + tau u'_c (c =
// 11, 21, 22, 31, 32, 33; FP32-mixed subtracts the Kahan compensation from
// u first), formed inside the row pass as the Green sources are: one CTA per
// x-row, twelve lines.  Output [12][n][n][n/2+1] complex float.
template <int M>
__global__ void __launch_bounds__(12 * M / 8) k_uij_rows(const float *__restrict__ u, const float *__restrict__ ud,
                                                         const float *__restrict__ cu, int64_t n3, float tau,
                                                         float2 *__restrict__ out, int sp,
                                                         const float4 *__restrict__ twff) {
  constexpr int N = 2 * M, TH = M / 8, LP = rowline_pitch<M>();
  extern __shared__ __align__(16) unsigned char rows_sm[];
  float2 *s = reinterpret_cast<float2 *>(rows_sm);
  float2 *tws = s + 12 * LP, *twc = tws + (M / 2 + 1);
  load_tw_rows<M>(tws, twc, twff);
  const int64_t row = blockIdx.x, nspec = (int64_t)N * N * sp;
  for (int idx = threadIdx.x; idx < 6 * M; idx += blockDim.x) {
    const int c = idx / M, m = idx % M;
    const int64_t x = c * n3 + row * N + 2 * m;
    float2 uv = *reinterpret_cast<const float2 *>(u + x);
    if (cu) {
      const float2 cv = *reinterpret_cast<const float2 *>(cu + x);
      uv.x -= cv.x;
      uv.y -= cv.y;
    }
    const float2 dv = *reinterpret_cast<const float2 *>(ud + x);
    s[c * LP + fswz(m)] = make_float2(tau * uv.x, tau * uv.y);
    s[(6 + c) * LP + fswz(m)] = make_float2(uv.x + tau * dv.x, uv.y + tau * dv.y);
  }
  __syncthreads();
  {
    const int ln = threadIdx.x / TH, j = threadIdx.x % TH;
    float2 *line = s + ln * LP;
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = line[fswz(j + r * TH)];
    __syncthreads();
    f_stockham<M, 1, false, true, true>(v, j, line, 1, twc, 1, [&](int i, float2 x) { line[fswz(i)] = x; });
  }
  __syncthreads();
  split_pairs<M, 12>(s, tws, [&](int b, int k, float2 x) { out[b * nspec + row * sp + k] = x; });
}

// The same twelve fields in FP64 (tau u_c and u_c + tau u'_c), split into
// float-float on the integer pipes, in the float-float row pass.  Two CTAs
// per x-row, six fields each; M threads, lines 6 and 7 scratch as in
// k_ff_gws_rows.
template <int M>
__global__ void __launch_bounds__(M) k_ff_uij_rows(const double *__restrict__ u, const double *__restrict__ ud,
                                                   int64_t n3, double tau, float4 *__restrict__ out,
                                                   const float4 *__restrict__ twff) {
  constexpr int N = 2 * M, NH = M + 1, TH = M / 8, LP = M + M / 8;
  __shared__ float4 s[8 * LP];
  __shared__ float4 tw[N];  // W_N^k, k < N
  load_tw(tw, twff, M);
  const int half = (int)(blockIdx.x & 1);
  const int64_t row = blockIdx.x >> 1, nhalf = (int64_t)N * N * NH;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const int64_t x = row * N + 2 * m;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const double2 uv = *reinterpret_cast<const double2 *>(u + c * n3 + x);
      double2 w;
      if (half == 0) {
        w = make_double2(tau * uv.x, tau * uv.y);
      } else {
        const double2 dv = *reinterpret_cast<const double2 *>(ud + c * n3 + x);
        w = make_double2(uv.x + tau * dv.x, uv.y + tau * dv.y);
      }
      s[c * LP + fpad(m)] = cx(f2_from_bits(w.x), f2_from_bits(w.y));
    }
    s[6 * LP + fpad(m)] = s[7 * LP + fpad(m)] = c_zero<float4>();
  }
  __syncthreads();
  {
    const int ln = threadIdx.x / TH, j = threadIdx.x % TH;
    float4 *line = s + ln * LP;
    float4 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = line[fpad(j + r * TH)];
    __syncthreads();
    f_stockham<M, 1, false>(v, j, line, 1, tw, 2, [&](int i, float4 x) { line[fpad(i)] = x; });  // W_M = W_N^2
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < 6 * NH; idx += blockDim.x) {
    const int b = idx / NH, k = idx % NH;
    out[(half * 6 + b) * nhalf + row * NH + k] = real_split<M>(s + b * LP, k, tw);
  }
}

// z pass of the complex-float half spectra through TMA.  Persistent CTAs
// walk tiles of kFzCols kx columns x L z-points (one ky row of one field);
// a tile arrives by cp.async.bulk.tensor in one of kFzStages shared-memory
// stages while the CTA transforms the one before, and leaves by a bulk
// tensor store from its own stage.  The spectra's rows are padded
// (axg_f32_spec_pitch) so that their byte stride suits TMA; the last kx
// block reaches past the pitch, where TMA loads zeros and drops the stores.
// Each z-line is 64 bytes wide in 512 planes a megabyte apart: the plain
// column kernel reached 0.53 of the DRAM peak on it, limited by the loads in
// flight.  A stage wait that runs out raises AXG_KERR_MBAR_TIMEOUT.
constexpr int kFzCols = 8;    // kx columns per tile: 64-byte boxes
constexpr int kFzStages = 2;  // 3 and 4 stages at one CTA per SM measured slower
constexpr int kFyCols = 4;    // kx columns per CTA of the y pass (32-byte rows, sector aligned at the padded pitch)

template <int L>
constexpr size_t zt_smem() {
  return (size_t)(kFzStages * L * kFzCols + (L + L / 8) * kFzCols + L) * sizeof(float2) + 8 * kFzStages + 16 + 128;
}

template <int L>
__global__ void __launch_bounds__(kFzCols * L / 8, (1024 / (kFzCols * L / 8)) < 32 ? 1024 / (kFzCols * L / 8) : 32)
    k_cols_z_tma(const __grid_constant__ CUtensorMap tm, int nkb, int ny, int ntiles,
                 const float4 *__restrict__ twff, int *err) {
  using namespace axg_tma;
  constexpr int TH = L / 8, LP = L + L / 8, TILE = L * kFzCols, BOX = L < 256 ? L : 256, S = kFzStages;
  constexpr uint32_t BYTES = TILE * sizeof(float2);
  extern __shared__ unsigned char zt_raw[];
  unsigned char *sm =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(zt_raw) + 127) & ~uintptr_t(127));
  float2 *tile = reinterpret_cast<float2 *>(sm);  // [S][L][kFzCols], dense as the TMA box
  float2 *xb = tile + S * TILE;                    // exchange lines, element i of column c at fpad(i) kFzCols + c
  float2 *tw = xb + LP * kFzCols;                  // W_L^k, k < L
  uint64_t *bars = reinterpret_cast<uint64_t *>(tw + L);
  int &fail = *reinterpret_cast<int *>(bars + S);
  load_tw(tw, twff, L / 2);
  const uint32_t bar0 = smem_u32(bars);
  if (threadIdx.x == 0) {
    for (int q = 0; q < S; ++q) mbar_init(bar0 + 8 * q, 1);
    fence_barrier_init();
    fail = 0;
  }
  __syncthreads();
  auto issue = [&](int t, int st) {  // tile t: (field, ky) = o, kx block kb
    const int o = t / nkb, kb = t % nkb;
    const uint32_t dst = smem_u32(tile + st * TILE), bar = bar0 + 8 * st;
    mbar_expect_tx(bar, BYTES);
#pragma unroll
    for (int h = 0; h < L / BOX; ++h)
      tma_load_4d(dst + h * BOX * kFzCols * (int)sizeof(float2), &tm, kb * kFzCols, o % ny, h * BOX, o / ny, bar);
  };
  if (threadIdx.x == 0)
    for (int q = 0; q < S - 1; ++q)
      if (blockIdx.x + q * (int)gridDim.x < ntiles) issue(blockIdx.x + q * gridDim.x, q);
  const int c = threadIdx.x % kFzCols, j = threadIdx.x / kFzCols;
  int i = 0;
  for (int t = blockIdx.x; t < ntiles; ++i, t += gridDim.x) {
    const int st = i % S;
    const int tn = t + (S - 1) * (int)gridDim.x;
    if (threadIdx.x == 0 && tn < ntiles) {
      bulk_wait_read0();  // the store of the previous tile, from the stage about to be refilled, has read it
      issue(tn, (i + S - 1) % S);
    }
    if (!mbar_wait_bounded(bar0 + 8 * st, (i / S) & 1)) fail = 1;
    __syncthreads();
    if (fail) break;
    float2 *tl = tile + st * TILE;
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = tl[(j + r * TH) * kFzCols + c];
    f_stockham<L, 1, false>(v, j, xb + c, kFzCols, tw, 1, [&](int ii, float2 z) { tl[ii * kFzCols + c] = z; });
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      const int o = t / nkb, kb = t % nkb;
      const uint32_t src = smem_u32(tl);
#pragma unroll
      for (int h = 0; h < L / BOX; ++h)
        tma_store_4d(&tm, src + h * BOX * kFzCols * (int)sizeof(float2), kb * kFzCols, o % ny, h * BOX, o / ny);
      bulk_commit();
    }
  }
  if (threadIdx.x == 0) {
    if (fail) {
      atomicCAS(err, 0, AXG_KERR_MBAR_TIMEOUT);
      for (int q = 1; q < S; ++q) mbar_wait_bounded(bar0 + 8 * ((i + q) % S), ((i + q) / S) & 1, 100000000LL);
    }
    bulk_wait0();
  }
}

// y and z passes in complex float of `batch` half spectra, rows of pitch sp
// (axg_f32_spec_pitch): the y pass by k_cols (kFyCols columns, 32-byte
// rows on sector boundaries), the z pass by k_cols_z_tma
template <int L>
int f_cols_t(axg_ctx *ctx, float2 *out, int batch, int sp, const float4 *tw) {
  constexpr int n = L, nh = L / 2 + 1;
  const int64_t plane = (int64_t)n * sp, vol = plane * n;
  const int nky = (nh + kFyCols - 1) / kFyCols;
  AXG_TRY((launch_cols<float2, L, kFyCols, false>(ctx, "fft_f32_y", (int64_t)batch * n * nky, out, nh, n, vol, plane,
                                                   (int64_t)sp, tw, 0)));
  CUtensorMap m;
  constexpr int BOX = L < 256 ? L : 256;
  const cuuint64_t dims[4] = {(cuuint64_t)sp, (cuuint64_t)n, (cuuint64_t)n, (cuuint64_t)batch};
  const cuuint64_t str[3] = {(cuuint64_t)sp * 8, (cuuint64_t)plane * 8, (cuuint64_t)vol * 8};
  const cuuint32_t box[4] = {kFzCols, 1, BOX, 1};
  AXG_TRY(axg_encode_tmap(ctx, &m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, out, dims, str, box));  // (re, im) float pairs
  constexpr size_t smem = zt_smem<L>();
  constexpr int threads = kFzCols * L / 8;
  AXG_TRY(allow_smem(ctx, k_cols_z_tma<L>, smem));
  AXG_CUDA_TRY(ctx, cudaFuncSetAttribute(k_cols_z_tma<L>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  int per_sm = 0, sms = 0;
  AXG_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cols_z_tma<L>, threads, smem));
  if (per_sm < 1) return axg_set_error(ctx, AXG_ERR_CUDA, "z-pass kernel does not fit on an SM");
  AXG_CUDA_TRY(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const int nkb = (nh + kFzCols - 1) / kFzCols, ntiles = batch * n * nkb;
  const int grid = std::min(ntiles, sms * per_sm);
  AXG_LAUNCH(ctx, "fft_f32_z", k_cols_z_tma<L>, (unsigned)grid, threads, smem, m, nkb, n, ntiles, tw, ctx->d_err);
  return AXG_OK;
}

template <int L>
int uij_r2c_t(axg_ctx *ctx, const float *u, const float *ud, const float *cu, float tau, float2 *out,
              const float4 *tw) {
  constexpr int n = L, M = L / 2;
  const int sp = axg_f32_spec_pitch(n);
  constexpr size_t smem = rows_f32_smem<M>(12);
  AXG_TRY(allow_smem(ctx, k_uij_rows<M>, smem));
  AXG_LAUNCH(ctx, "uij_rows_fp32", k_uij_rows<M>, (unsigned)((int64_t)n * n), 12 * M / 8, smem, u, ud, cu,
             (int64_t)n * n * n, tau, out, sp, tw);
  return f_cols_t<L>(ctx, out, 12, sp, tw);
}

template <int L>
int ff_uij_d2z_t(axg_ctx *ctx, const double *u, const double *ud, double tau, double2 *out, const float4 *tw) {
  constexpr int n = L, M = L / 2;
  float4 *f = reinterpret_cast<float4 *>(out);
  AXG_LAUNCH(ctx, "uij_rows_fp64", k_ff_uij_rows<M>, (unsigned)(2 * (int64_t)n * n), M, 0, u, ud,
             (int64_t)n * n * n, tau, f, tw);
  return d2z_cols_t<L>(ctx, f, 12, tw, false);
}

template <int L>
int gws_r2c_t(axg_ctx *ctx, const float2 *phi, float2 *out, float scale, const float4 *tw) {
  constexpr int n = L, M = L / 2;
  const int64_t rows = (int64_t)n * n;
  const int sp = axg_f32_spec_pitch(n);
  constexpr size_t smem = rows_f32_smem<M>(6 * kSrcRows);
  AXG_TRY(allow_smem(ctx, k_gws_rows<M>, smem));
  AXG_LAUNCH(ctx, "gw_source_rows_fp32", k_gws_rows<M>, (unsigned)(rows / kSrcRows), 6 * kSrcRows * M / 8, smem,
             phi, scale, out, sp, tw);
  return f_cols_t<L>(ctx, out, 6, sp, tw);
}

}  // namespace

// 16..512: the sizes the tests and the benchmark run; larger N keep cuFFT
bool axg_ff_fft_supported(int n) { return n >= 16 && n <= 512 && (n & (n - 1)) == 0; }

bool axg_ff_use(int n) {
  const char *env = std::getenv("AXG_FFT_FF");
  return axg_ff_fft_supported(n) && !(env && env[0] == '0');
}

namespace {
int ensure_twiddles(axg_ctx *ctx, int n) {
  if (ctx->ff_tw_n != n) {
    axg_free(ctx, (void **)&ctx->ff_tw);
    ctx->ff_tw_n = 0;
    // W_n^k = exp(-2 pi i k / n), k < n / 2, split into float-float on the host
    std::vector<float> h((size_t)n / 2 * 4);
    const double two_pi = 6.283185307179586476925286766559;
    for (int k = 0; k < n / 2; ++k) {
      const double c = std::cos(two_pi * k / n), s = -std::sin(two_pi * k / n);
      const float ch = (float)c, sh = (float)s;
      h[4 * k + 0] = ch;
      h[4 * k + 1] = (float)(c - (double)ch);
      h[4 * k + 2] = sh;
      h[4 * k + 3] = (float)(s - (double)sh);
    }
    AXG_TRY(axg_alloc(ctx, (void **)&ctx->ff_tw, h.size() * sizeof(float), "FFT twiddles"));
    AXG_CUDA_TRY(ctx, cudaMemcpy(ctx->ff_tw, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    ctx->ff_tw_n = n;
  }
  return AXG_OK;
}
}  // namespace

int axg_ff_z2z(axg_ctx *ctx, double2 *data, int n, int inverse) {
  if (!axg_ff_fft_supported(n)) return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "float-float FFT size");
  AXG_TRY(ensure_twiddles(ctx, n));
  const float4 *tw = reinterpret_cast<const float4 *>(ctx->ff_tw);
#define AXG_FF_Z2Z(L) \
  case L: return inverse ? z2z_t<L, true>(ctx, data, tw) : z2z_t<L, false>(ctx, data, tw);
  switch (n) {
    AXG_FF_Z2Z(16)
    AXG_FF_Z2Z(32)
    AXG_FF_Z2Z(64)
    AXG_FF_Z2Z(128)
    AXG_FF_Z2Z(256)
    AXG_FF_Z2Z(512)
    default: return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "float-float FFT size");
  }
#undef AXG_FF_Z2Z
}

int axg_ff_d2z(axg_ctx *ctx, const double *in, double2 *out, int n, int batch, bool keep_ff) {
  if (!axg_ff_fft_supported(n)) return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "float-float FFT size");
  AXG_TRY(ensure_twiddles(ctx, n));
  const float4 *tw = reinterpret_cast<const float4 *>(ctx->ff_tw);
  switch (n) {
    case 16: return d2z_t<16>(ctx, in, out, batch, tw, keep_ff);
    case 32: return d2z_t<32>(ctx, in, out, batch, tw, keep_ff);
    case 64: return d2z_t<64>(ctx, in, out, batch, tw, keep_ff);
    case 128: return d2z_t<128>(ctx, in, out, batch, tw, keep_ff);
    case 256: return d2z_t<256>(ctx, in, out, batch, tw, keep_ff);
    case 512: return d2z_t<512>(ctx, in, out, batch, tw, keep_ff);
    default: return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "float-float FFT size");
  }
}

int axg_gw_source_r2c_f32(axg_ctx *ctx, const float2 *phi, float2 *out, int n, float scale) {
  if (!axg_ff_fft_supported(n)) return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "FP32 source transform size");
  AXG_TRY(ensure_twiddles(ctx, n));
  const float4 *tw = reinterpret_cast<const float4 *>(ctx->ff_tw);
  switch (n) {
    case 16: return gws_r2c_t<16>(ctx, phi, out, scale, tw);
    case 32: return gws_r2c_t<32>(ctx, phi, out, scale, tw);
    case 64: return gws_r2c_t<64>(ctx, phi, out, scale, tw);
    case 128: return gws_r2c_t<128>(ctx, phi, out, scale, tw);
    case 256: return gws_r2c_t<256>(ctx, phi, out, scale, tw);
    case 512: return gws_r2c_t<512>(ctx, phi, out, scale, tw);
    default: return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "FP32 source transform size");
  }
}

int axg_gw_source_d2z_ff(axg_ctx *ctx, const double2 *phi, double d, double inv_d, int d_pow2, double2 *out, int n,
                         bool keep_ff) {
  if (!axg_ff_fft_supported(n)) return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "float-float FFT size");
  AXG_TRY(ensure_twiddles(ctx, n));
  const float4 *tw = reinterpret_cast<const float4 *>(ctx->ff_tw);
  switch (n) {
    case 16: return ff_gws_d2z_t<16>(ctx, phi, d, inv_d, d_pow2, out, tw, keep_ff);
    case 32: return ff_gws_d2z_t<32>(ctx, phi, d, inv_d, d_pow2, out, tw, keep_ff);
    case 64: return ff_gws_d2z_t<64>(ctx, phi, d, inv_d, d_pow2, out, tw, keep_ff);
    case 128: return ff_gws_d2z_t<128>(ctx, phi, d, inv_d, d_pow2, out, tw, keep_ff);
    case 256: return ff_gws_d2z_t<256>(ctx, phi, d, inv_d, d_pow2, out, tw, keep_ff);
    case 512: return ff_gws_d2z_t<512>(ctx, phi, d, inv_d, d_pow2, out, tw, keep_ff);
    default: return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "float-float FFT size");
  }
}

int axg_uij_r2c_f32(axg_ctx *ctx, const float *u, const float *ud, const float *cu, float tau, float2 *out, int n) {
  if (!axg_ff_fft_supported(n)) return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "FP32 u_ij transform size");
  AXG_TRY(ensure_twiddles(ctx, n));
  const float4 *tw = reinterpret_cast<const float4 *>(ctx->ff_tw);
  switch (n) {
    case 16: return uij_r2c_t<16>(ctx, u, ud, cu, tau, out, tw);
    case 32: return uij_r2c_t<32>(ctx, u, ud, cu, tau, out, tw);
    case 64: return uij_r2c_t<64>(ctx, u, ud, cu, tau, out, tw);
    case 128: return uij_r2c_t<128>(ctx, u, ud, cu, tau, out, tw);
    case 256: return uij_r2c_t<256>(ctx, u, ud, cu, tau, out, tw);
    case 512: return uij_r2c_t<512>(ctx, u, ud, cu, tau, out, tw);
    default: return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "FP32 u_ij transform size");
  }
}

int axg_uij_d2z_ff(axg_ctx *ctx, const double *u, const double *ud, double tau, double2 *out, int n) {
  if (!axg_ff_fft_supported(n)) return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "float-float FFT size");
  AXG_TRY(ensure_twiddles(ctx, n));
  const float4 *tw = reinterpret_cast<const float4 *>(ctx->ff_tw);
  switch (n) {
    case 16: return ff_uij_d2z_t<16>(ctx, u, ud, tau, out, tw);
    case 32: return ff_uij_d2z_t<32>(ctx, u, ud, tau, out, tw);
    case 64: return ff_uij_d2z_t<64>(ctx, u, ud, tau, out, tw);
    case 128: return ff_uij_d2z_t<128>(ctx, u, ud, tau, out, tw);
    case 256: return ff_uij_d2z_t<256>(ctx, u, ud, tau, out, tw);
    case 512: return ff_uij_d2z_t<512>(ctx, u, ud, tau, out, tw);
    default: return axg_set_error(ctx, AXG_ERR_UNSUPPORTED, "float-float FFT size");
  }
}
