// axg_defects.cu -- defect identification on the GPU (defects_3d.f90).
//
// This translation unit is compiled with -fmad=false: every floating-point
// expression below rounds each operation separately, exactly as IEEE host C
// does without contraction, and the FP64 atan2 / sin / cos are the
// deterministic versions of axg_detmath.h.  Cell flags, counts, plaquette
// windings and every per-cell fit (position, direction, length, velocity,
// wall area) are therefore bit-identical to a host evaluation of the same
// formulas.  FP32 phases (atan2f) serve only as a filter that decides the
// cells whose outcome cannot change within their error bound; all other
// cells go through the FP64 path.
//
// Passes (all O(N^3) passes are HBM-streaming, the fits are sparse):
//   1. phase     : ph[s] = atan2f(Im phi, Re phi), FP32         (4 B / site)
//   2. classify  : 8 corner phases, sort, largest circular gap -> int8 flags,
//                  warp-aggregated counts (defects_3d.f90:67-103, 309-349).
//                  Filtered: the FP32 phases are within 1e-6 of the FP64
//                  ones, and sorting moves no value by more than that, so a
//                  cell whose every decision (wall gap against wrap gap,
//                  largest gap against pi and 7 pi / 4) clears a 2e-5
//                  margin has the FP64 flags; any other cell is redone from
//                  phi with the deterministic FP64 atan2, as on the host.
//   3. winding   : three plaquettes per site, filtered the same way (a
//                  corner difference within the margin of +-pi is redone in
//                  FP64)
//   4. compaction: string and wall cells listed in cell order
//   5. fits      : string cells lane-scheduled from a counter -- the search
//                  of position_string (1001 random starts, screened in FP32,
//                  + Nelder-Mead, defects_3d.f90:435-603; the chi2 in
//                  float-float on the FP32 pipes, axg_ffchi2.h), string_length
//                  (1027-1056), velocity_string (605-692), position_wall
//                  (1058-1233)
//   6. sums      : add_string_length / add_wall_area without grouping
#include <cmath>

#include "axg_detmath.h"
#include "axg_ffchi2.h"
#include "axg_internal.h"

namespace {

constexpr double kRefPi = 3.14159265359;
constexpr double kRefTwoPi = 2 * kRefPi;
constexpr double kStringPhdiff = kRefPi;
constexpr double kRemovalPhdiff = 7 * kRefPi / 4;
constexpr int kMaxIter = 1000;
constexpr int kNumSimp = 4;

// The FP64 value of site s.  comp: the Kahan compensation of an FP32-mixed
// phi (else null); the value is then (double)v - (double)c, the snapshot
// axg_download returns, so the FP64 decisions are those of the host's
// classification of the downloaded field.
template <typename V>
__device__ __forceinline__ void load_c(const V *a, const V *comp, int64_t s, double &re, double &im) {
  const V v = a[s];
  re = (double)v.x;
  im = (double)v.y;
  if (comp) {
    const V c = comp[s];
    re = re - (double)c.x;
    im = im - (double)c.y;
  }
}

// FP32 phase of each site.  For an FP64 field a component outside the FP32
// normal range (and not zero) would lose relative precision in conversion:
// such sites get NaN and every cell touching them is classified in FP64.
template <typename V>
__global__ void k_phase32(const V *__restrict__ phi, float *__restrict__ ph, int64_t n3) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride) {
    const V v = phi[s];
    if constexpr (sizeof(v.x) == 4) {
      ph[s] = atan2f(v.y, v.x);
    } else {
      auto in_range = [](double x) {
        const long long b = __double_as_longlong(x) & 0x7fffffffffffffffLL;
        const int e = (int)(b >> 52);
        return b == 0 || (e >= 1023 - 126 && e <= 1023 + 127);
      };
      ph[s] = (in_range(v.x) && in_range(v.y)) ? atan2f((float)v.y, (float)v.x) : __int_as_float(0x7fc00000);
    }
  }
}

__device__ __forceinline__ void cswap(double &a, double &b) {
  const double lo = a < b ? a : b;
  const double hi = a < b ? b : a;
  a = lo;
  b = hi;
}

// Batcher-style 19-comparator sorting network for 8 values (ascending).
__device__ __forceinline__ void sort8(double v[8]) {
  cswap(v[0], v[1]); cswap(v[2], v[3]); cswap(v[4], v[5]); cswap(v[6], v[7]);
  cswap(v[0], v[2]); cswap(v[1], v[3]); cswap(v[4], v[6]); cswap(v[5], v[7]);
  cswap(v[1], v[2]); cswap(v[5], v[6]); cswap(v[0], v[4]); cswap(v[3], v[7]);
  cswap(v[1], v[5]); cswap(v[2], v[6]);
  cswap(v[1], v[4]); cswap(v[3], v[6]);
  cswap(v[2], v[4]); cswap(v[3], v[5]);
  cswap(v[3], v[4]);
}

__device__ __forceinline__ int64_t corner(int n, int ix, int iy, int iz, int c) {
  const int dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
  const int x = ix + dx == n ? 0 : ix + dx, y = iy + dy == n ? 0 : iy + dy,
            z = iz + dz == n ? 0 : iz + dz;
  return ((int64_t)z * n + y) * n + x;
}

// id_with_phase (defects_3d.f90:309-349) on sorted phases
__device__ __forceinline__ int8_t classify_sorted(const double pht[8], int which) {
  int8_t flag = 0;
  const double t = pht[0] - pht[7] + kRefTwoPi;
  double tmax = pht[1] - pht[0];
#pragma unroll
  for (int k = 1; k < 7; ++k) {
    const double g = pht[k + 1] - pht[k];
    tmax = g > tmax ? g : tmax;
  }
  if ((which & AXG_F_ID_WALLS) && tmax > t) {
    flag += 2;
  } else {
    tmax = t > tmax ? t : tmax;
  }
  if ((which & AXG_F_ID_STRINGS) && tmax < kStringPhdiff) flag += 1;
  if ((which & AXG_F_SPEC_EST) && tmax < kRemovalPhdiff) flag += 4;
  return flag;
}

// Three counters per block: warps tally ballots in registers, the block
// adds them in shared memory, and one thread adds the block's totals to the
// global counters (3 global atomics per block instead of 3 per warp pass).
struct BlockCount3 {
  unsigned long long c[3] = {0, 0, 0};
  __device__ __forceinline__ void add(bool a, bool b, bool d) {
    c[0] += __popc(__ballot_sync(0xffffffffu, a));
    c[1] += __popc(__ballot_sync(0xffffffffu, b));
    c[2] += __popc(__ballot_sync(0xffffffffu, d));
  }
  __device__ __forceinline__ void flush(unsigned long long *dst) {
    __shared__ unsigned long long sh[3];
    if (threadIdx.x < 3) sh[threadIdx.x] = 0;
    __syncthreads();
    if ((threadIdx.x & 31) == 0)
      for (int k = 0; k < 3; ++k)
        if (c[k]) atomicAdd(&sh[k], c[k]);
    __syncthreads();
    if (threadIdx.x < 3 && sh[threadIdx.x]) atomicAdd(&dst[threadIdx.x], sh[threadIdx.x]);
  }
};

// >> 4 (2 x 1e-6 phase error + FP32 rounding of a gap).  The phase error
// budget of 1e-6 covers atan2f (3 ulp) and, for an FP32-mixed field, the
// Kahan compensation the FP32 phase leaves out (|c| <= ulp(phi) / 2, so
// <= 1.2e-7 rad).
constexpr float kMargin = 2e-5f;

__device__ __forceinline__ void cswapf(float &a, float &b) {
  const float lo = fminf(a, b), hi = fmaxf(a, b);
  a = lo;
  b = hi;
}
__device__ __forceinline__ void sort8f(float v[8]) {
  cswapf(v[0], v[1]); cswapf(v[2], v[3]); cswapf(v[4], v[5]); cswapf(v[6], v[7]);
  cswapf(v[0], v[2]); cswapf(v[1], v[3]); cswapf(v[4], v[6]); cswapf(v[5], v[7]);
  cswapf(v[1], v[2]); cswapf(v[5], v[6]); cswapf(v[0], v[4]); cswapf(v[3], v[7]);
  cswapf(v[1], v[5]); cswapf(v[2], v[6]);
  cswapf(v[1], v[4]); cswapf(v[3], v[6]);
  cswapf(v[2], v[4]); cswapf(v[3], v[5]);
  cswapf(v[3], v[4]);
}

// id_with_phase on FP32 phases; false when a decision lies inside the margin
__device__ __forceinline__ bool classify_sorted_f(const float p[8], int which, int8_t &flag) {
  flag = 0;
  const float t = p[0] - p[7] + (float)kRefTwoPi;
  float tmax = p[1] - p[0];
#pragma unroll
  for (int k = 1; k < 7; ++k) tmax = fmaxf(tmax, p[k + 1] - p[k]);
  bool sure = true;
  if (which & AXG_F_ID_WALLS) {
    sure = fabsf(tmax - t) >= kMargin;
    if (tmax > t) flag += 2;
    else tmax = fmaxf(t, tmax);
  } else {
    tmax = fmaxf(t, tmax);
  }
  if (which & AXG_F_ID_STRINGS) {
    sure = sure && fabsf(tmax - (float)kStringPhdiff) >= kMargin;
    if (tmax < (float)kStringPhdiff) flag += 1;
  }
  if (which & AXG_F_SPEC_EST) {
    sure = sure && fabsf(tmax - (float)kRemovalPhdiff) >= kMargin;
    if (tmax < (float)kRemovalPhdiff) flag += 4;
  }
  return sure;
}

template <typename V>
__device__ __forceinline__ double phase64(const V *phi, const V *comp, int64_t s) {
  double re, im;
  load_c(phi, comp, s, re, im);
  return axd_atan2(im, re);
}

// The deterministic FP64 phase of every site, for the fits: each fitted cell
// reads its eight corners here instead of forming them (a string or wall
// cell's corners are shared with its neighbours, and the fits ran them as
// divergent FP64 chains at the start of every cell).
template <typename V>
__global__ void k_phase64_all(const V *__restrict__ phi, const V *__restrict__ cphi, int64_t n3,
                              double *__restrict__ ph) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n3; s += stride)
    ph[s] = phase64(phi, cphi, s);
}

template <typename V>
__global__ void k_classify(const float *__restrict__ ph, const V *__restrict__ phi, const V *__restrict__ cphi, int n,
                           int which,
                           int8_t *__restrict__ flags, unsigned long long *__restrict__ counts) {
  const int64_t n3 = (int64_t)n * n * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  BlockCount3 tally;
  // uniform trip count so every lane reaches the ballots
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n3; base += stride) {
    const int64_t s = base + threadIdx.x;
    int8_t f = 0;
    if (s < n3) {
      const int ix = (int)(s % n), iy = (int)((s / n) % n), iz = (int)(s / ((int64_t)n * n));
      float v[8];
      bool known = true;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        v[c] = ph[corner(n, ix, iy, iz, c)];
        known = known && !isnan(v[c]);
      }
      if (known) {
        sort8f(v);
        known = classify_sorted_f(v, which, f);
      }
      if (!known) {  // the FP64 classification of the host
        double d[8];
        for (int c = 0; c < 8; ++c) d[c] = phase64(phi, cphi, corner(n, ix, iy, iz, c));
        sort8(d);
        f = classify_sorted(d, which);
      }
      flags[s] = f;
    }
    tally.add((f & 1) != 0, (f & 2) != 0, (f & 4) != 0);
  }
  tally.flush(counts);
}

__device__ __forceinline__ double wrapd(double d) {
  const double pi = AXD_PI_HI, tp = 2 * AXD_PI_HI;
  if (d > pi) return d - tp;
  if (d <= -pi) return d + tp;
  return d;
}
__device__ __forceinline__ bool pierced(double a, double b, double c, double d) {
  double w = wrapd(b - a);
  w = w + wrapd(c - b);
  w = w + wrapd(d - c);
  w = w + wrapd(a - d);
  return w > AXD_PI_HI || w < -AXD_PI_HI;
}

// plaquette a-b-c-d on FP32 phases; false when a corner difference lies
// within the margin of the +-pi wrap or a phase is unknown
__device__ __forceinline__ bool pierced_f(float a, float b, float c, float d, bool &hit) {
  const float kPi = (float)AXD_PI_HI;
  const float ds[4] = {b - a, c - b, d - c, a - d};
  float w = 0.0f;
  bool sure = true;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float x = ds[k];
    sure = sure && fabsf(fabsf(x) - kPi) >= kMargin;  // false for NaN too
    w += x > kPi ? x - 2 * kPi : (x <= -kPi ? x + 2 * kPi : x);
  }
  hit = w > kPi || w < -kPi;
  return sure;
}

template <typename V>
__global__ void k_winding(const float *__restrict__ ph, const V *__restrict__ phi, const V *__restrict__ cphi, int n,
                          unsigned long long *__restrict__ counts) {
  const int64_t n2 = (int64_t)n * n, n3 = n2 * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  BlockCount3 tally;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n3; base += stride) {
    const int64_t s = base + threadIdx.x;
    bool hit[3] = {false, false, false};
    if (s < n3) {
      const int ix = (int)(s % n), iy = (int)((s / n) % n), iz = (int)(s / n2);
      const int x1 = ix + 1 == n ? 0 : ix + 1, y1 = iy + 1 == n ? 0 : iy + 1,
                z1 = iz + 1 == n ? 0 : iz + 1;
      auto S = [&](int x, int y, int z) { return ((int64_t)z * n + y) * n + x; };
      // corners of the x, y, z plaquettes (counts[0..2] = px, py, pz)
      const int64_t q[3][4] = {{S(ix, iy, iz), S(ix, y1, iz), S(ix, y1, z1), S(ix, iy, z1)},
                               {S(ix, iy, iz), S(ix, iy, z1), S(x1, iy, z1), S(x1, iy, iz)},
                               {S(ix, iy, iz), S(x1, iy, iz), S(x1, y1, iz), S(ix, y1, iz)}};
#pragma unroll
      for (int o = 0; o < 3; ++o) {
        if (!pierced_f(ph[q[o][0]], ph[q[o][1]], ph[q[o][2]], ph[q[o][3]], hit[o]))
          hit[o] = pierced(phase64(phi, cphi, q[o][0]), phase64(phi, cphi, q[o][1]), phase64(phi, cphi, q[o][2]),
                           phase64(phi, cphi, q[o][3]));
      }
    }
    tally.add(hit[0], hit[1], hit[2]);
  }
  tally.flush(counts);
}

// ---------------- compaction in cell order ----------------
constexpr int kChunk = 2048;  // cells per block
constexpr int kCThreads = 256;  // 8 consecutive cells per thread

__global__ void k_block_count(const int8_t *__restrict__ flags, int64_t n3, int *__restrict__ cs,
                              int *__restrict__ cw) {
  const int64_t b0 = (int64_t)blockIdx.x * kChunk + threadIdx.x * 8;
  int ns = 0, nw = 0;
  for (int k = 0; k < 8; ++k) {
    const int64_t s = b0 + k;
    if (s < n3) {
      const int8_t f = flags[s];
      ns += (f & 1) != 0;
      nw += (f & 2) != 0;
    }
  }
  __shared__ int sh[2][kCThreads];
  sh[0][threadIdx.x] = ns;
  sh[1][threadIdx.x] = nw;
  __syncthreads();
  for (int o = kCThreads / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + o];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    cs[blockIdx.x] = sh[0][0];
    cw[blockIdx.x] = sh[1][0];
  }
}

// exclusive scan of nb block counts (single block, sequential over chunks)
__global__ void k_scan_blocks(int *__restrict__ cs, int *__restrict__ cw, int nb) {
  __shared__ long long carry[2];
  __shared__ int sh[2][1024];
  if (threadIdx.x == 0) carry[0] = carry[1] = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += 1024) {
    const int i = base + threadIdx.x;
    const int a = i < nb ? cs[i] : 0, b = i < nb ? cw[i] : 0;
    sh[0][threadIdx.x] = a;
    sh[1][threadIdx.x] = b;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      int x0 = 0, x1 = 0;
      if ((int)threadIdx.x >= o) {
        x0 = sh[0][threadIdx.x - o];
        x1 = sh[1][threadIdx.x - o];
      }
      __syncthreads();
      sh[0][threadIdx.x] += x0;
      sh[1][threadIdx.x] += x1;
      __syncthreads();
    }
    if (i < nb) {
      cs[i] = (int)(carry[0] + sh[0][threadIdx.x] - a);
      cw[i] = (int)(carry[1] + sh[1][threadIdx.x] - b);
    }
    __syncthreads();
    if (threadIdx.x == 1023) {
      carry[0] += sh[0][1023];
      carry[1] += sh[1][1023];
    }
    __syncthreads();
  }
}

__global__ void k_compact(const int8_t *__restrict__ flags, int64_t n3, const int *__restrict__ offs,
                          const int *__restrict__ offw, int64_t *__restrict__ scell,
                          int64_t *__restrict__ wcell) {
  const int64_t b0 = (int64_t)blockIdx.x * kChunk + threadIdx.x * 8;
  int ns = 0, nw = 0;
  int8_t f[8];
  for (int k = 0; k < 8; ++k) {
    const int64_t s = b0 + k;
    f[k] = s < n3 ? flags[s] : 0;
    ns += (f[k] & 1) != 0;
    nw += (f[k] & 2) != 0;
  }
  __shared__ int sh[2][kCThreads];
  sh[0][threadIdx.x] = ns;
  sh[1][threadIdx.x] = nw;
  __syncthreads();
  for (int o = 1; o < kCThreads; o <<= 1) {
    int x0 = 0, x1 = 0;
    if ((int)threadIdx.x >= o) {
      x0 = sh[0][threadIdx.x - o];
      x1 = sh[1][threadIdx.x - o];
    }
    __syncthreads();
    sh[0][threadIdx.x] += x0;
    sh[1][threadIdx.x] += x1;
    __syncthreads();
  }
  int ps = offs[blockIdx.x] + sh[0][threadIdx.x] - ns;
  int pw = offw[blockIdx.x] + sh[1][threadIdx.x] - nw;
  for (int k = 0; k < 8; ++k) {
    if (f[k] & 1) scell[ps++] = b0 + k;
    if (f[k] & 2) wcell[pw++] = b0 + k;
  }
}

// ---------------- per-cell fits ----------------
// defects_3d.f90:1027-1056
__device__ double string_length(const double pos[3], const double dir[3]) {
  const double atmax = 0.867, atmax0 = 0.86602540378378444;
  double tp = atmax, tn = -atmax;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j <= 1; ++j) {
      double w = j - 0.5;
      w = w - pos[i];
      if (fabs(w) > atmax * fabs(dir[i])) continue;
      const double t = w / dir[i];
      if (t > 0) {
        if (t < tp) tp = t;
      } else {
        if (t > tn) tn = t;
      }
    }
  if (tp < atmax0 && tn > -atmax0) return tp - tn;
  return 0.0;
}

__device__ __forceinline__ bool out_of_box(const double t[4]) {
  const double mx[4] = {1.0, kRefPi, sqrt(3.0) / 2, kRefPi};
  const double mn[4] = {-1.0, -kRefPi, 0.0, -kRefPi};
  for (int k = 0; k < 4; ++k)
    if (t[k] > mx[k] || t[k] < mn[k]) return true;
  return false;
}

// Start point i of the random search (defects_3d.f90:463-470): four
// uniforms from two Philox draws, mapped onto the parameter box.
__device__ __forceinline__ void string_start(uint64_t seed, uint64_t cell, int i, double t[4]) {
  const double max_s[4] = {1.0, kRefPi, sqrt(3.0) / 2, kRefPi};
  const double min_s[4] = {-1.0, -kRefPi, 0.0, -kRefPi};
  double x[4];
  for (int k = 0; k < 4; k += 2) {
    const int j = i * 4 + k;
    const axd_u32x4 r = axd_draw(seed, 3u, (uint32_t)(j >> 1), cell);
    x[k] = axd_u01(r.v[0], r.v[1]);
    x[k + 1] = axd_u01(r.v[2], r.v[3]);
  }
  for (int k = 0; k < 4; ++k) t[k] = max_s[k] * x[k] + min_s[k] * (1 - x[k]);
}

// A lower bound of calc_chi2_string(ph, t) from an FP32 evaluation, or -inf
// where the FP32 value cannot be bounded (a corner too close to the string
// axis for its angle to be resolved, or a phase difference within the error
// of the +-pi wrap).  Error budget, all generous:
//   du, dv: angles and radius rounded to FP32, sqrt(1 - mu^2) from an FP64
//           product, CUDA sincosf (2 ulp), products and sums of terms below
//           2.4 in magnitude: |error| <= kDuv = 4e-6;
//   angle : atan2f (3 ulp of pi) plus the rotation of (du, dv) by an error
//           of kDuv at radius r: e = kAng + 2 kDuv / (r - 2 kDuv);
//   phase : FP32 rounding of ph, of the difference and of the wrap
//           constants, within kPh = 2e-6;
//   chi2  : a = <d^2> moves by at most (2 pi + E) E, b^2 = <d>^2 by at most
//           (2 pi + E + 2e-6)(E + 2e-6), FP32 summation by below 2e-5;
// and the total is doubled, plus 1e-4.
//
// Kept out of line: inlined into the search step (with its eight atan2f and
// two sincosf) it made the string-fit loop's code outgrow the instruction
// cache (ncu at 128^3: 9.1 "no instruction" stalls per issue); one copy took
// the 128^3 fits from 152 to 106 ms.
__device__ __noinline__ float chi2_string_lower(const float phf[8], const double t[4]) {
  constexpr float kDuv = 4e-6f, kAng = 2e-6f, kPh = 2e-6f;
  constexpr float kPiF = (float)kRefPi, kTwoPiF = (float)kRefTwoPi;
  const float mu = (float)t[0], ph = (float)t[1], rad = (float)t[2], ang = (float)t[3];
  float s4, c4, sp, cp;
  sincosf(ang, &s4, &c4);
  sincosf(ph, &sp, &cp);
  // 1 - mu^2 is formed in FP64: for |mu| near 1 the FP32 rounding of mu
  // alone would move sqrt(1 - mu^2) by up to 5e-4
  const float u0 = rad * c4, v0 = rad * s4, sm = sqrtf((float)((1.0 - t[0]) * (1.0 + t[0])));
  float a = 0.0f, b = 0.0f, E = 0.0f;
  for (int iz = 0; iz <= 1; ++iz) {
    const float z = iz - 0.5f;
    for (int iy = 0; iy <= 1; ++iy) {
      const float y = iy - 0.5f;
      for (int ix = 0; ix <= 1; ++ix) {
        const float x = ix - 0.5f;
        const int i = (iz * 2 + iy) * 2 + ix;
        const float du = -u0 + mu * (x * cp + y * sp) - z * sm;
        const float dv = -v0 - x * sp + y * cp;
        const float r = sqrtf(du * du + dv * dv);
        if (!(r > 8 * kDuv)) return -INFINITY;
        const float e = kAng + kPh + 2 * kDuv / (r - 2 * kDuv);
        float d = phf[i] - atan2f(dv, du);
        if (!(fabsf(fabsf(d) - kPiF) > e + kPh)) return -INFINITY;
        if (d >= kPiF)
          d = d - kTwoPiF;
        else if (d < -kPiF)
          d = d + kTwoPiF;
        a = a + d * d;
        b = b + d;
        E = fmaxf(E, e);
      }
    }
  }
  a = a / 8;
  b = b / 8;
  const float tp = (float)kRefTwoPi;
  const float bound = 2 * ((tp + E) * E + (tp + E + 2e-6f) * (E + 2e-6f) + 2e-5f) + 1e-4f;
  return (a - b * b) - bound;
}

// defects_3d.f90:435-603, as a per-lane state machine.
//
// The fit of one string cell is a random search over 1001 starts followed by
// a Nelder-Mead simplex of up to 1000 iterations (tol 0.05 on chi2).  In
// evolved fields about two thirds of the string cells never reach the
// tolerance and run all 1000 iterations.  Written as one loop per thread,
// a warp ran its slowest cell's iteration count, and the expansion,
// contraction and shrink branches one after another.  Here each lane holds
// the search state of one cell and advances it to its next chi2
// evaluation; every pass of the scheduling loop makes at most one chi2
// evaluation per lane, at a lane-specific point, so the 8 atan2 of the
// evaluations run on all active lanes together.  A lane whose cell is done
// writes the cell's results and takes the next cell from a global counter.
//
// The random search keeps kNumSimp + 1 of the starts, in the order drawn.
// Once that set is full, a start changes it only if its chi2 is at most the
// value in the last slot.  That value can rise (the first two starts are
// kept unsorted, defects_3d.f90:471-476, and a larger early value moves up
// the list), but never above the largest value kept at any earlier time.
// The starts are therefore screened with FP32 lower bounds
// (chi2_string_lower) against the largest kept value; only the starts that
// pass are evaluated, in draw order.  A screened-out start has a chi2 above
// any threshold the sequential search could have compared it with (the
// bound's 1e-4 margin covers the 1e-14 between the FP64 chi2 it was
// derived for and the float-float chi2 the search uses).  Every chi2 that
// enters a decision or the kept state is the float-float value of
// axd_chi2_string_ff (axg_ffchi2.h), which the CPU restatement evaluates
// too, so the fit is bit-identical to its sequential search.
struct StringSearch {
  double p_s[5][4], chi2_s[5], c_s[4], t_s[4], s_s[4], chi2;
  int n0, i, it, stage;
  bool expand;
};

enum : int {
  kSearch = 0,
  kNmStart,
  kNmReflect,
  kNmSecondPrep,
  kNmSecond,
  kShrink1,  // kShrink1 .. kShrink1 + kNumSimp - 1: shrink vertices 1..kNumSimp
  kNmSort = kShrink1 + kNumSimp,
  kFinished
};

__device__ __forceinline__ void search_init(StringSearch &S) {
  for (int a = 0; a < 5; ++a) {
    S.chi2_s[a] = 0.0;
    for (int k = 0; k < 4; ++k) S.p_s[a][k] = 0.0;
  }
  S.n0 = -1;
  S.i = 0;
  S.it = 0;
  S.stage = kSearch;
  S.expand = false;
  S.chi2 = 0.0;
}

// the random-search bookkeeping of one exactly evaluated start (t_s, chi2)
__device__ __forceinline__ void search_insert(StringSearch &S, double chi2) {
  if (S.n0 <= 0) {
    S.n0 = S.n0 + 1;
    S.chi2_s[S.n0] = chi2;
    for (int k = 0; k < 4; ++k) S.p_s[S.n0][k] = S.t_s[k];
    return;
  }
  if (S.n0 < kNumSimp || chi2 <= S.chi2_s[S.n0]) {
    S.n0 = S.n0 + 1 < kNumSimp ? S.n0 + 1 : kNumSimp;
    int i0 = S.n0;
    while (chi2 <= S.chi2_s[i0 - 1]) {
      if (i0 <= kNumSimp) {
        S.chi2_s[i0] = S.chi2_s[i0 - 1];
        for (int k = 0; k < 4; ++k) S.p_s[i0][k] = S.p_s[i0 - 1][k];
      }
      i0 = i0 - 1;
      if (i0 == 0) break;
    }
    S.chi2_s[i0] = chi2;
    for (int k = 0; k < 4; ++k) S.p_s[i0][k] = S.t_s[k];
  }
}

// the expansion / contraction decision with the second point's chi2
__device__ __forceinline__ void search_second(StringSearch &S, double chi2s) {
  if (S.expand) {
    if (S.chi2 <= chi2s) {
      S.chi2_s[kNumSimp] = S.chi2;
      for (int k = 0; k < 4; ++k) S.p_s[kNumSimp][k] = S.t_s[k];
    } else {
      S.chi2_s[kNumSimp] = chi2s;
      for (int k = 0; k < 4; ++k) S.p_s[kNumSimp][k] = S.s_s[k];
    }
    S.stage = kNmSort;
  } else if (chi2s <= S.chi2_s[kNumSimp]) {
    S.chi2_s[kNumSimp] = chi2s;
    for (int k = 0; k < 4; ++k) S.p_s[kNumSimp][k] = S.s_s[k];
    S.stage = kNmSort;
  } else {
    S.stage = kShrink1;
  }
}

// Advance S to its next chi2 evaluation; true with the point in P, false
// when the lane has none this pass (screening budget spent, or finished).
__device__ bool search_prepare(StringSearch &S, const float phf[8], uint64_t seed, uint64_t cell, double P[4],
                               int screen) {
  const double chi2max = 8 * kRefPi * kRefPi, tol = 0.05;
  for (;;) {
    if (S.stage == kSearch) {
      if (S.i > kMaxIter) {
        S.stage = kNmStart;
        continue;
      }
      if (S.n0 < kNumSimp) {  // filling the kept set: no screen
        string_start(seed, cell, S.i, S.t_s);
        for (int k = 0; k < 4; ++k) P[k] = S.t_s[k];
        return true;
      }
      double thr = S.chi2_s[0];
      for (int k = 1; k <= kNumSimp; ++k) thr = S.chi2_s[k] > thr ? S.chi2_s[k] : thr;
      for (int k = 0; k <= kNumSimp; ++k)
        if (S.chi2_s[k] != S.chi2_s[k]) thr = INFINITY;
      for (int cnt = 0; cnt < screen && S.i <= kMaxIter; ++cnt) {
        string_start(seed, cell, S.i, S.t_s);
        if (!((double)chi2_string_lower(phf, S.t_s) > thr)) {
          for (int k = 0; k < 4; ++k) P[k] = S.t_s[k];
          return true;
        }
        S.i = S.i + 1;
      }
      if (S.i > kMaxIter) {
        S.stage = kNmStart;
        continue;
      }
      return false;
    }
    if (S.stage == kNmStart) {
      if (!(S.chi2_s[0] > tol && S.it < kMaxIter)) {
        S.stage = kFinished;
        return false;
      }
      S.it = S.it + 1;
      for (int k = 0; k < 4; ++k) S.c_s[k] = 0.0;
      for (int i0 = 0; i0 < kNumSimp; ++i0)
        for (int k = 0; k < 4; ++k) S.c_s[k] = S.c_s[k] + S.p_s[i0][k];
      static_assert(kNumSimp == 4, "the centroid scaling below is 1 / kNumSimp");
      for (int k = 0; k < 4; ++k) S.c_s[k] = S.c_s[k] * 0.25;  // exact: the same value as / kNumSimp
      for (int k = 0; k < 4; ++k) S.t_s[k] = 2 * S.c_s[k] - S.p_s[kNumSimp][k];
      if (out_of_box(S.t_s)) {
        S.chi2 = chi2max;
        S.stage = kNmSecondPrep;
        continue;
      }
      for (int k = 0; k < 4; ++k) P[k] = S.t_s[k];
      S.stage = kNmReflect;
      return true;
    }
    if (S.stage == kNmSecondPrep) {
      S.expand = S.chi2 < S.chi2_s[kNumSimp];
      if (S.expand)
        for (int k = 0; k < 4; ++k) S.s_s[k] = 3 * S.c_s[k] - 4 * S.p_s[kNumSimp][k];
      else
        for (int k = 0; k < 4; ++k) S.s_s[k] = 1.5 * S.c_s[k] - 0.5 * S.p_s[kNumSimp][k];
      if (out_of_box(S.s_s)) {
        search_second(S, chi2max);
        continue;
      }
      for (int k = 0; k < 4; ++k) P[k] = S.s_s[k];
      S.stage = kNmSecond;
      return true;
    }
    if (S.stage == kNmSort) {
      for (int i0 = kNumSimp - 1; i0 >= 0; --i0)
        for (int m = 0; m <= i0; ++m)
          if (S.chi2_s[m] > S.chi2_s[m + 1]) {
            for (int k = 0; k < 4; ++k) {
              const double tt = S.p_s[m][k];
              S.p_s[m][k] = S.p_s[m + 1][k];
              S.p_s[m + 1][k] = tt;
            }
            const double c = S.chi2_s[m];
            S.chi2_s[m] = S.chi2_s[m + 1];
            S.chi2_s[m + 1] = c;
          }
      S.stage = kNmStart;
      continue;
    }
    if (S.stage >= kShrink1 && S.stage < kNmSort) {  // shrink towards the best vertex
      const int j = S.stage - kShrink1 + 1;
      for (int k = 0; k < 4; ++k) S.p_s[j][k] = 0.5 * (S.p_s[j][k] + S.p_s[0][k]);
      for (int k = 0; k < 4; ++k) P[k] = S.p_s[j][k];
      return true;
    }
    return false;  // kFinished
  }
}

// S takes the chi2 of the point search_prepare returned
__device__ void search_consume(StringSearch &S, double v) {
  if (S.stage == kSearch) {
    search_insert(S, v);
    S.i = S.i + 1;
  } else if (S.stage == kNmReflect) {
    S.chi2 = v;
    S.stage = kNmSecondPrep;
  } else if (S.stage == kNmSecond) {
    search_second(S, v);
  } else {
    const int j = S.stage - kShrink1 + 1;
    S.chi2_s[j] = v;
    S.stage = j < kNumSimp ? S.stage + 1 : kNmSort;
  }
}

// position, direction, goodness of fit and length from the best vertex
__device__ void string_result(const StringSearch &S, double pos[3], double dir[3], double *gof, double *sl) {
  const double mu = S.p_s[0][0], phi = S.p_s[0][1];
  double s4, c4, sp, cp;
  axd_sincos(S.p_s[0][3], &s4, &c4);
  const double u0 = S.p_s[0][2] * c4, v0 = S.p_s[0][2] * s4;
  const double chi2 = S.chi2_s[0];
  axd_sincos(phi, &sp, &cp);
  const double sq = sqrt(1.0 - mu * mu);
  dir[0] = sq * cp;
  dir[1] = sq * sp;
  dir[2] = mu;
  pos[0] = u0 * mu * cp - v0 * sp;
  pos[1] = u0 * mu * sp + v0 * cp;
  pos[2] = -(u0 * sqrt(1 - mu * mu));
  *gof = exp(-chi2 / 2);
  *sl = string_length(pos, dir);
}

// reference BLAS dspr ('U')
__device__ void dspr_u(int n, double alpha, const double *x, double *ap) {
  int kk = 0;
  for (int j = 0; j < n; ++j) {
    if (x[j] != 0.0) {
      const double temp = alpha * x[j];
      int k = kk;
      for (int i = 0; i <= j; ++i) {
        ap[k] = ap[k] + x[i] * temp;
        ++k;
      }
    }
    kk += j + 1;
  }
}

// reference LAPACK dpptrf + dpptri ('U') on a packed 4x4
__device__ void pp_inverse4(double *ap) {
  const int n = 4;
  int jj = 0;
  for (int j = 1; j <= n; ++j) {
    const int jc = jj + 1;
    jj = jj + j;
    if (j > 1) {
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
    const double ajj = ap[jj - 1] - dot;
    if (ajj <= 0.0) {
      ap[jj - 1] = ajj;
      return;
    }
    ap[jj - 1] = sqrt(ajj);
  }
  int jc = 1;
  for (int j = 1; j <= n; ++j) {
    ap[jc + j - 2] = 1.0 / ap[jc + j - 2];
    const double ajj = -ap[jc + j - 2];
    double *x = ap + (jc - 1);
    int kk = 1;
    for (int jx = 1; jx <= j - 1; ++jx) {
      if (x[jx - 1] != 0.0) {
        const double temp = x[jx - 1];
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
  jj = 0;
  for (int j = 1; j <= n; ++j) {
    const int jc2 = jj + 1;
    jj = jj + j;
    if (j > 1) dspr_u(j - 1, 1.0, ap + (jc2 - 1), ap);
    const double ajj = ap[jj - 1];
    for (int i = 0; i < j; ++i) ap[jc2 - 1 + i] = ajj * ap[jc2 - 1 + i];
  }
}

// defects_3d.f90:605-692 (VEL=0)
template <typename V>
__device__ void velocity_string(const V *phi, const V *cphi, const V *phid, int n, double dspa, int ix, int iy,
                                int iz, const double pos[3], double vel[3]) {
  double wr[4] = {0, 0, 0, 0}, wi[4] = {0, 0, 0, 0}, dr[4] = {0, 0, 0, 0}, di[4] = {0, 0, 0, 0};
  double mat[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0}, mat0[10];
  double d[4];
  d[0] = 1.0;
  for (int k = 0; k <= 1; ++k) {
    const int zz = iz + k == n ? 0 : iz + k;
    d[3] = k - pos[2] - 0.5;
    for (int j = 0; j <= 1; ++j) {
      const int yy = iy + j == n ? 0 : iy + j;
      d[2] = j - pos[1] - 0.5;
      for (int i = 0; i <= 1; ++i) {
        const int xx = ix + i == n ? 0 : ix + i;
        d[1] = i - pos[0] - 0.5;
        const int64_t s = ((int64_t)zz * n + yy) * n + xx;
        double pr, pi_, qr, qi;
        load_c(phi, cphi, s, pr, pi_);
        load_c(phid, (const V *)nullptr, s, qr, qi);
        for (int l = 0; l < 4; ++l) {
          wr[l] = wr[l] + d[l] * pr;
          wi[l] = wi[l] + d[l] * pi_;
          dr[l] = dr[l] + d[l] * qr;
          di[l] = di[l] + d[l] * qi;
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
  for (int l = 0; l < 10; ++l) {
    mat[l] /= 8;
    mat0[l] = mat[l];
  }
  pp_inverse4(mat0);
  double w0r[4] = {0, 0, 0, 0}, w0i[4] = {0, 0, 0, 0}, d0r[4] = {0, 0, 0, 0}, d0i[4] = {0, 0, 0, 0};
  for (int ii = 1; ii <= 4; ++ii)
    for (int jj = 1; jj <= 4; ++jj) {
      int kk = ii > jj ? ii : jj;
      kk = kk * (kk - 1) / 2 + (ii < jj ? ii : jj);
      const double m = mat0[kk - 1];
      w0r[ii - 1] = w0r[ii - 1] + m * wr[jj - 1];
      w0i[ii - 1] = w0i[ii - 1] + m * wi[jj - 1];
      d0r[ii - 1] = d0r[ii - 1] + m * dr[jj - 1];
      d0i[ii - 1] = d0i[ii - 1] + m * di[jj - 1];
    }
  const double x = d0r[0], y = d0i[0];
  double a = 0, b = 0, c = 0;
  for (int l = 1; l < 4; ++l) {
    a = a + w0r[l] * w0r[l];
    b = b + w0r[l] * w0i[l];
    c = c + w0i[l] * w0i[l];
  }
  const double det = a * c - b * b;
  for (int l = 1; l < 4; ++l) {
    const double v = (x * c - y * b) * w0r[l] + (-(x * b) + y * a) * w0i[l];
    vel[l - 1] = -v / det * dspa;
  }
}

// defects_3d.f90:1058-1233
// The 20 x 20 grid of wall directions of position_wall (defects_3d.f90:
// 1135-1160): d0 = (sqrt(1 - mu^2) cos phi, sqrt(1 - mu^2) sin phi, mu) for
// mu = ((2 imu - 20) - 1) / 20, phi = pi ((2 iphi - 1) - 20) / 20, in the
// reference's operations; the same for every cell, so k_wall_fit forms it
// once per CTA in shared memory.
struct WallGrid {
  double d0[400][4];  // d0 and phi
  float f[400][3];    // d0 rounded to FP32, for the screen of position_wall
};

__device__ void wall_grid_fill(WallGrid &g) {
  for (int idx = threadIdx.x; idx < 400; idx += blockDim.x) {
    const int imu = idx / 20 + 1, iphi = idx % 20 + 1;
    const double mu = ((double)(-20 + 2 * imu) - 1.0) / 20;
    const double phi = kRefPi * ((2 * iphi - 1.0) - 20) / 20;
    double sp, cp;
    axd_sincos(phi, &sp, &cp);
    const double sq = sqrt(1 - mu * mu);
    g.d0[idx][0] = sq * cp;
    g.d0[idx][1] = sq * sp;
    g.d0[idx][2] = mu;
    g.d0[idx][3] = phi;
    for (int k = 0; k < 3; ++k) g.f[idx][k] = (float)g.d0[idx][k];
  }
}

// The direction search of position_wall screened in FP32.  Per direction
// the reference forms d_i = pp_i . d0, W = sum d_i, S = sum d_i^2 and
// chi2 = S - m w^2 with w = max(W, 0) / m, i.e. chi2 = S - max(W, 0)^2 / m.
// With |pp| < 0.87 (each component in (-0.5, 0.5)), |d0| = 1 and m <= 12,
// the FP32 value differs from the FP64 one by less than kWallScreenErr:
// inputs rounded to FP32 and three products and two sums move d by < 5e-7,
// so W by < 1.3e-5 and S by < 2e-5; max(W, 0)^2 / m is Lipschitz in W
// (either branch of the reference's w < 0 test), < 9e-5 for |W| <= 10.4;
// the remaining roundings are below 1e-5.  The FP32 error is thus below
// 1.3e-4; the screen allows 1e-3.  A direction whose FP32 value exceeds the
// smallest FP32 value by more than twice that cannot hold the FP64 minimum,
// so evaluating only the others in FP64, in the reference's loop order and
// with its strict-less update, selects the same direction and w.
constexpr float kWallScreenErr = 1e-3f;

__device__ void position_wall(const double ph[8], const WallGrid &grid, double pos[3], double dir[3], double *gof,
                              double *wa) {
  double pp[12][3], th[12], uv[12][2], sn[8], cs[8];
  for (int i = 0; i < 8; ++i) axd_sincos(ph[i], &sn[i], &cs[i]);
  int m = 0;
  for (int iz = 0; iz <= 1; ++iz)
    for (int iy = 0; iy <= 1; ++iy) {
      const double u = sn[(iz * 2 + iy) * 2 + 0], v = sn[(iz * 2 + iy) * 2 + 1];
      if (u * v < 0.0) {
        pp[m][0] = (u + v) / (u - v) / 2;
        pp[m][1] = iy - 0.5;
        pp[m][2] = iz - 0.5;
        ++m;
      }
    }
  for (int iy = 0; iy <= 1; ++iy)
    for (int ix = 0; ix <= 1; ++ix) {
      const double u = sn[(0 * 2 + iy) * 2 + ix], v = sn[(1 * 2 + iy) * 2 + ix];
      if (u * v < 0.0) {
        pp[m][0] = ix - 0.5;
        pp[m][1] = iy - 0.5;
        pp[m][2] = (u + v) / (u - v) / 2;
        ++m;
      }
    }
  for (int iz = 0; iz <= 1; ++iz)
    for (int ix = 0; ix <= 1; ++ix) {
      const double u = sn[(iz * 2 + 0) * 2 + ix], v = sn[(iz * 2 + 1) * 2 + ix];
      if (u * v < 0.0) {
        pp[m][0] = ix - 0.5;
        pp[m][1] = (u + v) / (u - v) / 2;
        pp[m][2] = iz - 0.5;
        ++m;
      }
    }
  if (m < 3) {
    for (int k = 0; k < 3; ++k) pos[k] = dir[k] = 0.0;
    *gof = 0.0;
    *wa = 0.0;
    return;
  }
  float ppf[12][3];
  for (int i = 0; i < m; ++i)
    for (int k = 0; k < 3; ++k) ppf[i][k] = (float)pp[i][k];
  auto screen = [&](int idx) {
    const float *g = grid.f[idx];
    float W = 0.0f, S = 0.0f;
    for (int i = 0; i < m; ++i) {
      const float d = ppf[i][0] * g[0] + ppf[i][1] * g[1] + ppf[i][2] * g[2];
      W += d;
      S += d * d;
    }
    const float wp = fmaxf(W, 0.0f);
    return S - wp * wp / (float)m;
  };
  float fmin = INFINITY;
  for (int idx = 0; idx < 400; ++idx) fmin = fminf(fmin, screen(idx));
  const float fcut = fmin + 2 * kWallScreenErr;
  double chi2min = 6.0, mut = 0.0, phit = 0.0, wt = 0.0;
  for (int imu = 1; imu <= 20; ++imu) {
    for (int iphi = 1; iphi <= 20; ++iphi) {
      if (!(screen((imu - 1) * 20 + (iphi - 1)) <= fcut)) continue;
      const double *d0 = grid.d0[(imu - 1) * 20 + (iphi - 1)];
      const double mu = d0[2], phi = d0[3];
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
  const double sqt = sqrt(1 - mut * mut);
  double d0[3] = {sqt * cpt, sqt * spt, mut};
  int num = 0;
  for (int iz = 0; iz <= 1; ++iz)
    for (int iy = 0; iy <= 1; ++iy)
      for (int ix = 0; ix <= 1; ++ix) {
        const double disp[3] = {ix - 0.5, iy - 0.5, iz - 0.5};
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
  const double dir1[3] = {mut * cpt, mut * spt, -sqrt(1 - mut * mut)};
  const double dir2[3] = {-spt, cpt, 0.0};
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
        const double w = th[j - 1];
        th[j - 1] = th[j];
        th[j] = w;
        const double a = uv[j - 1][0], b = uv[j - 1][1];
        uv[j - 1][0] = uv[j][0];
        uv[j - 1][1] = uv[j][1];
        uv[j][0] = a;
        uv[j][1] = b;
      }
  double area = 0.0;
  double w = th[m - 1] - kRefTwoPi;
  double u = sqrt(uv[m - 1][0] * uv[m - 1][0] + uv[m - 1][1] * uv[m - 1][1]);
  for (int i = 0; i < m; ++i) {
    const double v = sqrt(uv[i][0] * uv[i][0] + uv[i][1] * uv[i][1]);
    w = th[i] - w;
    area = area + 0.5 * u * v * axd_sin(w);
    u = v;
    w = th[i];
  }
  *wa = area;
}

// FP32 screens per start-phase pass of a lane (search_prepare): a pass
// screens at most this many random starts, so lanes in the start phase hold
// the warp's Nelder-Mead lanes back for a few FP32 bounds only (8 measured
// fastest of 2..32 at 128^3).
constexpr int kScreenPerPass = 8;

// String fits, lane-scheduled: each lane takes cells from *next (zero at
// launch) and advances its search one chi2 evaluation per pass (see
// search_prepare); the grid is sized to the resident CTAs.  The float-float
// chi2 is a long chain of dependent FP32 operations, so the kernel is bound
// by latency: capped at 96 registers (a few spills) it holds 5 CTAs per SM
// instead of 3 (128^3: 237 -> 158 ms; 4, 6 and 8 CTAs measured slower).
template <typename V>
__global__ void __launch_bounds__(128, 5) k_string_fit(const V *__restrict__ phi, const V *__restrict__ cphi,
                                                    const double *__restrict__ ph64, const V *__restrict__ phid, int n,
                                                    double dspa, uint64_t seed, const int64_t *__restrict__ cells,
                                                    int64_t ncell, double *__restrict__ out,
                                                    unsigned long long *__restrict__ next) {
  StringSearch S;
  axd_ff pcf[8];  // corner phases as float-float pairs (the chi2 runs in float-float)
  float phf[8];
  int64_t k = -1, s = 0;
  auto fetch = [&]() {
    k = (int64_t)atomicAdd(next, 1ull);
    if (k >= ncell) {
      k = -1;
      return;
    }
    s = cells[k];
    const int ix = (int)(s % n), iy = (int)((s / n) % n), iz = (int)(s / ((int64_t)n * n));
    for (int c = 0; c < 8; ++c) {
      const double pc = ph64[corner(n, ix, iy, iz, c)];
      pcf[c] = axd_ff_from(pc);
      phf[c] = (float)pc;
    }
    search_init(S);
  };
  fetch();
  for (;;) {
    if (k >= 0 && S.stage == kFinished) {
      const int ix = (int)(s % n), iy = (int)((s / n) % n), iz = (int)(s / ((int64_t)n * n));
      double pos[3], dir[3], vel[3], gof, l;
      string_result(S, pos, dir, &gof, &l);
      velocity_string(phi, cphi, phid, n, dspa, ix, iy, iz, pos, vel);
      double *r = out + 13 * k;
      r[0] = pos[0] + ix + 0.5;
      r[1] = pos[1] + iy + 0.5;
      r[2] = pos[2] + iz + 0.5;
      r[3] = dir[0];
      r[4] = dir[1];
      r[5] = dir[2];
      r[6] = vel[0];
      r[7] = vel[1];
      r[8] = vel[2];
      r[9] = gof;
      r[10] = l;
      r[11] = (double)s;
      r[12] = -1.0;
      fetch();
    }
    if (__all_sync(0xffffffffu, k < 0)) break;
    double P[4];
    const bool need = k >= 0 && search_prepare(S, phf, seed, (uint64_t)s, P, kScreenPerPass);
    __syncwarp();
    if (need) search_consume(S, axd_chi2_string_ff(pcf, P));
  }
}

__global__ void __launch_bounds__(128) k_wall_fit(const double *__restrict__ ph64, int n,
                                                  const int64_t *__restrict__ cells,
                                                  int64_t ncell, double *__restrict__ out) {
  __shared__ WallGrid grid;
  wall_grid_fill(grid);
  __syncthreads();
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ncell) return;
  const int64_t s = cells[k];
  const int ix = (int)(s % n), iy = (int)((s / n) % n), iz = (int)(s / ((int64_t)n * n));
  double pc[8];
  for (int c = 0; c < 8; ++c) pc[c] = ph64[corner(n, ix, iy, iz, c)];
  double pos[3], dir[3], gof, a;
  position_wall(pc, grid, pos, dir, &gof, &a);
  double *r = out + 10 * k;
  r[0] = pos[0] + ix + 0.5;
  r[1] = pos[1] + iy + 0.5;
  r[2] = pos[2] + iz + 0.5;
  r[3] = dir[0];
  r[4] = dir[1];
  r[5] = dir[2];
  r[6] = gof;
  r[7] = a;
  r[8] = (double)s;
  r[9] = -1.0;
}

// add_string_length / add_wall_area sums (one block; fixed-order tree)
__global__ void k_defect_sums(const double *__restrict__ strs, int64_t ns,
                              const double *__restrict__ walls, int64_t nw, double *__restrict__ out) {
  __shared__ double sh[5][256];
  double a[5] = {0, 0, 0, 0, 0};  // sl, sqrt(v2), v2, gamma, count of v2<1
  double wsum = 0.0;
  for (int64_t k = threadIdx.x; k < ns; k += blockDim.x) {
    const double *r = strs + 13 * k;
    a[0] = a[0] + r[10];
    double v2 = r[6] * r[6] + r[7] * r[7];
    v2 = v2 + r[8] * r[8];
    if (v2 < 1.0) {
      a[1] = a[1] + sqrt(v2);
      a[2] = a[2] + v2;
      a[3] = a[3] + 1 / sqrt(1 - v2);
      a[4] = a[4] + 1.0;
    }
  }
  for (int64_t k = threadIdx.x; k < nw; k += blockDim.x) wsum = wsum + walls[10 * k + 7];
  for (int q = 0; q < 5; ++q) sh[q][threadIdx.x] = a[q];
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int q = 0; q < 5; ++q) sh[q][threadIdx.x] = sh[q][threadIdx.x] + sh[q][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 5; ++q) out[q] = sh[q][0];
  __syncthreads();
  sh[0][threadIdx.x] = wsum;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[0][threadIdx.x] = sh[0][threadIdx.x] + sh[0][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[5] = sh[0][0];
}

// ---------------- grouping (defects_3d.f90:1235-1652, 1735-2143) ----------------
// Connected components of the fitted positions under the periodic distance
// threshold: the partition the reference's grouping produces on one rank and
// one thread.  Hash grid of G^3 cells (cell side >= threshold) + lock-free
// union-find linking the larger root under the smaller, so the final label
// of every point is the smallest list index of its component.
constexpr int kUfMaxRetries = 1 << 20;

__device__ double lat_dist_periodic(int n, const double *a, const double *b) {
  double s = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double dp = fabs(a[k] - b[k]);
    const double e = (double)n - dp;
    const double m = dp < e ? dp : e;
    s = s + m * m;
  }
  return sqrt(s);
}

__device__ int uf_find(volatile int *par, int x) {
  while (true) {
    const int p = par[x];
    if (p == x) return x;
    const int gp = par[p];
    if (gp != p) par[x] = gp;  // path halving: a valid ancestor, benign race
    x = p;
  }
}

__device__ void uf_union(int *par, int a, int b, int *err) {
  for (int it = 0; it < kUfMaxRetries; ++it) {
    a = uf_find(par, a);
    b = uf_find(par, b);
    if (a == b) return;
    if (a > b) {
      const int t = a;
      a = b;
      b = t;
    }
    const int old = atomicCAS(&par[b], b, a);
    if (old == b) return;
    b = old;
  }
  atomicExch(err, AXG_KERR_BOUNDS);
}

__device__ __forceinline__ int cell_of(double x, int n, int G) {
  double w = x - floor(x / n) * n;  // into [0, n)
  int c = (int)(w * G / n);
  return c < 0 ? 0 : (c >= G ? G - 1 : c);
}

__global__ void k_grp_init(int *par, int np) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < np) par[i] = i;
}

__global__ void k_grp_count(const double *rows, int width, int np, int n, int G, int *cell, int *count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double *r = rows + (int64_t)width * i;
  const int c = (cell_of(r[2], n, G) * G + cell_of(r[1], n, G)) * G + cell_of(r[0], n, G);
  cell[i] = c;
  atomicAdd(&count[c], 1);
}

__global__ void k_scan_int(int *a, int m) {
  __shared__ long long carry;
  __shared__ int sh[1024];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < m; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < m ? a[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int x = (int)threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += x;
      __syncthreads();
    }
    if (i < m) a[i] = (int)(carry + sh[threadIdx.x] - v);
    __syncthreads();
    if (threadIdx.x == 1023) carry += sh[1023];
    __syncthreads();
  }
}

__global__ void k_grp_scatter(const int *cell, int np, const int *start, int *fill, int *sorted) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const int c = cell[i];
  sorted[start[c] + atomicAdd(&fill[c], 1)] = i;
}

__global__ void k_grp_link(const double *rows, int width, int np, int n, int G, double th, const int *cell,
                           const int *start, const int *count, const int *sorted, int *par, int *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double *ri = rows + (int64_t)width * i;
  const int c = cell[i];
  const int cx = c % G, cy = (c / G) % G, cz = c / (G * G);
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int nc = ((cz + dz + G) % G * G + (cy + dy + G) % G) * G + (cx + dx + G) % G;
        for (int q = start[nc]; q < start[nc] + count[nc]; ++q) {
          const int j = sorted[q];
          if (j <= i) continue;
          if (lat_dist_periodic(n, ri, rows + (int64_t)width * j) <= th) uf_union(par, i, j, err);
        }
      }
}

__global__ void k_grp_link_all(const double *rows, int width, int np, int n, double th, int *par, int *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double *ri = rows + (int64_t)width * i;
  for (int j = i + 1; j < np; ++j)
    if (lat_dist_periodic(n, ri, rows + (int64_t)width * j) <= th) uf_union(par, i, j, err);
}

__global__ void k_grp_label(double *rows, int width, int gcol, int vcol, int np, int *par, double *tot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const int g = uf_find(par, i);
  rows[(int64_t)width * i + gcol] = (double)g;
  atomicAdd(&tot[g], rows[(int64_t)width * i + vcol]);
}

__global__ void k_grp_out(const int *par, const double *tot, int np, double t2, double t3, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np || par[i] != i) return;
  atomicAdd(&out[0], tot[i]);
  if (tot[i] > t2) atomicAdd(&out[1], tot[i]);
  if (tot[i] > t3) atomicAdd(&out[2], tot[i]);
  atomicAdd(&out[3], 1.0);
}

int grid_for(int64_t count, int per = 256) {
  int64_t b = (count + per - 1) / per;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b < 1 ? 1 : b);
}

int ensure_scratch(axg_ctx *ctx) {
  if (!ctx->phase) AXG_TRY(axg_alloc(ctx, (void **)&ctx->phase, (size_t)ctx->n3 * 4, "phase"));
  if (!ctx->flags) AXG_TRY(axg_alloc(ctx, (void **)&ctx->flags, (size_t)ctx->n3, "defect flags"));
  return AXG_OK;
}

int compute_phases(axg_ctx *ctx) {
  AXG_TRY(ensure_scratch(ctx));
  const void *phi = ctx->phi[ctx->cur];
  if (ctx->p.precision == AXG_PREC_FP32_MIXED)
    AXG_LAUNCH(ctx, "defect_phase_fp32", k_phase32<float2>, grid_for(ctx->n3), 256, 0,
               (const float2 *)phi, ctx->phase, ctx->n3);
  else
    AXG_LAUNCH(ctx, "defect_phase_fp64", k_phase32<double2>, grid_for(ctx->n3), 256, 0,
               (const double2 *)phi, ctx->phase, ctx->n3);
  return AXG_OK;
}

// grouping_strings / grouping_walls + the grouped branch of add_string_length
// / add_wall_area: out = (all, groups above t2, groups above t3, #groups)
int group_and_sum(axg_ctx *ctx, double *rows, int width, int gcol, int vcol, int64_t np64, double th, double t2,
                  double t3, double out[4]) {
  const int np = (int)np64;
  const int n = (int)ctx->n;
  int G = (int)std::floor(n / th);
  if (G > 64) G = 64;
  const bool grid = G >= 3;
  const int ncell = grid ? G * G * G : 1;
  int *ib = nullptr;
  double *db = nullptr;
  int rc = AXG_OK;
  auto cleanup = axg_on_exit([&] {
    cudaStreamSynchronize(ctx->stream);
    axg_free(ctx, (void **)&ib);
    axg_free(ctx, (void **)&db);
  });
  AXG_TRY(axg_alloc(ctx, (void **)&ib, sizeof(int) * ((size_t)4 * np + 3 * (size_t)ncell + 4), "grouping"));
  do {
    if ((rc = axg_alloc(ctx, (void **)&db, sizeof(double) * ((size_t)np + 4), "group totals"))) break;
    int *par = ib, *cell = ib + np, *sorted = ib + 2 * np, *count = ib + 3 * (size_t)np,
        *start = count + ncell, *fill = start + ncell;
    double *tot = db, *dout = db + np;
    AXG_CUDA_TRY(ctx, cudaMemsetAsync(ib + 3 * (size_t)np, 0, sizeof(int) * 3 * (size_t)ncell, ctx->stream));
    AXG_CUDA_TRY(ctx, cudaMemsetAsync(db, 0, sizeof(double) * ((size_t)np + 4), ctx->stream));
    const int blocks = (np + 255) / 256;
    AXG_LAUNCH(ctx, "group_init", k_grp_init, blocks, 256, 0, par, np);
    if (grid) {
      AXG_LAUNCH(ctx, "group_count", k_grp_count, blocks, 256, 0, rows, width, np, n, G, cell, count);
      AXG_CUDA_TRY(ctx, cudaMemcpyAsync(start, count, sizeof(int) * ncell, cudaMemcpyDeviceToDevice, ctx->stream));
      AXG_LAUNCH(ctx, "group_scan", k_scan_int, 1, 1024, 0, start, ncell);
      AXG_LAUNCH(ctx, "group_scatter", k_grp_scatter, blocks, 256, 0, cell, np, start, fill, sorted);
      AXG_LAUNCH(ctx, "group_link", k_grp_link, blocks, 256, 0, rows, width, np, n, G, th, cell, start, count, sorted,
                 par, ctx->d_err);
    } else {
      AXG_LAUNCH(ctx, "group_link_all", k_grp_link_all, blocks, 256, 0, rows, width, np, n, th, par, ctx->d_err);
    }
    AXG_LAUNCH(ctx, "group_label", k_grp_label, blocks, 256, 0, rows, width, gcol, vcol, np, par, tot);
    AXG_LAUNCH(ctx, "group_out", k_grp_out, blocks, 256, 0, par, tot, np, t2, t3, dout);
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(out, dout, sizeof(double) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    rc = axg_evo_check_error(ctx);
  } while (0);
  return rc;
}

// grouping threshold max(2, (width^2 hor)^(1/3)) (defects_3d.f90:1245-1246)
double group_threshold(double wid, double hor) {
  const double th = std::pow(wid * wid * hor, 1.0 / 3.0);
  return th > 2.0 ? th : 2.0;
}

}  // namespace

int axg_def_classify(axg_ctx *ctx, int which, int64_t counts[3]) {
  AXG_TRY(compute_phases(ctx));
  AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_cnt, 0, 3 * sizeof(unsigned long long), ctx->stream));
  if (ctx->p.precision == AXG_PREC_FP32_MIXED)
    AXG_LAUNCH(ctx, "defect_classify", k_classify<float2>, grid_for(ctx->n3), 256, 0, ctx->phase,
               (const float2 *)ctx->phi[ctx->cur], (const float2 *)ctx->cphi, (int)ctx->n, which, ctx->flags,
               ctx->d_cnt);
  else
    AXG_LAUNCH(ctx, "defect_classify", k_classify<double2>, grid_for(ctx->n3), 256, 0, ctx->phase,
               (const double2 *)ctx->phi[ctx->cur], (const double2 *)nullptr, (int)ctx->n, which, ctx->flags,
               ctx->d_cnt);
  unsigned long long h[3];
  AXG_CUDA_TRY(ctx, cudaMemcpyAsync(h, ctx->d_cnt, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < 3; ++k) counts[k] = (int64_t)h[k];
  ctx->flags_valid = true;
  ctx->last_ns = counts[0];
  ctx->last_nw = counts[1];
  ctx->last_nm = counts[2];
  return AXG_OK;
}

int axg_def_winding(axg_ctx *ctx, int64_t counts[3]) {
  AXG_TRY(compute_phases(ctx));
  AXG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_cnt + 3, 0, 3 * sizeof(unsigned long long), ctx->stream));
  if (ctx->p.precision == AXG_PREC_FP32_MIXED)
    AXG_LAUNCH(ctx, "string_winding", k_winding<float2>, grid_for(ctx->n3), 256, 0, ctx->phase,
               (const float2 *)ctx->phi[ctx->cur], (const float2 *)ctx->cphi, (int)ctx->n, ctx->d_cnt + 3);
  else
    AXG_LAUNCH(ctx, "string_winding", k_winding<double2>, grid_for(ctx->n3), 256, 0, ctx->phase,
               (const double2 *)ctx->phi[ctx->cur], (const double2 *)nullptr, (int)ctx->n, ctx->d_cnt + 3);
  unsigned long long h[3];
  AXG_CUDA_TRY(ctx, cudaMemcpyAsync(h, ctx->d_cnt + 3, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < 3; ++k) counts[k] = (int64_t)h[k];
  return AXG_OK;
}

int axg_def_id_defects(axg_ctx *ctx, double tau, double sl[3], double wa[3], double svel[3],
                       int64_t counts[3]) {
  const int which = ctx->p.flags & (AXG_F_ID_STRINGS | AXG_F_ID_WALLS | AXG_F_SPEC_EST);
  AXG_TRY(axg_def_classify(ctx, which, counts));
  const int64_t ns = counts[0], nw = counts[1];
  const int nb = (int)((ctx->n3 + kChunk - 1) / kChunk);
  int *bc = nullptr;
  int64_t *cells = nullptr;
  int rc = AXG_OK;
  AXG_TRY(axg_alloc(ctx, (void **)&bc, (size_t)nb * 2 * sizeof(int), "block counts"));
  do {
    if ((rc = axg_alloc(ctx, (void **)&cells, (size_t)(ns + nw + 1) * 8, "defect cells"))) break;
    if (ns > ctx->cap_strings) {
      axg_free(ctx, (void **)&ctx->d_strings);
      if ((rc = axg_alloc(ctx, (void **)&ctx->d_strings, (size_t)ns * 13 * 8, "string list"))) break;
      ctx->cap_strings = ns;
    }
    if (nw > ctx->cap_walls) {
      axg_free(ctx, (void **)&ctx->d_walls);
      if ((rc = axg_alloc(ctx, (void **)&ctx->d_walls, (size_t)nw * 10 * 8, "wall list"))) break;
      ctx->cap_walls = nw;
    }
    AXG_LAUNCH(ctx, "defect_block_count", k_block_count, nb, kCThreads, 0, ctx->flags, ctx->n3, bc,
               bc + nb);
    AXG_LAUNCH(ctx, "defect_scan", k_scan_blocks, 1, 1024, 0, bc, bc + nb, nb);
    AXG_LAUNCH(ctx, "defect_compact", k_compact, nb, kCThreads, 0, ctx->flags, ctx->n3, bc, bc + nb,
               cells, cells + ns);
    const int n = (int)ctx->n;
    const bool f32 = ctx->p.precision == AXG_PREC_FP32_MIXED;
    if (ns + nw > 0) {
      if (!ctx->phase64) AXG_TRY(axg_alloc(ctx, (void **)&ctx->phase64, (size_t)ctx->n3 * 8, "FP64 phases"));
      if (f32)
        AXG_LAUNCH(ctx, "fit_phases_fp64", k_phase64_all<float2>, grid_for(ctx->n3), 256, 0,
                   (const float2 *)ctx->phi[ctx->cur], (const float2 *)ctx->cphi, ctx->n3, ctx->phase64);
      else
        AXG_LAUNCH(ctx, "fit_phases_fp64", k_phase64_all<double2>, grid_for(ctx->n3), 256, 0,
                   (const double2 *)ctx->phi[ctx->cur], (const double2 *)nullptr, ctx->n3, ctx->phase64);
    }
    if (ns > 0) {
      // resident CTAs only: lanes take cells from a counter (d_cnt[8])
      int per_sm = 0, sms = 0;
      AXG_CUDA_TRY(ctx, f32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_string_fit<float2>, 128, 0)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_string_fit<double2>, 128, 0));
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
      int64_t grid = (int64_t)std::max(per_sm, 1) * std::max(sms, 1);
      grid = std::min<int64_t>(grid, (ns + 127) / 128);
      unsigned long long *next = ctx->d_cnt + 8;
      AXG_CUDA_TRY(ctx, cudaMemsetAsync(next, 0, sizeof(unsigned long long), ctx->stream));
      if (f32)
        AXG_LAUNCH(ctx, "string_fit_fp32", k_string_fit<float2>, (unsigned)grid, 128, 0,
                   (const float2 *)ctx->phi[ctx->cur], (const float2 *)ctx->cphi, ctx->phase64,
                   (const float2 *)ctx->phid, n, ctx->p.dspa, (uint64_t)ctx->p.seed, cells, ns, ctx->d_strings,
                   next);
      else
        AXG_LAUNCH(ctx, "string_fit_fp64", k_string_fit<double2>, (unsigned)grid, 128, 0,
                   (const double2 *)ctx->phi[ctx->cur], (const double2 *)nullptr, ctx->phase64,
                   (const double2 *)ctx->phid, n, ctx->p.dspa, (uint64_t)ctx->p.seed, cells, ns, ctx->d_strings,
                   next);
    }
    if (nw > 0) {
      AXG_LAUNCH(ctx, "wall_fit", k_wall_fit, (unsigned)((nw + 127) / 128), 128, 0, ctx->phase64, n, cells + ns,
                 nw, ctx->d_walls);
    }
    AXG_LAUNCH(ctx, "defect_sums", k_defect_sums, 1, 256, 0, ctx->d_strings, ns, ctx->d_walls, nw,
               ctx->d_red);
    double h[6];
    if (cudaMemcpyAsync(h, ctx->d_red, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
      rc = axg_set_error(ctx, AXG_ERR_CUDA, "defect sums");
      break;
    }
    sl[0] = sl[1] = sl[2] = h[0];
    if (h[4] > 0) {
      svel[0] = h[1] / h[4];
      svel[1] = h[2] / h[4];
      svel[2] = h[3] / h[4];
    } else {
      svel[0] = svel[1] = svel[2] = 0.0;
    }
    wa[0] = wa[1] = wa[2] = h[5];
    const double kPi = 3.14159265359, hor = tau / ctx->p.dspa;
    if ((ctx->p.flags & AXG_F_GROUP_STRINGS) && ns > 0) {
      double g[4];
      const double th = group_threshold(ctx->p.width_cr / ctx->p.dspa / tau, hor);
      if ((rc = group_and_sum(ctx, ctx->d_strings, 13, 12, 10, ns, th, 2 * hor, 2 * kPi * hor, g))) break;
      sl[0] = g[0];
      sl[1] = g[1];
      sl[2] = g[2];
    }
    if ((ctx->p.flags & AXG_F_GROUP_WALLS) && nw > 0) {
      double g[4];
      const double th = group_threshold(ctx->p.thickness_cr / ctx->p.dspa / tau, hor);
      if ((rc = group_and_sum(ctx, ctx->d_walls, 10, 9, 7, nw, th, kPi * hor * hor, 4 * kPi * hor * hor, g))) break;
      wa[0] = g[0];
      wa[1] = g[1];
      wa[2] = g[2];
    }
    ctx->last_ns = ns;
    ctx->last_nw = nw;
  } while (0);
  cudaStreamSynchronize(ctx->stream);
  axg_free(ctx, (void **)&bc);
  axg_free(ctx, (void **)&cells);
  return rc;
}

extern "C" {

int axg_classify_cells(axg_ctx *ctx, int which, int64_t counts[3]) {
  if (!ctx || !counts) return AXG_ERR_ARG;
  return axg_def_classify(ctx, which & 7, counts);
}

int axg_download_defect_flags(axg_ctx *ctx, int8_t *flags) {
  if (!ctx || !flags) return AXG_ERR_ARG;
  if (!ctx->flags || !ctx->flags_valid)
    return axg_set_error(ctx, AXG_ERR_STATE, "no classification since the last state change");
  AXG_CUDA_TRY(ctx, cudaMemcpyAsync(flags, ctx->flags, (size_t)ctx->n3, cudaMemcpyDeviceToHost, ctx->stream));
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return AXG_OK;
}

int axg_string_winding(axg_ctx *ctx, int64_t counts[3]) {
  if (!ctx || !counts) return AXG_ERR_ARG;
  return axg_def_winding(ctx, counts);
}

int axg_id_defects(axg_ctx *ctx, int64_t idx, double tau, double sl[3], double wa[3], double svel[3],
                   int64_t counts[3]) {
  (void)idx;
  if (!ctx || !sl || !wa || !svel || !counts) return AXG_ERR_ARG;
  return axg_def_id_defects(ctx, tau, sl, wa, svel, counts);
}

int axg_download_defect_lists(axg_ctx *ctx, double *strings, int64_t max_strings, double *walls,
                              int64_t max_walls) {
  if (!ctx) return AXG_ERR_ARG;
  const int64_t ns = std::min(max_strings, ctx->last_ns), nw = std::min(max_walls, ctx->last_nw);
  if (strings && ns > 0 && ctx->d_strings)
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(strings, ctx->d_strings, (size_t)ns * 13 * 8, cudaMemcpyDeviceToHost, ctx->stream));
  if (walls && nw > 0 && ctx->d_walls)
    AXG_CUDA_TRY(ctx, cudaMemcpyAsync(walls, ctx->d_walls, (size_t)nw * 10 * 8, cudaMemcpyDeviceToHost, ctx->stream));
  AXG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return AXG_OK;
}

}  // extern "C"
