/*
 * axg_detmath.h -- deterministic FP64 math shared by the CUDA kernels and the
 * C restatement used to check them.
 *
 * Every operation here is an IEEE-754 correctly rounded primitive (+, -, *, /,
 * sqrt, fused multiply-add) written through the AXD_* macros, which map to the
 * non-contractible __d*_rn / __fma_rn intrinsics in device code and to plain C
 * operators plus fma() in host code (host code must be compiled with
 * -ffp-contract=off).  The results are therefore bit-identical on the GPU and
 * on any IEEE host, which is what makes the string / wall / mask flags of the
 * cell classification (defects_3d.f90:70-96, 309-349) bit-exact between the
 * GPU path and the CPU restatement.
 *
 * The reference obtains cell-corner phases as aimag(log(phi))
 * (defects_3d.f90:92), i.e. the principal argument atan2(Im, Re).  axd_atan2
 * below is a project-written atan2:
 *   n = min(|x|,|y|), d = max(|x|,|y|), t = n / d in [0,1];
 *   k = round(8 t) from an FP32 ratio of n and d (bit fields only), c = k/8;
 *   atan t = atan(c) + atan(r),  r = (n - c d)/(d + c n) (one division, the
 *   numerator and denominator each one fused multiply-add), |r| <= 1/16 +
 *   2^-20;
 *   atan(r) = r - r^3/3 + r^5/5 - ... - r^15/15 (Taylor series of atan, the
 *   first omitted term is below 1e-18 relative);
 *   atan(k/8) is tabulated as a double-double (hi + lo) computed to 300 bits.
 * The quadrant is restored with pi/2 and pi carried as double-doubles.  This
 * is the classical table-driven argument reduction (e.g. J.-M. Muller,
 * "Elementary Functions", ch. 6); accuracy is 1 ulp.  Forming r from n and d
 * instead of from the rounded ratio t saves a division and the rounding of
 * t (the earlier form, r = (t - c)/(1 + t c), reached 2 ulp).
 *
 * axd_sincos reduces by pi/2 with a three-part Cody-Waite constant and uses
 * the Taylor series of sin / cos to degree 17 / 18 on |r| <= pi/4.
 *
 * The Philox4x32-10 counter-based generator follows J. K. Salmon, M. A. Moraes,
 * R. O. Dror, D. E. Shaw, "Parallel random numbers: as easy as 1, 2, 3"
 * (SC'11): multipliers 0xD2511F53 / 0xCD9E8D57, Weyl key increments
 * 0x9E3779B9 / 0xBB67AE85, ten rounds.
 */
#ifndef AXG_DETMATH_H
#define AXG_DETMATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define AXD_FN static __host__ __device__ __forceinline__
#else
#include <math.h>
#define AXD_FN static inline
#endif

#if defined(__CUDA_ARCH__)
#define AXD_ADD(a, b) __dadd_rn((a), (b))
#define AXD_SUB(a, b) __dsub_rn((a), (b))
#define AXD_MUL(a, b) __dmul_rn((a), (b))
#define AXD_DIV(a, b) __ddiv_rn((a), (b))
#define AXD_FMA(a, b, c) __fma_rn((a), (b), (c))
#define AXD_SQRT(a) __dsqrt_rn((a))
#define AXF_MUL(a, b) __fmul_rn((a), (b))
#define AXF_ADD(a, b) __fadd_rn((a), (b))
#define AXF_DIV(a, b) __fdiv_rn((a), (b))
#else
#define AXD_ADD(a, b) ((a) + (b))
#define AXD_SUB(a, b) ((a) - (b))
#define AXD_MUL(a, b) ((a) * (b))
#define AXD_DIV(a, b) ((a) / (b))
#define AXD_FMA(a, b, c) fma((a), (b), (c))
#define AXD_SQRT(a) sqrt((a))
#define AXF_MUL(a, b) ((a) * (b))
#define AXF_ADD(a, b) ((a) + (b))
#define AXF_DIV(a, b) ((a) / (b))
#endif

/* pi, pi/2 as double-doubles (hi + lo). */
#define AXD_PI_HI 3.141592653589793
#define AXD_PI_LO 1.2246467991473532e-16
#define AXD_PIO2_HI 1.5707963267948966
#define AXD_PIO2_LO 6.123233995736766e-17
#define AXD_TWO_OVER_PI 0.6366197723675814
/* pi/2 split for Cody-Waite reduction: P1, P2 carry 33 significant bits. */
#define AXD_CW_P1 1.5707963267341256
#define AXD_CW_P2 6.077100506303966e-11
#define AXD_CW_P3 2.0222662487959506e-21

AXD_FN double axd_atan_tab_hi(int k) {
  switch (k) {
    case 1: return 0.12435499454676144;
    case 2: return 0.24497866312686414;
    case 3: return 0.35877067027057225;
    case 4: return 0.4636476090008061;
    case 5: return 0.5585993153435624;
    case 6: return 0.6435011087932844;
    case 7: return 0.7188299996216245;
    case 8: return 0.7853981633974483;
    default: return 0.0;
  }
}

AXD_FN double axd_atan_tab_lo(int k) {
  switch (k) {
    case 1: return -3.1253241424539383e-18;
    case 2: return 1.0698755618734451e-17;
    case 3: return -2.4623815582638635e-17;
    case 4: return 2.2698777452961687e-17;
    case 5: return -5.4556305485916264e-18;
    case 6: return 1.5834785051444286e-17;
    case 7: return -2.1478388444456983e-17;
    case 8: return 3.061616997868383e-17;
    default: return 0.0;
  }
}

AXD_FN double axd_fabs(double v) {
  union { double d; uint64_t u; } b;
  b.d = v;
  b.u &= 0x7fffffffffffffffULL;
  return b.d;
}

AXD_FN int axd_signbit(double v) {
  union { double d; uint64_t u; } b;
  b.d = v;
  return (int)(b.u >> 63);
}

AXD_FN double axd_copysign(double mag, double sgn) {
  union { double d; uint64_t u; } m, s;
  m.d = mag;
  s.d = sgn;
  m.u = (m.u & 0x7fffffffffffffffULL) | (s.u & 0x8000000000000000ULL);
  return m.d;
}

AXD_FN uint64_t axd_bits(double v) {
  union { double d; uint64_t u; } b;
  b.d = v;
  return b.u;
}

AXD_FN float axd_f_from_bits(uint32_t v) {
  union { float f; uint32_t u; } b;
  b.u = v;
  return b.f;
}

/* k = round(8 n / d) for magnitudes 0 <= n <= d (d > 0): the FP32 ratio of
 * n and d, both scaled by d's exponent and cut to 24 significant bits from
 * their bit fields (no FP64 instruction; a subnormal or out-of-range n
 * counts as 0).  The bucket can be the neighbouring one only where 8 t lies
 * within 2^-20 of a half-integer, so |r| <= 1/16 + 2^-20 in axd_atan2. */
AXD_FN int axd_atan_bucket(double n, double d) {
  const uint64_t bn = axd_bits(n), bd = axd_bits(d);
  const int en = (int)(bn >> 52), ed = (int)(bd >> 52);
  const int e = en - ed + 127;
  const float nf = (e >= 1 && en > 0) ? axd_f_from_bits(((uint32_t)e << 23) | (uint32_t)((bn >> 29) & 0x7fffffu)) : 0.0f;
  const float df = axd_f_from_bits((127u << 23) | (uint32_t)((bd >> 29) & 0x7fffffu));
  const int k = (int)AXF_ADD(AXF_MUL(AXF_DIV(nf, df), 8.0f), 0.5f);
  return k > 8 ? 8 : k;
}

/* atan(r) = r + r r2 P(r2), P = -1/3 + r2/5 - r2^2/7 + ... - r2^6/15 */
AXD_FN double axd_atan_series(double r) {
  double r2 = AXD_MUL(r, r);
  double p = -0.06666666666666667;
  p = AXD_FMA(p, r2, 0.07692307692307693);
  p = AXD_FMA(p, r2, -0.09090909090909091);
  p = AXD_FMA(p, r2, 0.1111111111111111);
  p = AXD_FMA(p, r2, -0.14285714285714285);
  p = AXD_FMA(p, r2, 0.2);
  p = AXD_FMA(p, r2, -0.3333333333333333);
  return AXD_FMA(AXD_MUL(r, r2), p, r);
}

/* atan(n / d) for 0 <= n <= d as hi + lo pieces; the low-order part is
 * returned, the table value in *hi_out. */
AXD_FN double axd_atan_ratio_parts(double n, double d, double *hi_out) {
  const int k = axd_atan_bucket(n, d);
  const double c = (double)k * 0.125; /* exact */
  const double r = AXD_DIV(AXD_FMA(-c, d, n), AXD_FMA(c, n, d));
  *hi_out = axd_atan_tab_hi(k);
  return AXD_ADD(axd_atan_tab_lo(k), axd_atan_series(r)); /* low-order part */
}

/* Principal argument of x + i y in [-pi, pi]; C99 atan2 semantics for zeros. */
AXD_FN double axd_atan2(double y, double x) {
  if (x != x || y != y) return AXD_ADD(x, y);
  double ax = axd_fabs(x), ay = axd_fabs(y);
  if (ay == 0.0) {
    if (axd_signbit(x)) return axd_copysign(AXD_ADD(AXD_PI_HI, AXD_PI_LO), y);
    return y;
  }
  if (ax == 0.0) return axd_copysign(AXD_ADD(AXD_PIO2_HI, AXD_PIO2_LO), y);
  int swap = ay > ax;
  double num = swap ? ax : ay;
  double den = swap ? ay : ax;
  double hi;
  double lo = axd_atan_ratio_parts(num, den, &hi);
  double a;
  if (swap) {
    /* pi/2 - (hi + lo) */
    double s = AXD_SUB(AXD_PIO2_LO, lo);
    a = AXD_ADD(AXD_SUB(AXD_PIO2_HI, hi), s);
    if (axd_signbit(x)) {
      /* pi - a, with a in [pi/4, pi/2] */
      a = AXD_ADD(AXD_SUB(AXD_PI_HI, a), AXD_PI_LO);
    }
  } else {
    if (axd_signbit(x)) {
      /* pi - (hi + lo) */
      double s = AXD_SUB(AXD_PI_LO, lo);
      a = AXD_ADD(AXD_SUB(AXD_PI_HI, hi), s);
    } else {
      a = AXD_ADD(hi, lo);
    }
  }
  return axd_copysign(a, y);
}

/* sin and cos of x for |x| < 1e6 (Cody-Waite reduction by pi/2). */
AXD_FN void axd_sincos(double x, double *s_out, double *c_out) {
  double kf = AXD_MUL(x, AXD_TWO_OVER_PI);
#if defined(__CUDA_ARCH__)
  kf = rint(kf);
#else
  kf = rint(kf);
#endif
  double r = AXD_FMA(-kf, AXD_CW_P1, x);
  r = AXD_FMA(-kf, AXD_CW_P2, r);
  r = AXD_FMA(-kf, AXD_CW_P3, r);
  double r2 = AXD_MUL(r, r);
  /* sin r = r + r*r2*S(r2) */
  double ps = 2.8114572543455206e-15;
  ps = AXD_FMA(ps, r2, -7.647163731819816e-13);
  ps = AXD_FMA(ps, r2, 1.6059043836821613e-10);
  ps = AXD_FMA(ps, r2, -2.505210838544172e-08);
  ps = AXD_FMA(ps, r2, 2.7557319223985893e-06);
  ps = AXD_FMA(ps, r2, -0.0001984126984126984);
  ps = AXD_FMA(ps, r2, 0.008333333333333333);
  ps = AXD_FMA(ps, r2, -0.16666666666666666);
  double sr = AXD_FMA(AXD_MUL(r, r2), ps, r);
  /* cos r = 1 + r2*C(r2) */
  double pc = -1.5619206968586225e-16;
  pc = AXD_FMA(pc, r2, 4.779477332387385e-14);
  pc = AXD_FMA(pc, r2, -1.1470745597729725e-11);
  pc = AXD_FMA(pc, r2, 2.08767569878681e-09);
  pc = AXD_FMA(pc, r2, -2.755731922398589e-07);
  pc = AXD_FMA(pc, r2, 2.48015873015873e-05);
  pc = AXD_FMA(pc, r2, -0.001388888888888889);
  pc = AXD_FMA(pc, r2, 0.041666666666666664);
  pc = AXD_FMA(pc, r2, -0.5);
  double cr = AXD_FMA(r2, pc, 1.0);
  long long q = ((long long)kf) & 3;
  if (q == 0) { *s_out = sr; *c_out = cr; }
  else if (q == 1) { *s_out = cr; *c_out = -sr; }
  else if (q == 2) { *s_out = -sr; *c_out = -cr; }
  else { *s_out = -cr; *c_out = sr; }
}

AXD_FN double axd_sin(double x) { double s, c; axd_sincos(x, &s, &c); return s; }
AXD_FN double axd_cos(double x) { double s, c; axd_sincos(x, &s, &c); return c; }

/* ---------------- Philox4x32-10 ---------------- */
typedef struct { uint32_t v[4]; } axd_u32x4;

AXD_FN void axd_mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

AXD_FN axd_u32x4 axd_philox4x32_10(axd_u32x4 ctr, uint32_t k0, uint32_t k1) {
  for (int round = 0; round < 10; ++round) {
    if (round > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t hi0, lo0, hi1, lo1;
    axd_mulhilo32(0xD2511F53u, ctr.v[0], &hi0, &lo0);
    axd_mulhilo32(0xCD9E8D57u, ctr.v[2], &hi1, &lo1);
    axd_u32x4 o;
    o.v[0] = hi1 ^ ctr.v[1] ^ k0;
    o.v[1] = lo1;
    o.v[2] = hi0 ^ ctr.v[3] ^ k1;
    o.v[3] = lo0;
    ctr = o;
  }
  return ctr;
}

/* 53-bit uniform in (0,1] from two 32-bit words (never returns 0). */
AXD_FN double axd_u01_open0(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6); /* 53 bits */
  return ((double)m + 1.0) * 1.1102230246251565e-16;            /* 2^-53 */
}

/* 53-bit uniform in [0,1). */
AXD_FN double axd_u01(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)m * 1.1102230246251565e-16;
}

/*
 * Counter layout used for every random draw of this project:
 *   key   = (seed_lo, seed_hi)
 *   ctr   = (index_lo, index_hi, stream, realisation)
 * `index` is the 64-bit linear index of the object (Fourier mode, cell, ...)
 * and `stream` separates independent uses (phi, phidot, fit starts ...).
 */
AXD_FN axd_u32x4 axd_draw(uint64_t seed, uint32_t stream, uint32_t realisation, uint64_t index) {
  axd_u32x4 c;
  c.v[0] = (uint32_t)index;
  c.v[1] = (uint32_t)(index >> 32);
  c.v[2] = stream;
  c.v[3] = realisation;
  return axd_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

#endif /* AXG_DETMATH_H */
