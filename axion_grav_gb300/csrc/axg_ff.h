// axg_ff.h -- float-float arithmetic for FP64-accuracy work on the FP32
// pipes (GB300 issues FP64 at 1/64 of its FP32 rate).
//
// A value is an unevaluated sum hi + lo of two floats, about 48 significant
// bits.  Every operation goes through the round-once intrinsics
// (__fadd_rn, __fmul_rn, __fmaf_rn), which the compiler never contracts, so
// the error-free transformations below stay exact:
//   f2_add  : Dekker's two-sum of the high parts, the low parts added, one
//             renormalisation (error below 2^-47 (|a| + |b|));
//   f2_dot2 : a b + s c d (s = +-1) as a two-term dot product: the exact
//             high products through FMAs, their two-sum and the low-part
//             cross terms, left unnormalised for the add that consumes it;
//   f2_mul  : a b likewise, unnormalised.
#ifndef AXG_FF_H
#define AXG_FF_H

#include <cuda_runtime.h>

struct F2 {
  float h, l;
};

__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  const float s = __fadd_rn(a.h, b.h);
  const float v = __fsub_rn(s, a.h);
  float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, v)), __fsub_rn(b.h, v));
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  const float h = __fadd_rn(s, e);
  return {h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ F2 f2_neg(F2 a) { return {-a.h, -a.l}; }

__device__ __forceinline__ F2 f2_sub(F2 a, F2 b) { return f2_add(a, f2_neg(b)); }

__device__ __forceinline__ F2 f2_dot2(F2 a, F2 b, F2 c, F2 d, float sg) {
  const float p1 = __fmul_rn(a.h, b.h), p2 = __fmul_rn(sg * c.h, d.h);
  const float s = __fadd_rn(p1, p2), v = __fsub_rn(s, p1);
  const float e0 = __fadd_rn(__fsub_rn(p1, __fsub_rn(s, v)), __fsub_rn(p2, v));
  const float e1 = __fmaf_rn(a.h, b.h, -p1), e2 = __fmaf_rn(sg * c.h, d.h, -p2);
  float t = __fmul_rn(sg * c.l, d.h);
  t = __fmaf_rn(sg * c.h, d.l, t);
  t = __fmaf_rn(a.l, b.h, t);
  t = __fmaf_rn(a.h, b.l, t);
  return {s, __fadd_rn(__fadd_rn(e0, __fadd_rn(e1, e2)), t)};
}

// a b, unnormalised (the exact high product through an FMA plus the cross
// terms of the low parts)
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return {p, e};
}

__device__ __forceinline__ F2 f2_half(F2 a) { return {__fmul_rn(a.h, 0.5f), __fmul_rn(a.l, 0.5f)}; }  // exact

__device__ __forceinline__ F2 f2_from(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}

// x = h + l from the bit fields of x, no FP64 instruction (for kernels whose
// FP64 pipe is busy with other work): h is x truncated to 24 significant
// bits (sign, rebiased exponent and the top 23 mantissa bits moved into a
// float), l the remaining 29 mantissa bits as an integer, converted to float
// (rounded to 24 bits) and scaled by the power of two of their place.
// |l| < ulp(h), about 48 significant bits in all.  Exponents outside
// [2^-74, 2^128), zeros, subnormals and non-finite x take f2_from.
__device__ __forceinline__ F2 f2_from_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e < 949u || e > 1150u) return f2_from(x);
  const unsigned sign = hi & 0x80000000u;
  const float h = __uint_as_float(sign | ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
  const float l = __fmul_rn(__uint2float_rn(lo & 0x1fffffffu), __uint_as_float((e - 948u) << 23));
  return {h, __uint_as_float(__float_as_uint(l) | sign)};
}

__device__ __forceinline__ double f2_to(F2 a) { return (double)a.h + (double)a.l; }

#endif  // AXG_FF_H
