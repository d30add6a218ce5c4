/*
 * axg_ffchi2.h -- the chi2 of the string fit (defects_3d.f90:385-433) in
 * float-float arithmetic, shared by the CUDA kernels and the C restatement
 * that checks them.
 *
 * GB300 issues FP64 at 1/64 of its FP32 rate, and the string fits of
 * id_defects evaluate this chi2 about 10^3 times per string cell (1001
 * random starts screened in FP32, then up to 1000 Nelder-Mead iterations),
 * each with eight atan2 and two sin/cos.  In FP64 that was the whole cost of
 * the fits.  Here every value is an unevaluated sum hi + lo of two floats
 * (about 48 significant bits) and every operation an IEEE-754 correctly
 * rounded FP32 primitive (+, -, *, /, sqrt, fused multiply-add) written
 * through the AXF_* macros: the __f*_rn intrinsics in device code, plain
 * float operators and fmaf / sqrtf / rintf in host code (compiled with
 * -ffp-contract=off).  The result is bit-identical on the GPU and on any
 * IEEE host, and within about 1e-14 of the FP64 chi2 (a CPU test compares
 * the two).
 *
 * The float-float primitives are the error-free transformations of Dekker
 * and Knuth (two-sum, product by fused multiply-add) with one
 * renormalisation, as in T. J. Dekker, "A floating-point technique for
 * extending the available precision", Numer. Math. 18 (1971).
 *   sin / cos : x in [-pi, pi] reduced by k pi/2 (pi/2 in three floats),
 *               Taylor series to r^17 / r^16 on |r| <= pi/4 (the terms
 *               from r^10 on in FP32);
 *   atan2     : the table-driven reduction of axd_atan2 (axg_detmath.h),
 *               atan(n/d) = atan(k/8) + atan(r), r = (n - c d)/(d + c n),
 *               atan(r) = r + r r^2 Q(r^2) with Q to r^14 (the terms past
 *               r^6 in FP32, where they lie below 2^-32 of r).
 */
#ifndef AXG_FFCHI2_H
#define AXG_FFCHI2_H

#include "axg_detmath.h"

/* AXD_UNROLL unrolls a loop with constant trip count in device code;
 * AXD_NOINL keeps one copy of a large function in device code (the fully
 * inlined chi2, eight atan2 and two sin/cos, overflowed the instruction
 * cache: most issue slots then stalled on instruction fetch) */
#if defined(__CUDACC__)
#define AXD_UNROLL _Pragma("unroll")
#define AXD_NOUNROLL _Pragma("unroll 1")
#define AXD_NOINL static __host__ __device__ __noinline__
#else
#define AXD_UNROLL
#define AXD_NOUNROLL
#define AXD_NOINL static
#endif

#if defined(__CUDA_ARCH__)
#define AXF_SUB(a, b) __fsub_rn((a), (b))
#define AXF_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define AXF_SQRT(a) __fsqrt_rn((a))
#define AXF_RINT(a) rintf((a))
#define AXF_FROM_D(x) __double2float_rn((x))
#else
#define AXF_SUB(a, b) ((a) - (b))
#define AXF_FMA(a, b, c) fmaf((a), (b), (c))
#define AXF_SQRT(a) sqrtf((a))
#define AXF_RINT(a) rintf((a))
#define AXF_FROM_D(x) ((float)(x))
#endif

typedef struct {
  float h, l;
} axd_ff;

AXD_FN axd_ff axd_ff_mk(float h, float l) {
  axd_ff r;
  r.h = h;
  r.l = l;
  return r;
}

/* |a| >= |b| or a == 0 */
AXD_FN axd_ff axd_ff_fast2sum(float a, float b) {
  const float s = AXF_ADD(a, b);
  return axd_ff_mk(s, AXF_SUB(b, AXF_SUB(s, a)));
}

AXD_FN axd_ff axd_ff_add(axd_ff a, axd_ff b) {
  const float s = AXF_ADD(a.h, b.h);
  const float v = AXF_SUB(s, a.h);
  float e = AXF_ADD(AXF_SUB(a.h, AXF_SUB(s, v)), AXF_SUB(b.h, v));
  e = AXF_ADD(e, AXF_ADD(a.l, b.l));
  return axd_ff_fast2sum(s, e);
}

AXD_FN axd_ff axd_ff_neg(axd_ff a) { return axd_ff_mk(-a.h, -a.l); }
AXD_FN axd_ff axd_ff_sub(axd_ff a, axd_ff b) { return axd_ff_add(a, axd_ff_neg(b)); }

AXD_FN axd_ff axd_ff_mul(axd_ff a, axd_ff b) {
  const float p = AXF_MUL(a.h, b.h);
  float e = AXF_FMA(a.h, b.h, -p);
  e = AXF_FMA(a.h, b.l, e);
  e = AXF_FMA(a.l, b.h, e);
  return axd_ff_fast2sum(p, e);
}

AXD_FN axd_ff axd_ff_mulf(axd_ff a, float f) {
  const float p = AXF_MUL(a.h, f);
  float e = AXF_FMA(a.h, f, -p);
  e = AXF_FMA(a.l, f, e);
  return axd_ff_fast2sum(p, e);
}

/* a / b: the float quotient of the high parts, corrected once by the
 * float-float remainder */
AXD_FN axd_ff axd_ff_div(axd_ff a, axd_ff b) {
  const float q1 = AXF_DIV(a.h, b.h);
  const axd_ff r = axd_ff_sub(a, axd_ff_mulf(b, q1));
  return axd_ff_fast2sum(q1, AXF_DIV(r.h, b.h));
}

/* sqrt(a), a >= 0: the float root corrected once by the remainder */
AXD_FN axd_ff axd_ff_sqrt(axd_ff a) {
  if (!(a.h > 0.0f)) return axd_ff_mk(0.0f, 0.0f);
  const float s = AXF_SQRT(a.h);
  const axd_ff r = axd_ff_sub(a, axd_ff_mulf(axd_ff_mk(s, 0.0f), s));
  return axd_ff_fast2sum(s, AXF_DIV(r.h, AXF_MUL(2.0f, s)));
}

AXD_FN axd_ff axd_ff_from(double x) {
  const float h = AXF_FROM_D(x);
  return axd_ff_mk(h, AXF_FROM_D(AXD_SUB(x, (double)h)));
}

AXD_FN double axd_ff_to(axd_ff a) { return AXD_ADD((double)a.h, (double)a.l); }

/* a >= b, a > b on the (renormalised) pairs */
AXD_FN int axd_ff_ge(axd_ff a, axd_ff b) { return a.h > b.h || (a.h == b.h && a.l >= b.l); }
AXD_FN int axd_ff_gt(axd_ff a, axd_ff b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }

/* sin and cos of x, |x| <= pi (+ a few ulp), as float-float pairs */
AXD_NOINL void axd_ff_sincos(axd_ff x, axd_ff *s_out, axd_ff *c_out) {
  /* pi/2 = P1 + P2 + P3 to about 2^-76; k P_i is exact for |k| <= 2 */
  const float P1 = 1.5707963705062866f, P2 = -4.371138828673793e-08f, P3 = -1.7151245100058819e-15f;
  const float kf = AXF_RINT(AXF_MUL(x.h, 0.6366197723675814f));
  axd_ff r = axd_ff_add(x, axd_ff_mk(-AXF_MUL(kf, P1), 0.0f));
  r = axd_ff_add(r, axd_ff_mk(-AXF_MUL(kf, P2), 0.0f));
  r = axd_ff_add(r, axd_ff_mk(-AXF_MUL(kf, P3), 0.0f));
  const int q = (int)kf & 3;
  const axd_ff r2 = axd_ff_mul(r, r);
  /* (-1)^k / (2k+1)! and (-1)^k / (2k)! as float-float pairs */
  const float ks[9][2] = {{1.0f, 0.0f},
                          {-0.1666666716337204f, 4.967053879312289e-09f},
                          {0.008333333767950535f, -4.34617203337595e-10f},
                          {-0.00019841270113829523f, 2.725596874933456e-12f},
                          {2.7557318844628753e-06f, 3.793571224297229e-14f},
                          {-2.5052107943679403e-08f, -4.4176230446483665e-16f},
                          {1.6059044372074283e-10f, -5.352526511562726e-18f},
                          {-7.647163609812713e-13f, -1.2200710471178288e-20f},
                          {2.8114573589663704e-15f, -1.0462084739763658e-22f}};
  const float kc[9][2] = {{1.0f, 0.0f},
                          {-0.5f, 0.0f},
                          {0.0416666679084301f, -1.2417634698280722e-09f},
                          {-0.0013888889225199819f, 3.3631094437103215e-11f},
                          {2.4801587642286904e-05f, -3.40699609366682e-13f},
                          {-2.755731998149713e-07f, 7.575112209051195e-15f},
                          {2.0876755879584152e-09f, 1.1082839147459852e-16f},
                          {-1.147074536050896e-11f, -2.372207689231238e-19f},
                          {4.7794772561329454e-14f, 7.62544404448643e-22f}};
  /* the terms from r^10 on lie below 3e-9 of the result, so their float
   * rounding stays below 2^-50 of it: they are summed in FP32 */
  const float t = r2.h;
  float fs = ks[8][0], fc = kc[8][0];
  AXD_UNROLL
  for (int k = 7; k >= 5; --k) {
    fs = AXF_FMA(fs, t, ks[k][0]);
    fc = AXF_FMA(fc, t, kc[k][0]);
  }
  axd_ff ps = axd_ff_mk(fs, 0.0f), pc = axd_ff_mk(fc, 0.0f);
  AXD_UNROLL
  for (int k = 4; k >= 0; --k) {
    ps = axd_ff_add(axd_ff_mul(ps, r2), axd_ff_mk(ks[k][0], ks[k][1]));
    pc = axd_ff_add(axd_ff_mul(pc, r2), axd_ff_mk(kc[k][0], kc[k][1]));
  }
  const axd_ff s0 = axd_ff_mul(ps, r), c0 = pc;
  /* x = q pi/2 + r */
  axd_ff sn = (q & 1) ? c0 : s0, cs = (q & 1) ? s0 : c0;
  if (q == 2 || q == 3) sn = axd_ff_neg(sn);
  if (q == 1 || q == 2) cs = axd_ff_neg(cs);
  *s_out = sn;
  *c_out = cs;
}

/* atan(k/8), k = 0..8, as a float-float pair (from the double-double
 * values of axg_detmath.h), by selects */
AXD_FN axd_ff axd_ff_atan_tab(int k) {
  const float tab[9][2] = {{0.0f, 0.0f},
                           {0.12435499578714371f, -1.240382241363136e-09f},
                           {0.244978666305542f, -3.1786777654474463e-09f},
                           {0.3587706685066223f, 1.7639498750554594e-09f},
                           {0.46364760398864746f, 5.01215868808913e-09f},
                           {0.5585992932319641f, 2.2111597886009804e-08f},
                           {0.6435011029243469f, 5.868937336117597e-09f},
                           {0.7188299894332886f, 1.0188335508587443e-08f},
                           {0.7853981852531433f, -2.1855694143368964e-08f}};
  axd_ff r = axd_ff_mk(0.0f, 0.0f);
  AXD_UNROLL
  for (int i = 1; i < 9; ++i)
    if (k == i) r = axd_ff_mk(tab[i][0], tab[i][1]);
  return r;
}

/* the principal argument of x + i y as a float-float pair (0 when both are
 * zero) */
AXD_NOINL axd_ff axd_ff_atan2(axd_ff y, axd_ff x) {
  /* pi/2, pi as float-float pairs */
  const axd_ff pio2 = axd_ff_mk(1.5707963705062866f, -4.371138828673793e-08f);
  const axd_ff pi = axd_ff_mk(3.1415927410125732f, -8.742277657347586e-08f);
  const int sgnx = x.h < 0.0f || (x.h == 0.0f && x.l < 0.0f);
  const int sgny = y.h < 0.0f || (y.h == 0.0f && y.l < 0.0f);
  const axd_ff ax = sgnx ? axd_ff_neg(x) : x, ay = sgny ? axd_ff_neg(y) : y;
  const int swap = axd_ff_gt(ay, ax);
  const axd_ff n = swap ? ax : ay, d = swap ? ay : ax;
  if (!(d.h > 0.0f)) return axd_ff_mk(0.0f, 0.0f);
  int k = (int)AXF_ADD(AXF_MUL(AXF_DIV(n.h, d.h), 8.0f), 0.5f);
  k = k < 0 ? 0 : (k > 8 ? 8 : k);
  const float c = AXF_MUL((float)k, 0.125f); /* exact */
  const axd_ff r = axd_ff_div(axd_ff_sub(n, axd_ff_mulf(d, c)), axd_ff_add(d, axd_ff_mulf(n, c)));
  /* atan(r) = r + r r2 Q(r2), Q = -1/3 + r2/5 - r2^2/7 + r2^3 q(r2) */
  const axd_ff r2 = axd_ff_mul(r, r);
  const float t = r2.h;
  float q = -0.06666666666666667f;
  q = AXF_FMA(q, t, 0.07692307692307693f);
  q = AXF_FMA(q, t, -0.09090909090909091f);
  q = AXF_FMA(q, t, 0.1111111111111111f);
  axd_ff Q = axd_ff_add(axd_ff_mulf(r2, q), axd_ff_mk(-0.1428571492433548f, 6.38621200366174e-09f));
  Q = axd_ff_add(axd_ff_mul(Q, r2), axd_ff_mk(0.20000000298023224f, -2.9802322831784522e-09f));
  Q = axd_ff_add(axd_ff_mul(Q, r2), axd_ff_mk(-0.3333333432674408f, 9.934107758624577e-09f));
  const axd_ff at = axd_ff_add(r, axd_ff_mul(axd_ff_mul(r, r2), Q));
  axd_ff a = axd_ff_add(axd_ff_atan_tab(k), at);
  if (swap) a = axd_ff_sub(pio2, a);
  if (sgnx) a = axd_ff_sub(pi, a);
  return sgny ? axd_ff_neg(a) : a;
}

/* defects_3d.f90:385-433: chi2 of the straight-string model pr = (mu, phi,
 * radius, angle) against the corner phases ph[8] (float-float, from
 * axd_ff_from of the FP64 phases), corner i = (iz 2 + iy) 2 + ix at
 * offsets (ix, iy, iz) - 1/2:
 *   du = -u0 + mu (x cos phi + y sin phi) - z sqrt(1 - mu^2),
 *   dv = -v0 - x sin phi + y cos phi,  (u0, v0) = radius (cos, sin) angle,
 *   d = ph - atan2(dv, du) wrapped into [-pi, pi) (the reference's
 *   truncated pi), chi2 = <d^2> - <d>^2. */
AXD_FN double axd_chi2_string_ff(const axd_ff ph[8], const double pr[4]) {
  const axd_ff refpi = axd_ff_mk(3.1415927410125732f, -8.742257051608249e-08f);
  const axd_ff tworefpi = axd_ff_mk(6.2831854820251465f, -1.7484514103216497e-07f);
  axd_ff s4, c4, sp, cp;
  axd_ff_sincos(axd_ff_from(pr[3]), &s4, &c4);
  axd_ff_sincos(axd_ff_from(pr[1]), &sp, &cp);
  const axd_ff rad = axd_ff_from(pr[2]), mu = axd_ff_from(pr[0]);
  const axd_ff u0 = axd_ff_mul(rad, c4), v0 = axd_ff_mul(rad, s4);
  const axd_ff sm = axd_ff_sqrt(axd_ff_sub(axd_ff_mk(1.0f, 0.0f), axd_ff_mul(mu, mu)));
  /* x cos phi etc. for x = +-1/2 are exact halvings */
  const axd_ff hcp = axd_ff_mulf(cp, 0.5f), hsp = axd_ff_mulf(sp, 0.5f), hsm = axd_ff_mulf(sm, 0.5f);
  axd_ff a = axd_ff_mk(0.0f, 0.0f), b = axd_ff_mk(0.0f, 0.0f);
  AXD_NOUNROLL
  for (int i = 0; i < 8; ++i) {
    const int ix = i & 1, iy = (i >> 1) & 1, iz = i >> 2;
    const axd_ff xc = ix ? hcp : axd_ff_neg(hcp), ys = iy ? hsp : axd_ff_neg(hsp);
    const axd_ff xs = ix ? hsp : axd_ff_neg(hsp), yc = iy ? hcp : axd_ff_neg(hcp);
    const axd_ff zs = iz ? hsm : axd_ff_neg(hsm);
    const axd_ff du = axd_ff_sub(axd_ff_add(axd_ff_neg(u0), axd_ff_mul(mu, axd_ff_add(xc, ys))), zs);
    const axd_ff dv = axd_ff_add(axd_ff_sub(axd_ff_neg(v0), xs), yc);
    axd_ff d = axd_ff_sub(ph[i], axd_ff_atan2(dv, du));
    if (axd_ff_ge(d, refpi))
      d = axd_ff_sub(d, tworefpi);
    else if (axd_ff_gt(axd_ff_neg(refpi), d))
      d = axd_ff_add(d, tworefpi);
    a = axd_ff_add(a, axd_ff_mul(d, d));
    b = axd_ff_add(b, d);
  }
  a = axd_ff_mulf(a, 0.125f);
  b = axd_ff_mulf(b, 0.125f);
  return axd_ff_to(axd_ff_sub(a, axd_ff_mul(b, b)));
}

#endif /* AXG_FFCHI2_H */
