// axg_gw_source.h -- the FP64 Green's-function sources at one site
// (grav_waves.f90:323-356 data1_to_arr_dphi and :209-232): the central
// differences d_i phi = (phi(x + e_i) - phi(x - e_i)) / d, d = 2 dx, then
// S_ij = 2 ((d_i phi)_re (d_j phi)_re + (d_i phi)_im (d_j phi)_im) for
// (i, j) = (1,1),(2,1),(2,2),(3,1),(3,2),(3,3), in the reference's operation
// order.  The division by d is a multiplication by 1/d when d is a power of
// two (the same single rounding), and the factor 2 is exact.
#ifndef AXG_GW_SOURCE_H
#define AXG_GW_SOURCE_H

#include "axg_detmath.h"
#include "axg_internal.h"

// xr[k], xi[k]: the raw differences (or their sums over a coarse cell) of
// direction k; divided by d, then the six products
__device__ __forceinline__ void gw_sources_from_diff(const double xr[3], const double xi[3], double d, double inv_d,
                                                     int d_pow2, double S[6]) {
  double dr[3], di[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    dr[k] = d_pow2 ? axg_mul_pow2(xr[k], inv_d) : AXD_DIV(xr[k], d);
    di[k] = d_pow2 ? axg_mul_pow2(xi[k], inv_d) : AXD_DIV(xi[k], d);
  }
  int c = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j, ++c)
      S[c] = axg_mul_pow2(AXD_ADD(AXD_MUL(dr[i], dr[j]), AXD_MUL(di[i], di[j])), 2.0);  // == r1 + r1
}

// pa[k], pb[k]: phi at x + e_k and x - e_k, k = x, y, z
__device__ __forceinline__ void gw_sources_fp64(const double2 pa[3], const double2 pb[3], double d, double inv_d,
                                                int d_pow2, double S[6]) {
  double xr[3], xi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    xr[k] = AXD_SUB(pa[k].x, pb[k].x);
    xi[k] = AXD_SUB(pa[k].y, pb[k].y);
  }
  gw_sources_from_diff(xr, xi, d, inv_d, d_pow2, S);
}

#endif  // AXG_GW_SOURCE_H
