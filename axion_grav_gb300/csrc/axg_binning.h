// axg_binning.h -- shell binning shared by the spectra.
//
// Every shell bin the spectra use (nint(q/dq + 0.5) linear bins of
// grav_waves.f90:279 and spectrum.f90:538, the log bins) is a function of
// the integer |k|^2 alone, q = sqrt(|k|^2) dk.  axg_bin_table evaluates the
// same FP64 expressions once per |k|^2 on the host and keeps the table on the
// device, so a binning kernel does one 2-byte load per k instead of an FP64
// square root, division and rounding.  Kernels add into shared-memory bins
// through warp_bin_add: the lanes of a warp that hold the same bin are summed
// by shuffles and one lane adds the sum.
#pragma once
#include <cstdint>

#include "axg_internal.h"

enum axg_bin_kind {
  AXG_BIN_GW = 0,        // q > 0, linear or log bins (grav_waves.f90:279, log edges)
  AXG_BIN_SPECTRUM = 1,  // linear bins, bin 1 includes k = 0 (spectrum.f90:538)
};

// Device table of bins (-1: outside) indexed by |k|^2 in [0, 3 (m/2)^2] for an
// m^3 lattice; edges (nb + 1 values) only for log bins.  Cached in the context.
int axg_bin_table(axg_ctx *ctx, int kind, int m, double dwav, double dq, int nb, int logmode,
                  const double *edges, const int16_t **d_tab);

#ifdef __CUDACC__
// All 32 lanes must call this (b < 0: nothing to add).
__device__ __forceinline__ void warp_bin_add(double *sv, double *sw, int b, double v, double w) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  unsigned pending = __ballot_sync(full, b >= 0);
  while (pending) {
    const int leader = __ffs(pending) - 1;
    const int b0 = __shfl_sync(full, b, leader);
    const bool mine = b == b0;
    double x = mine ? v : 0.0, y = mine ? w : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_xor_sync(full, x, o);
      y += __shfl_xor_sync(full, y, o);
    }
    if (lane == leader) {
      atomicAdd(&sv[b0], x);
      atomicAdd(&sw[b0], y);
    }
    pending &= ~__ballot_sync(full, mine);
  }
}

__device__ __forceinline__ int kint_bin(int j, int n) { return (j + n / 2) % n - n / 2; }
#endif
