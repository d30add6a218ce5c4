// axg_binning.h -- shell binning shared by the spectra.
//
// Every shell bin the spectra use (nint(q/dq + 0.5) linear bins of
// grav_waves.f90:279 and spectrum.f90:538, the log bins) is a function of
// the integer |k|^2 alone, q = sqrt(|k|^2) dk.  axg_bin_table evaluates the
// same FP64 expressions once per |k|^2 on the host and keeps the table on the
// device, so a binning kernel does one 2-byte load per k instead of an FP64
// square root, division and rounding.  Kernels add into shared-memory bins
// through BinRun: each lane sums a short run of consecutive k-sites privately
// and adds to the shared bin only when its bin changes.
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
// Per-lane run accumulation: each lane walks kRun consecutive k-sites (along
// kx, so |k|^2 and the bin change slowly), sums privately and adds to the
// shared bins only when its bin changes.  FP64 work per site is one add.
constexpr int kRun = 4;

struct BinRun {
  int bin = -1;
  double v = 0.0;
  unsigned w = 0;  // count (or Hermitian weight sum, <= 2 per site)
  __device__ __forceinline__ void add(double *sv, double *sw, int b, double val, unsigned wt) {
    if (b != bin) {
      flush(sv, sw);
      bin = b;
      v = 0.0;
      w = 0;
    }
    if (b >= 0) {
      v += val;
      w += wt;
    }
  }
  __device__ __forceinline__ void flush(double *sv, double *sw) {
    if (bin >= 0 && w) {
      atomicAdd(&sv[bin], v);
      atomicAdd(&sw[bin], (double)w);
    }
    bin = -1;
  }
};

// first site of this lane's run and the stride between runs of one lane
__device__ __forceinline__ int64_t run_start() {
  return ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kRun;
}
__device__ __forceinline__ int64_t run_stride() { return (int64_t)gridDim.x * blockDim.x * kRun; }
#endif
