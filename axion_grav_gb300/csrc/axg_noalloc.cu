// axg_noalloc.cu -- volume moments of caller-owned device fields, allocating
// nothing.
//
// axg_field_moments (axg_ic.cu) reduces through a buffer that the context
// allocated with cudaMalloc.  Some callers cannot allocate device memory at
// the point where they want these diagnostics: a host code whose whole device
// memory is already handed to its own allocator or pool (a large lattice run
// typically reserves almost all HBM for its fields), or code that must not
// call into the allocator at that point (cudaMalloc / cudaFree can
// synchronise the device and stall work already queued by the caller).
// axg_field_moments_noalloc serves them: the caller passes its own device
// arrays and a host output, and the only scratch -- one partial sum per
// z-plane -- lives in the file-scope array below, which is part of the
// library image: every GPU that loads the library holds it until the process
// exits.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "axg_internal.h"

namespace {

// One row of four partial sums per z-plane (at most kNoallocMaxPlanes planes,
// i.e. ngrid <= 2048) plus one row for the four totals: 64 KiB + 32 B.
constexpr int kNoallocMaxPlanes = 2048;
static __device__ __align__(256) double g_plane_partials[kNoallocMaxPlanes + 1][4];

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// One block per z-plane: the four per-site terms of axg_field_moments summed
// over the plane, written (not accumulated) into partials[z].
__global__ void k_moments_planes(const double2 *__restrict__ phi, const double2 *__restrict__ phid, int n,
                                 double idx2, double A, double B, double C, double D,
                                 double (*__restrict__ partials)[4]) {
  const int z = blockIdx.x;
  const int64_t n2 = (int64_t)n * n;
  double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  for (int64_t r = threadIdx.x; r < n2; r += blockDim.x) {
    const int ix = (int)(r % n), iy = (int)(r / n);
    const int64_t s = z * n2 + r;
    const double2 c = phi[s], d = phid[s];
    const double a = c.x, b = c.y;
    const double m = a * a + b * b;
    a0 += m;
    a1 += d.x * d.x + d.y * d.y;
    const int64_t nb[3] = {z * n2 + (int64_t)iy * n + (ix + 1 == n ? 0 : ix + 1),
                           z * n2 + (int64_t)(iy + 1 == n ? 0 : iy + 1) * n + ix,
                           (int64_t)(z + 1 == n ? 0 : z + 1) * n2 + (int64_t)iy * n + ix};
    double g = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double2 e = phi[nb[k]];
      const double dr = e.x - a, di = e.y - b;
      g += dr * dr + di * di;
    }
    a2 += g * idx2;
    a3 += 0.5 * A * m * m + B * m + 2 * C * a + D * (a * a - b * b);
  }
  __shared__ double sh[4][32];
  const double v[4] = {warp_sum(a0), warp_sum(a1), warp_sum(a2), warp_sum(a3)};
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 4; ++k) sh[k][threadIdx.x >> 5] = v[k];
  __syncthreads();
  if (threadIdx.x < 32) {
    for (int k = 0; k < 4; ++k) {
      double x = threadIdx.x < (blockDim.x >> 5) ? sh[k][threadIdx.x] : 0.0;
      x = warp_sum(x);
      if (threadIdx.x == 0) partials[z][k] = x;
    }
  }
}

// Sum the n plane partials in plane order (one warp per moment).
__global__ void k_moments_total(const double (*__restrict__ partials)[4], int n, double inv_n3,
                                double *__restrict__ out4) {
  const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double x = 0.0;
  for (int z = lane; z < n; z += 32) x += partials[z][k];
  x = warp_sum(x);
  if (lane == 0) out4[k] = x * inv_n3;
}

// Device address of g_plane_partials, looked up once per device.
std::mutex g_mu;
double (*g_addr[64])[4] = {};

int plane_partials_address(int dev, double (**out)[4], std::string *msg) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev < 0 || dev >= 64) {
    *msg = "device ordinal out of range";
    return AXG_ERR_ARG;
  }
  if (!g_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_plane_partials);
    if (e != cudaSuccess) {
      *msg = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return AXG_ERR_CUDA;
    }
    g_addr[dev] = reinterpret_cast<double (*)[4]>(p);
  }
  *out = g_addr[dev];
  return AXG_OK;
}

}  // namespace

extern "C" int axg_field_moments_noalloc(const axg_params *p, const double *d_phi, const double *d_phidot,
                                         double tau, double out[4], void *stream) {
  if (!p || !d_phi || !d_phidot || !out || !(tau > 0)) return axg_set_error(nullptr, AXG_ERR_ARG, "null argument or tau <= 0");
  const int n = p->ngrid;
  if (n < 2) return axg_set_error(nullptr, AXG_ERR_ARG, "ngrid < 2");
  if (n > kNoallocMaxPlanes)
    return axg_set_error(nullptr, AXG_ERR_ARG,
                         "axg_field_moments_noalloc: ngrid " + std::to_string(n) + " exceeds its scratch limit of " +
                             std::to_string(kNoallocMaxPlanes) + " z-planes");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return axg_set_error(nullptr, AXG_ERR_CUDA, "cudaGetDevice");
  double(*partials)[4] = nullptr;
  std::string msg;
  const int rc = plane_partials_address(dev, &partials, &msg);
  if (rc != AXG_OK) return axg_set_error(nullptr, rc, msg);
  double f[4], pot[4];
  axg_kick_coeffs(p, tau, 0.0, f, pot);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_moments_planes<<<n, 256, 0, st>>>(reinterpret_cast<const double2 *>(d_phi),
                                      reinterpret_cast<const double2 *>(d_phidot), n, 1.0 / (p->dspa * p->dspa),
                                      pot[0], pot[1], pot[2], pot[3], partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return axg_set_error(nullptr, AXG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  // every row a call reads was written by this call, so nothing needs clearing
  double *totals = partials[kNoallocMaxPlanes];
  k_moments_total<<<1, 128, 0, st>>>(partials, n, 1.0 / ((double)n * n * n), totals);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, totals, sizeof(double) * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return axg_set_error(nullptr, AXG_ERR_CUDA, std::string("moments: ") + cudaGetErrorString(e));
  return AXG_OK;
}
