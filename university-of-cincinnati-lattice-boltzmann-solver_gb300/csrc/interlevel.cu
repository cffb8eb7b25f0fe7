// Coarse-fine transfer between two D3Q27 levels (refinement ratio 2, nodal
// indexing: fine node X lies on coarse node X/2 when every coordinate is even).
//
// explosion: every fine ghost node (state 1e7 .. 1.1e9, the reference's
//   encoding for fine nodes outside the level's valid region) takes the
//   nodal bilinear interpolation of the coarse level's populations: the mean
//   of the 1, 2, 4 or 8 coarse nodes around it (interlevel_interpolation.f95:
//   161-257 with amrex_interp_node_bilinear); a population that comes out
//   negative or NaN sends the node to the entropic equilibrium of the
//   interpolated density and velocity (the reference falls back to the coarse
//   equilibrium, interlevel_interpolation.f95:405-427).
// coalescence: every coarse node under a valid fine node takes the fine
//   node's populations (nodal injection, fine_to_coarse.f95:30-64 with
//   amrex_average_down_nodes).
//
// Both act on the post-collision populations each level keeps between steps;
// the maps (level indices) are built once on the host.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "lattice.cuh"

namespace elbm {
namespace {

template <typename T>
__device__ __forceinline__ double pop_value(const T* p, int64_t plane, int j, int64_t n);
template <>
__device__ __forceinline__ double pop_value<double>(const double* p, int64_t plane, int j, int64_t n) {
  return p[(int64_t)j * plane + n];
}
template <>
__device__ __forceinline__ double pop_value<float>(const float* p, int64_t plane, int j, int64_t n) {
  return (double)p[(int64_t)j * plane + n] + w27(j);  // FP32 storage holds deviations from w
}
template <typename T>
__device__ __forceinline__ void put_value(T* p, int64_t plane, int j, int64_t n, double f);
template <>
__device__ __forceinline__ void put_value<double>(double* p, int64_t plane, int j, int64_t n, double f) {
  p[(int64_t)j * plane + n] = f;
}
template <>
__device__ __forceinline__ void put_value<float>(float* p, int64_t plane, int j, int64_t n, double f) {
  p[(int64_t)j * plane + n] = (float)(f - w27(j));
}

// Entropic D3Q27 equilibrium f_i = rho w_i prod_k psi(u_k) zeta(u_k)^c_ik.
__device__ __forceinline__ double feq27(int i, double rho, const double u[3]) {
  double f = rho * w27(i);
  const int c[3] = {cx27(i), cy27(i), cz27(i)};
  for (int k = 0; k < 3; ++k) {
    const double s = sqrt(1.0 + 3.0 * u[k] * u[k]);
    f *= 2.0 - s;
    if (c[k] == 1) f *= (2.0 * u[k] + s) / (1.0 - u[k]);
    if (c[k] == -1) f *= (1.0 - u[k]) / (2.0 * u[k] + s);
  }
  return f;
}

// One thread per fine ghost node; src holds 8 coarse level indices per ghost
// node (unused slots repeat the first) and cnt how many are distinct.
template <typename T>
__global__ void explode_kernel(const T* __restrict__ coarse, int64_t cplane, T* __restrict__ fine, int64_t fplane,
                               const int32_t* __restrict__ ghost, const int32_t* __restrict__ src,
                               const uint8_t* __restrict__ cnt, int64_t n, unsigned long long* __restrict__ repaired) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const int k = cnt[g];
  const double inv = 1.0 / (double)k;  // k in {1, 2, 4, 8}: exact
  double f[Q27];
  bool bad = false;
  for (int j = 0; j < Q27; ++j) {
    double s = 0.0;
    for (int m = 0; m < k; ++m) s += pop_value(coarse, cplane, j, (int64_t)src[8 * g + m]);
    f[j] = s * inv;
    bad |= !(f[j] >= 0.0);
  }
  if (bad) {
    double rho = 0.0, j3[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < Q27; ++j) {
      rho += f[j];
      j3[0] += cx27(j) * f[j];
      j3[1] += cy27(j) * f[j];
      j3[2] += cz27(j) * f[j];
    }
    const double u[3] = {j3[0] / rho, j3[1] / rho, j3[2] / rho};
    for (int j = 0; j < Q27; ++j) f[j] = feq27(j, rho, u);
    atomicAdd(repaired, 1ull);
  }
  const int64_t dst = ghost[g];
  for (int j = 0; j < Q27; ++j) put_value(fine, fplane, j, dst, f[j]);
}

// One thread per (coarse node, population).
template <typename T>
__global__ void average_down_kernel(const T* __restrict__ fine, int64_t fplane, T* __restrict__ coarse, int64_t cplane,
                                    const int32_t* __restrict__ dst, const int32_t* __restrict__ src, int64_t n) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * Q27) return;
  const int64_t p = e / Q27;
  const int j = (int)(e % Q27);
  coarse[(int64_t)j * cplane + dst[p]] = fine[(int64_t)j * fplane + src[p]];
}

}  // namespace

void launch_explode(bool fp32, const void* coarse, int64_t cplane, void* fine, int64_t fplane, const int32_t* ghost,
                    const int32_t* src, const uint8_t* cnt, int64_t n, unsigned long long* repaired, cudaStream_t s) {
  if (n <= 0) return;
  const unsigned grid = (unsigned)((n + 127) / 128);
  if (fp32)
    explode_kernel<float><<<grid, 128, 0, s>>>((const float*)coarse, cplane, (float*)fine, fplane, ghost, src, cnt, n,
                                               repaired);
  else
    explode_kernel<double><<<grid, 128, 0, s>>>((const double*)coarse, cplane, (double*)fine, fplane, ghost, src, cnt,
                                                n, repaired);
}

void launch_average_down(bool fp32, const void* fine, int64_t fplane, void* coarse, int64_t cplane, const int32_t* dst,
                         const int32_t* src, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  const unsigned grid = (unsigned)((n * Q27 + 255) / 256);
  if (fp32)
    average_down_kernel<float><<<grid, 256, 0, s>>>((const float*)fine, fplane, (float*)coarse, cplane, dst, src, n);
  else
    average_down_kernel<double><<<grid, 256, 0, s>>>((const double*)fine, fplane, (double*)coarse, cplane, dst, src,
                                                     n);
}

}  // namespace elbm
