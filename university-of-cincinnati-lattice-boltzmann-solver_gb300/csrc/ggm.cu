// Refinement tagging by the gradient of the gradient magnitude (GGM) of a
// macroscopic field of a D3Q39 level, on the device, from the fields the step
// keeps (GGM/derivatives/calculate_grad_mag.f95, calculate_gradgrad_mag.f95,
// GGM/populate_q.f95, derivatives/modules/derivatives.f95:644-760):
//   gm  = |grad q| with the second-order "windage" differences of every axis,
//   ggm = |grad gm| the same way, and a tag where ggm >= the level's limit.
// The differences pick their points from the node's link codes (a point is
// used when the link to it is >= 0), the reference's quirks kept: the central
// form is (q(-1) - q(+1)) / 2, and the up-wind form for a non-positive wind
// reads q(-1), q(-2) while it tests the links to +1, +2.  Points outside the
// box on a non-periodic axis hold the freestream value of q (the initial
// value of the nodes outside an external-flow domain) and gm = 0 there.
// Also the microphone sampler of the output (weighted node sums on the device).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "kernels.cuh"

namespace elbm {
namespace {

struct GgmArgs {
  const double* macro;  // rho, u, v, w, T planes
  int64_t plane;
  int nx, ny, nz, periodic;
  const uint16_t* mask;  // per node: bits 0-11 links +1,+2,-1,-2 of x, y, z >= 0; 12 node >= 0; 13 node == -666;
                         // 14: 0 <= node < 100000
  int variable, scheme;  // populate_q variable (1-8); 0 central, 1 up-wind, 2 down-wind
  double fs[5];          // freestream rho, u, v, w, T
};

__device__ __forceinline__ double q_of(int var, double rho, double u, double v, double w, double T) {
  switch (var) {
    case 1: return rho;
    case 2: return u;
    case 3: return v;
    case 4: return w;
    case 5: return rho * (T + (u * u + v * v + w * w) / 2.0);  // calculate_flow_variables.f95: press
    case 6: return T;
    case 7: return sqrt(u * u + v * v + w * w);
    default: return 0.5 * rho * sqrt(u * u + v * v + w * w);  // calculate_v_mag.f95 choice 2
  }
}

__device__ __forceinline__ int64_t ggm_node(const GgmArgs& a, int x, int y, int z) {
  if (a.periodic & 1) x = (x % a.nx + a.nx) % a.nx;
  else if (x < 0 || x >= a.nx) return -1;
  if (a.periodic & 2) y = (y % a.ny + a.ny) % a.ny;
  else if (y < 0 || y >= a.ny) return -1;
  if (a.periodic & 4) z = (z % a.nz + a.nz) % a.nz;
  else if (z < 0 || z >= a.nz) return -1;
  return ((int64_t)z * a.ny + y) * a.nx + x;
}

// derivative_windage_secondord (and _firstord for its fall-backs); q: q0, q+1, q+2, q-1, q-2;
// s: link bits +1, +2, -1, -2
__device__ double windage2(const double (&q)[5], const bool (&s)[4], double wind, int scheme) {
  const bool p1 = s[0], p2 = s[1], m1 = s[2], m2 = s[3];
  if (scheme == 0) {
    if (p1 && m1) return (q[3] - q[1]) / 2.0;
    if (p1) return q[1] - q[0];
    if (m1) return q[0] - q[3];
    return 0.0;
  }
  const bool pos = scheme == 1 ? wind > 0.0 : wind < 0.0;
  if (pos) {
    if (m1 && m2) return (3 * q[0] - 4 * q[3] + q[4]) / 2;
    return m1 ? q[3] - q[0] : 0.0;  // first order: the -1 point
  }
  if (p1 && p2) return (-3 * q[0] + 4 * q[3] - q[4]) / 2;
  return p1 ? q[0] - q[1] : 0.0;  // first order: the +1 point
}

__global__ void ggm_gm_kernel(const GgmArgs a, double* __restrict__ gm) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = (int64_t)a.nx * a.ny * a.nz;
  if (n >= N) return;
  const uint16_t m = a.mask[n];
  if (!((m >> 12) & 1u) && !((m >> 13) & 1u)) {  // state < 0 and not -666: solid
    gm[n] = 0.0;
    return;
  }
  const int x = (int)(n % a.nx), y = (int)((n / a.nx) % a.ny), z = (int)(n / ((int64_t)a.nx * a.ny));
  auto q_at = [&](int64_t k) -> double {
    if (k < 0) return q_of(a.variable, a.fs[0], a.fs[1], a.fs[2], a.fs[3], a.fs[4]);
    return q_of(a.variable, a.macro[k], a.macro[a.plane + k], a.macro[2 * a.plane + k], a.macro[3 * a.plane + k],
                a.macro[4 * a.plane + k]);
  };
  double sum = 0.0;
  for (int ax = 0; ax < 3; ++ax) {
    const int dx = ax == 0, dy = ax == 1, dz = ax == 2;
    const double q[5] = {q_at(n), q_at(ggm_node(a, x + dx, y + dy, z + dz)),
                         q_at(ggm_node(a, x + 2 * dx, y + 2 * dy, z + 2 * dz)),
                         q_at(ggm_node(a, x - dx, y - dy, z - dz)), q_at(ggm_node(a, x - 2 * dx, y - 2 * dy, z - 2 * dz))};
    const bool s[4] = {(bool)((m >> (4 * ax)) & 1u), (bool)((m >> (4 * ax + 1)) & 1u),
                       (bool)((m >> (4 * ax + 2)) & 1u), (bool)((m >> (4 * ax + 3)) & 1u)};
    const double d = windage2(q, s, a.macro[(1 + ax) * a.plane + n], a.scheme);
    sum = (ax == 0) ? d * d : sum + d * d;
  }
  gm[n] = sqrt(sum);
}

__global__ void ggm_tag_kernel(const GgmArgs a, const double* __restrict__ gm, double limit, double* __restrict__ ggm,
                               uint8_t* __restrict__ tags, unsigned long long* ntag) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = (int64_t)a.nx * a.ny * a.nz;
  if (n >= N) return;
  const uint16_t m = a.mask[n];
  double g = 0.0;
  if ((m >> 12) & 1u) {
    const int x = (int)(n % a.nx), y = (int)((n / a.nx) % a.ny), z = (int)(n / ((int64_t)a.nx * a.ny));
    auto gm_at = [&](int64_t k) -> double { return k < 0 ? 0.0 : gm[k]; };
    double sum = 0.0;
    for (int ax = 0; ax < 3; ++ax) {
      const int dx = ax == 0, dy = ax == 1, dz = ax == 2;
      const double q[5] = {gm[n], gm_at(ggm_node(a, x + dx, y + dy, z + dz)),
                           gm_at(ggm_node(a, x + 2 * dx, y + 2 * dy, z + 2 * dz)),
                           gm_at(ggm_node(a, x - dx, y - dy, z - dz)),
                           gm_at(ggm_node(a, x - 2 * dx, y - 2 * dy, z - 2 * dz))};
      const bool s[4] = {(bool)((m >> (4 * ax)) & 1u), (bool)((m >> (4 * ax + 1)) & 1u),
                         (bool)((m >> (4 * ax + 2)) & 1u), (bool)((m >> (4 * ax + 3)) & 1u)};
      const double d = windage2(q, s, a.macro[(1 + ax) * a.plane + n], a.scheme);
      sum = (ax == 0) ? d * d : sum + d * d;
    }
    g = sqrt(sum);
  }
  if (ggm) ggm[n] = g;
  const bool t = ((m >> 12) & 1u) && g >= limit;
  tags[n] = t ? 1 : 0;
  if (t) atomicAdd(ntag, 1ull);
}

// Predictive splitting (GGM/PGS/predictive_splitter.f95:36-316), after the GGM tags of
// the same variable: for a node with state >= 0 whose velocity has a dominant component
// (|u| > 5|v| and > 5|w|, else v, else w), scan along that axis on the side the flow comes
// from (u > 0: from pgs_reach nodes upstream, or the box edge, towards the node, taking the
// farthest hit; u <= 0: from the node outwards, taking the nearest) for a node with
// 0 <= state < 100000 and ggm >= 2 sensitivity, and tag the nodes with state >= 0 from
// the hit to the node; with no dominant component, tag every node within pgs_reach on the
// three axes (both sides) with 0 <= state < 100000 and ggm >= 3 sensitivity.  The scan
// stays inside the box (the reference's FABs add nghosts ghost nodes to its reach).
__global__ void ggm_pgs_kernel(const GgmArgs a, const double* __restrict__ ggm, double sens, int reach,
                               uint8_t* __restrict__ tags) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = (int64_t)a.nx * a.ny * a.nz;
  if (n >= N || !((a.mask[n] >> 12) & 1u)) return;
  const int p3[3] = {(int)(n % a.nx), (int)((n / a.nx) % a.ny), (int)(n / ((int64_t)a.nx * a.ny))};
  const int dim[3] = {a.nx, a.ny, a.nz};
  const int64_t stride[3] = {1, a.nx, (int64_t)a.nx * a.ny};
  const double vel[3] = {a.macro[a.plane + n], a.macro[2 * a.plane + n], a.macro[3 * a.plane + n]};
  const double pgs_limit = 2 * sens, pgs_upper = 3 * sens;
  auto eligible = [&](int64_t k) { return ((a.mask[k] >> 14) & 1u) != 0; };
  auto lo_of = [&](int ax) { return (p3[ax] - 0 > reach) ? p3[ax] - reach : 0; };
  auto hi_of = [&](int ax) { return (dim[ax] - 1 - p3[ax] > reach) ? p3[ax] + reach : dim[ax] - 1; };
  int ax = -1;
  if (fabs(vel[0]) > 5 * fabs(vel[1]) && fabs(vel[0]) > 5 * fabs(vel[2])) ax = 0;
  else if (fabs(vel[1]) > 5 * fabs(vel[0]) && fabs(vel[1]) > 5 * fabs(vel[2])) ax = 1;
  else if (fabs(vel[2]) > 5 * fabs(vel[1]) && fabs(vel[2]) > 5 * fabs(vel[0])) ax = 2;
  const int64_t base = n - (int64_t)p3[ax < 0 ? 0 : ax] * stride[ax < 0 ? 0 : ax];
  if (ax >= 0) {
    int hit = -1;
    if (vel[ax] > 0.0) {
      for (int q = lo_of(ax); q <= p3[ax]; ++q) {
        const int64_t k = base + q * stride[ax];
        if (eligible(k) && ggm[k] >= pgs_limit) {
          hit = q;
          break;
        }
      }
      if (hit >= 0)
        for (int q = hit; q <= p3[ax]; ++q)
          if ((a.mask[base + q * stride[ax]] >> 12) & 1u) tags[base + q * stride[ax]] = 1;
    } else {
      for (int q = p3[ax]; q <= hi_of(ax); ++q) {
        const int64_t k = base + q * stride[ax];
        if (eligible(k) && ggm[k] >= pgs_limit) {
          hit = q;
          break;
        }
      }
      if (hit >= 0)
        for (int q = p3[ax]; q <= hit; ++q)
          if ((a.mask[base + q * stride[ax]] >> 12) & 1u) tags[base + q * stride[ax]] = 1;
    }
    return;
  }
  for (int b = 0; b < 3; ++b) {
    const int64_t bb = n - (int64_t)p3[b] * stride[b];
    for (int q = lo_of(b); q <= hi_of(b); ++q) {
      const int64_t k = bb + q * stride[b];
      if (eligible(k) && ggm[k] >= pgs_upper) tags[k] = 1;
    }
  }
}

// mic_write.f95:45-110: per microphone the weighted sums over its 8 nodes of
// pressure, T, rho, u, v, w (pressure = rho (T + |u|^2 / 2) as the flow variables keep it)
__global__ void mic_sample_kernel(const double* __restrict__ macro, int64_t plane, int nmic,
                                  const int32_t* __restrict__ nodes, const double* __restrict__ wts,
                                  double* __restrict__ out) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmic) return;
  double p = 0.0, T = 0.0, r = 0.0, u = 0.0, v = 0.0, w = 0.0;
  for (int b = 0; b < 8; ++b) {
    const int64_t n = nodes[8 * m + b];
    const double wt = wts[8 * m + b];
    const double rho = macro[n], uu = macro[plane + n], vv = macro[2 * plane + n], ww = macro[3 * plane + n],
                 tt = macro[4 * plane + n];
    p = p + wt * (rho * (tt + (uu * uu + vv * vv + ww * ww) / 2.0));
    T = T + wt * tt;
    r = r + wt * rho;
    u = u + wt * uu;
    v = v + wt * vv;
    w = w + wt * ww;
  }
  out[6 * m + 0] = p;
  out[6 * m + 1] = T;
  out[6 * m + 2] = r;
  out[6 * m + 3] = u;
  out[6 * m + 4] = v;
  out[6 * m + 5] = w;
}

}  // namespace

void launch_mic_sample(const double* macro, int64_t plane, int nmic, const int32_t* nodes, const double* wts,
                       double* out, cudaStream_t s) {
  mic_sample_kernel<<<(unsigned)((nmic + 127) / 128), 128, 0, s>>>(macro, plane, nmic, nodes, wts, out);
}

void launch_ggm(const double* macro, int64_t plane, int nx, int ny, int nz, int periodic, const uint16_t* mask,
                int variable, int scheme, const double* fs, double limit, double* gm, double* ggm, uint8_t* tags,
                unsigned long long* ntag, cudaStream_t s) {
  GgmArgs a{macro, plane, nx, ny, nz, periodic, mask, variable, scheme, {fs[0], fs[1], fs[2], fs[3], fs[4]}};
  const int64_t N = (int64_t)nx * ny * nz;
  const unsigned blocks = (unsigned)((N + 255) / 256);
  ggm_gm_kernel<<<blocks, 256, 0, s>>>(a, gm);
  ggm_tag_kernel<<<blocks, 256, 0, s>>>(a, gm, limit, ggm, tags, ntag);
}

void launch_ggm_pgs(const double* macro, int64_t plane, int nx, int ny, int nz, const uint16_t* mask,
                    const double* ggm, double sensitivity, int reach, uint8_t* tags, cudaStream_t s) {
  GgmArgs a{macro, plane, nx, ny, nz, 0, mask, 0, 0, {0, 0, 0, 0, 0}};
  const int64_t N = (int64_t)nx * ny * nz;
  ggm_pgs_kernel<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(a, ggm, sensitivity, reach, tags);
}

}  // namespace elbm
