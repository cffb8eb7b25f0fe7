// Host-side solid marking and wall-link fractions from a closed triangulated
// surface, in the reference's `state` encoding.
//
// The reference builds these at set-up in lbgrid/: fluid_or_solid (ray
// casting), state_directions, and inter_bb_setup.f95:44-246, which for every
// fluid node and direction finds where the link crosses a surface triangle
// and stores the crossing as state = -1001 - floor(|x - x_w| / link_dist * 1e9)
// (linking/modules/linkwise.f95:45-57, link_dist = |c_i| dx, link_info.f95:27).
// Only links from a fluid node to a solid node are searched, as in the
// reference, so a wall link never joins two fluid nodes.  This file produces
// the same encoding with a uniform-grid acceleration of the triangle search
// (the reference tests every triangle for every link).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/elbm_gb300.h"
#include "kernels39.cuh"
#include "lattice.cuh"

namespace {

struct Tri {
  double v[3][3];
  double n[3];  // (v1 - v0) x (v2 - v0)
  double lo[3], hi[3];
};

// Segment p0 -> p1 against one triangle: the plane parameter t in (0, 1] and
// an inside test by signed volumes, like inter_bb_setup.f95:90-150 and
// lbgrid/utilities/tri_volume.f95.  Returns t, or -1 when there is no crossing.
__host__ __device__ double seg_tri(const Tri& T, const double p0[3], const double p1[3]) {
  const double dotv = T.n[0] * T.v[0][0] + T.n[1] * T.v[0][1] + T.n[2] * T.v[0][2];
  const double upper = dotv - (p0[0] * T.n[0] + p0[1] * T.n[1] + p0[2] * T.n[2]);
  const double lower = (p1[0] - p0[0]) * T.n[0] + (p1[1] - p0[1]) * T.n[1] + (p1[2] - p0[2]) * T.n[2];
  if (lower == 0.0) return -1.0;
  const double t = upper / lower;
  if (!(t > 0.0 && t <= 1.0)) return -1.0;
  const double xc[3] = {p0[0] + t * (p1[0] - p0[0]), p0[1] + t * (p1[1] - p0[1]), p0[2] + t * (p1[2] - p0[2])};
  // signed volumes of the node, the crossing and each edge (tri_volume.f95:25-40)
  double e[3][3];
  for (int k = 0; k < 3; ++k)
    for (int a = 0; a < 3; ++a) e[k][a] = T.v[k][a] - p0[a];
  const double r[3] = {xc[0] - p0[0], xc[1] - p0[1], xc[2] - p0[2]};
  auto vol = [&](const double* a, const double* b) {
    return r[0] * (a[1] * b[2] - a[2] * b[1]) + r[1] * (a[2] * b[0] - a[0] * b[2]) + r[2] * (a[0] * b[1] - a[1] * b[0]);
  };
  const double v1 = vol(e[0], e[1]), v2 = -vol(e[0], e[2]), v3 = vol(e[1], e[2]);
  const bool pos = v1 >= 0.0 && v2 >= 0.0 && v3 >= 0.0, neg = v1 <= 0.0 && v2 <= 0.0 && v3 <= 0.0;
  return (pos || neg) ? t : -1.0;
}

// +x ray from p against one triangle, with half-open edge rules in the yz
// plane so that rays through shared edges and vertices count once.
__host__ __device__ bool ray_x_crosses(const Tri& T, const double p[3]) {
  const double y = p[1], z = p[2];
  // barycentric in the yz projection
  const double y0 = T.v[0][1], z0 = T.v[0][2], y1 = T.v[1][1], z1 = T.v[1][2], y2 = T.v[2][1], z2 = T.v[2][2];
  const double det = (y1 - y0) * (z2 - z0) - (y2 - y0) * (z1 - z0);
  if (det == 0.0) return false;
  auto edge = [&](double ay, double az, double by, double bz) {
    const double w = (by - ay) * (z - az) - (bz - az) * (y - ay);
    if (w != 0.0) return w;
    // on the edge line: own it when the edge is "top or left" (consistent tie-break)
    const bool top_left = (bz > az) || (bz == az && by < ay);
    return top_left ? 1e-300 : -1e-300;
  };
  double w0 = edge(y1, z1, y2, z2), w1 = edge(y2, z2, y0, z0), w2 = edge(y0, z0, y1, z1);
  if (det < 0.0) {
    w0 = -w0;
    w1 = -w1;
    w2 = -w2;
  }
  if (!(w0 > 0.0 && w1 > 0.0 && w2 > 0.0)) return false;
  // x of the plane at (y, z)
  const double nx = T.n[0];
  if (nx == 0.0) return false;
  const double xs = T.v[0][0] - (T.n[1] * (y - y0) + T.n[2] * (z - z0)) / nx;
  return xs > p[0];
}

}  // namespace

namespace {

// The triangles with their normals and bounding boxes, and a uniform grid of
// cells of 2 dx over the surface's bounding box listing the triangles that
// touch each cell and its neighbours (compressed rows).
struct TriGrid {
  std::vector<Tri> T;
  double glo[3], ghi[3], cell;
  int gn[3];
  std::vector<int32_t> start, tris;  // per cell: tris[start[c] .. start[c + 1])
};

void build_tri_grid(int ntri, const double* tri, double dx, TriGrid& G, double reach = 1.0) {
  G.T.resize(ntri);
  for (int c = 0; c < 3; ++c) {
    G.glo[c] = INFINITY;
    G.ghi[c] = -INFINITY;
  }
  for (int k = 0; k < ntri; ++k) {
    Tri& t = G.T[k];
    for (int v = 0; v < 3; ++v)
      for (int a = 0; a < 3; ++a) t.v[v][a] = tri[9 * k + 3 * v + a];
    const double a[3] = {t.v[1][0] - t.v[0][0], t.v[1][1] - t.v[0][1], t.v[1][2] - t.v[0][2]};
    const double b[3] = {t.v[2][0] - t.v[0][0], t.v[2][1] - t.v[0][1], t.v[2][2] - t.v[0][2]};
    t.n[0] = a[1] * b[2] - a[2] * b[1];
    t.n[1] = a[2] * b[0] - a[0] * b[2];
    t.n[2] = a[0] * b[1] - a[1] * b[0];
    for (int c = 0; c < 3; ++c) {
      t.lo[c] = std::min({t.v[0][c], t.v[1][c], t.v[2][c]});
      t.hi[c] = std::max({t.v[0][c], t.v[1][c], t.v[2][c]});
      G.glo[c] = std::min(G.glo[c], t.lo[c]);
      G.ghi[c] = std::max(G.ghi[c], t.hi[c]);
    }
  }
  // cells of 2 dx (D3Q27 links are at most sqrt(3) dx long) or of the longest D3Q39 link
  G.cell = std::max(2.0, reach) * dx;
  for (int c = 0; c < 3; ++c) G.gn[c] = std::max(1, (int)std::ceil((G.ghi[c] - G.glo[c]) / G.cell) + 1);
  const size_t ncell = (size_t)G.gn[0] * G.gn[1] * G.gn[2];
  std::vector<std::vector<int32_t>> lists(ncell);
  for (int k = 0; k < ntri; ++k) {
    int lo[3], hi[3];
    for (int c = 0; c < 3; ++c) {
      lo[c] = std::max(0, (int)std::floor((G.T[k].lo[c] - G.glo[c]) / G.cell) - 1);
      hi[c] = std::min(G.gn[c] - 1, (int)std::floor((G.T[k].hi[c] - G.glo[c]) / G.cell) + 1);
    }
    for (int c2 = lo[2]; c2 <= hi[2]; ++c2)
      for (int c1 = lo[1]; c1 <= hi[1]; ++c1)
        for (int c0 = lo[0]; c0 <= hi[0]; ++c0) lists[((size_t)c2 * G.gn[1] + c1) * G.gn[0] + c0].push_back(k);
  }
  G.start.assign(ncell + 1, 0);
  for (size_t c = 0; c < ncell; ++c) G.start[c + 1] = G.start[c] + (int32_t)lists[c].size();
  G.tris.resize(G.start[ncell]);
  for (size_t c = 0; c < ncell; ++c) std::copy(lists[c].begin(), lists[c].end(), G.tris.begin() + G.start[c]);
}

// The ray starts a tiny irrational offset off the lattice line, so that it passes
// through no vertex or edge of a surface built on lattice points.
constexpr double kRayDy = 7.548776662466927e-7, kRayDz = 5.698402909980532e-7;

// The wall code of link q of fluid node (i, j, k) towards a solid node (linkwise.f95:56):
// the nearest crossing among the triangles of the 27 cells around the node.
__host__ __device__ int32_t wall_code(const Tri* T, const int32_t* start, const int32_t* tris, const double* glo,
                                      double cell, const int* gn, const double p0[3], int q, double dx) {
  const int gc[3] = {(int)floor((p0[0] - glo[0]) / cell), (int)floor((p0[1] - glo[1]) / cell),
                     (int)floor((p0[2] - glo[2]) / cell)};
  const int c[3] = {elbm::cx27(q), elbm::cy27(q), elbm::cz27(q)};
  const double p1[3] = {p0[0] + c[0] * dx, p0[1] + c[1] * dx, p0[2] + c[2] * dx};
  double tbest = INFINITY;
  for (int d2 = -1; d2 <= 1; ++d2)
    for (int d1 = -1; d1 <= 1; ++d1)
      for (int d0 = -1; d0 <= 1; ++d0) {
        const int g0 = gc[0] + d0, g1 = gc[1] + d1, g2 = gc[2] + d2;
        if (g0 < 0 || g1 < 0 || g2 < 0 || g0 >= gn[0] || g1 >= gn[1] || g2 >= gn[2]) continue;
        const size_t cc = ((size_t)g2 * gn[1] + g1) * gn[0] + g0;
        for (int32_t e = start[cc]; e < start[cc + 1]; ++e) {
          const double tt = seg_tri(T[tris[e]], p0, p1);
          if (tt > 0.0 && tt < tbest) tbest = tt;
        }
      }
  if (tbest == INFINITY) tbest = 1.0;  // the link ends in a solid node without a recorded crossing
  const double len = sqrt((double)(c[0] * c[0] + c[1] * c[1] + c[2] * c[2])) * dx;
  const double dist = tbest * len;
  return -1001 - (int32_t)floor(dist / len * 1e9);
}

// The nearest crossing t in (0, 1] of the segment p0 -> p0 + c dx with the
// triangles of the cells around p0 (cells at least as long as the segment),
// 1 when none is found (a link that ends in a solid node without a recorded
// crossing), as the wall code -1001 - floor(t 1e9) (linkwise.f95:56).
__host__ __device__ int32_t seg_code(const Tri* T, const int32_t* start, const int32_t* tris, const double* glo,
                                     double cell, const int* gn, const double p0[3], const int c[3], double dx) {
  const int gc[3] = {(int)floor((p0[0] - glo[0]) / cell), (int)floor((p0[1] - glo[1]) / cell),
                     (int)floor((p0[2] - glo[2]) / cell)};
  const double p1[3] = {p0[0] + c[0] * dx, p0[1] + c[1] * dx, p0[2] + c[2] * dx};
  double tbest = INFINITY;
  for (int d2 = -1; d2 <= 1; ++d2)
    for (int d1 = -1; d1 <= 1; ++d1)
      for (int d0 = -1; d0 <= 1; ++d0) {
        const int g0 = gc[0] + d0, g1 = gc[1] + d1, g2 = gc[2] + d2;
        if (g0 < 0 || g1 < 0 || g2 < 0 || g0 >= gn[0] || g1 >= gn[1] || g2 >= gn[2]) continue;
        const size_t cc = ((size_t)g2 * gn[1] + g1) * gn[0] + g0;
        for (int32_t e = start[cc]; e < start[cc + 1]; ++e) {
          const double tt = seg_tri(T[tris[e]], p0, p1);
          if (tt > 0.0 && tt < tbest) tbest = tt;
        }
      }
  if (tbest == INFINITY) tbest = 1.0;
  return -1001 - (int32_t)floor(tbest * 1e9);
}

// The D3Q39 link vectors of a level and the rule that makes link i a wall
// link: on the shifted lattice (shifted_state_directions.f95:54-68) when the
// upstream node x - c_i is solid, the crossing searched from x towards it; on
// the unshifted lattice (state_directions.f95:696) when the downstream node
// x + c_i is solid, searched towards it.  seg[i] is the searched segment's
// direction, +-c_i.
struct Links39Geo {
  int seg[39][3];
  int periodic;
};

Links39Geo links39_geo(int shifted, int pfd, int periodic) {
  elbm::Lattice39 L;
  elbm::build_lattice39(shifted, pfd, L);
  Links39Geo G{};
  const int sgn = shifted ? -1 : 1;
  for (int i = 0; i < 39; ++i) {
    G.seg[i][0] = sgn * L.cx[i];
    G.seg[i][1] = sgn * L.cy[i];
    G.seg[i][2] = sgn * L.cz[i];
  }
  G.periodic = periodic;
  return G;
}

// Index of (i, j, k) with periodic wrap, -1 outside the box on a non-periodic axis.
__host__ __device__ int64_t geo_node(int i, int j, int k, int nx, int ny, int nz, int periodic) {
  if (periodic & 1) i = ((i % nx) + nx) % nx;
  else if (i < 0 || i >= nx) return -1;
  if (periodic & 2) j = ((j % ny) + ny) % ny;
  else if (j < 0 || j >= ny) return -1;
  if (periodic & 4) k = ((k % nz) + nz) % nz;
  else if (k < 0 || k >= nz) return -1;
  return ((int64_t)k * ny + j) * nx + i;
}

// The D3Q39 codes of node n: a solid node gets node type -1001 and -666 on its
// links; a fluid node's links whose searched neighbour is solid get wall codes.
__host__ __device__ void links39_node(const Tri* T, const int32_t* start, const int32_t* tris, const double* glo,
                                      double cell, const int* gn, int nx, int ny, int nz, const double* origin,
                                      double dx, const Links39Geo& G, const uint8_t* solid, int64_t n,
                                      int32_t* state) {
  const int64_t N = (int64_t)nx * ny * nz;
  if (solid[n]) {
    state[n] = -1001;
    for (int q = 1; q < 39; ++q) state[(int64_t)q * N + n] = -666;
    return;
  }
  const int i = (int)(n % nx), j = (int)((n / nx) % ny), k = (int)(n / ((int64_t)nx * ny));
  const double p0[3] = {origin[0] + i * dx, origin[1] + j * dx, origin[2] + k * dx};
  for (int q = 1; q < 39; ++q) {
    const int64_t m = geo_node(i + G.seg[q][0], j + G.seg[q][1], k + G.seg[q][2], nx, ny, nz, G.periodic);
    if (m < 0 || !solid[m]) continue;
    state[(int64_t)q * N + n] = seg_code(T, start, tris, glo, cell, gn, p0, G.seg[q], dx);
  }
}

// Solid nodes by +x ray casting (host).
void mark_solid_host(const TriGrid& G, int nx, int ny, int nz, const double* origin, double dx,
                     std::vector<uint8_t>& solid) {
  const std::vector<Tri>& T = G.T;
  const int ntri = (int)T.size();
  solid.assign((size_t)nx * ny * nz, 0);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j) {
      const double y = origin[1] + (j + kRayDy) * dx, z = origin[2] + (k + kRayDz) * dx;
      if (y < G.glo[1] || y > G.ghi[1] || z < G.glo[2] || z > G.ghi[2]) continue;
      std::vector<int> cand;
      for (int t = 0; t < ntri; ++t)
        if (T[t].lo[1] <= y && y <= T[t].hi[1] && T[t].lo[2] <= z && z <= T[t].hi[2]) cand.push_back(t);
      if (cand.empty()) continue;
      for (int i = 0; i < nx; ++i) {
        const double p[3] = {origin[0] + i * dx, y, z};
        if (p[0] > G.ghi[0]) break;
        int cross = 0;
        for (int t : cand) cross += ray_x_crosses(T[t], p) ? 1 : 0;
        if (cross & 1) solid[((int64_t)k * ny + j) * nx + i] = 1;
      }
    }
}

// ---- device path ----
constexpr int kRowCand = 4096;  // candidate triangles of one +x ray held in shared memory

// One block per (j, k) row: the triangles whose yz box holds the ray, then the
// crossing parity of every node of the row (fluid_or_solid by ray casting).
__global__ void mark_solid_kernel(const Tri* __restrict__ T, int ntri, int nx, int ny, int nz, double3 origin,
                                  double dx, double3 glo, double3 ghi, uint8_t* __restrict__ solid,
                                  int* __restrict__ overflow) {
  __shared__ int32_t cand[kRowCand];
  __shared__ int ncand;
  const int j = blockIdx.x % ny, k = blockIdx.x / ny;
  const double y = origin.y + (j + kRayDy) * dx, z = origin.z + (k + kRayDz) * dx;
  if (threadIdx.x == 0) ncand = 0;
  __syncthreads();
  const bool in = !(y < glo.y || y > ghi.y || z < glo.z || z > ghi.z);
  if (in)
    for (int t = threadIdx.x; t < ntri; t += blockDim.x)
      if (T[t].lo[1] <= y && y <= T[t].hi[1] && T[t].lo[2] <= z && z <= T[t].hi[2]) {
        const int slot = atomicAdd(&ncand, 1);
        if (slot < kRowCand) cand[slot] = t;
      }
  __syncthreads();
  const int nc = ncand;
  if (nc > kRowCand && threadIdx.x == 0) atomicExch(overflow, 1);
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    const int64_t n = ((int64_t)k * ny + j) * nx + i;
    uint8_t s = 0;
    const double p[3] = {origin.x + i * dx, y, z};
    if (in && nc > 0 && nc <= kRowCand && !(p[0] > ghi.x)) {
      int cross = 0;
      for (int e = 0; e < nc; ++e) cross += ray_x_crosses(T[cand[e]], p) ? 1 : 0;
      s = (uint8_t)(cross & 1);
    }
    solid[n] = s;
  }
}

// One thread per node: solid nodes -1001 on every component; the links of a
// fluid node that end in a solid node get their wall code.
__global__ void mark_links_kernel(const Tri* __restrict__ T, const int32_t* __restrict__ start,
                                  const int32_t* __restrict__ tris, int nx, int ny, int nz, double3 origin, double dx,
                                  double3 glo, double cell, int3 gn, const uint8_t* __restrict__ solid,
                                  int32_t* __restrict__ state) {
  const int64_t N = (int64_t)nx * ny * nz;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  if (solid[n]) {
    for (int q = 0; q < elbm::Q27; ++q) state[(int64_t)q * N + n] = -1001;
    return;
  }
  const int i = (int)(n % nx), j = (int)((n / nx) % ny), k = (int)(n / ((int64_t)nx * ny));
  const double p0[3] = {origin.x + i * dx, origin.y + j * dx, origin.z + k * dx};
  const double g0[3] = {glo.x, glo.y, glo.z};
  const int gnn[3] = {gn.x, gn.y, gn.z};
  for (int q = 1; q < elbm::Q27; ++q) {
    const int it = i + elbm::cx27(q), jt = j + elbm::cy27(q), kt = k + elbm::cz27(q);
    if (!(it >= 0 && jt >= 0 && kt >= 0 && it < nx && jt < ny && kt < nz && solid[((int64_t)kt * ny + jt) * nx + it]))
      continue;
    state[(int64_t)q * N + n] = wall_code(T, start, tris, g0, cell, gnn, p0, q, dx);
  }
}

// One thread per node: the D3Q39 codes (links39_node).
__global__ void mark_links39_kernel(const Tri* __restrict__ T, const int32_t* __restrict__ start,
                                    const int32_t* __restrict__ tris, int nx, int ny, int nz, double3 origin,
                                    double dx, double3 glo, double cell, int3 gn, const Links39Geo G,
                                    const uint8_t* __restrict__ solid, int32_t* __restrict__ state) {
  const int64_t N = (int64_t)nx * ny * nz;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const double o[3] = {origin.x, origin.y, origin.z}, g0[3] = {glo.x, glo.y, glo.z};
  const int gnn[3] = {gn.x, gn.y, gn.z};
  links39_node(T, start, tris, g0, cell, gnn, nx, ny, nz, o, dx, G, solid, n, state);
}

// The longest searched D3Q39 segment in lattice units.
double seg39_reach(const Links39Geo& G) {
  double r = 0.0;
  for (int q = 0; q < 39; ++q)
    r = std::max(r, std::sqrt((double)(G.seg[q][0] * G.seg[q][0] + G.seg[q][1] * G.seg[q][1] + G.seg[q][2] * G.seg[q][2])));
  return std::ceil(r);
}

}  // namespace

namespace elbm {

// elbm_mark_triangles39 on the device.
int mark_triangles39_device(int nx, int ny, int nz, const double* origin, double dx, int ntri, const double* tri,
                            int shifted, int pfd, int periodic, int32_t* state, cudaStream_t s, std::string& why) {
  const Links39Geo LG = links39_geo(shifted, pfd, periodic);
  TriGrid G;
  build_tri_grid(ntri, tri, dx, G, seg39_reach(LG));
  const int64_t N = (int64_t)nx * ny * nz;
  Tri* dT = nullptr;
  int32_t *dstart = nullptr, *dtris = nullptr, *dstate = nullptr;
  uint8_t* dsolid = nullptr;
  int* dover = nullptr;
  auto release = [&]() {
    cudaFree(dT);
    cudaFree(dstart);
    cudaFree(dtris);
    cudaFree(dstate);
    cudaFree(dsolid);
    cudaFree(dover);
  };
  if (cudaMalloc(&dT, sizeof(Tri) * ntri) || cudaMalloc(&dstart, sizeof(int32_t) * G.start.size()) ||
      cudaMalloc(&dtris, sizeof(int32_t) * std::max<size_t>(G.tris.size(), 1)) ||
      cudaMalloc(&dstate, sizeof(int32_t) * 39 * N) || cudaMalloc(&dsolid, N) || cudaMalloc(&dover, sizeof(int))) {
    release();
    why = "device memory";
    return ELBM_E_CUDA;
  }
  cudaMemcpyAsync(dT, G.T.data(), sizeof(Tri) * ntri, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dstart, G.start.data(), sizeof(int32_t) * G.start.size(), cudaMemcpyHostToDevice, s);
  if (!G.tris.empty())
    cudaMemcpyAsync(dtris, G.tris.data(), sizeof(int32_t) * G.tris.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dstate, state, sizeof(int32_t) * 39 * N, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(dover, 0, sizeof(int), s);
  const double3 o = make_double3(origin[0], origin[1], origin[2]);
  mark_solid_kernel<<<(unsigned)((int64_t)ny * nz), 128, 0, s>>>(
      dT, ntri, nx, ny, nz, o, dx, make_double3(G.glo[0], G.glo[1], G.glo[2]),
      make_double3(G.ghi[0], G.ghi[1], G.ghi[2]), dsolid, dover);
  mark_links39_kernel<<<(unsigned)((N + 127) / 128), 128, 0, s>>>(
      dT, dstart, dtris, nx, ny, nz, o, dx, make_double3(G.glo[0], G.glo[1], G.glo[2]), G.cell,
      make_int3(G.gn[0], G.gn[1], G.gn[2]), LG, dsolid, dstate);
  int over = 0;
  cudaMemcpyAsync(&over, dover, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(state, dstate, sizeof(int32_t) * 39 * N, cudaMemcpyDeviceToHost, s);
  const cudaError_t e = cudaStreamSynchronize(s);
  release();
  if (e != cudaSuccess) {
    why = cudaGetErrorString(e);
    return ELBM_E_CUDA;
  }
  if (over) {
    why = "more than 4096 triangles along one +x ray of the lattice; use elbm_mark_triangles39";
    return ELBM_E_UNSUPPORTED;
  }
  return ELBM_OK;
}

// elbm_mark_triangles on the device (the C-ABI entry takes the context's stream).
int mark_triangles_device(int nx, int ny, int nz, const double* origin, double dx, int ntri, const double* tri,
                          int32_t* state, cudaStream_t s, std::string& why) {
  TriGrid G;
  build_tri_grid(ntri, tri, dx, G);
  const int64_t N = (int64_t)nx * ny * nz;
  Tri* dT = nullptr;
  int32_t *dstart = nullptr, *dtris = nullptr, *dstate = nullptr;
  uint8_t* dsolid = nullptr;
  int* dover = nullptr;
  auto release = [&]() {
    cudaFree(dT);
    cudaFree(dstart);
    cudaFree(dtris);
    cudaFree(dstate);
    cudaFree(dsolid);
    cudaFree(dover);
  };
  if (cudaMalloc(&dT, sizeof(Tri) * ntri) || cudaMalloc(&dstart, sizeof(int32_t) * G.start.size()) ||
      cudaMalloc(&dtris, sizeof(int32_t) * std::max<size_t>(G.tris.size(), 1)) ||
      cudaMalloc(&dstate, sizeof(int32_t) * Q27 * N) || cudaMalloc(&dsolid, N) || cudaMalloc(&dover, sizeof(int))) {
    release();
    why = "device memory";
    return ELBM_E_CUDA;
  }
  cudaMemcpyAsync(dT, G.T.data(), sizeof(Tri) * ntri, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dstart, G.start.data(), sizeof(int32_t) * G.start.size(), cudaMemcpyHostToDevice, s);
  if (!G.tris.empty())
    cudaMemcpyAsync(dtris, G.tris.data(), sizeof(int32_t) * G.tris.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dstate, state, sizeof(int32_t) * Q27 * N, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(dover, 0, sizeof(int), s);
  const double3 o = make_double3(origin[0], origin[1], origin[2]);
  mark_solid_kernel<<<(unsigned)((int64_t)ny * nz), 128, 0, s>>>(
      dT, ntri, nx, ny, nz, o, dx, make_double3(G.glo[0], G.glo[1], G.glo[2]),
      make_double3(G.ghi[0], G.ghi[1], G.ghi[2]), dsolid, dover);
  mark_links_kernel<<<(unsigned)((N + 127) / 128), 128, 0, s>>>(
      dT, dstart, dtris, nx, ny, nz, o, dx, make_double3(G.glo[0], G.glo[1], G.glo[2]), G.cell,
      make_int3(G.gn[0], G.gn[1], G.gn[2]), dsolid, dstate);
  int over = 0;
  cudaMemcpyAsync(&over, dover, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(state, dstate, sizeof(int32_t) * Q27 * N, cudaMemcpyDeviceToHost, s);
  const cudaError_t e = cudaStreamSynchronize(s);
  release();
  if (e != cudaSuccess) {
    why = cudaGetErrorString(e);
    return ELBM_E_CUDA;
  }
  if (over) {
    why = "more than 4096 triangles along one +x ray of the lattice; use elbm_mark_triangles";
    return ELBM_E_UNSUPPORTED;
  }
  return ELBM_OK;
}

}  // namespace elbm

extern "C" int elbm_mark_triangles(int nx, int ny, int nz, const double* origin, double dx, int ntri,
                                   const double* tri, int32_t* state) {
  using namespace elbm;
  if (nx < 1 || ny < 1 || nz < 1 || !origin || !(dx > 0.0) || ntri < 1 || !tri || !state) return ELBM_E_ARG;
  const int64_t N = (int64_t)nx * ny * nz;
  TriGrid G;
  build_tri_grid(ntri, tri, dx, G);
  const std::vector<Tri>& T = G.T;
  const double* glo = G.glo;
  const double* ghi = G.ghi;
  auto coord = [&](int i, int a) { return origin[a] + i * dx; };
  // 1) solid nodes: odd number of +x ray crossings (fluid_or_solid by ray casting)
  std::vector<uint8_t> solid(N, 0);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j) {
      const double y = origin[1] + (j + kRayDy) * dx, z = origin[2] + (k + kRayDz) * dx;
      if (y < glo[1] || y > ghi[1] || z < glo[2] || z > ghi[2]) continue;
      std::vector<int> cand;
      for (int t = 0; t < ntri; ++t)
        if (T[t].lo[1] <= y && y <= T[t].hi[1] && T[t].lo[2] <= z && z <= T[t].hi[2]) cand.push_back(t);
      if (cand.empty()) continue;
      for (int i = 0; i < nx; ++i) {
        const double p[3] = {coord(i, 0), y, z};
        if (p[0] > ghi[0]) break;
        int cross = 0;
        for (int t : cand) cross += ray_x_crosses(T[t], p) ? 1 : 0;
        if (cross & 1) solid[((int64_t)k * ny + j) * nx + i] = 1;
      }
    }
  // 2) codes: solid nodes -1001; wall links of fluid nodes carry the crossing fraction
  for (int64_t n = 0; n < N; ++n) {
    if (!solid[n]) continue;
    for (int q = 0; q < Q27; ++q) state[(int64_t)q * N + n] = -1001;
  }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int64_t n = ((int64_t)k * ny + j) * nx + i;
        if (solid[n]) continue;
        const double p0[3] = {coord(i, 0), coord(j, 1), coord(k, 2)};
        for (int q = 1; q < Q27; ++q) {
          // only links from a fluid node to a solid node are wall links
          // (inter_bb_setup.f95:36-40: same-type neighbours skip the crossing search)
          const int it = i + D3Q27::cx[q], jt = j + D3Q27::cy[q], kt = k + D3Q27::cz[q];
          if (!(it >= 0 && jt >= 0 && kt >= 0 && it < nx && jt < ny && kt < nz && solid[((int64_t)kt * ny + jt) * nx + it]))
            continue;
          state[(int64_t)q * N + n] = wall_code(T.data(), G.start.data(), G.tris.data(), glo, G.cell, G.gn, p0, q, dx);
        }
      }
  return ELBM_OK;
}

extern "C" int elbm_mark_triangles39(int nx, int ny, int nz, const double* origin, double dx, int ntri,
                                     const double* tri, int shifted, int primary_flow_dir, int periodic,
                                     int32_t* state) {
  using namespace elbm;
  if (nx < 1 || ny < 1 || nz < 1 || !origin || !(dx > 0.0) || ntri < 1 || !tri || !state || periodic < 0 ||
      periodic > 7 || primary_flow_dir < 1 || primary_flow_dir > 6)
    return ELBM_E_ARG;
  const Links39Geo LG = links39_geo(shifted, primary_flow_dir, periodic);
  TriGrid G;
  build_tri_grid(ntri, tri, dx, G, seg39_reach(LG));
  std::vector<uint8_t> solid;
  mark_solid_host(G, nx, ny, nz, origin, dx, solid);
  const int64_t N = (int64_t)nx * ny * nz;
  for (int64_t n = 0; n < N; ++n)
    links39_node(G.T.data(), G.start.data(), G.tris.data(), G.glo, G.cell, G.gn, nx, ny, nz, origin, dx, LG,
                 solid.data(), n, state);
  return ELBM_OK;
}
