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
#include <vector>

#include "../../include/elbm_gb300.h"
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
double seg_tri(const Tri& T, const double p0[3], const double p1[3]) {
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
bool ray_x_crosses(const Tri& T, const double p[3]) {
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

extern "C" int elbm_mark_triangles(int nx, int ny, int nz, const double* origin, double dx, int ntri,
                                   const double* tri, int32_t* state) {
  using namespace elbm;
  if (nx < 1 || ny < 1 || nz < 1 || !origin || !(dx > 0.0) || ntri < 1 || !tri || !state) return ELBM_E_ARG;
  const int64_t N = (int64_t)nx * ny * nz;
  std::vector<Tri> T(ntri);
  double glo[3] = {INFINITY, INFINITY, INFINITY}, ghi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int k = 0; k < ntri; ++k) {
    Tri& t = T[k];
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
      glo[c] = std::min(glo[c], t.lo[c]);
      ghi[c] = std::max(ghi[c], t.hi[c]);
    }
  }
  // uniform grid over the surface's bounding box, cells of 2 dx, listing triangles
  const double cell = 2.0 * dx;
  int gn[3];
  for (int c = 0; c < 3; ++c) gn[c] = std::max(1, (int)std::ceil((ghi[c] - glo[c]) / cell) + 1);
  std::vector<std::vector<int>> grid((size_t)gn[0] * gn[1] * gn[2]);
  auto gidx = [&](int i, int j, int k) { return ((size_t)k * gn[1] + j) * gn[0] + i; };
  for (int k = 0; k < ntri; ++k) {
    int lo[3], hi[3];
    for (int c = 0; c < 3; ++c) {
      lo[c] = std::max(0, (int)std::floor((T[k].lo[c] - glo[c]) / cell) - 1);
      hi[c] = std::min(gn[c] - 1, (int)std::floor((T[k].hi[c] - glo[c]) / cell) + 1);
    }
    for (int c2 = lo[2]; c2 <= hi[2]; ++c2)
      for (int c1 = lo[1]; c1 <= hi[1]; ++c1)
        for (int c0 = lo[0]; c0 <= hi[0]; ++c0) grid[gidx(c0, c1, c2)].push_back(k);
  }
  auto coord = [&](int i, int a) { return origin[a] + i * dx; };
  // 1) solid nodes: odd number of +x ray crossings (fluid_or_solid by ray casting).
  // The ray starts a tiny irrational offset off the lattice line, so that it passes
  // through no vertex or edge of a surface built on lattice points.
  constexpr double kRayDy = 7.548776662466927e-7, kRayDz = 5.698402909980532e-7;
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
        bool near_solid = false;
        for (int q = 1; q < Q27 && !near_solid; ++q) {
          const int it = i + D3Q27::cx[q], jt = j + D3Q27::cy[q], kt = k + D3Q27::cz[q];
          near_solid = it >= 0 && jt >= 0 && kt >= 0 && it < nx && jt < ny && kt < nz &&
                       solid[((int64_t)kt * ny + jt) * nx + it];
        }
        if (!near_solid) continue;
        const int gc[3] = {(int)std::floor((p0[0] - glo[0]) / cell), (int)std::floor((p0[1] - glo[1]) / cell),
                           (int)std::floor((p0[2] - glo[2]) / cell)};
        for (int q = 1; q < Q27; ++q) {
          const int c[3] = {D3Q27::cx[q], D3Q27::cy[q], D3Q27::cz[q]};
          // only links from a fluid node to a solid node are wall links
          // (inter_bb_setup.f95:36-40: same-type neighbours skip the crossing search)
          const int it = i + c[0], jt = j + c[1], kt = k + c[2];
          if (!(it >= 0 && jt >= 0 && kt >= 0 && it < nx && jt < ny && kt < nz && solid[((int64_t)kt * ny + jt) * nx + it]))
            continue;
          const double p1[3] = {p0[0] + c[0] * dx, p0[1] + c[1] * dx, p0[2] + c[2] * dx};
          double tbest = INFINITY;
          for (int d2 = -1; d2 <= 1; ++d2)
            for (int d1 = -1; d1 <= 1; ++d1)
              for (int d0 = -1; d0 <= 1; ++d0) {
                const int g0 = gc[0] + d0, g1 = gc[1] + d1, g2 = gc[2] + d2;
                if (g0 < 0 || g1 < 0 || g2 < 0 || g0 >= gn[0] || g1 >= gn[1] || g2 >= gn[2]) continue;
                for (int t : grid[gidx(g0, g1, g2)]) {
                  const double tt = seg_tri(T[t], p0, p1);
                  if (tt > 0.0 && tt < tbest) tbest = tt;
                }
              }
          if (tbest == INFINITY) tbest = 1.0;  // the link ends in a solid node without a recorded crossing
          // linkwise.f95:56: -1001 - floor(|x - x_w| / link_dist * 1e9)
          const double len = std::sqrt((double)(c[0] * c[0] + c[1] * c[1] + c[2] * c[2])) * dx;
          const double dist = tbest * len;
          state[(int64_t)q * N + n] = -1001 - (int32_t)std::floor(dist / len * 1e9);
        }
      }
  return ELBM_OK;
}
