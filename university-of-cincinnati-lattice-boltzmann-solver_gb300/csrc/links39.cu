// Host-side decoding of D3Q39 link codes into pull-form link words.
//
// The reference streams by a push loop (looping/timestepping/streaming.f95:
// 266-481): direction outermost, then z, y, x; every boundary rule first
// rewrites fout(x, i) in place (bounce-back swaps fout(x, i) and
// fout(x, opp(i)); inlets, outlets and the freestream put an equilibrium;
// pure outflow copies fout(x, opp(i))), then writes fi(x, opp(i)); on the
// shifted lattice the interior push happens as well.  A later write to the
// same post-streaming slot replaces an earlier one, and a slot nothing writes
// keeps last step's value.  This file runs that loop once on symbols: every
// fout entry is "population k of node m" or "equilibrium table t, population
// p", every write carries its loop position, and the last write of each slot
// wins.  A node whose 39 slots all end up as the plain pull fout(y - c_j, j)
// is a bulk node; the others get 39 link words.
//
// Interpolated wall links (codes -1001 - q 1e9, streaming.f95:478-1133) write
// a value that the step computes from the node's targets (target_finder.f95,
// then shifted_ibb.f95 on the shifted lattice or interpolative_bounceback_bc.f95
// on the unshifted one).  target_finder sums
// the node's post-streaming slots as the loop has left them at the node's
// first wall link, so the decoder also records, for such nodes, the last
// write of every slot up to that point.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/elbm_gb300.h"
#include "kernels39.cuh"
#include "links39.h"

namespace elbm {
namespace {

struct Sym {
  int8_t kind = 0;  // 0 none, 1 fout(node, pop), 2 equilibrium(table, pop), 3 wall value(pop)
  int8_t pop = 0;
  int8_t table = 0;
  int64_t node = -1;
};

// inviscid_edge.f95 (D3Q39 branch): the specular reflection j of an inviscid
// link (-11/-12) of direction i and the displacement d of the node that
// receives fout(x, i).  Per axis where the unshifted velocity has a component:
// the unit link along it being -11 reflects it (displacement 0 for speed-1
// diagonals, -c/2 for speed-2 ones), else for speed-2 diagonals the speed-2
// link being -11 reflects it (displacement +c/2), else it keeps c.  Axis
// directions always reflect: displacement 0 for speed 1; for speed 2, -c/2
// when the unit link along the axis is -11, else +c/2; for speed 3, +2c/3
// when the unit and the speed-2 links along it are both -11, 0 when only the
// speed-2 one is, else -2c/3.  On the shifted lattice the routine then adds
// the shift (the primary flow direction's unit vector, :1230-1243); the
// caller does that.  The reference's table departs from this in two entries, kept here:
// direction 9 (1-based) with x and y (x and z) reflecting goes to 12 (11), and
// direction 27 with only y reflecting is displaced by the opposite y.
bool inviscid39(const Lattice39& U, int i, const int32_t* code, int& j, int (&d)[3]) {
  const int c[3] = {U.cx[i], U.cy[i], U.cz[i]};
  const int sp = std::max(std::abs(c[0]), std::max(std::abs(c[1]), std::abs(c[2])));
  const int nz = (c[0] != 0) + (c[1] != 0) + (c[2] != 0);
  int r[3] = {c[0], c[1], c[2]};
  bool refl[3] = {false, false, false};
  if (nz == 1) {
    for (int a = 0; a < 3; ++a) {
      r[a] = -c[a];
      d[a] = 0;
      if (c[a] == 0) continue;
      const int side = c[a] < 0 ? 3 : 0;
      const bool unit = code[1 + a + side] == -11, two = code[15 + a + side] == -11;
      if (sp == 2) d[a] = unit ? -c[a] / 2 : c[a] / 2;
      else if (sp == 3) d[a] = (unit && two) ? (2 * c[a]) / 3 : two ? 0 : -(2 * c[a]) / 3;
    }
  } else {
    for (int a = 0; a < 3; ++a) {
      d[a] = c[a];
      if (c[a] == 0) continue;
      const int side = c[a] < 0 ? 3 : 0;
      if (code[1 + a + side] == -11) {
        r[a] = -c[a];
        d[a] = sp == 1 ? 0 : -c[a] / 2;
        refl[a] = true;
      } else if (sp == 2 && code[15 + a + side] == -11) {
        r[a] = -c[a];
        d[a] = c[a] / 2;
        refl[a] = true;
      }
    }
    if (!refl[0] && !refl[1] && !refl[2]) return false;
    if (i == 8 && refl[0] && refl[1] && !refl[2]) {
      r[0] = 1, r[1] = 1, r[2] = -1;
    } else if (i == 8 && refl[0] && refl[2] && !refl[1]) {
      r[0] = 1, r[1] = -1, r[2] = 1;
    }
    if (i == 26 && !refl[0] && refl[1]) d[1] = -d[1];
  }
  for (int k = 0; k < Q39; ++k)
    if (U.cx[k] == r[0] && U.cy[k] == r[1] && U.cz[k] == r[2]) {
      j = k;
      return true;
    }
  return false;
}

bool fluid39(int32_t s0) {
  if (s0 < 0) return false;
  if (s0 >= 1000 && s0 < 51000) return false;
  if (s0 >= 200 && s0 < 299) return false;
  return true;
}

}  // namespace

int decode_links39(const int32_t* st, int ngs, int nx, int ny, int nz, int periodic, int shifted, int pfd,
                   const int32_t* inlet_type, const int32_t* outlet_type, Links39& out, std::string& why) {
  Lattice39 L;
  build_lattice39(shifted, pfd, L);
  const int fx = nx + 2 * ngs, fy = ny + 2 * ngs, fz = nz + 2 * ngs;
  const int64_t fplane = (int64_t)fx * fy * fz;
  const int64_t N = (int64_t)nx * ny * nz;
  auto sidx = [&](int x, int y, int z) { return ((int64_t)(z + ngs) * fy + (y + ngs)) * fx + (x + ngs); };
  auto code = [&](int i, int x, int y, int z) { return st[(int64_t)i * fplane + sidx(x, y, z)]; };
  // target of a push from (x, y, z) along c_i: wrap periodic axes, -1 outside the box
  auto target = [&](int x, int y, int z, int i, int& tx, int& ty, int& tz) -> int64_t {
    tx = x + L.cx[i];
    ty = y + L.cy[i];
    tz = z + L.cz[i];
    if (periodic & 1) tx = ((tx % nx) + nx) % nx;
    else if (tx < 0 || tx >= nx) return -1;
    if (periodic & 2) ty = ((ty % ny) + ny) % ny;
    else if (ty < 0 || ty >= ny) return -1;
    if (periodic & 4) tz = ((tz % nz) + nz) % nz;
    else if (tz < 0 || tz >= nz) return -1;
    return ((int64_t)tz * ny + ty) * nx + tx;
  };
  // node index of (x, y, z) with periodic wrap, -1 outside the box
  auto node_at = [&](int x, int y, int z) -> int64_t {
    if (periodic & 1) x = ((x % nx) + nx) % nx;
    else if (x < 0 || x >= nx) return -1;
    if (periodic & 2) y = ((y % ny) + ny) % ny;
    else if (y < 0 || y >= ny) return -1;
    if (periodic & 4) z = ((z % nz) + nz) % nz;
    else if (z < 0 || z >= nz) return -1;
    return ((int64_t)z * ny + y) * nx + x;
  };
  Lattice39 L0;  // the unshifted set: erp = its opposites (linking/modules/linkwise.f95:39)
  build_lattice39(0, pfd, L0);
  auto is_wall = [](int32_t c) { return c <= -1001 && c >= -1100000000; };
  // nodes with wall links; "adjacent" ones (a wall among components 1..14, streaming.f95:492)
  // take their targets at their first wall link, loop position (i0, node)
  std::vector<int32_t> adj(N, -1);
  std::vector<int64_t> k0;
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const int32_t s0 = code(0, x, y, z);
        if (s0 >= 0 && !fluid39(s0)) {
          why = "a node with state >= 0 that does not collide (200..298, 1000..50999)";
          return ELBM_E_UNSUPPORTED;
        }
        if (s0 < 0) continue;
        int i0 = -1, adjacent = 0;
        for (int i = 1; i < Q39; ++i) {
          const int32_t c = code(i, x, y, z);
          if (is_wall(c) && i0 < 0) i0 = i;
          if (i < 15 && c < -1000) adjacent = 1;
        }
        if (i0 >= 0 && shifted && pfd != 1) {
          why = "interpolated wall links on the shifted lattice need primary_flow_dir 1";
          return ELBM_E_UNSUPPORTED;
        }
        if (i0 >= 0 && adjacent) {
          const int64_t n = ((int64_t)z * ny + y) * nx + x;
          adj[n] = (int32_t)k0.size();
          k0.push_back(((int64_t)i0 * N + n) * 2);
        }
      }
  // last write of every post-streaming slot: loop position (direction, node, then 0 for the
  // push and 1 for the node's own boundary write) and symbol; and for the adjacent wall nodes
  // the last write up to the push at their first wall link
  std::vector<int64_t> key((size_t)N * Q39, -1);
  std::vector<Sym> val((size_t)N * Q39);
  std::vector<int64_t> skey(k0.size() * Q39, -1);
  std::vector<Sym> sval(k0.size() * Q39);
  auto emit = [&](int64_t t, int j, int64_t k, const Sym& v) {
    const size_t e = (size_t)t * Q39 + j;
    if (k > key[e]) {
      key[e] = k;
      val[e] = v;
    }
    const int32_t a = adj[t];
    if (a >= 0 && k <= k0[a] && k > skey[(size_t)a * Q39 + j]) {
      skey[(size_t)a * Q39 + j] = k;
      sval[(size_t)a * Q39 + j] = v;
    }
  };
  Sym fo[Q39];
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const int64_t n = ((int64_t)z * ny + y) * nx + x;
        const int32_t s0 = code(0, x, y, z);
        if (s0 < 0) continue;
        for (int i = 0; i < Q39; ++i) {
          fo[i].kind = 1;
          fo[i].node = n;
          fo[i].pop = (int8_t)i;
        }
        for (int i = 0; i < Q39; ++i) {
          const int64_t kpos = ((int64_t)i * N + n) * 2;  // loop order: i, then z, y, x
          int tx, ty, tz;
          const int64_t t = target(x, y, z, i, tx, ty, tz);
          if (i == 0 && shifted) {
            // the rest population moves only onto a node with state >= 0
            if (t >= 0 && code(0, tx, ty, tz) >= 0) emit(t, 0, kpos, fo[0]);
            continue;
          }
          const int32_t c = (i == 0) ? s0 : code(i, x, y, z);
          if (c >= 0 && c <= 1100000000) {
            if (t >= 0) emit(t, i, kpos, fo[i]);
            continue;
          }
          if (c == -666) continue;
          if (c == -11 || c == -12) {
            // streaming.f95:370-382: the shifted push, then fi(x + d, j) = fout(x, i); a reflection
            // landing outside the box leaves it, like a push across a face
            if (shifted && t >= 0) emit(t, i, kpos, fo[i]);
            int32_t codes[Q39];
            for (int q = 0; q < Q39; ++q) codes[q] = code(q, x, y, z);
            int j = 0, d[3];
            // no branch of inviscid_edge.f95 applies (no unit or speed-2 axis link of the direction is
            // -11, e.g. where a wall link took one): the reference writes nothing for this link
            if (!inviscid39(L0, i, codes, j, d)) continue;
            if (shifted) d[(pfd - 1) % 3] += pfd <= 3 ? 1 : -1;  // the shift, inviscid_edge.f95:1230-1243
            const int64_t r = node_at(x + d[0], y + d[1], z + d[2]);
            if (r >= 0) emit(r, j, kpos + 1, fo[i]);
            continue;
          }
          if (is_wall(c)) {
            // streaming.f95:482-486: the shifted lattice pushes onto a node with state >= 0; the
            // closure (shifted_ibb, or interpolative_bounceback_bc of direction opp(i) on the
            // unshifted lattice) rewrites fout(x, i) in place, then fi(x, opp(i)) = fout(x, i)
            // (opp(i) = i on the shifted lattice)
            if (shifted && t >= 0 && code(0, tx, ty, tz) >= 0) emit(t, i, kpos, fo[i]);
            fo[i].kind = 3;
            fo[i].pop = (int8_t)i;
            fo[i].node = -1;
            emit(n, L.opp[i], kpos + 1, fo[i]);
            continue;
          }
          if (shifted && t >= 0) emit(t, i, kpos, fo[i]);
          const int o = L.opp[i];
          Sym eq;
          eq.kind = 2;
          eq.pop = (int8_t)o;
          if (c == -10) {
            const Sym tmp = fo[i];
            fo[i] = fo[o];
            fo[o] = tmp;
          } else if (c == -5) {
          } else if (c == -8 || c == -1000) {
            eq.table = 0;
            fo[i] = eq;
          } else if (c <= -100 && c >= -199) {
            const int k = -c - 100;
            if (k < 1 || k > 8) {
              why = "inlet number outside 1..8";
              return ELBM_E_UNSUPPORTED;
            }
            const int ty2 = inlet_type[k - 1];
            if (ty2 == 1 || ty2 == 2 || ty2 == 4) eq.table = (int8_t)k;
            else if (ty2 == 3) eq.table = 0;
            else {
              why = "unsupported inlet type";
              return ELBM_E_UNSUPPORTED;
            }
            fo[i] = eq;
          } else if (c <= -200 && c >= -299) {
            const int k = -c - 200;
            if (k < 1 || k > 8) {
              why = "outlet number outside 1..8";
              return ELBM_E_UNSUPPORTED;
            }
            const int ty2 = outlet_type[k - 1];
            if (ty2 == 1 || ty2 == 4) {
              eq.table = (int8_t)(8 + k);
              fo[i] = eq;
            } else if (ty2 == 2) {
              eq.table = (int8_t)k;  // press_temp_bc.f95:26-27 reads the inlet table
              fo[i] = eq;
            } else if (ty2 == 3) {
              eq.table = 0;
              fo[i] = eq;
            } else if (ty2 == 6) {
              fo[i] = fo[o];  // pure_outflow_bc.f95:19-20
            } else {
              why = "unsupported outlet type";
              return ELBM_E_UNSUPPORTED;
            }
          } else if (c <= -300 && c >= -499) {
            emit(n, i, kpos + 1, fo[i]);
            continue;
          } else {
            why = "unsupported D3Q39 link code " + std::to_string(c);
            return ELBM_E_UNSUPPORTED;
          }
          emit(n, o, kpos + 1, fo[i]);
        }
      }
  // link word of a symbol seen from node (x, y, z); false when it cannot be encoded
  auto encode = [&](const Sym& v, bool written, int x, int y, int z, uint32_t& w) -> bool {
    if (!written || v.kind == 0) {
      w = link39(L39_STALE, 0, 0, 0, 0, 0);
      return true;
    }
    if (v.kind == 2) {
      w = link39(L39_EQ, v.pop, v.table, 0, 0, 0);
      return true;
    }
    if (v.kind == 3) {
      w = link39(L39_WALL, v.pop, 0, 0, 0, 0);
      return true;
    }
    // fout(m, k): displacement from this node, minimal image on periodic axes
    const int mx = (int)(v.node % nx), my = (int)((v.node / nx) % ny), mz = (int)(v.node / ((int64_t)nx * ny));
    int dx = mx - x, dy = my - y, dz = mz - z;
    if (periodic & 1) dx = ((dx % nx) + nx + nx / 2) % nx - nx / 2;
    if (periodic & 2) dy = ((dy % ny) + ny + ny / 2) % ny - ny / 2;
    if (periodic & 4) dz = ((dz % nz) + nz + nz / 2) % nz - nz / 2;
    if (dx < -4 || dx > 4 || dy < -4 || dy > 4 || dz < -4 || dz > 4) return false;
    w = link39(L39_PULL, v.pop, 0, dx, dy, dz);
    return true;
  };
  // link classes of the repair (damp_it.f95:64-177)
  out.dmask.assign(N, 0ull);
  out.gmask.assign(N, 0);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        uint64_t m = 0;
        for (int i = 0; i < Q39; ++i) {
          const int32_t c = code(i, x, y, z);
          if (shifted ? c >= -500 : c >= 0) m |= 1ull << i;
        }
        if (code(0, x, y, z) >= -500) m |= 1ull << 63;
        out.dmask[((int64_t)z * ny + y) * nx + x] = m;
        int32_t cs[Q39];
        for (int i = 0; i < Q39; ++i) cs[i] = code(i, x, y, z);
        out.gmask[((int64_t)z * ny + y) * nx + x] = ggm_mask39(cs);
      }
  // classify the fluid nodes and encode the boundary records
  out.ntype.assign(N, 0);
  out.bidx.assign(N, -1);
  out.words.clear();
  out.bnodes.clear();
  out.walls.clear();
  out.recwall.clear();
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const int64_t n = ((int64_t)z * ny + y) * nx + x;
        if (!fluid39(code(0, x, y, z))) continue;
        uint32_t w[Q39];
        bool bulk = true, wall = false;
        for (int j = 0; j < Q39; ++j) {
          const Sym& v = val[(size_t)n * Q39 + j];
          if (!encode(v, key[(size_t)n * Q39 + j] >= 0, x, y, z, w[j])) {
            why = "a slot reads a node more than 4 links away (box too small on a periodic axis)";
            return ELBM_E_UNSUPPORTED;
          }
          if (w[j] != link39(L39_PULL, j, 0, -L.cx[j], -L.cy[j], -L.cz[j])) bulk = false;
          if (j > 0 && is_wall(code(j, x, y, z))) wall = true;
        }
        if (bulk && !wall) {
          out.ntype[n] = 1;
          continue;
        }
        out.ntype[n] = wall ? 3 : 2;
        out.bidx[n] = (int32_t)out.bnodes.size();
        out.bnodes.push_back((int32_t)n);
        out.words.insert(out.words.end(), w, w + Q39);
        out.recwall.push_back(wall ? (int32_t)out.walls.size() : -1);
        if (!wall) continue;
        Wall39Rec r{};
        r.node = (int32_t)n;
        r.rec = out.bidx[n];
        r.adjacent = adj[n] >= 0;
        for (int j = 0; j < Q39; ++j) {
          r.code[j] = code(j, x, y, z);
          r.upass[j] = -1;
          r.snap[j] = link39(L39_STALE, 0, 0, 0, 0, 0);
        }
        if (r.adjacent) {
          const size_t a = (size_t)adj[n];
          for (int j = 0; j < Q39; ++j) {
            const Sym& v = sval[a * Q39 + j];
            if (v.kind == 3 || !encode(v, skey[a * Q39 + j] >= 0, x, y, z, r.snap[j])) {
              why = "target_finder would read a slot this decoder cannot express";
              return ELBM_E_UNSUPPORTED;
            }
          }
          // target_finder.f95:36-58 (unshifted): velocity and temperature of node x + c_opp(j) when
          // that link is fluid, else of the node itself
          for (int j = 1; j < Q39 && !shifted; ++j) {
            if (!is_wall(r.code[j]) || r.code[L.opp[j]] < 0) continue;
            const int o = L.opp[j];
            const int64_t m = node_at(x + L.cx[o], y + L.cy[o], z + L.cz[o]);
            if (m < 0) {
              why = "target_finder reads the velocity of a node outside the box";
              return ELBM_E_UNSUPPORTED;
            }
            r.upass[o] = (int32_t)m;
          }
          // target_finder.f95:95-125 (shifted): velocity and temperature of node x + c_j where link
          // erp(j) is null, else of node x + c_5 (1-based)
          for (int j = 1; j < Q39 && shifted; ++j) {
            if (!is_wall(r.code[j])) continue;
            const int src = r.code[L0.opp[j]] == -666 ? j : 4;
            const int64_t m = node_at(x + L.cx[src], y + L.cy[src], z + L.cz[src]);
            if (m < 0) {
              why = "target_finder reads the velocity of a node outside the box";
              return ELBM_E_UNSUPPORTED;
            }
            r.upass[src] = (int32_t)m;
          }
        }
        static const int SX[7] = {0, 1, 0, 0, -1, 0, 0}, SY[7] = {0, 0, 1, 0, 0, -1, 0},
                         SZ[7] = {0, 0, 0, 1, 0, 0, -1};
        for (int j = 0; j < 7; ++j) {
          const int64_t m = node_at(x + SX[j], y + SY[j], z + SZ[j]);
          r.sidx[j] = (int32_t)m;
          r.st[j] = m < 0 ? -666 : code(0, (int)(m % nx), (int)((m / nx) % ny), (int)(m / ((int64_t)nx * ny)));
          r.tidx[j] = -1;
          if (!r.adjacent && r.st[j] >= 0) {
            const int64_t mt = node_at(x + L.cx[j], y + L.cy[j], z + L.cz[j]);
            if (mt < 0) {
              why = "the wall stencil reads a temperature outside the box";
              return ELBM_E_UNSUPPORTED;
            }
            r.tidx[j] = (int32_t)mt;
          }
        }
        out.walls.push_back(r);
      }
  return ELBM_OK;
}

}  // namespace elbm

extern "C" int elbm_links39_tables(int nx, int ny, int nz, const int32_t* state, int ngrow_state, int periodic,
                                   int shifted, int primary_flow_dir, const int32_t* inlet_type,
                                   const int32_t* outlet_type, uint8_t* ntype, int32_t* rec_node, uint32_t* words,
                                   int64_t capacity, int64_t* nrec) {
  using namespace elbm;
  if (nx < 1 || ny < 1 || nz < 1 || !state || ngrow_state < 0 || periodic < 0 || periodic > 7 || !inlet_type ||
      !outlet_type || !ntype || !nrec || primary_flow_dir < 1 || primary_flow_dir > 6)
    return ELBM_E_ARG;
  Links39 L;
  std::string why;
  const int rc = decode_links39(state, ngrow_state, nx, ny, nz, periodic, shifted, primary_flow_dir, inlet_type,
                                outlet_type, L, why);
  if (rc) return rc;
  *nrec = (int64_t)L.bnodes.size();
  for (size_t n = 0; n < L.ntype.size(); ++n) ntype[n] = L.ntype[n];
  if ((int64_t)L.bnodes.size() > capacity) return ELBM_E_ARG;
  for (size_t r = 0; r < L.bnodes.size(); ++r) {
    if (rec_node) rec_node[r] = L.bnodes[r];
    if (words)
      for (int j = 0; j < 39; ++j) words[r * 39 + j] = L.words[r * 39 + j];
  }
  return ELBM_OK;
}
