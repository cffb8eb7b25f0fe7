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
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/elbm_gb300.h"
#include "kernels39.cuh"
#include "links39.h"

namespace elbm {
namespace {

struct Sym {
  int8_t kind = 0;  // 0 none, 1 fout(node, pop), 2 equilibrium(table, pop)
  int8_t pop = 0;
  int8_t table = 0;
  int64_t node = -1;
};

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
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const int32_t s0 = code(0, x, y, z);
        if (s0 >= 0 && !fluid39(s0)) {
          why = "a node with state >= 0 that does not collide (200..298, 1000..50999)";
          return ELBM_E_UNSUPPORTED;
        }
      }
  // last write of every post-streaming slot: loop position and symbol
  std::vector<int64_t> key((size_t)N * Q39, -1);
  std::vector<Sym> val((size_t)N * Q39);
  auto emit = [&](int64_t t, int j, int64_t k, const Sym& v) {
    const size_t e = (size_t)t * Q39 + j;
    if (k > key[e]) {
      key[e] = k;
      val[e] = v;
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
          const int64_t kpos = (int64_t)i * N + n;  // loop order: i, then z, y, x
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
            emit(n, i, kpos, fo[i]);
            continue;
          } else {
            why = "unsupported D3Q39 link code " + std::to_string(c);
            return ELBM_E_UNSUPPORTED;
          }
          emit(n, o, kpos, fo[i]);
        }
      }
  // classify the fluid nodes and encode the boundary records
  out.ntype.assign(N, 0);
  out.bidx.assign(N, -1);
  out.words.clear();
  out.bnodes.clear();
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const int64_t n = ((int64_t)z * ny + y) * nx + x;
        if (!fluid39(code(0, x, y, z))) continue;
        uint32_t w[Q39];
        bool bulk = true;
        for (int j = 0; j < Q39; ++j) {
          const Sym& v = val[(size_t)n * Q39 + j];
          if (key[(size_t)n * Q39 + j] < 0 || v.kind == 0) {
            w[j] = link39(L39_STALE, 0, 0, 0, 0, 0);
            bulk = false;
            continue;
          }
          if (v.kind == 2) {
            w[j] = link39(L39_EQ, v.pop, v.table, 0, 0, 0);
            bulk = false;
            continue;
          }
          // fout(m, k): displacement from this node, minimal image on periodic axes
          const int mx = (int)(v.node % nx), my = (int)((v.node / nx) % ny), mz = (int)(v.node / ((int64_t)nx * ny));
          int dx = mx - x, dy = my - y, dz = mz - z;
          if (periodic & 1) dx = ((dx % nx) + nx + nx / 2) % nx - nx / 2;
          if (periodic & 2) dy = ((dy % ny) + ny + ny / 2) % ny - ny / 2;
          if (periodic & 4) dz = ((dz % nz) + nz + nz / 2) % nz - nz / 2;
          if (dx < -4 || dx > 4 || dy < -4 || dy > 4 || dz < -4 || dz > 4) {
            why = "a slot reads a node more than 4 links away (box too small on a periodic axis)";
            return ELBM_E_UNSUPPORTED;
          }
          w[j] = link39(L39_PULL, v.pop, 0, dx, dy, dz);
          if (!(v.pop == j && dx == -L.cx[j] && dy == -L.cy[j] && dz == -L.cz[j])) bulk = false;
        }
        if (bulk) {
          out.ntype[n] = 1;
        } else {
          out.ntype[n] = 2;
          out.bidx[n] = (int32_t)out.bnodes.size();
          out.bnodes.push_back((int32_t)n);
          out.words.insert(out.words.end(), w, w + Q39);
        }
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
