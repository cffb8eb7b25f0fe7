// Lattice tables shared by host and device code.
//
// D3Q27 ordering follows the reference's own D3Q27 table
// (linking/modules/linkwise.f95:25-32, cx_27/cy_27/cz_27/opp_27) so that the
// per-direction link codes of an AMReX `state` FAB can be consumed unchanged.
// D3Q39 ordering follows general/background_calcs/directions_and_weights.f95:463-471
// (unshifted opposites :502-504; the Galilean-shifted set uses opp(i) = i, :494-496).
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define ELBM_HD __host__ __device__ __forceinline__
#else
#define ELBM_HD inline
#endif

namespace elbm {

constexpr int Q27 = 27;
constexpr int Q39 = 39;

// Host copies of the D3Q27 table (linkwise.f95:25-32, converted to 0-based indices).
struct D3Q27 {
  static constexpr int cx[Q27] = {0, 1, 0, 0, -1, 0, 0, 1, 0, -1, 0, 1, 1, -1, -1, 1, 0, -1, 0, 1, 1, 1, 1, -1, -1, -1, -1};
  static constexpr int cy[Q27] = {0, 0, 1, 0, 0, -1, 0, 1, 1, 1, 1, 0, 0, 0, 0, -1, -1, -1, -1, 1, 1, -1, -1, 1, 1, -1, -1};
  static constexpr int cz[Q27] = {0, 0, 0, 1, 0, 0, -1, 0, -1, 0, 1, 1, -1, -1, 1, 0, -1, 0, 1, 1, -1, 1, -1, 1, -1, 1, -1};
  static constexpr int opp[Q27] = {0, 4, 5, 6, 1, 2, 3, 17, 18, 15, 16, 13, 14, 11, 12, 9, 10, 7, 8, 26, 25, 24, 23, 22, 21, 20, 19};
};

// The same table for device code, packed two bits per direction (c + 1), so
// that fully unrolled loops fold every lookup into an immediate.
ELBM_HD constexpr int cx27(int i) { return (int)((0x2a9182919459ull >> (2 * i)) & 3ull) - 1; }
ELBM_HD constexpr int cy27(int i) { return (int)((0x28280156a9165ull >> (2 * i)) & 3ull) - 1; }
ELBM_HD constexpr int cz27(int i) { return (int)((0x888a460a44595ull >> (2 * i)) & 3ull) - 1; }

// 1-D weights of the product-form D3Q27 set at T0 = 1/3: w(0) = 2/3, w(+-1) = 1/6.
ELBM_HD constexpr double w1d(int c) { return c == 0 ? 2.0 / 3.0 : 1.0 / 6.0; }
ELBM_HD constexpr double w27(int i) { return w1d(cx27(i)) * w1d(cy27(i)) * w1d(cz27(i)); }

// Index of the velocity (a,b,c) in the D3Q27 table, -1 when absent.
ELBM_HD constexpr int find27(int a, int b, int c) {
  for (int i = 0; i < Q27; ++i)
    if (cx27(i) == a && cy27(i) == b && cz27(i) == c) return i;
  return -1;
}
ELBM_HD constexpr int opp27(int i) { return find27(-cx27(i), -cy27(i), -cz27(i)); }

// Boundary link word (one uint16 per population of a boundary node, pull form).
//   bits 0-4  : source population (PULL) or equilibrium table (EQ)
//   bits 5-9  : source node offset (dx+1) + 3(dy+1) + 9(dz+1), dx,dy,dz in {-1,0,1}; 13 = the node itself
//   bits 10-12: kind
// LK_IBB: interpolated bounce-back; source population = the wall-ward one, the
// offset field holds the second fluid node (13 = none; kOffXbox = a node of
// another box, its level index in the cross-box array), the fraction is in a
// float array.
// LK_XBOX: pull the source population from a node of another box of the level,
// whose level index is in the cross-box array (one int32 per population of a
// boundary record).
enum LinkKind : uint16_t { LK_PULL = 0, LK_EQ = 1, LK_IBB = 2, LK_KEEP = 3, LK_XBOX = 4 };
constexpr int kOffXbox = 27;
ELBM_HD constexpr uint16_t link_word(int kind, int pop, int off) {
  return (uint16_t)((kind << 10) | (off << 5) | pop);
}
ELBM_HD constexpr int lw_kind(uint16_t w) { return (w >> 10) & 7; }
ELBM_HD constexpr int lw_pop(uint16_t w) { return w & 31; }
ELBM_HD constexpr int lw_off(uint16_t w) { return (w >> 5) & 31; }
ELBM_HD constexpr int off_code(int dx, int dy, int dz) { return (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1); }

// Equilibrium tables: 0 = freestream, 1..8 = inlets 1..8, 9..16 = outlets 1..8.
constexpr int kEqTables = 17;

// Node classes stored in the per-node type byte.
enum NodeType : uint8_t { NT_SKIP = 0, NT_BULK = 1, NT_BOUNDARY = 2 };

}  // namespace elbm
