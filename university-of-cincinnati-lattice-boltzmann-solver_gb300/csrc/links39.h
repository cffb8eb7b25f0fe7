// Pull-form link tables of a D3Q39 box (csrc/links39.cu).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "kernels39.cuh"

namespace elbm {

struct Links39 {
  std::vector<uint8_t> ntype;   // per node: 0 neither pushes nor collides, 1 bulk, 2 boundary record,
                                //   3 boundary record with interpolated wall links
  std::vector<int32_t> bidx;    // per node: boundary record or -1
  std::vector<int32_t> bnodes;  // per record: node
  std::vector<uint32_t> words;  // 39 per record
  std::vector<Wall39Rec> walls; // nodes with interpolated wall links
  std::vector<int32_t> recwall; // per record: wall record or -1
  // per node, for the negative-population repair: bit i (0..38) link i interior (state >= 0;
  // shifted lattice: >= -500), bit 63 node type >= -500
  std::vector<uint64_t> dmask;
  // per node, for the GGM differences: bits 0-11 the links to x+1, x+2, x-1, x-2, then y, z (state
  // components 2, 16, 5, 19 / 3, 17, 6, 20 / 4, 18, 7, 21, 1-based) >= 0; bit 12 node >= 0; bit 13 node == -666;
  // bit 14 0 <= node < 100000 (the cells predictive splitting scans)
  std::vector<uint16_t> gmask;
};

// The GGM mask of one node from its 39 state components.
inline uint16_t ggm_mask39(const int32_t* code) {
  static const int comp[12] = {1, 15, 4, 18, 2, 16, 5, 19, 3, 17, 6, 20};
  uint16_t m = 0;
  for (int k = 0; k < 12; ++k)
    if (code[comp[k]] >= 0) m |= (uint16_t)(1u << k);
  if (code[0] >= 0) m |= 1u << 12;
  if (code[0] == -666) m |= 1u << 13;
  if (code[0] >= 0 && code[0] < 100000) m |= 1u << 14;
  return m;
}

int decode_links39(const int32_t* st, int ngs, int nx, int ny, int nz, int periodic, int shifted, int pfd,
                   const int32_t* inlet_type, const int32_t* outlet_type, Links39& out, std::string& why);

}  // namespace elbm
