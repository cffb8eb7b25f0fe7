// Internal kernel interface of libelbm_gb300 (not part of the C ABI).
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "lattice.cuh"

namespace elbm {

// Solid nodes and wall links of a triangulated surface on the device (csrc/geometry.cu);
// state is the host array, read and written back.
int mark_triangles_device(int nx, int ny, int nz, const double* origin, double dx, int ntri, const double* tri,
                          int32_t* state, cudaStream_t s, std::string& why);
// D3Q39 codes (shifted or unshifted lattice) from a triangulated surface on the device.
int mark_triangles39_device(int nx, int ny, int nz, const double* origin, double dx, int ntri, const double* tri,
                            int shifted, int pfd, int periodic, int32_t* state, cudaStream_t s, std::string& why);

// Device-side statistics of one or more steps (accumulated with atomics).
struct DevStats {
  unsigned long long node_updates;
  unsigned long long newton_iters;
  unsigned long long exact_nodes;
  unsigned long long fallbacks;
  unsigned long long max_dH_bits;  // bit pattern of a non-negative double (monotone in value)
  unsigned long long dh_over;      // check mode: nodes with |dH| above the tolerance
  unsigned long long guess_misses; // learned alpha: guesses that needed the Newton fallback
  unsigned int status;
  unsigned int pad;
};
static_assert(sizeof(DevStats) == 64, "DevStats is half a cache line");

// A context keeps kStatSlots DevStats slots, kStatStride apart (one 128-byte
// line each).  The D3Q27 step kernels send a warp's updates to the slot of its
// block (block index mod kStatSlots), so that the atomics of a big level do not
// all queue at one L2 line; the other kernels use slot 0 and the host adds the
// slots up.
constexpr int kStatSlots = 64;
constexpr int kStatStride = 2;
constexpr size_t kStatBytes = sizeof(DevStats) * kStatSlots * kStatStride;

// One box of a level as the tensor-copy (TMA) step variant walks it: tiles of
// TX x TY nodes (TX = 1 << tx_log2 in {32, 64, 128}, TY = 256 / TX) in x, y,
// one z plane each; tiles numbered box after box, x fastest.
struct WsBox {
  int64_t base;   // level index of the box's node (0, 0, 0)
  int64_t tile0;  // first tile of the box
  int nx, ny, nz;
  int tx_log2;
  int tiles_x, tiles_y;
};
// Nodes per tile of the tensor-copy variant and the widest tile it uses.
constexpr int kWsTileNodes = 256;
constexpr int kWsMaxTileX = 128;

// Arguments of one fused D3Q27 step on a single box (valid region, no ghosts).
struct Step27Args {
  const void* src;  // post-collision populations of the previous step, Q planes
  void* dst;        // post-collision populations of this step
  int64_t plane;    // elements between population planes (>= N, padded)
  int nx, ny, nz;   // box dimensions when the level has one box
  int64_t N;        // nodes of the level (all boxes, each padded to whole 32-node chunks)
  int nbox;               // boxes of the level
  const int32_t* chunk_box;  // box of every 32-node chunk (nbox > 1)
  const int4* boxdim;        // nx, ny, nz of every box (nbox > 1)
  const int32_t* xsrc;       // cross-box source index per population of a boundary record (-1: none)
  unsigned long long* work_counter;  // chunk counter of the persistent variant (zeroed before each launch)
  // negative post-collision populations: (node * 27 + population) entries for the repair (nullptr: off)
  unsigned long long* neg_list;
  unsigned long long* neg_count;
  long long neg_cap;
  // FP32 path: nodes with some |Delta_i / f_i| > 0.1 are listed here by the step kernel and
  // finished by a second kernel (nullptr: solved in place)
  uint32_t* defer_list;
  unsigned long long* defer_count;
  long long defer_cap;
  int defer_on;           // 0 inside the kernel that finishes the listed nodes
  const uint8_t* ntype;   // NodeType per node
  const int32_t* bidx;    // boundary record per boundary node
  const uint16_t* words;  // Q link words per boundary record
  const void* qfrac;      // Q wall fractions per boundary record (LK_IBB links), FP64 or FP32 like the populations
  const void* eq;         // kEqTables x Q equilibria (FP64: f; FP32: deviations)
  double beta;
  double tol_alpha;
  double tol_dH;
  int max_newton;
  int alpha_mode;
  int check_dH;
  float* alpha_out;       // optional per-node alpha (FP32)
  DevStats* stats;
  const float* mlp;       // learned-alpha weights, FP32 (ELBM_ALPHA_LEARNED)
  int variant;            // kernel variant chosen by the autotuner
  // tensor-copy variant: one CUtensorMap per box over the source buffer (4-D: x, y, z,
  // population), the boxes' tilings and the level's tile count (nullptr: not eligible)
  const void* ws_maps;
  const WsBox* ws_boxes;
  int64_t ws_ntiles;
  // boundary nodes: level node index of every boundary record (the FP32 step kernels update the
  // bulk nodes, a second kernel these)
  const int32_t* bnode;
  int64_t nbnd;
  // resolved sources of the boundary records' pulls, Q x nbnd (nullptr: decode the link words)
  const uint32_t* rsrc;
  // harvesting of (populations, alpha) records for training (nullptr: off)
  float* harvest;
  unsigned long long* harvest_count;
  long long harvest_cap;
  int harvest_stride;
  // one-box levels whose 27 planes stay below 2^31 elements: the element offset of each pull,
  // population j of node n at n + pull_off[j] (the offset variant reads them as kernel parameters)
  int pull_off_ok;
  int32_t pull_off[27];
};

// 0: direct; 1, 4, 5, 6, 7: direct with registers capped for 4, 5, 6, 8, 7 blocks of 128 threads
// per SM; 2: bulk-copy staged; 3: persistent warps taking chunks from a counter (4 blocks per SM);
// 8: warp-specialised, tensor copies (TMA) of 256-node tiles into a shared-memory ring;
// 9: direct, the 27 pull offsets of a one-box level precomputed (kernel parameters)
constexpr int kFp32Variants = 10;
constexpr int kVariantTma = 8;
constexpr int kVariantOff = 9;
// Bytes allocated before and after each population buffer (never written):
// room for the staged kernel's row-segment copies that start 4 floats before
// a plane or run up to a tile past its end.
constexpr size_t kPopGuardBytes = 1024;

// Brings the allocation-free upload's module and staging buffer onto `device`
// (current) and records the buffer's address (csrc/noalloc.cu); elbm_create calls it.
cudaError_t noalloc_setup(int device);

void launch_d3q27_fp64(const Step27Args& a, cudaStream_t s);
void upload_alpha_mlp(const float* w_host, cudaStream_t s);
void launch_d3q27_fp32(const Step27Args& a, cudaStream_t s);
// Negative-population repair: find (full scan of a.src, optional), then compute
// every repaired value from the unrepaired field a.src, then scatter into a.src.
constexpr long long kDampCap = 1ll << 22;
void launch_damp27_scan(const Step27Args& a, bool fp32, cudaStream_t s);
void launch_damp27_fix(const Step27Args& a, bool fp32, void* vals, cudaStream_t s);
void launch_explode(bool fp32, const void* coarse, int64_t cplane, void* fine, int64_t fplane, const int32_t* ghost,
                    const int32_t* src, const uint8_t* cnt, int64_t n, unsigned long long* repaired, cudaStream_t s);
void launch_average_down(bool fp32, const void* fine, int64_t fplane, void* coarse, int64_t cplane, const int32_t* dst,
                         const int32_t* src, int64_t n, cudaStream_t s);

}  // namespace elbm
