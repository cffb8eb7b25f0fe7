// Internal interface of the D3Q39 kernels (not part of the C ABI).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace elbm {

// Lattice tables of general/background_calcs/directions_and_weights.f95:463-780,
// after the optional Galilean shift; filled on the host, read from constant memory.
struct Lattice39 {
  int cx[39], cy[39], cz[39], opp[39];
  int ucx[39], ucy[39], ucz[39], erp[39];  // the unshifted set and its opposites
  double cmag[39];
  int phi[13][39];  // 1, cx, cy, cz, cx2, cy2, cz2, cxcy, cxcz, cycz, cx c2, cy c2, cz c2
  int yi[27][39];
  int kroen[27][39];
};

// Scalars of one level (background calculations of the reference).
struct D3Q39Dev {
  int shifted, primary_flow_dir, turbulent, lvl, startup_timesteps, max_lm_iters;
  double gama, t_ref, rho_ref, p_ref, mu_ref, kappa_ref, gas_const_R, const_vol, const_press, molec_weight;
  double dt, elbm_epsilon, init_beta_1, init_beta_2, beta_1_scaling, beta_2_scaling;
  double su_lm[13];                    // start-up multipliers (su_chi .. su_lambda_z)
  double fs_u, fs_v, fs_w, fs_temp;    // freestream velocity and temperature
};

// A fluid node with interpolated wall links (codes -1001 - q 1e9): what
// target_finder and the wall closure read for it.
struct Wall39Rec {
  int32_t node;       // box node
  int32_t rec;        // its boundary record
  int32_t adjacent;   // a wall link among directions 1..14: targets from target_finder plus a Newton solve
  int32_t pad;
  int32_t code[39];   // the node's state components (0: node type)
  uint32_t snap[39];  // adjacent nodes: the post-streaming slot as target_finder finds it (link word)
  int32_t upass[39];  // node whose previous macroscopic values target_finder takes for direction j (-1: none)
  int32_t st[7];      // node types of the stencil rest, +x, +y, +z, -x, -y, -z (-666 outside the box)
  int32_t sidx[7];    // stencil nodes (-1 outside the box)
  int32_t tidx[7];    // non-adjacent nodes: temperature source of each fluid stencil node (one lattice shift on)
};

struct Step39Args {
  const double* fsrc;
  const double* gsrc;
  double* fdst;
  double* gdst;
  double* lm;      // 13 planes, read and written in place (node-local)
  double* w_vel;   // previous step's w, read and written in place (node-local)
  double* alpha;   // optional
  double* macro;   // optional: rho, u, v, w, T planes
  int64_t plane;
  int nx, ny, nz;
  int64_t N;
  int step;        // timestep(amr_max_lvl) of this step
  D3Q39Dev k;
  DevStats* stats;
  // link codes (nullptr ntype: periodic box, every node a plain pull)
  int periodic;               // bit 0/1/2: x/y/z wrap
  const uint8_t* ntype;       // 0 skip, 1 bulk (plain pulls), 2 boundary
  const int32_t* bidx;        // boundary record per node
  const uint32_t* words;      // 39 per record: kind | pop << 2 | table << 8 | offset << 13
  const double* eqf;          // 17 x 39 boundary equilibria of f (0 freestream, 1-8 inlets, 9-16 outlets)
  const double* eqg;          // same for g
  double* fprev;              // 39 per record: post-streaming f of the previous step
  double* gprev;
  // interpolated wall links (nwall records; the step's macro planes hold the previous step's fields)
  const Wall39Rec* walls;
  int64_t nwall;
  const int32_t* recwall;     // per boundary record: its wall record or -1
  double* wallf;              // 39 per wall record: the wall values of f, then g, of this step
  double* wallg;
  // FP32 storage (fsrc32 set): f and g held as float deviations from a per-direction reference
  // (ref: 39 values for f, then 39 for g); the step computes in FP64 as with FP64 storage
  const float* fsrc32;
  const float* gsrc32;
  float* fdst32;
  float* gdst32;
  const double* ref;
};

// Link words of D3Q39 boundary records.
enum Link39Kind : uint32_t { L39_STALE = 0, L39_PULL = 1, L39_EQ = 2, L39_WALL = 3 };
__host__ __device__ constexpr uint32_t link39(uint32_t kind, int pop, int table, int dx, int dy, int dz) {
  return kind | ((uint32_t)pop << 2) | ((uint32_t)table << 8) |
         ((uint32_t)((dx + 4) + 9 * (dy + 4) + 81 * (dz + 4)) << 13);
}

// One box's latest D3Q39 state as the coarse-fine transfer reads or writes it.
struct Box39View {
  double* f;
  double* g;
  double* lm;     // 13 planes
  double* w_vel;
  double* alpha;
  double* macro;  // rho, u, v, w, T planes
  int64_t plane;
};

void build_lattice39(int shifted, int primary_flow_dir, Lattice39& L);
void upload_lattice39(const Lattice39& L, cudaStream_t s);
void launch_d3q39_fp64(const Step39Args& a, cudaStream_t s);
void launch_d3q39_walls(const Step39Args& a, cudaStream_t s);
void launch_d3q39_init(const Step39Args& a, const double* lm0, unsigned long long* capped, cudaStream_t s);
void launch_mic_sample(const double* macro, int64_t plane, int nmic, const int32_t* nodes, const double* wts,
                       double* out, cudaStream_t s);
void launch_ggm(const double* macro, int64_t plane, int nx, int ny, int nz, int periodic, const uint16_t* mask,
                int variable, int scheme, const double* fs, double limit, double* gm, double* ggm, uint8_t* tags,
                unsigned long long* ntag, cudaStream_t s);
// coarse-fine transfer: coarse / fine are device tables of box views; counters[0] counts ghost
// nodes with a repaired population, counters[1] multiplier solves that hit the iteration cap
void launch_d3q39_explode(const Box39View* coarse, const Box39View& fine, const int32_t* ghost, const int32_t* src,
                          const uint16_t* sbox, const uint8_t* cnt, int64_t n, const D3Q39Dev& k, int step,
                          unsigned long long* counters, cudaStream_t s);
void launch_d3q39_average_down(const Box39View* fine, const Box39View& coarse, const int32_t* dst, const int32_t* src,
                               const uint16_t* sbox, int64_t n, cudaStream_t s);
void launch_ggm_pgs(const double* macro, int64_t plane, int nx, int ny, int nz, const uint16_t* mask,
                    const double* ggm, double sensitivity, int reach, uint8_t* tags, cudaStream_t s);
// dmask nullptr: a box without link codes (every link interior)
// src, dst: FP64 planes, or (ref set) float deviations from ref
void launch_d3q39_damp_links(const void* src, void* dst, const double* ref, const unsigned long long* dmask, int nx,
                             int ny, int nz, int64_t plane, int periodic, int shifted, const int* lo, const int* hi,
                             const double* eq, DevStats* stats, cudaStream_t s);

}  // namespace elbm
