// C ABI of libelbm_gb300: level registry, link decoding, host<->device copies
// and the per-level step driver.  Declarations and reference citations live in
// include/elbm_gb300.h.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/elbm_gb300.h"
#include "kernels.cuh"
#include "kernels39.cuh"
#include "links39.h"
#include "mlp.cuh"
#include <algorithm>
#include <array>
#include <random>
#include "lattice.cuh"

using namespace elbm;

namespace {

// Device buffer.  `guard` extra elements on either side of the usable range
// are allocated but never written: the staged step kernel's bulk copies of row
// segments may start a few elements before a plane and end after it.
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  T* base = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n), base(o.base) { o.p = o.base = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      reset();
      p = o.p;
      n = o.n;
      base = o.base;
      o.p = o.base = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { reset(); }
  void reset() {
    if (base) cudaFree(base);
    p = base = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count, size_t guard = 0) {
    reset();
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&base, (count + 2 * guard) * sizeof(T));
    if (e == cudaSuccess) {
      n = count;
      p = base + guard;
    } else {
      base = nullptr;
    }
    return e;
  }
};

struct Box {
  int lo[3], hi[3];
  int nx, ny, nz;
  int64_t N, plane;
  // D3Q27: the box's nodes are [base, base + N) of the level-wide arrays, and
  // its decoded links wait on the host until every box of the level has them
  int64_t base = 0;
  std::vector<uint8_t> h_ntype;
  std::vector<int64_t> h_bnodes;   // boundary nodes (box-local index)
  std::vector<uint16_t> h_words;   // Q per boundary node
  std::vector<double> h_qfrac;     // Q per boundary node
  std::vector<int32_t> h_xsrc;     // Q per boundary node (level index of a cross-box source, -1: none)
  std::vector<int64_t> h_ghost;    // fine ghost nodes (state 1e7 .. 1.1e9), box-local index
  DevBuf<double> staging;  // FP64 packed staging for FP32 conversion
  // D3Q39: populations, g populations, multipliers, previous w, alpha and macroscopic fields
  DevBuf<uint8_t> buf[2];
  int cur = 0;
  DevBuf<uint8_t> gbuf[2];
  int gcur = 0;
  // FP32 storage: per-direction reference of f (39) then g (39), fixed at the first upload or
  // initial state (the per-direction mean of the box), and an FP64 staging plane set for transfers
  DevBuf<double> ref39, stage39;
  bool ref39_set = false;
  DevBuf<double> lm, w_vel, alpha64, macro;
  // D3Q39 link codes (elbm_set_links39)
  bool links39 = false;
  DevBuf<uint8_t> ntype39;
  DevBuf<int32_t> bidx39, bnodes39;
  DevBuf<uint32_t> words39;
  DevBuf<double> fprev39, gprev39;
  int64_t nrec39 = 0;
  // interpolated wall links: per-node records, record -> wall map, this step's wall values
  DevBuf<Wall39Rec> walls39;
  DevBuf<int32_t> recwall39;
  DevBuf<double> wallf39, wallg39;
  int64_t nwall39 = 0;
  DevBuf<unsigned long long> dmask39;  // link classes of the repair, per node
  DevBuf<uint16_t> gmask39;            // links of the GGM differences, per node
  bool macro_set = false;  // elbm_upload_macro39 since the last elbm_upload_level39
  int64_t fluid_nodes = 0, boundary_nodes = 0;
  bool links_set = false, data_set = false;
};

struct Level {
  bool registered = false;
  int lattice = 0, storage = 0, ngrow = 0;
  std::vector<std::unique_ptr<Box>> boxes;
  elbm_d3q27_params p27{};
  elbm_d3q39_params p39{};
  bool params_set = false;
  bool mlp_set = false;  // learned-alpha weights uploaded
  DevBuf<float> mlp_w;   // the level's network weights (FP32 master copy; BF16 in the tensor-core kernel)
  int variant = 0;  // FP32 D3Q27 kernel variant picked by elbm_autotune
  DevBuf<uint8_t> eq;  // kEqTables x Q, FP64 or FP32 deviations
  DevBuf<double> eq39f, eq39g;  // D3Q39 boundary equilibria of f and g, kEqTables x 39
  // A D3Q39 level of several boxes is held as one internal box (the sheet) over their bounding
  // box, so that links, wall targets and the repair reach across box faces in place: sub39 holds
  // the caller's boxes (lo, hi); a box's state waits here until every box has one (then the sheet's
  // state is assembled and decoded once), and the per-box calls that complete the sheet's
  // populations, fields and initial state are counted
  std::vector<std::array<int32_t, 6>> sub39;
  std::vector<std::vector<int32_t>> sub39_state;
  std::vector<int> sub39_ngrow;
  std::vector<uint8_t> sub39_have_pops, sub39_have_macro, sub39_have_init;
  elbm_d3q39_bc sub39_bc{};
  double fs39[4] = {0, 0, 0, 0};  // D3Q39 freestream u, v, w, T (interpolated wall links)
  // D3Q27: every box of the level in one set of arrays (one launch per step)
  int64_t plane = 0;        // nodes per population plane: the boxes, each padded to whole 32-node chunks
  DevBuf<uint8_t> pop[2];   // population ping-pong (bytes: FP64 or FP32)
  int cur = 0;              // buffer holding the latest post-collision state
  DevBuf<uint8_t> ntype;    // per node
  DevBuf<int32_t> bidx;     // per node: boundary record or -1
  DevBuf<uint16_t> words;   // Q per boundary record
  DevBuf<uint8_t> qfrac;    // Q per boundary record, FP64 or FP32 like the populations
  DevBuf<int32_t> xsrc;     // Q per boundary record
  DevBuf<int32_t> bnode;    // level node index of every boundary record
  int64_t nrec = 0;         // boundary records of the level
  DevBuf<uint32_t> rsrc;    // resolved pull sources of the records, Q x nrec (empty: level too large)
  DevBuf<int32_t> chunk_box;
  DevBuf<int4> boxdim;
  DevBuf<float> alpha;      // per node (record_alpha)
  DevBuf<unsigned long long> work;  // chunk counter of the persistent step variant
  // tensor-copy step variant (FP32): 2 x nbox tensor maps (buffer 0's boxes, then buffer 1's),
  // the boxes' tilings and the level's tile count; empty when the level is not eligible
  DevBuf<uint8_t> ws_maps;
  DevBuf<WsBox> ws_boxes;
  int64_t ws_ntiles = 0;
  std::string ws_why;  // why the level has no tensor-copy tables (empty: it has them)
  DevBuf<uint32_t> defer_list;      // FP32: strongly non-equilibrium nodes of the step, finished apart
  DevBuf<unsigned long long> defer_count;
  // negative-population repair: (node * 27 + population) list, its count, repaired values
  DevBuf<unsigned long long> damp_list, damp_count;
  DevBuf<double> damp_vals;
  bool links_ready = false; // every box's links decoded and uploaded
  // coarse-fine transfer with level lvl - 1 (elbm_interlevel_setup)
  DevBuf<int32_t> il_ghost, il_src, il_down_dst, il_down_src;
  DevBuf<uint8_t> il_cnt;
  DevBuf<unsigned long long> il_repaired;
  int64_t il_nghost = 0, il_ndown = 0;
  bool il_ready = false;
  // the same for two D3Q39 levels: ghost lists of the fine boxes (box k: entries il39_goff[k] ..
  // il39_goff[k + 1]) with their coarse sources as (box, local index), coalescence lists of the
  // coarse boxes (offsets il39_doff) with their fine sources; device tables of both levels' box views
  DevBuf<int32_t> il39_ghost, il39_gsrc, il39_ddst, il39_dsrc;
  DevBuf<uint16_t> il39_gbox, il39_dbox;
  DevBuf<uint8_t> il39_gcnt;
  std::vector<int64_t> il39_goff, il39_doff;
  DevBuf<Box39View> il39_cview, il39_fview;
  std::vector<Box39View> il39_hcview, il39_hfview;
  DevBuf<unsigned long long> il39_counters;
};

}  // namespace

struct elbm_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  std::vector<Level> levels;
  DevBuf<DevStats> stats;
  // CUDA graph of two coarse cycles of the AMR sub-cycle (elbm_amr_run)
  cudaGraphExec_t amr_exec = nullptr;
  int amr_nlev = 0;
  uint64_t amr_key = 0;  // fingerprint of the level set-up the graph was captured for
};

namespace {

int fail(elbm_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

int cuda_fail(elbm_ctx* c, cudaError_t e, const char* what) {
  return fail(c, ELBM_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CUDA_TRY(call, what)                          \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
  } while (0)

Level* get_level(elbm_ctx* c, int lvl) {
  if (!c || lvl < 0 || lvl >= (int)c->levels.size() || !c->levels[lvl].registered) return nullptr;
  return &c->levels[lvl];
}

Box* get_box(elbm_ctx* c, int lvl, int box, Level** lv_out = nullptr) {
  Level* lv = get_level(c, lvl);
  if (!lv || box < 0 || box >= (int)lv->boxes.size()) return nullptr;
  if (lv_out) *lv_out = lv;
  return lv->boxes[box].get();
}

bool node_is_fluid(int32_t s0) {
  // collision.f95:157-159 skips state < 0, 1000 <= state < 51000, 200 <= state < 299
  if (s0 < 0) return false;
  if (s0 >= 1000 && s0 < 51000) return false;
  if (s0 >= 200 && s0 < 299) return false;
  return true;
}

// Fine nodes outside the level's valid region, filled from the coarse level
// (loop.f95:71-89: 1e7 .. 1.1e9 ghost).
bool node_is_ghost(int32_t s0) { return s0 >= 10000000 && s0 <= 1100000000; }

size_t elem_size(int storage) { return storage == ELBM_STORE_FP64 ? sizeof(double) : sizeof(float); }

// Post-streaming slots of the D3Q39 boundary records before the first step:
// the node's own populations (fi = fout at the start).
// ref: nullptr for FP64 storage, else the FP32 deviations' reference (f, then g)
template <typename T>
__global__ void stale39_init_kernel(const T* __restrict__ f, const T* __restrict__ g,
                                    const int32_t* __restrict__ bnodes, int64_t nrec, int64_t plane,
                                    const double* __restrict__ ref, double* __restrict__ fprev,
                                    double* __restrict__ gprev) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nrec * 39) return;
  const int64_t r = e / 39;
  const int j = (int)(e % 39);
  fprev[e] = (double)f[(int64_t)j * plane + bnodes[r]] + (ref ? ref[j] : 0.0);
  gprev[e] = (double)g[(int64_t)j * plane + bnodes[r]] + (ref ? ref[39 + j] : 0.0);
}

void launch_stale39_init(Box& b, cudaStream_t s) {
  if (b.nrec39 <= 0) return;
  const int64_t n = b.nrec39 * 39;
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (b.ref39.p)
    stale39_init_kernel<float><<<grid, 256, 0, s>>>((const float*)b.buf[b.cur].p, (const float*)b.gbuf[b.gcur].p,
                                                   b.bnodes39.p, b.nrec39, b.plane, b.ref39.p, b.fprev39.p,
                                                   b.gprev39.p);
  else
    stale39_init_kernel<double><<<grid, 256, 0, s>>>((const double*)b.buf[b.cur].p, (const double*)b.gbuf[b.gcur].p,
                                                    b.bnodes39.p, b.nrec39, b.plane, nullptr, b.fprev39.p,
                                                    b.gprev39.p);
}

// FP32 D3Q39 storage: per-plane sums of an FP64 plane set (for the reference), and the
// conversions between FP64 planes and float deviations from the reference.
// Per-block partial sums of each of 39 planes (plane j, block k at j * gridDim.x + k); the host
// adds them in block order, so that the reference (and every FP32 value) is the same run after run.
__global__ void plane_sums39_kernel(const double* __restrict__ src, int64_t N, int64_t plane,
                                    double* __restrict__ parts) {
  __shared__ double part[256];
  const int j = blockIdx.y;
  double acc = 0.0;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    acc += src[(int64_t)j * plane + n];
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) parts[(int64_t)j * gridDim.x + blockIdx.x] = part[0];
}

__global__ void to_dev39_kernel(const double* __restrict__ src, float* __restrict__ dst, int64_t N, int64_t plane,
                                const double* __restrict__ ref) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (n < N) dst[(int64_t)j * plane + n] = (float)(src[(int64_t)j * plane + n] - ref[j]);
}

__global__ void from_dev39_kernel(const float* __restrict__ src, double* __restrict__ dst, int64_t N, int64_t plane,
                                  const double* __restrict__ ref) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (n < N) dst[(int64_t)j * plane + n] = (double)src[(int64_t)j * plane + n] + ref[j];
}

// The FP64 f and g planes in b.stage39 (f first, then g) into the FP32 buffers 0, fixing the
// reference at the per-direction mean when the box has none yet.
cudaError_t stage39_to_fp32(Box& b, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  const int64_t half = b.plane * 39;
  if (!b.ref39_set) {
    const unsigned gx = (unsigned)std::min<int64_t>((b.N + 255) / 256, 512);
    DevBuf<double> parts;
    if ((e = parts.alloc((size_t)78 * gx)) != cudaSuccess) return e;
    plane_sums39_kernel<<<dim3(gx, 39), 256, 0, s>>>(b.stage39.p, b.N, b.plane, parts.p);
    plane_sums39_kernel<<<dim3(gx, 39), 256, 0, s>>>(b.stage39.p + half, b.N, b.plane, parts.p + (size_t)39 * gx);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    std::vector<double> hp((size_t)78 * gx), h(78);
    if ((e = cudaMemcpyAsync(hp.data(), parts.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, s)) !=
        cudaSuccess)
      return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    for (int j = 0; j < 78; ++j) {
      double acc = 0.0;
      for (unsigned k = 0; k < gx; ++k) acc += hp[(size_t)j * gx + k];
      h[j] = acc / (double)b.N;
    }
    if ((e = cudaMemcpyAsync(b.ref39.p, h.data(), 78 * sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    b.ref39_set = true;
  }
  const dim3 grid((unsigned)((b.N + 255) / 256), 39);
  to_dev39_kernel<<<grid, 256, 0, s>>>(b.stage39.p, (float*)b.buf[0].p, b.N, b.plane, b.ref39.p);
  to_dev39_kernel<<<grid, 256, 0, s>>>(b.stage39.p + half, (float*)b.gbuf[0].p, b.N, b.plane, b.ref39.p + 39);
  return cudaGetLastError();
}

// ---- conversion kernels between the FP64 host layout and FP32 deviations ----
__global__ void to_dev32_kernel(const double* __restrict__ f, float* __restrict__ d, int64_t N, int64_t plane) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (n >= N) return;
  d[(int64_t)j * plane + n] = (float)(f[(int64_t)j * N + n] - w27(j));
}
__global__ void from_dev32_kernel(const float* __restrict__ d, double* __restrict__ f, int64_t N, int64_t plane) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (n >= N) return;
  f[(int64_t)j * N + n] = (double)d[(int64_t)j * plane + n] + w27(j);
}

// Copy the valid region of a host FAB (ngrow ghosts, ncomp comps) into a
// packed device array with component stride `plane` (elements of size es).
template <typename T>
cudaError_t fab_to_packed(const T* host, T* dev, const Box& b, int ngrow, int ncomp, int64_t plane, cudaStream_t s) {
  const int fx = b.nx + 2 * ngrow, fy = b.ny + 2 * ngrow, fz = b.nz + 2 * ngrow;
  if (ngrow == 0) {
    // whole component planes: plain copies (one when the device planes are not padded)
    if (plane == b.N) return cudaMemcpyAsync(dev, host, (size_t)b.N * ncomp * sizeof(T), cudaMemcpyHostToDevice, s);
    for (int q = 0; q < ncomp; ++q) {
      const cudaError_t e = cudaMemcpyAsync(dev + (int64_t)q * plane, host + (int64_t)q * b.N, (size_t)b.N * sizeof(T),
                                            cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  for (int q = 0; q < ncomp; ++q) {
    cudaMemcpy3DParms p{};
    p.srcPtr = make_cudaPitchedPtr((void*)(host + (int64_t)q * fx * fy * fz), fx * sizeof(T), fx, fy);
    p.srcPos = make_cudaPos(ngrow * sizeof(T), ngrow, ngrow);
    p.dstPtr = make_cudaPitchedPtr((void*)(dev + (int64_t)q * plane), b.nx * sizeof(T), b.nx, b.ny);
    p.dstPos = make_cudaPos(0, 0, 0);
    p.extent = make_cudaExtent(b.nx * sizeof(T), b.ny, b.nz);
    p.kind = cudaMemcpyHostToDevice;
    cudaError_t e = cudaMemcpy3DAsync(&p, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T>
cudaError_t packed_to_fab(const T* dev, T* host, const Box& b, int ngrow, int ncomp, int64_t plane, cudaStream_t s) {
  const int fx = b.nx + 2 * ngrow, fy = b.ny + 2 * ngrow, fz = b.nz + 2 * ngrow;
  if (ngrow == 0) {
    if (plane == b.N) return cudaMemcpyAsync(host, dev, (size_t)b.N * ncomp * sizeof(T), cudaMemcpyDeviceToHost, s);
    for (int q = 0; q < ncomp; ++q) {
      const cudaError_t e = cudaMemcpyAsync(host + (int64_t)q * b.N, dev + (int64_t)q * plane, (size_t)b.N * sizeof(T),
                                            cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  for (int q = 0; q < ncomp; ++q) {
    cudaMemcpy3DParms p{};
    p.srcPtr = make_cudaPitchedPtr((void*)(dev + (int64_t)q * plane), b.nx * sizeof(T), b.nx, b.ny);
    p.srcPos = make_cudaPos(0, 0, 0);
    p.dstPtr = make_cudaPitchedPtr((void*)(host + (int64_t)q * fx * fy * fz), fx * sizeof(T), fx, fy);
    p.dstPos = make_cudaPos(ngrow * sizeof(T), ngrow, ngrow);
    p.extent = make_cudaExtent(b.nx * sizeof(T), b.ny, b.nz);
    p.kind = cudaMemcpyDeviceToHost;
    cudaError_t e = cudaMemcpy3DAsync(&p, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// The same copies for a sub-box of a box: the caller's box of a multi-box D3Q39
// level inside the internal sheet, at offset off, of size n (nodes per axis).
template <typename T>
cudaError_t sub_copy(T* host, T* dev, const Box& b, const int (&off)[3], const int (&n)[3], int ngrow, int ncomp,
                     int64_t plane, bool to_dev, cudaStream_t s) {
  const int fx = n[0] + 2 * ngrow, fy = n[1] + 2 * ngrow, fz = n[2] + 2 * ngrow;
  for (int q = 0; q < ncomp; ++q) {
    cudaPitchedPtr hp = make_cudaPitchedPtr((void*)(host + (int64_t)q * fx * fy * fz), fx * sizeof(T), fx, fy);
    cudaPitchedPtr dp = make_cudaPitchedPtr((void*)(dev + (int64_t)q * plane), b.nx * sizeof(T), b.nx, b.ny);
    const cudaPos hpos = make_cudaPos(ngrow * sizeof(T), ngrow, ngrow);
    const cudaPos dpos = make_cudaPos(off[0] * sizeof(T), off[1], off[2]);
    cudaMemcpy3DParms p{};
    p.srcPtr = to_dev ? hp : dp;
    p.srcPos = to_dev ? hpos : dpos;
    p.dstPtr = to_dev ? dp : hp;
    p.dstPos = to_dev ? dpos : hpos;
    p.extent = make_cudaExtent(n[0] * sizeof(T), n[1], n[2]);
    p.kind = to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    const cudaError_t e = cudaMemcpy3DAsync(&p, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// The caller's box k of a D3Q39 level: the internal box holding it, the box's
// offset in it and its size.  A single-box level is its own sheet.
struct Sub39 {
  Box* b = nullptr;
  int off[3] = {0, 0, 0};
  int n[3] = {0, 0, 0};
  bool whole = true;  // the caller's box is the whole internal box
};

Sub39 get_sub39(elbm_ctx* c, int lvl, int box, Level** lv_out) {
  Sub39 r;
  Level* lv = get_level(c, lvl);
  if (!lv || lv->lattice != ELBM_D3Q39 || lv->boxes.empty()) return r;
  if (lv_out) *lv_out = lv;
  if (lv->sub39.empty()) {
    if (box < 0 || box >= (int)lv->boxes.size()) return r;
    r.b = lv->boxes[box].get();
    r.n[0] = r.b->nx;
    r.n[1] = r.b->ny;
    r.n[2] = r.b->nz;
    return r;
  }
  if (box < 0 || box >= (int)lv->sub39.size()) return r;
  r.b = lv->boxes[0].get();
  r.whole = false;
  for (int a = 0; a < 3; ++a) {
    r.off[a] = lv->sub39[box][a] - r.b->lo[a];
    r.n[a] = lv->sub39[box][3 + a] - lv->sub39[box][a] + 1;
  }
  return r;
}

// Host-to-device (or back) copy of ncomp component planes of the caller's box.
template <typename T>
cudaError_t sub39_copy(const Sub39& u, T* host, T* dev, int ngrow, int ncomp, int64_t plane, bool to_dev,
                       cudaStream_t s) {
  if (u.whole)
    return to_dev ? fab_to_packed((const T*)host, dev, *u.b, ngrow, ncomp, plane, s)
                  : packed_to_fab((const T*)dev, host, *u.b, ngrow, ncomp, plane, s);
  return sub_copy(host, dev, *u.b, u.off, u.n, ngrow, ncomp, plane, to_dev, s);
}

// Pull-form decoding of one population's link (see include/elbm_gb300.h and
// the push rules of looping/timestepping/streaming.f95:365-481).
// Returns 0 and the link word, or a negative error code.
// Level index of the node at global coordinates (gx, gy, gz), -1 when no box
// of the level holds it.
int64_t level_index(const Level& lv, int gx, int gy, int gz) {
  for (const auto& bp : lv.boxes) {
    const Box& b = *bp;
    if (gx < b.lo[0] || gx > b.hi[0] || gy < b.lo[1] || gy > b.hi[1] || gz < b.lo[2] || gz > b.hi[2]) continue;
    return b.base + ((int64_t)(gz - b.lo[2]) * b.ny + (gy - b.lo[1])) * b.nx + (gx - b.lo[0]);
  }
  return -1;
}

// The state FAB around one node of a box: is the node at box-local offset
// (dx, dy, dz) fluid?  1 yes, 0 no, -1 outside the FAB (its ghost cells included).
struct StateView {
  const int32_t* st;
  int64_t fab_plane, sidx;
  const int* sstride;
  int g, x, y, z;
  const Box* b;
  int fluid(int dx, int dy, int dz) const {
    const int sx = x + dx, sy = y + dy, sz = z + dz;
    if (sx < -g || sy < -g || sz < -g || sx >= b->nx + g || sy >= b->ny + g || sz >= b->nz + g) return -1;
    return node_is_fluid(st[sidx + (int64_t)dx * sstride[0] + (int64_t)dy * sstride[1] + (int64_t)dz * sstride[2]])
               ? 1
               : 0;
  }
  bool inside(int dx, int dy, int dz) const {
    const int sx = x + dx, sy = y + dy, sz = z + dz;
    return sx >= 0 && sy >= 0 && sz >= 0 && sx < b->nx && sy < b->ny && sz < b->nz;
  }
};

int decode_link27(const int32_t* st, int64_t fab_plane, int64_t sidx, const int sstride[3], int ngs, int x, int y,
                  int z, const Box& b, const Level& lv, int j, bool ghost, uint16_t& word, double& qf, int32_t& xs,
                  bool& interior, std::string& why) {
  qf = 0.0;
  xs = -1;
  const StateView sv{st, fab_plane, sidx, sstride, ngs, x, y, z, &b};
  const int i = D3Q27::opp[j];  // the link that leaves x along -c_j
  const int32_t code = st[(int64_t)i * fab_plane + sidx];
  interior = false;
  if (code >= 0) {
    const int dx = -D3Q27::cx[j], dy = -D3Q27::cy[j], dz = -D3Q27::cz[j];
    if (!sv.inside(dx, dy, dz)) {
      // the source lies in another box of the level (AMReX fills this box's
      // ghost cells from it; here the step reads it in place)
      const int64_t li = level_index(lv, b.lo[0] + x + dx, b.lo[1] + y + dy, b.lo[2] + z + dz);
      if (li < 0 && ghost) {
        // outermost ghost shell: the coarse level refills this node before it matters
        word = link_word(LK_KEEP, j, 0);
        return 0;
      }
      if (li < 0) {
        why = "fluid link leaves the level's boxes (coarse-fine or domain edge without a boundary code)";
        return ELBM_E_UNSUPPORTED;
      }
      xs = (int32_t)li;
      word = link_word(LK_XBOX, j, 0);
      return 0;
    }
    word = link_word(LK_PULL, j, off_code(dx, dy, dz));
    interior = true;
    return 0;
  }
  if (code == -10 || code == -5) {  // bounceback.f95:13-19 (halfway bounce-back), null_bc
    word = link_word(LK_PULL, i, off_code(0, 0, 0));
    return 0;
  }
  if (code == -11 || code == -12) {  // inviscid_edge.f95: specular reflection
    const int c[3] = {D3Q27::cx[j], D3Q27::cy[j], D3Q27::cz[j]};
    int src_c[3] = {c[0], c[1], c[2]}, disp[3] = {c[0], c[1], c[2]};
    bool any = false;
    for (int a = 0; a < 3; ++a) {
      if (c[a] == 0) continue;
      int card[3] = {0, 0, 0};
      card[a] = -c[a];
      const int k = find27(card[0], card[1], card[2]);
      const int32_t cc = st[(int64_t)k * fab_plane + sidx];
      if (cc == -11 || cc == -12) {
        src_c[a] = -c[a];
        disp[a] = 0;
        any = true;
      }
    }
    const int src_pop = find27(src_c[0], src_c[1], src_c[2]);
    const int dx = -disp[0], dy = -disp[1], dz = -disp[2];
    int64_t li = -1;
    bool ok = any && src_pop != j && sv.fluid(dx, dy, dz) == 1;
    if (ok && !sv.inside(dx, dy, dz)) {
      li = level_index(lv, b.lo[0] + x + dx, b.lo[1] + y + dy, b.lo[2] + z + dz);
      ok = li >= 0;
    }
    if (ok && li >= 0) {
      xs = (int32_t)li;
      word = link_word(LK_XBOX, src_pop, 0);
    } else if (ok) {
      word = link_word(LK_PULL, src_pop, off_code(dx, dy, dz));
    } else {
      word = link_word(LK_PULL, i, off_code(0, 0, 0));
    }
    return 0;
  }
  if (code == -3 || code == -8 || code == -1000) {  // freestream_bc.f95, freestream_edge_bc.f95
    word = link_word(LK_EQ, 0, 0);
    return 0;
  }
  if (code <= -100 && code >= -199) {  // inlet_bc.f95:21-53
    const int k = -code - 100;
    if (k < 1 || k > 8) {
      why = "inlet number outside 1..8";
      return ELBM_E_UNSUPPORTED;
    }
    word = link_word(LK_EQ, k, 0);
    return 0;
  }
  if (code <= -200 && code >= -299) {  // outlet_bc.f95:23-58
    const int k = -code - 200;
    if (k < 1 || k > 8) {
      why = "outlet number outside 1..8";
      return ELBM_E_UNSUPPORTED;
    }
    const int t = lv.p27.outlet_type[k - 1];
    if (t == 1 || t == 4) word = link_word(LK_EQ, 8 + k, 0);
    else if (t == 2) word = link_word(LK_EQ, k, 0);  // press_temp_bc.f95:26-27 reads the inlet table
    else if (t == 3) word = link_word(LK_EQ, 0, 0);
    else if (t == 6) word = link_word(LK_PULL, j, off_code(0, 0, 0));  // pure_outflow_bc.f95:19-20
    else {
      why = "unsupported outlet type";
      return ELBM_E_UNSUPPORTED;
    }
    return 0;
  }
  if (code == -666 || code == -1001) {  // null / plain solid: nothing streams in
    word = link_word(LK_KEEP, j, 0);
    return 0;
  }
  if (code < -1001) {
    // wall link with the packed fraction of linkwise.f95:56; decoded as in
    // interpolative_bounceback_bc.f95:66: q = |state + 1001| / 1e9
    const double q = std::fabs((double)code + 1001.0) / 1e9;
    qf = q;
    // the second fluid node of the interpolation, x + c_j (one step away from the wall)
    const int dx = D3Q27::cx[j], dy = D3Q27::cy[j], dz = D3Q27::cz[j];
    int off = off_code(0, 0, 0);
    if (sv.fluid(dx, dy, dz) == 1) {
      if (sv.inside(dx, dy, dz)) {
        off = off_code(dx, dy, dz);
      } else {
        const int64_t li = level_index(lv, b.lo[0] + x + dx, b.lo[1] + y + dy, b.lo[2] + z + dz);
        if (li >= 0) {
          xs = (int32_t)li;
          off = kOffXbox;
        }
      }
    }
    word = link_word(LK_IBB, i, off);
    return 0;
  }
  why = "unsupported link code " + std::to_string(code);
  return ELBM_E_UNSUPPORTED;
}


int finish_stats(elbm_ctx* c, elbm_stats* out) {
  if (!out) return ELBM_OK;
  DevStats slots[kStatSlots * kStatStride];
  CUDA_TRY(cudaMemcpyAsync(slots, c->stats.p, kStatBytes, cudaMemcpyDeviceToHost, c->stream), "stats");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  // the slots added up (maxima and flags combined)
  DevStats ds{};
  for (int k = 0; k < kStatSlots; ++k) {
    const DevStats& s = slots[k * kStatStride];
    ds.node_updates += s.node_updates;
    ds.newton_iters += s.newton_iters;
    ds.exact_nodes += s.exact_nodes;
    ds.fallbacks += s.fallbacks;
    ds.max_dH_bits = std::max(ds.max_dH_bits, s.max_dH_bits);
    ds.dh_over += s.dh_over;
    ds.guess_misses += s.guess_misses;
    ds.status |= s.status;
  }
  float ms = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "elapsed");
  std::memset(out, 0, sizeof *out);
  out->node_updates = (int64_t)ds.node_updates;
  out->newton_iters = (int64_t)ds.newton_iters;
  out->exact_path_nodes = (int64_t)ds.exact_nodes;
  out->fallbacks = (int64_t)ds.fallbacks;
  out->status = ds.status;
  double mx;
  std::memcpy(&mx, &ds.max_dH_bits, sizeof mx);
  out->max_abs_dH = mx;
  out->dh_over_tol = (int64_t)ds.dh_over;
  out->guess_misses = (int64_t)ds.guess_misses;
  out->kernel_ms = ms;
  return ELBM_OK;
}

// The level's scalars in the form the D3Q39 kernels read.
D3Q39Dev dev39(const elbm_d3q39_params& p, const Level& lv) {
  D3Q39Dev k{};
  k.shifted = p.shifted;
  k.primary_flow_dir = p.primary_flow_dir;
  k.turbulent = p.turbulent;
  k.lvl = p.lvl;
  k.startup_timesteps = p.startup_timesteps;
  k.max_lm_iters = p.max_lm_iters;
  k.gama = p.gama;
  k.t_ref = p.t_ref;
  k.rho_ref = p.rho_ref;
  k.p_ref = p.p_ref;
  k.mu_ref = p.mu_ref;
  k.kappa_ref = p.kappa_ref;
  k.gas_const_R = p.gas_const_R;
  k.const_vol = p.const_vol;
  k.const_press = p.const_press;
  k.molec_weight = p.molec_weight;
  k.dt = p.dt;
  k.elbm_epsilon = p.elbm_epsilon;
  k.init_beta_1 = p.init_beta_1;
  k.init_beta_2 = p.init_beta_2;
  k.beta_1_scaling = p.beta_1_scaling;
  k.beta_2_scaling = p.beta_2_scaling;
  for (int r = 0; r < 13; ++r) k.su_lm[r] = p.su_lm[r];
  k.fs_u = lv.fs39[0];
  k.fs_v = lv.fs39[1];
  k.fs_w = lv.fs39[2];
  k.fs_temp = lv.fs39[3];
  return k;
}

// D3Q39 level steps: fused stream/flow-variables/collision, then the optional repair.
int step39(elbm_ctx* c, Level& lv, int nsteps) {
  const elbm_d3q39_params& p = lv.p39;
  for (auto& bp : lv.boxes) {
    if (!bp->data_set)
      return fail(c, ELBM_E_STATE,
                  lv.sub39.empty() ? "populations missing"
                                   : "populations missing: a level of several boxes steps once every box has been "
                                     "uploaded (elbm_upload_level39 or elbm_init_level39)");
    if (!bp->links39 && p.periodic != 7)
      return fail(c, ELBM_E_STATE, "a D3Q39 box that is not periodic on every axis needs elbm_set_links39");
    if (bp->nwall39 > 0 && !bp->macro_set)
      return fail(c, ELBM_E_STATE, "interpolated wall links need the macroscopic fields (elbm_upload_macro39)");
  }
  CUDA_TRY(cudaEventRecord(c->ev0, c->stream), "event");
  for (int s = 0; s < nsteps; ++s) {
    for (auto& bp : lv.boxes) {
      Box& b = *bp;
      Step39Args a{};
      if (lv.storage == ELBM_STORE_FP32_DEV) {
        a.fsrc32 = (const float*)b.buf[b.cur].p;
        a.gsrc32 = (const float*)b.gbuf[b.gcur].p;
        a.fdst32 = (float*)b.buf[b.cur ^ 1].p;
        a.gdst32 = (float*)b.gbuf[b.gcur ^ 1].p;
        a.ref = b.ref39.p;
      } else {
        a.fsrc = (const double*)b.buf[b.cur].p;
        a.gsrc = (const double*)b.gbuf[b.gcur].p;
        a.fdst = (double*)b.buf[b.cur ^ 1].p;
        a.gdst = (double*)b.gbuf[b.gcur ^ 1].p;
      }
      a.lm = b.lm.p;
      a.w_vel = b.w_vel.p;
      a.alpha = b.alpha64.p;
      a.macro = b.macro.p;
      a.plane = b.plane;
      a.nx = b.nx;
      a.ny = b.ny;
      a.nz = b.nz;
      a.N = b.N;
      a.step = lv.p39.timestep;
      a.stats = c->stats.p;
      a.periodic = p.periodic;
      if (b.links39) {
        a.ntype = b.ntype39.p;
        a.bidx = b.bidx39.p;
        a.words = b.words39.p;
        a.eqf = lv.eq39f.p;
        a.eqg = lv.eq39g.p;
        a.fprev = b.fprev39.p;
        a.gprev = b.gprev39.p;
        a.walls = b.walls39.p;
        a.nwall = b.nwall39;
        a.recwall = b.recwall39.p;
        a.wallf = b.wallf39.p;
        a.wallg = b.wallg39.p;
      }
      a.k = dev39(p, lv);
      if (a.nwall > 0) {
        launch_d3q39_walls(a, c->stream);
        CUDA_TRY(cudaGetLastError(), "d3q39 wall launch");
      }
      launch_d3q39_fp64(a, c->stream);
      CUDA_TRY(cudaGetLastError(), "d3q39 step launch");
      b.cur ^= 1;
      b.gcur ^= 1;
      b.macro_set = true;  // the step wrote the fields
      if (p.damp) {
        // damp_it.f95:64-177 on the new state, its fout part, then its gout part (the same rules;
        // outside the box each set's freestream equilibrium); a box without link codes is periodic
        // on every axis
        const bool f32 = lv.storage == ELBM_STORE_FP32_DEV;
        launch_d3q39_damp_links(b.buf[b.cur].p, b.buf[b.cur ^ 1].p, f32 ? b.ref39.p : nullptr,
                                b.links39 ? b.dmask39.p : nullptr, b.nx, b.ny, b.nz, b.plane, p.periodic, p.shifted,
                                b.lo, b.hi, b.links39 ? lv.eq39f.p : nullptr, c->stats.p, c->stream);
        CUDA_TRY(cudaGetLastError(), "d3q39 damp launch");
        b.cur ^= 1;
        launch_d3q39_damp_links(b.gbuf[b.gcur].p, b.gbuf[b.gcur ^ 1].p, f32 ? b.ref39.p + 39 : nullptr,
                                b.links39 ? b.dmask39.p : nullptr, b.nx, b.ny, b.nz, b.plane, p.periodic, p.shifted,
                                b.lo, b.hi, b.links39 ? lv.eq39g.p : nullptr, c->stats.p, c->stream);
        CUDA_TRY(cudaGetLastError(), "d3q39 damp launch (g)");
        b.gcur ^= 1;
      }
    }
    lv.p39.timestep += 1;  // steps_counter.f95:18-31
  }
  CUDA_TRY(cudaEventRecord(c->ev1, c->stream), "event");
  return ELBM_OK;
}

}  // namespace

namespace {

// Tensor maps and tilings of the tensor-copy step variant (csrc/d3q27_step.cu,
// d3q27_fp32_ws_kernel) for a D3Q27 FP32 level.  Per box and population
// buffer a 4-D map (x, y, z, population) over the box's nodes, with a copy
// box of (TX + 8) x TY x 1 x 1 floats: TX = 32, 64 or 128 by the box's width
// (the narrowest that holds a row), TY = 256 / TX.  Levels with a box whose
// rows are not whole 16-byte units (nx % 4 != 0), or whose maps the driver
// does not accept, leave the tables empty and step with the other variants.
int build_ws_tables(elbm_ctx* c, Level& lv) {
  lv.ws_maps.reset();
  lv.ws_boxes.reset();
  lv.ws_ntiles = 0;
  lv.ws_why.clear();
  for (auto& b : lv.boxes)
    if (b->nx % 4 != 0) {
      lv.ws_why = "a box's rows are not whole 16-byte units (nx % 4 != 0)";
      return ELBM_OK;
    }
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    // the driver's tensor-map encoder, through the runtime (no link-time dependency on libcuda)
    for (unsigned ver : {12000u, (unsigned)CUDA_VERSION}) {
      void* fn = nullptr;
      cudaDriverEntryPointQueryResult q{};
      const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, ver, cudaEnableDefault, &q);
      if (e == cudaSuccess && q == cudaDriverEntryPointSuccess && fn) {
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        break;
      }
      char why[160];
      snprintf(why, sizeof why, "cuTensorMapEncodeTiled not available (runtime error %d, query result %d)", (int)e,
               (int)q);
      lv.ws_why = why;
    }
    if (!encode) return ELBM_OK;
    lv.ws_why.clear();
  }
  const int nbox = (int)lv.boxes.size();
  std::vector<WsBox> wb(nbox);
  std::vector<CUtensorMap> maps(2 * (size_t)nbox);
  int64_t tiles = 0;
  for (int k = 0; k < nbox; ++k) {
    const Box& b = *lv.boxes[k];
    const int txl = b.nx <= 32 ? 5 : (b.nx <= 64 ? 6 : 7);
    const int TX = 1 << txl, TY = kWsTileNodes / TX;
    WsBox& w = wb[k];
    w.base = b.base;
    w.tile0 = tiles;
    w.nx = b.nx;
    w.ny = b.ny;
    w.nz = b.nz;
    w.tx_log2 = txl;
    w.tiles_x = (b.nx + TX - 1) / TX;
    w.tiles_y = (b.ny + TY - 1) / TY;
    tiles += (int64_t)w.tiles_x * w.tiles_y * b.nz;
    for (int buf = 0; buf < 2; ++buf) {
      const cuuint64_t dims[4] = {(cuuint64_t)b.nx, (cuuint64_t)b.ny, (cuuint64_t)b.nz, (cuuint64_t)Q27};
      const cuuint64_t strides[3] = {(cuuint64_t)b.nx * 4, (cuuint64_t)b.nx * b.ny * 4, (cuuint64_t)lv.plane * 4};
      const cuuint32_t box[4] = {(cuuint32_t)(TX + 8), (cuuint32_t)TY, 1, 1};
      const cuuint32_t estr[4] = {1, 1, 1, 1};
      void* base = lv.pop[buf].p + (size_t)b.base * sizeof(float);
      const CUresult r = encode(&maps[(size_t)buf * nbox + k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides,
                                box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r != CUDA_SUCCESS) {
        char why[160];
        snprintf(why, sizeof why, "the driver rejected the tensor map of box %d (CUresult %d)", k, (int)r);
        lv.ws_why = why;
        return ELBM_OK;
      }
    }
  }
  static_assert(sizeof(CUtensorMap) == 128, "tensor map size");
  CUDA_TRY(lv.ws_maps.alloc(maps.size() * sizeof(CUtensorMap)), "tensor maps");
  CUDA_TRY(cudaMemcpy(lv.ws_maps.p, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice),
           "tensor maps");
  CUDA_TRY(lv.ws_boxes.alloc(nbox), "tile boxes");
  CUDA_TRY(cudaMemcpy(lv.ws_boxes.p, wb.data(), nbox * sizeof(WsBox), cudaMemcpyHostToDevice), "tile boxes");
  lv.ws_ntiles = tiles;
  return ELBM_OK;
}

}  // namespace

extern "C" {

int elbm_create(int device, elbm_ctx** out) {
  if (!out) return ELBM_E_ARG;
  *out = nullptr;
  auto c = std::make_unique<elbm_ctx>();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return ELBM_E_CUDA;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return ELBM_E_CUDA;
  if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) return ELBM_E_CUDA;
  if (c->stats.alloc((size_t)kStatSlots * kStatStride) != cudaSuccess) return ELBM_E_CUDA;
  if (cudaMemset(c->stats.p, 0, kStatBytes) != cudaSuccess) return ELBM_E_CUDA;
  // reserve the allocation-free upload's staging buffer on this device now (csrc/noalloc.cu)
  if (noalloc_setup(device) != cudaSuccess) return ELBM_E_CUDA;
  *out = c.release();
  return ELBM_OK;
}

void elbm_destroy(elbm_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->amr_exec) cudaGraphExecDestroy(c->amr_exec);
  c->levels.clear();
  c->stats.reset();
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* elbm_last_error_string(const elbm_ctx* c) { return c ? c->err.c_str() : "null context"; }

int elbm_level_register(elbm_ctx* c, int lvl, int lattice, int storage, int nbox, const int32_t* lo_hi, int ngrow) {
  if (!c) return ELBM_E_ARG;
  if (lvl < 0 || lvl > 30) return fail(c, ELBM_E_ARG, "level %d out of range", lvl);
  if (lattice != ELBM_D3Q27 && lattice != ELBM_D3Q39) return fail(c, ELBM_E_UNSUPPORTED, "lattice %d", lattice);
  if (storage != ELBM_STORE_FP64 && storage != ELBM_STORE_FP32_DEV) return fail(c, ELBM_E_ARG, "bad storage %d", storage);
  if (nbox < 1) return fail(c, ELBM_E_ARG, "nbox=%d", nbox);
  if (!lo_hi || ngrow < 0) return fail(c, ELBM_E_ARG, "null lo_hi or negative ngrow");
  for (int k = 0; k < nbox; ++k)
    for (int m = 0; m < k; ++m) {
      bool overlap = true;
      for (int a = 0; a < 3; ++a)
        overlap &= lo_hi[6 * k + a] <= lo_hi[6 * m + 3 + a] && lo_hi[6 * m + a] <= lo_hi[6 * k + 3 + a];
      if (overlap) return fail(c, ELBM_E_ARG, "boxes %d and %d overlap", m, k);
    }
  if (lattice == ELBM_D3Q39 && nbox > 1) {
    // one internal box over the boxes' bounding box (nodes outside every box stay inactive)
    int32_t bb[6] = {lo_hi[0], lo_hi[1], lo_hi[2], lo_hi[3], lo_hi[4], lo_hi[5]};
    for (int k = 1; k < nbox; ++k)
      for (int a = 0; a < 3; ++a) {
        if (lo_hi[6 * k + 3 + a] < lo_hi[6 * k + a]) return fail(c, ELBM_E_ARG, "empty box %d", k);
        bb[a] = std::min(bb[a], lo_hi[6 * k + a]);
        bb[3 + a] = std::max(bb[3 + a], lo_hi[6 * k + 3 + a]);
      }
    if (const int rc = elbm_level_register(c, lvl, lattice, storage, 1, bb, ngrow)) return rc;
    Level& lv = c->levels[lvl];
    for (int k = 0; k < nbox; ++k)
      lv.sub39.push_back({lo_hi[6 * k], lo_hi[6 * k + 1], lo_hi[6 * k + 2], lo_hi[6 * k + 3], lo_hi[6 * k + 4],
                          lo_hi[6 * k + 5]});
    lv.sub39_state.assign(nbox, {});
    lv.sub39_ngrow.assign(nbox, 0);
    lv.sub39_have_pops.assign(nbox, 0);
    lv.sub39_have_macro.assign(nbox, 0);
    lv.sub39_have_init.assign(nbox, 0);
    return ELBM_OK;
  }
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  if ((int)c->levels.size() <= lvl) c->levels.resize(lvl + 1);
  Level& lv = c->levels[lvl];
  lv = Level();
  lv.lattice = lattice;
  lv.storage = storage;
  lv.ngrow = ngrow;
  for (int k = 0; k < nbox; ++k) {
    auto b = std::make_unique<Box>();
    for (int a = 0; a < 3; ++a) {
      b->lo[a] = lo_hi[6 * k + a];
      b->hi[a] = lo_hi[6 * k + 3 + a];
      if (b->hi[a] < b->lo[a]) return fail(c, ELBM_E_ARG, "empty box %d", k);
    }
    b->nx = b->hi[0] - b->lo[0] + 1;
    b->ny = b->hi[1] - b->lo[1] + 1;
    b->nz = b->hi[2] - b->lo[2] + 1;
    b->N = (int64_t)b->nx * b->ny * b->nz;
    b->base = lv.plane;
    lv.plane += (b->N + 31) / 32 * 32;
    if (lattice == ELBM_D3Q39) {
      b->plane = (b->N + 31) / 32 * 32;
      const size_t bytes = (size_t)b->plane * 39 * elem_size(storage);
      for (int s = 0; s < 2; ++s) CUDA_TRY(b->buf[s].alloc(bytes), "population buffers");
      for (int s = 0; s < 2; ++s) CUDA_TRY(b->gbuf[s].alloc(bytes), "g buffers");
      CUDA_TRY(b->lm.alloc((size_t)b->plane * 13), "multipliers");
      CUDA_TRY(b->w_vel.alloc((size_t)b->plane), "w");
      CUDA_TRY(b->alpha64.alloc((size_t)b->plane), "alpha");
      CUDA_TRY(b->macro.alloc((size_t)b->plane * 5), "macro");
      // defined fields for nodes no upload covers (a multi-box level's uncovered nodes)
      CUDA_TRY(cudaMemset(b->macro.p, 0, b->macro.n * sizeof(double)), "macro");
      if (storage == ELBM_STORE_FP32_DEV) CUDA_TRY(b->ref39.alloc(78), "FP32 reference");
    }
    lv.boxes.push_back(std::move(b));
  }
  if (lattice == ELBM_D3Q27) {
    if (lv.plane > INT32_MAX) return fail(c, ELBM_E_ARG, "a level holds at most 2^31 - 1 nodes");
    for (auto& b : lv.boxes) b->plane = lv.plane;
    const size_t bytes = (size_t)lv.plane * Q27 * elem_size(storage);
    for (int s = 0; s < 2; ++s) CUDA_TRY(lv.pop[s].alloc(bytes, kPopGuardBytes), "population buffers");
    CUDA_TRY(lv.ntype.alloc(lv.plane), "node types");
    CUDA_TRY(lv.work.alloc(1), "work counter");
    if (storage == ELBM_STORE_FP32_DEV) {
      CUDA_TRY(lv.defer_list.alloc(std::max<size_t>((size_t)lv.plane / 8, 4096)), "deferred-node list");
      CUDA_TRY(lv.defer_count.alloc(1), "deferred-node count");
    }
    CUDA_TRY(cudaMemsetAsync(lv.ntype.p, 0, lv.plane, c->stream), "memset");
    std::vector<int32_t> cb(lv.plane / 32);
    std::vector<int4> bd(nbox);
    for (int k = 0; k < nbox; ++k) {
      const Box& b = *lv.boxes[k];
      for (int64_t ch = b.base / 32; ch < (b.base + b.N + 31) / 32; ++ch) cb[ch] = k;
      bd[k] = make_int4(b.nx, b.ny, b.nz, 0);
    }
    CUDA_TRY(lv.chunk_box.alloc(cb.size()), "chunk boxes");
    CUDA_TRY(cudaMemcpy(lv.chunk_box.p, cb.data(), cb.size() * sizeof(int32_t), cudaMemcpyHostToDevice), "chunk boxes");
    CUDA_TRY(lv.boxdim.alloc(nbox), "box dims");
    CUDA_TRY(cudaMemcpy(lv.boxdim.p, bd.data(), bd.size() * sizeof(int4), cudaMemcpyHostToDevice), "box dims");
  }
  CUDA_TRY(lv.eq.alloc(kEqTables * Q27 * sizeof(double)), "eq tables");
  if (lattice == ELBM_D3Q27 && storage == ELBM_STORE_FP32_DEV)
    if (const int rc = build_ws_tables(c, lv)) return rc;
  lv.registered = true;
  return ELBM_OK;
}

}  // extern "C"

namespace {

int damp_buffers(elbm_ctx* c, Level& lv) {
  if (!lv.damp_list.p) CUDA_TRY(lv.damp_list.alloc(kDampCap), "repair list");
  if (!lv.damp_count.p) CUDA_TRY(lv.damp_count.alloc(1), "repair count");
  if (!lv.damp_vals.p) CUDA_TRY(lv.damp_vals.alloc(kDampCap), "repair values");
  return ELBM_OK;
}

}  // namespace

extern "C" {

int elbm_set_d3q27_params(elbm_ctx* c, int lvl, const elbm_d3q27_params* p) {
  Level* lv = get_level(c, lvl);
  if (!lv || !p) return fail(c, ELBM_E_ARG, "unknown level or null params");
  if (lv->lattice != ELBM_D3Q27) return fail(c, ELBM_E_ARG, "level %d is not a D3Q27 level", lvl);
  if (!(p->nu > 0.0) || p->max_newton < 1 || p->alpha_mode < 0 || p->alpha_mode > 2 || p->damp < 0 || p->damp > 1)
    return fail(c, ELBM_E_ARG, "bad D3Q27 parameters");
  if (p->damp) {
    CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
    if (const int rc = damp_buffers(c, *lv)) return rc;
  }
  if (p->alpha_mode == ELBM_ALPHA_LEARNED && (!lv->mlp_set || lv->storage != ELBM_STORE_FP32_DEV))
    return fail(c, ELBM_E_STATE, "learned alpha needs an FP32-storage level and weights (elbm_set_alpha_mlp)");
  lv->p27 = *p;
  lv->params_set = true;
  double tab[kEqTables][Q27];
  for (int j = 0; j < Q27; ++j) {
    tab[0][j] = p->fs_feq[j];
    for (int k = 0; k < 8; ++k) {
      tab[1 + k][j] = p->inl_feq[k][j];
      tab[9 + k][j] = p->outl_feq[k][j];
    }
  }
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  if (lv->storage == ELBM_STORE_FP64) {
    CUDA_TRY(cudaMemcpyAsync(lv->eq.p, tab, sizeof tab, cudaMemcpyHostToDevice, c->stream), "eq upload");
  } else {
    float tf[kEqTables][Q27];
    for (int t = 0; t < kEqTables; ++t)
      for (int j = 0; j < Q27; ++j) tf[t][j] = (float)(tab[t][j] - w27(j));
    CUDA_TRY(cudaMemcpyAsync(lv->eq.p, tf, sizeof tf, cudaMemcpyHostToDevice, c->stream), "eq upload");
  }
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  return ELBM_OK;
}

int elbm_set_links(elbm_ctx* c, int lvl, int box, const int32_t* state, int ngrow_state) {
  Level* lv = nullptr;
  Box* b = get_box(c, lvl, box, &lv);
  if (!b || !state || ngrow_state < 0) return fail(c, ELBM_E_ARG, "unknown level/box or null state");
  if (lv->lattice != ELBM_D3Q27) return fail(c, ELBM_E_UNSUPPORTED, "link tables of D3Q39 levels are not supported");
  if (!lv->params_set) return fail(c, ELBM_E_STATE, "set the level parameters before the links");
  const int g = ngrow_state;
  const int fx = b->nx + 2 * g, fy = b->ny + 2 * g, fz = b->nz + 2 * g;
  const int64_t fab_plane = (int64_t)fx * fy * fz;
  const int sstride[3] = {1, fx, fx * fy};
  std::vector<uint8_t> nt(b->N, NT_SKIP);
  std::vector<uint16_t> words;
  std::vector<double> qfr;
  std::vector<int32_t> xsv;
  std::vector<int64_t> bnodes, ghosts;
  int64_t fluid = 0;
  std::string why;
  for (int z = 0; z < b->nz; ++z)
    for (int y = 0; y < b->ny; ++y)
      for (int x = 0; x < b->nx; ++x) {
        const int64_t n = ((int64_t)z * b->ny + y) * b->nx + x;
        const int64_t s = ((int64_t)(z + g) * fy + (y + g)) * fx + (x + g);
        if (!node_is_fluid(state[s])) continue;
        ++fluid;
        const bool ghost = node_is_ghost(state[s]);
        if (ghost) ghosts.push_back(n);
        uint16_t w[Q27];
        double qv[Q27] = {0.0};
        int32_t xv[Q27];
        bool all_interior = true;
        w[0] = link_word(LK_PULL, 0, off_code(0, 0, 0));
        xv[0] = -1;
        for (int j = 1; j < Q27; ++j) {
          bool interior;
          const int rc = decode_link27(state, fab_plane, s, sstride, g, x, y, z, *b, *lv, j, ghost, w[j], qv[j],
                                       xv[j], interior, why);
          if (rc) return fail(c, rc, "node (%d,%d,%d) population %d: %s", x + b->lo[0], y + b->lo[1], z + b->lo[2], j,
                              why.c_str());
          all_interior &= interior;
        }
        if (all_interior) {
          nt[n] = NT_BULK;
        } else {
          nt[n] = NT_BOUNDARY;
          bnodes.push_back(n);
          words.insert(words.end(), w, w + Q27);
          qfr.insert(qfr.end(), qv, qv + Q27);
          xsv.insert(xsv.end(), xv, xv + Q27);
        }
      }
  b->h_ntype.swap(nt);
  b->h_bnodes.swap(bnodes);
  b->h_words.swap(words);
  b->h_qfrac.swap(qfr);
  b->h_xsrc.swap(xsv);
  b->h_ghost.swap(ghosts);
  b->fluid_nodes = fluid;
  b->boundary_nodes = (int64_t)b->h_bnodes.size();
  b->links_set = true;
  // once every box has its links, the level-wide tables go to the device
  lv->links_ready = false;
  lv->il_ready = false;
  for (auto& bp : lv->boxes)
    if (!bp->links_set) return ELBM_OK;
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  std::vector<uint8_t> lnt(lv->plane, NT_SKIP);
  std::vector<int32_t> lbi(lv->plane, -1);
  std::vector<uint16_t> lw;
  std::vector<double> lq;
  std::vector<int32_t> lx;
  std::vector<int32_t> lbn;
  int32_t rec = 0;
  for (auto& bp : lv->boxes) {
    const Box& bb = *bp;
    std::memcpy(&lnt[bb.base], bb.h_ntype.data(), bb.N);
    for (size_t k = 0; k < bb.h_bnodes.size(); ++k) {
      lbi[bb.base + bb.h_bnodes[k]] = rec++;
      lbn.push_back((int32_t)(bb.base + bb.h_bnodes[k]));
    }
    lw.insert(lw.end(), bb.h_words.begin(), bb.h_words.end());
    lq.insert(lq.end(), bb.h_qfrac.begin(), bb.h_qfrac.end());
    lx.insert(lx.end(), bb.h_xsrc.begin(), bb.h_xsrc.end());
  }
  CUDA_TRY(cudaMemcpy(lv->ntype.p, lnt.data(), lv->plane, cudaMemcpyHostToDevice), "node types");
  CUDA_TRY(lv->bidx.alloc(lv->plane), "boundary index");
  CUDA_TRY(cudaMemcpy(lv->bidx.p, lbi.data(), lv->plane * sizeof(int32_t), cudaMemcpyHostToDevice), "boundary index");
  CUDA_TRY(lv->words.alloc(std::max<size_t>(lw.size(), 1)), "link words");
  if (!lw.empty())
    CUDA_TRY(cudaMemcpy(lv->words.p, lw.data(), lw.size() * sizeof(uint16_t), cudaMemcpyHostToDevice), "words");
  CUDA_TRY(lv->bnode.alloc(std::max<size_t>(lbn.size(), 1)), "boundary nodes");
  if (!lbn.empty())
    CUDA_TRY(cudaMemcpy(lv->bnode.p, lbn.data(), lbn.size() * sizeof(int32_t), cudaMemcpyHostToDevice), "bnodes");
  lv->nrec = (int64_t)lbn.size();
  // resolved sources (one word per record and population, population-major): the element of the
  // source buffer for pulls within or across boxes and for kept values, 2^31 + the table entry for
  // equilibrium links, all ones for interpolated bounce-back (decoded from its word in the kernel)
  lv->rsrc.reset();
  if (lv->nrec > 0 && (int64_t)Q27 * lv->plane < (int64_t(1) << 31)) {
    std::vector<uint32_t> rs((size_t)Q27 * lv->nrec);
    int64_t r = 0;
    for (auto& bp : lv->boxes) {
      const Box& bb = *bp;
      for (size_t k = 0; k < bb.h_bnodes.size(); ++k, ++r) {
        const int64_t n = bb.base + bb.h_bnodes[k];
        for (int j = 0; j < Q27; ++j) {
          const uint16_t w = bb.h_words[k * Q27 + j];
          const int kind = lw_kind(w), pop = lw_pop(w), off = lw_off(w);
          uint32_t v = 0xffffffffu;
          if (kind == LK_PULL) {
            const int64_t sn = n + (off % 3 - 1) + (int64_t)((off / 3) % 3 - 1) * bb.nx +
                               (int64_t)(off / 9 - 1) * bb.nx * bb.ny;
            v = (uint32_t)((int64_t)pop * lv->plane + sn);
          } else if (kind == LK_XBOX) {
            v = (uint32_t)((int64_t)pop * lv->plane + bb.h_xsrc[k * Q27 + j]);
          } else if (kind == LK_KEEP) {
            v = (uint32_t)((int64_t)j * lv->plane + n);
          } else if (kind == LK_EQ) {
            v = 0x80000000u | (uint32_t)(pop * Q27 + j);
          }
          rs[(size_t)j * lv->nrec + r] = v;
        }
      }
    }
    CUDA_TRY(lv->rsrc.alloc(rs.size()), "resolved sources");
    CUDA_TRY(cudaMemcpy(lv->rsrc.p, rs.data(), rs.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "rsrc");
  }
  CUDA_TRY(lv->xsrc.alloc(std::max<size_t>(lx.size(), 1)), "cross-box sources");
  if (!lx.empty())
    CUDA_TRY(cudaMemcpy(lv->xsrc.p, lx.data(), lx.size() * sizeof(int32_t), cudaMemcpyHostToDevice), "cross-box");
  const size_t qes = elem_size(lv->storage);
  CUDA_TRY(lv->qfrac.alloc(std::max<size_t>(lq.size(), 1) * qes), "wall fractions");
  if (!lq.empty()) {
    std::vector<uint8_t> qbytes(lq.size() * qes);
    for (size_t k = 0; k < lq.size(); ++k) {
      if (qes == sizeof(double)) {
        std::memcpy(&qbytes[k * qes], &lq[k], sizeof(double));
      } else {
        const float v = (float)lq[k];
        std::memcpy(&qbytes[k * qes], &v, sizeof(float));
      }
    }
    CUDA_TRY(cudaMemcpy(lv->qfrac.p, qbytes.data(), qbytes.size(), cudaMemcpyHostToDevice), "fractions");
  }
  lv->links_ready = true;
  return ELBM_OK;
}

int elbm_upload_level(elbm_ctx* c, int lvl, int box, const double* fout) {
  Level* lv = nullptr;
  Box* b = get_box(c, lvl, box, &lv);
  if (!b || !fout) return fail(c, ELBM_E_ARG, "unknown level/box or null data");
  if (lv->lattice != ELBM_D3Q27) return fail(c, ELBM_E_ARG, "use elbm_upload_level39 for D3Q39 levels");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  const size_t es = elem_size(lv->storage);
  uint8_t* cur = lv->pop[lv->cur].p + b->base * es;
  uint8_t* other = lv->pop[lv->cur ^ 1].p + b->base * es;
  if (lv->storage == ELBM_STORE_FP64) {
    CUDA_TRY(fab_to_packed(fout, (double*)cur, *b, lv->ngrow, Q27, lv->plane, c->stream), "upload");
  } else {
    if (!b->staging.p) CUDA_TRY(b->staging.alloc((size_t)b->N * Q27), "staging");
    CUDA_TRY(fab_to_packed(fout, b->staging.p, *b, lv->ngrow, Q27, b->N, c->stream), "upload");
    dim3 grid((unsigned)((b->N + 255) / 256), Q27);
    to_dev32_kernel<<<grid, 256, 0, c->stream>>>(b->staging.p, (float*)cur, b->N, lv->plane);
    CUDA_TRY(cudaGetLastError(), "to_dev32");
  }
  // both buffers start identical so that nodes a step never writes stay defined
  CUDA_TRY(cudaMemcpy2DAsync(other, lv->plane * es, cur, lv->plane * es, b->N * es, Q27, cudaMemcpyDeviceToDevice,
                             c->stream),
           "copy");
  b->data_set = true;
  return ELBM_OK;
}

int elbm_download_level(elbm_ctx* c, int lvl, int box, double* fout) {
  Level* lv = nullptr;
  Box* b = get_box(c, lvl, box, &lv);
  if (!b || !fout) return fail(c, ELBM_E_ARG, "unknown level/box or null data");
  if (lv->lattice != ELBM_D3Q27) return fail(c, ELBM_E_ARG, "use elbm_download_level39 for D3Q39 levels");
  if (!b->data_set) return fail(c, ELBM_E_STATE, "no populations uploaded");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  const size_t es = elem_size(lv->storage);
  const uint8_t* cur = lv->pop[lv->cur].p + b->base * es;
  if (lv->storage == ELBM_STORE_FP64) {
    CUDA_TRY(packed_to_fab((const double*)cur, fout, *b, lv->ngrow, Q27, lv->plane, c->stream), "download");
  } else {
    if (!b->staging.p) CUDA_TRY(b->staging.alloc((size_t)b->N * Q27), "staging");
    dim3 grid((unsigned)((b->N + 255) / 256), Q27);
    from_dev32_kernel<<<grid, 256, 0, c->stream>>>((const float*)cur, b->staging.p, b->N, lv->plane);
    CUDA_TRY(cudaGetLastError(), "from_dev32");
    CUDA_TRY(packed_to_fab((const double*)b->staging.p, fout, *b, lv->ngrow, Q27, b->N, c->stream), "download");
  }
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  return ELBM_OK;
}

int elbm_download_alpha(elbm_ctx* c, int lvl, int box, double* alpha) {
  Level* lv = nullptr;
  Box* b = get_box(c, lvl, box, &lv);
  if (!b || !alpha) return fail(c, ELBM_E_ARG, "unknown level/box or null data");
  if (lv->lattice != ELBM_D3Q27) return fail(c, ELBM_E_ARG, "use elbm_download_level39 for D3Q39 levels");
  if (!lv->alpha.p) return fail(c, ELBM_E_STATE, "alpha recording is off (record_alpha = 0)");
  std::vector<float> tmp(b->N);
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  CUDA_TRY(cudaMemcpyAsync(tmp.data(), lv->alpha.p + b->base, b->N * sizeof(float), cudaMemcpyDeviceToHost,
                           c->stream),
           "alpha");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  for (int64_t n = 0; n < b->N; ++n) alpha[n] = tmp[n];
  return ELBM_OK;
}

// The arguments of one D3Q27 step over every box of a level.
// The offset variant serves one-box levels whose 27 planes stay below 2^31 elements.
bool off_variant_ok(const Level& lv) {
  if (lv.boxes.size() != 1) return false;
  const Box& b = *lv.boxes[0];
  return (int64_t)Q27 * lv.plane + (int64_t)b.nx * b.ny + b.nx + 1 < ((int64_t)1 << 31);
}

Step27Args level_args27(elbm_ctx* c, Level& lv) {
  const elbm_d3q27_params& p = lv.p27;
  Step27Args a{};
  a.src = lv.pop[lv.cur].p;
  a.dst = lv.pop[lv.cur ^ 1].p;
  a.plane = lv.plane;
  a.N = lv.plane;
  a.nbox = (int)lv.boxes.size();
  a.nx = lv.boxes[0]->nx;
  a.ny = lv.boxes[0]->ny;
  a.nz = lv.boxes[0]->nz;
  a.chunk_box = lv.chunk_box.p;
  a.boxdim = lv.boxdim.p;
  a.xsrc = lv.xsrc.p;
  a.work_counter = lv.work.p;
  a.ntype = lv.ntype.p;
  a.bidx = lv.bidx.p;
  a.words = lv.words.p;
  a.qfrac = lv.qfrac.p;
  a.eq = lv.eq.p;
  a.beta = 1.0 / (2.0 * p.nu / (1.0 / 3.0) + 1.0);
  a.tol_alpha = p.tol_alpha;
  a.tol_dH = p.tol_dH;
  a.max_newton = p.max_newton;
  a.alpha_mode = p.alpha_mode;
  a.check_dH = p.check_dH;
  a.stats = c->stats.p;
  a.variant = lv.variant;
  a.mlp = lv.mlp_set ? lv.mlp_w.p : nullptr;
  a.defer_list = lv.defer_list.p;
  a.defer_count = lv.defer_count.p;
  a.defer_cap = (long long)lv.defer_list.n;
  a.bnode = lv.bnode.p;
  a.nbnd = lv.nrec;
  a.rsrc = lv.rsrc.p;
  if (off_variant_ok(lv)) {
    const Box& b = *lv.boxes[0];
    a.pull_off_ok = 1;
    for (int j = 0; j < Q27; ++j)
      a.pull_off[j] = (int32_t)((int64_t)j * lv.plane - (cx27(j) + (int64_t)cy27(j) * b.nx + (int64_t)cz27(j) * b.nx * b.ny));
  }
  if (lv.ws_maps.p) {
    a.ws_maps = lv.ws_maps.p + (size_t)lv.cur * lv.boxes.size() * sizeof(CUtensorMap);
    a.ws_boxes = lv.ws_boxes.p;
    a.ws_ntiles = lv.ws_ntiles;
  }
  return a;
}

// One step of a D3Q27 level (no host synchronisation: capturable); with
// p27.damp, the step lists the negative populations it writes and the repair
// follows on the new state (collision then damp_it, loop.f95:133-139).
void enqueue_step27_args(elbm_ctx* c, Level& lv, Step27Args a) {
  const bool damp = lv.p27.damp && lv.damp_list.p;
  if (damp) {
    cudaMemsetAsync(lv.damp_count.p, 0, sizeof(unsigned long long), c->stream);
    a.neg_list = lv.damp_list.p;
    a.neg_count = lv.damp_count.p;
    a.neg_cap = kDampCap;
  }
  if (lv.storage == ELBM_STORE_FP64) launch_d3q27_fp64(a, c->stream);
  else launch_d3q27_fp32(a, c->stream);
  lv.cur ^= 1;
  if (damp) {
    Step27Args r = a;
    r.src = lv.pop[lv.cur].p;
    launch_damp27_fix(r, lv.storage == ELBM_STORE_FP32_DEV, lv.damp_vals.p, c->stream);
  }
}

int ready27(elbm_ctx* c, Level& lv) {
  for (auto& bp : lv.boxes)
    if (!bp->links_set || !bp->data_set) return fail(c, ELBM_E_STATE, "links or populations missing");
  if (!lv.links_ready) return fail(c, ELBM_E_STATE, "link tables not uploaded");
  return ELBM_OK;
}

int elbm_level_step(elbm_ctx* c, int lvl, int nsteps, elbm_stats* out) {
  Level* lv = get_level(c, lvl);
  if (!lv) return fail(c, ELBM_E_ARG, "unknown level %d", lvl);
  if (nsteps < 0) return fail(c, ELBM_E_ARG, "negative step count");
  if (!lv->params_set) return fail(c, ELBM_E_STATE, "level parameters not set");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  CUDA_TRY(cudaMemsetAsync(c->stats.p, 0, kStatBytes, c->stream), "stats reset");
  if (lv->lattice == ELBM_D3Q39) {
    const int rc = step39(c, *lv, nsteps);
    if (rc) return rc;
    return finish_stats(c, out);
  }
  const elbm_d3q27_params& p = lv->p27;
  if (const int rc = ready27(c, *lv)) return rc;
  if (p.record_alpha && !lv->alpha.p) {
    CUDA_TRY(lv->alpha.alloc(lv->plane), "alpha buffer");
    CUDA_TRY(cudaMemsetAsync(lv->alpha.p, 0, lv->plane * sizeof(float), c->stream), "memset");
  }
  CUDA_TRY(cudaEventRecord(c->ev0, c->stream), "event");
  for (int s = 0; s < nsteps; ++s) {
    Step27Args a = level_args27(c, *lv);
    a.alpha_out = (p.record_alpha && s == nsteps - 1) ? lv->alpha.p : nullptr;
    enqueue_step27_args(c, *lv, a);
    CUDA_TRY(cudaGetLastError(), "step kernel launch");
  }
  CUDA_TRY(cudaEventRecord(c->ev1, c->stream), "event");
  return finish_stats(c, out);
}

static_assert(kFp32Variants == ELBM_KERNEL_VARIANTS, "variant count of the C ABI");

int elbm_autotune(elbm_ctx* c, int lvl, int reps, int* chosen, double* ms_per_variant) {
  Level* lv = get_level(c, lvl);
  if (!lv || reps < 1) return fail(c, ELBM_E_ARG, "unknown level or reps < 1");
  if (lv->lattice != ELBM_D3Q27 || lv->storage != ELBM_STORE_FP32_DEV || !lv->params_set) {
    if (chosen) *chosen = 0;
    return ELBM_OK;  // a single kernel variant exists for the other paths
  }
  if (const int rc = ready27(c, *lv)) return rc;
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  float best = INFINITY;
  int best_v = 0;
  for (int v = 0; v < kFp32Variants; ++v) {
    if ((v == kVariantTma && !lv->ws_maps.p) || (v == kVariantOff && !off_variant_ok(*lv))) {
      if (ms_per_variant) ms_per_variant[v] = INFINITY;  // not available for this level
      continue;
    }
    CUDA_TRY(cudaEventRecord(c->ev0, c->stream), "event");
    for (int r = 0; r < reps + 1; ++r) {
      if (r == 1) CUDA_TRY(cudaEventRecord(c->ev0, c->stream), "event");
      // read the current state, write the other buffer, do not swap: the level does not advance
      Step27Args a = level_args27(c, *lv);
      a.check_dH = 0;
      a.variant = v;
      launch_d3q27_fp32(a, c->stream);
      CUDA_TRY(cudaGetLastError(), "autotune launch");
    }
    CUDA_TRY(cudaEventRecord(c->ev1, c->stream), "event");
    CUDA_TRY(cudaEventSynchronize(c->ev1), "sync");
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "elapsed");
    ms /= reps;
    if (ms_per_variant) ms_per_variant[v] = ms;
    if (ms < best) {
      best = ms;
      best_v = v;
    }
  }
  lv->variant = best_v;
  if (chosen) *chosen = best_v;
  CUDA_TRY(cudaMemsetAsync(c->stats.p, 0, kStatBytes, c->stream), "stats reset");
  return ELBM_OK;
}

int elbm_set_kernel_variant(elbm_ctx* c, int lvl, int variant) {
  if (!c) return ELBM_E_ARG;
  Level* lv = get_level(c, lvl);
  if (!lv || variant < 0 || variant >= kFp32Variants) return fail(c, ELBM_E_ARG, "unknown level or variant");
  if (variant == kVariantTma && !lv->ws_maps.p)
    return fail(c, ELBM_E_UNSUPPORTED, "the tensor-copy step variant does not serve this level: %s",
                lv->ws_why.empty() ? "not a D3Q27 level with FP32 deviation storage" : lv->ws_why.c_str());
  if (variant == kVariantOff && !off_variant_ok(*lv))
    return fail(c, ELBM_E_UNSUPPORTED, "the offset step variant serves one-box levels below 2^31 elements per 27 planes");
  lv->variant = variant;
  return ELBM_OK;
}

int elbm_set_alpha_mlp(elbm_ctx* c, int lvl, const float* weights) {
  Level* lv = get_level(c, lvl);
  if (!lv || !weights) return fail(c, ELBM_E_ARG, "unknown level or null weights");
  for (int k = 0; k < kMlpParams; ++k)
    if (!std::isfinite(weights[k])) return fail(c, ELBM_E_ARG, "non-finite weight %d", k);
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  if (!lv->mlp_w.p) CUDA_TRY(lv->mlp_w.alloc(kMlpParams), "weights");
  CUDA_TRY(cudaMemcpyAsync(lv->mlp_w.p, weights, kMlpParams * sizeof(float), cudaMemcpyHostToDevice, c->stream),
           "weights");
  upload_alpha_mlp(weights, c->stream);
  CUDA_TRY(cudaGetLastError(), "weights upload");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  lv->mlp_set = true;
  return ELBM_OK;
}

int elbm_alpha_harvest(elbm_ctx* c, int lvl, int nsteps, int stride, float* records, int64_t capacity,
                       int64_t* count) {
  Level* lv = get_level(c, lvl);
  if (!lv || nsteps < 1 || stride < 1 || !records || capacity < 1 || !count)
    return fail(c, ELBM_E_ARG, "bad harvest arguments");
  if (lv->lattice != ELBM_D3Q27 || lv->storage != ELBM_STORE_FP32_DEV || !lv->params_set ||
      lv->p27.alpha_mode != ELBM_ALPHA_NEWTON)
    return fail(c, ELBM_E_STATE, "harvesting needs an FP32-storage D3Q27 level with Newton alpha");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  DevBuf<float> buf;
  DevBuf<unsigned long long> cnt;
  CUDA_TRY(buf.alloc((size_t)capacity * kMlpRecord), "harvest buffer");
  CUDA_TRY(cnt.alloc(1), "harvest counter");
  CUDA_TRY(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), c->stream), "memset");
  CUDA_TRY(cudaMemsetAsync(c->stats.p, 0, kStatBytes, c->stream), "stats reset");
  if (const int rc = ready27(c, *lv)) return rc;
  for (int s = 0; s < nsteps; ++s) {
    Step27Args a = level_args27(c, *lv);
    a.check_dH = 0;
    a.harvest = buf.p;
    a.harvest_count = cnt.p;
    a.harvest_cap = capacity;
    a.harvest_stride = stride;
    launch_d3q27_fp32(a, c->stream);
    CUDA_TRY(cudaGetLastError(), "harvest launch");
    lv->cur ^= 1;
  }
  unsigned long long n = 0;
  CUDA_TRY(cudaMemcpyAsync(&n, cnt.p, sizeof n, cudaMemcpyDeviceToHost, c->stream), "count");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  const int64_t m = (int64_t)std::min<unsigned long long>(n, (unsigned long long)capacity);
  CUDA_TRY(cudaMemcpy(records, buf.p, (size_t)m * kMlpRecord * sizeof(float), cudaMemcpyDeviceToHost), "records");
  *count = m;
  return ELBM_OK;
}

int elbm_alpha_mlp_infer(elbm_ctx* c, const float* weights, const float* x, int64_t n, float* out,
                         uint32_t* status) {
  if (!c || !weights || !x || n < 1 || !out) return fail(c, ELBM_E_ARG, "bad inference arguments");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  DevBuf<float> w, xd, od;
  DevBuf<unsigned> st;
  CUDA_TRY(w.alloc(kMlpParams), "w");
  CUDA_TRY(xd.alloc((size_t)n * kMlpIn), "x");
  CUDA_TRY(od.alloc((size_t)n), "out");
  CUDA_TRY(st.alloc(1), "status");
  CUDA_TRY(cudaMemcpyAsync(w.p, weights, kMlpParams * sizeof(float), cudaMemcpyHostToDevice, c->stream), "w");
  CUDA_TRY(cudaMemcpyAsync(xd.p, x, (size_t)n * kMlpIn * sizeof(float), cudaMemcpyHostToDevice, c->stream), "x");
  CUDA_TRY(cudaMemsetAsync(st.p, 0, sizeof(unsigned), c->stream), "memset");
  mlp_tc_infer(w.p, xd.p, n, od.p, st.p, c->stream);
  CUDA_TRY(cudaGetLastError(), "inference launch");
  CUDA_TRY(cudaMemcpyAsync(out, od.p, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, c->stream), "out");
  unsigned sh = 0;
  CUDA_TRY(cudaMemcpyAsync(&sh, st.p, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream), "status");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  if (status) *status = sh;
  return ELBM_OK;
}

int elbm_alpha_mlp_grad(elbm_ctx* c, const float* weights, const float* records, int64_t n, float* grad,
                        double* loss) {
  if (!c || !weights || !records || n < 1 || !grad) return fail(c, ELBM_E_ARG, "bad gradient arguments");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  DevBuf<float> w, rec, scratch, g;
  DevBuf<double> l;
  CUDA_TRY(w.alloc(kMlpParams), "w");
  CUDA_TRY(rec.alloc((size_t)n * kMlpRecord), "records");
  CUDA_TRY(scratch.alloc((size_t)n * kMlpScratch), "scratch");
  CUDA_TRY(g.alloc(kMlpParams), "grad");
  CUDA_TRY(l.alloc(1), "loss");
  CUDA_TRY(cudaMemcpyAsync(w.p, weights, kMlpParams * sizeof(float), cudaMemcpyHostToDevice, c->stream), "w");
  CUDA_TRY(cudaMemcpyAsync(rec.p, records, (size_t)n * kMlpRecord * sizeof(float), cudaMemcpyHostToDevice, c->stream),
           "records");
  CUDA_TRY(cudaMemsetAsync(g.p, 0, kMlpParams * sizeof(float), c->stream), "memset");
  CUDA_TRY(cudaMemsetAsync(l.p, 0, sizeof(double), c->stream), "memset");
  mlp_batch_grad(w.p, rec.p, n, scratch.p, g.p, l.p, c->stream);
  CUDA_TRY(cudaGetLastError(), "grad launch");
  CUDA_TRY(cudaMemcpyAsync(grad, g.p, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, c->stream), "grad");
  double lh = 0.0;
  CUDA_TRY(cudaMemcpyAsync(&lh, l.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "loss");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  if (loss) *loss = lh / (double)n;
  return ELBM_OK;
}

int elbm_alpha_mlp_train(elbm_ctx* c, const float* records, int64_t n, int epochs, int batch, float lr, uint64_t seed,
                         float* weights, double* loss_per_epoch) {
  if (!c || !records || n < 1 || epochs < 1 || batch < 1 || !(lr > 0.f) || !weights)
    return fail(c, ELBM_E_ARG, "bad training arguments");
  if ((uint64_t)n > 0xffffffffull) return fail(c, ELBM_E_ARG, "at most 2^32 - 1 records");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  const int64_t B = std::min<int64_t>(batch, n);
  DevBuf<float> w, m, v, g, rec, bat, scratch;
  DevBuf<double> l;
  DevBuf<uint32_t> perm;
  CUDA_TRY(w.alloc(kMlpParams), "w");
  CUDA_TRY(m.alloc(kMlpParams), "m");
  CUDA_TRY(v.alloc(kMlpParams), "v");
  CUDA_TRY(g.alloc(kMlpParams), "g");
  CUDA_TRY(rec.alloc((size_t)n * kMlpRecord), "records");
  CUDA_TRY(bat.alloc((size_t)B * kMlpRecord), "batch");
  CUDA_TRY(scratch.alloc((size_t)B * kMlpScratch), "scratch");
  CUDA_TRY(l.alloc(1), "loss");
  CUDA_TRY(perm.alloc((size_t)n), "permutation");
  CUDA_TRY(cudaMemcpyAsync(w.p, weights, kMlpParams * sizeof(float), cudaMemcpyHostToDevice, c->stream), "w");
  CUDA_TRY(cudaMemcpyAsync(rec.p, records, (size_t)n * kMlpRecord * sizeof(float), cudaMemcpyHostToDevice, c->stream),
           "records");
  CUDA_TRY(cudaMemsetAsync(m.p, 0, kMlpParams * sizeof(float), c->stream), "m");
  CUDA_TRY(cudaMemsetAsync(v.p, 0, kMlpParams * sizeof(float), c->stream), "v");
  std::mt19937_64 rng(seed);
  std::vector<uint32_t> hp((size_t)n);
  int t = 0;
  for (int e = 0; e < epochs; ++e) {
    for (int64_t k = 0; k < n; ++k) hp[k] = (uint32_t)k;
    std::shuffle(hp.begin(), hp.end(), rng);
    CUDA_TRY(cudaMemcpyAsync(perm.p, hp.data(), (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream),
             "perm");
    CUDA_TRY(cudaMemsetAsync(l.p, 0, sizeof(double), c->stream), "memset");
    int64_t seen = 0;
    for (int64_t off = 0; off + B <= n; off += B) {
      mlp_gather_batch(rec.p, perm.p, off, B, bat.p, c->stream);
      CUDA_TRY(cudaMemsetAsync(g.p, 0, kMlpParams * sizeof(float), c->stream), "memset");
      mlp_batch_grad(w.p, bat.p, B, scratch.p, g.p, l.p, c->stream);
      mlp_adam(w.p, g.p, m.p, v.p, lr, ++t, c->stream);
      CUDA_TRY(cudaGetLastError(), "train launch");
      seen += B;
    }
    double lh = 0.0;
    CUDA_TRY(cudaMemcpyAsync(&lh, l.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "loss");
    CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
    if (loss_per_epoch) loss_per_epoch[e] = seen ? lh / (double)seen : 0.0;
  }
  CUDA_TRY(cudaMemcpy(weights, w.p, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost), "weights");
  return ELBM_OK;
}

namespace {

// (box, box-local index) of level coordinates, or box -1.
int box_of(const Level& lv, int gx, int gy, int gz, int64_t& local) {
  for (size_t k = 0; k < lv.boxes.size(); ++k) {
    const Box& b = *lv.boxes[k];
    if (gx < b.lo[0] || gx > b.hi[0] || gy < b.lo[1] || gy > b.hi[1] || gz < b.lo[2] || gz > b.hi[2]) continue;
    local = ((int64_t)(gz - b.lo[2]) * b.ny + (gy - b.lo[1])) * b.nx + (gx - b.lo[0]);
    return (int)k;
  }
  return -1;
}

// The maps of the coarse-fine transfer between two D3Q39 levels (boxes with link codes).
int interlevel_setup39(elbm_ctx* c, Level* fl, Level* cl) {
  if (fl->boxes.size() > 65535 || cl->boxes.size() > 65535) return fail(c, ELBM_E_ARG, "too many boxes");
  for (const auto* lv : {fl, cl})
    for (const auto& bp : lv->boxes)
      if (!bp->links39) return fail(c, ELBM_E_STATE, "set the links of both levels first (elbm_set_links39)");
  // explosion: each fine ghost node from the 1, 2, 4 or 8 coarse nodes around it (z-, y-, x-major)
  std::vector<int32_t> gidx, gsrc;
  std::vector<uint16_t> gbox;
  std::vector<uint8_t> gcnt;
  std::vector<int64_t> goff{0};
  for (const auto& bp : fl->boxes) {
    const Box& b = *bp;
    for (int64_t n : b.h_ghost) {
      const int X[3] = {b.lo[0] + (int)(n % b.nx), b.lo[1] + (int)((n / b.nx) % b.ny),
                        b.lo[2] + (int)(n / ((int64_t)b.nx * b.ny))};
      int lo[3], hi[3];
      for (int a = 0; a < 3; ++a) {
        lo[a] = (X[a] - ((X[a] % 2 + 2) % 2)) / 2;          // floor(X / 2)
        hi[a] = ((X[a] % 2 + 2) % 2) ? lo[a] + 1 : lo[a];  // odd: the next coarse node too
      }
      int32_t src[8];
      uint16_t sb[8];
      int k = 0;
      for (int cz = lo[2]; cz <= hi[2]; ++cz)
        for (int cy = lo[1]; cy <= hi[1]; ++cy)
          for (int cxx = lo[0]; cxx <= hi[0]; ++cxx) {
            int64_t li = 0;
            const int bi = box_of(*cl, cxx, cy, cz, li);
            if (bi < 0)
              return fail(c, ELBM_E_UNSUPPORTED, "fine ghost node (%d,%d,%d) lies outside the coarse level", X[0], X[1],
                          X[2]);
            src[k] = (int32_t)li;
            sb[k++] = (uint16_t)bi;
          }
      for (int m = k; m < 8; ++m) {
        src[m] = src[0];
        sb[m] = sb[0];
      }
      gidx.push_back((int32_t)n);
      gsrc.insert(gsrc.end(), src, src + 8);
      gbox.insert(gbox.end(), sb, sb + 8);
      gcnt.push_back((uint8_t)k);
    }
    goff.push_back((int64_t)gidx.size());
  }
  // coalescence: coarse nodes (not skipped) under a valid fine node (not skipped, not a ghost)
  std::vector<int32_t> ddst, dsrc;
  std::vector<uint16_t> dbox;
  std::vector<int64_t> doff{0};
  for (const auto& bp : cl->boxes) {
    const Box& b = *bp;
    for (int64_t n = 0; n < b.N; ++n) {
      if (b.h_ntype[n] == 0) continue;
      const int C[3] = {b.lo[0] + (int)(n % b.nx), b.lo[1] + (int)((n / b.nx) % b.ny),
                        b.lo[2] + (int)(n / ((int64_t)b.nx * b.ny))};
      int64_t li = 0;
      const int fb = box_of(*fl, 2 * C[0], 2 * C[1], 2 * C[2], li);
      if (fb < 0) continue;
      const Box& f = *fl->boxes[fb];
      if (f.h_ntype[li] == 0 || std::binary_search(f.h_ghost.begin(), f.h_ghost.end(), li)) continue;
      ddst.push_back((int32_t)n);
      dsrc.push_back((int32_t)li);
      dbox.push_back((uint16_t)fb);
    }
    doff.push_back((int64_t)ddst.size());
  }
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  auto put = [&](auto& buf, const auto& v) -> cudaError_t {
    cudaError_t e = buf.alloc(std::max<size_t>(v.size(), 1));
    if (e == cudaSuccess && !v.empty())
      e = cudaMemcpy(buf.p, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice);
    return e;
  };
  CUDA_TRY(put(fl->il39_ghost, gidx), "interlevel map");
  CUDA_TRY(put(fl->il39_gsrc, gsrc), "interlevel map");
  CUDA_TRY(put(fl->il39_gbox, gbox), "interlevel map");
  CUDA_TRY(put(fl->il39_gcnt, gcnt), "interlevel map");
  CUDA_TRY(put(fl->il39_ddst, ddst), "interlevel map");
  CUDA_TRY(put(fl->il39_dsrc, dsrc), "interlevel map");
  CUDA_TRY(put(fl->il39_dbox, dbox), "interlevel map");
  CUDA_TRY(fl->il39_cview.alloc(cl->boxes.size()), "box views");
  CUDA_TRY(fl->il39_fview.alloc(fl->boxes.size()), "box views");
  CUDA_TRY(fl->il39_counters.alloc(2), "interlevel counters");
  fl->il39_goff.swap(goff);
  fl->il39_doff.swap(doff);
  fl->il_nghost = (int64_t)gidx.size();
  fl->il_ndown = (int64_t)ddst.size();
  fl->il_ready = true;
  return ELBM_OK;
}

Box39View view39(Box& b) {
  return Box39View{(double*)b.buf[b.cur].p, (double*)b.gbuf[b.gcur].p, b.lm.p, b.w_vel.p, b.alpha64.p, b.macro.p,
                   b.plane};
}

// Upload the box views of a level (their ping-pong halves change every step).
cudaError_t views39(elbm_ctx* c, Level& lv, std::vector<Box39View>& host, DevBuf<Box39View>& dev) {
  host.clear();
  for (auto& bp : lv.boxes) host.push_back(view39(*bp));
  return cudaMemcpyAsync(dev.p, host.data(), host.size() * sizeof(Box39View), cudaMemcpyHostToDevice, c->stream);
}

}  // namespace

int elbm_interlevel_setup(elbm_ctx* c, int lvl) {
  Level* fl = get_level(c, lvl);
  Level* cl = lvl >= 1 ? get_level(c, lvl - 1) : nullptr;
  if (!fl || !cl) return fail(c, ELBM_E_ARG, "levels %d and %d must both be registered", lvl - 1, lvl);
  if (fl->lattice == ELBM_D3Q39 && cl->lattice == ELBM_D3Q39) {
    if (fl->storage != ELBM_STORE_FP64 || cl->storage != ELBM_STORE_FP64)
      return fail(c, ELBM_E_UNSUPPORTED, "D3Q39 coarse-fine transfer joins two levels of FP64 storage");
    return interlevel_setup39(c, fl, cl);
  }
  if (fl->lattice != ELBM_D3Q27 || cl->lattice != ELBM_D3Q27 || fl->storage != cl->storage)
    return fail(c, ELBM_E_UNSUPPORTED, "coarse-fine transfer joins two D3Q27 levels of the same storage or two D3Q39 levels");
  if (!fl->links_ready || !cl->links_ready) return fail(c, ELBM_E_STATE, "set the links of both levels first");
  // explosion map: each fine ghost node from the 1, 2, 4 or 8 coarse nodes around it
  std::vector<int32_t> gidx, gsrc;
  std::vector<uint8_t> gcnt;
  for (const auto& bp : fl->boxes) {
    const Box& b = *bp;
    for (int64_t n : b.h_ghost) {
      const int X[3] = {b.lo[0] + (int)(n % b.nx), b.lo[1] + (int)((n / b.nx) % b.ny), b.lo[2] + (int)(n / ((int64_t)b.nx * b.ny))};
      int lo[3], hi[3];
      for (int a = 0; a < 3; ++a) {
        lo[a] = (X[a] - ((X[a] % 2 + 2) % 2)) / 2;          // floor(X / 2)
        hi[a] = ((X[a] % 2 + 2) % 2) ? lo[a] + 1 : lo[a];  // odd: the next coarse node too
      }
      int32_t src[8];
      int k = 0;
      for (int cz = lo[2]; cz <= hi[2]; ++cz)
        for (int cy = lo[1]; cy <= hi[1]; ++cy)
          for (int cxx = lo[0]; cxx <= hi[0]; ++cxx) {
            const int64_t li = level_index(*cl, cxx, cy, cz);
            if (li < 0)
              return fail(c, ELBM_E_UNSUPPORTED, "fine ghost node (%d,%d,%d) lies outside the coarse level", X[0], X[1],
                          X[2]);
            src[k++] = (int32_t)li;
          }
      for (int m = k; m < 8; ++m) src[m] = src[0];
      gidx.push_back((int32_t)(b.base + n));
      gsrc.insert(gsrc.end(), src, src + 8);
      gcnt.push_back((uint8_t)k);
    }
  }
  // coalescence map: coarse fluid nodes under a valid fine fluid node
  std::vector<int32_t> ddst, dsrc;
  for (const auto& bp : cl->boxes) {
    const Box& b = *bp;
    for (int64_t n = 0; n < b.N; ++n) {
      if (b.h_ntype[n] == NT_SKIP) continue;
      const int C[3] = {b.lo[0] + (int)(n % b.nx), b.lo[1] + (int)((n / b.nx) % b.ny), b.lo[2] + (int)(n / ((int64_t)b.nx * b.ny))};
      const int64_t fi = level_index(*fl, 2 * C[0], 2 * C[1], 2 * C[2]);
      if (fi < 0) continue;
      // the fine node must be a valid fluid node (not a ghost, not solid)
      bool valid = false;
      for (const auto& fp : fl->boxes) {
        const Box& fb = *fp;
        if (fi < fb.base || fi >= fb.base + fb.N) continue;
        const int64_t ln = fi - fb.base;
        valid = fb.h_ntype[ln] != NT_SKIP && !std::binary_search(fb.h_ghost.begin(), fb.h_ghost.end(), ln);
      }
      if (!valid) continue;
      ddst.push_back((int32_t)(b.base + n));
      dsrc.push_back((int32_t)fi);
    }
  }
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  fl->il_nghost = (int64_t)gidx.size();
  fl->il_ndown = (int64_t)ddst.size();
  CUDA_TRY(fl->il_ghost.alloc(std::max<size_t>(gidx.size(), 1)), "interlevel map");
  CUDA_TRY(fl->il_src.alloc(std::max<size_t>(gsrc.size(), 1)), "interlevel map");
  CUDA_TRY(fl->il_cnt.alloc(std::max<size_t>(gcnt.size(), 1)), "interlevel map");
  CUDA_TRY(fl->il_down_dst.alloc(std::max<size_t>(ddst.size(), 1)), "interlevel map");
  CUDA_TRY(fl->il_down_src.alloc(std::max<size_t>(dsrc.size(), 1)), "interlevel map");
  CUDA_TRY(fl->il_repaired.alloc(1), "interlevel counter");
  if (!gidx.empty()) {
    CUDA_TRY(cudaMemcpy(fl->il_ghost.p, gidx.data(), gidx.size() * 4, cudaMemcpyHostToDevice), "map");
    CUDA_TRY(cudaMemcpy(fl->il_src.p, gsrc.data(), gsrc.size() * 4, cudaMemcpyHostToDevice), "map");
    CUDA_TRY(cudaMemcpy(fl->il_cnt.p, gcnt.data(), gcnt.size(), cudaMemcpyHostToDevice), "map");
  }
  if (!ddst.empty()) {
    CUDA_TRY(cudaMemcpy(fl->il_down_dst.p, ddst.data(), ddst.size() * 4, cudaMemcpyHostToDevice), "map");
    CUDA_TRY(cudaMemcpy(fl->il_down_src.p, dsrc.data(), dsrc.size() * 4, cudaMemcpyHostToDevice), "map");
  }
  fl->il_ready = true;
  return ELBM_OK;
}

int elbm_fill_fine_ghosts(elbm_ctx* c, int lvl, int64_t* repaired) {
  Level* fl = get_level(c, lvl);
  Level* cl = lvl >= 1 ? get_level(c, lvl - 1) : nullptr;
  if (!fl || !cl) return fail(c, ELBM_E_ARG, "unknown levels");
  if (!fl->il_ready) return fail(c, ELBM_E_STATE, "call elbm_interlevel_setup first");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  if (fl->lattice == ELBM_D3Q39) {
    for (const auto& bp : cl->boxes)
      if (!bp->data_set || !bp->macro_set)
        return fail(c, ELBM_E_STATE, "the coarse level needs its populations and fields (a step, "
                                     "elbm_upload_macro39 or elbm_init_level39)");
    for (const auto& bp : fl->boxes)
      if (!bp->data_set) return fail(c, ELBM_E_STATE, "populations missing on the fine level");
    CUDA_TRY(cudaMemsetAsync(fl->il39_counters.p, 0, 2 * sizeof(unsigned long long), c->stream), "memset");
    CUDA_TRY(views39(c, *cl, fl->il39_hcview, fl->il39_cview), "box views");
    const D3Q39Dev k = dev39(fl->p39, *fl);
    for (size_t bi = 0; bi < fl->boxes.size(); ++bi) {
      const int64_t o = fl->il39_goff[bi], n = fl->il39_goff[bi + 1] - o;
      launch_d3q39_explode(fl->il39_cview.p, view39(*fl->boxes[bi]), fl->il39_ghost.p + o, fl->il39_gsrc.p + 8 * o,
                           fl->il39_gbox.p + 8 * o, fl->il39_gcnt.p + o, n, k, fl->p39.timestep,
                           fl->il39_counters.p, c->stream);
      CUDA_TRY(cudaGetLastError(), "explosion launch");
    }
    if (repaired) {
      unsigned long long r[2] = {0, 0};
      CUDA_TRY(cudaMemcpyAsync(r, fl->il39_counters.p, sizeof r, cudaMemcpyDeviceToHost, c->stream), "counters");
      CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
      *repaired = (int64_t)r[0];
      if (r[1]) return fail(c, ELBM_E_NUMERIC, "%llu ghost-node multiplier solves hit the iteration cap", r[1]);
    }
    return ELBM_OK;
  }
  CUDA_TRY(cudaMemsetAsync(fl->il_repaired.p, 0, sizeof(unsigned long long), c->stream), "memset");
  launch_explode(fl->storage == ELBM_STORE_FP32_DEV, cl->pop[cl->cur].p, cl->plane, fl->pop[fl->cur].p, fl->plane,
                 fl->il_ghost.p, fl->il_src.p, fl->il_cnt.p, fl->il_nghost, fl->il_repaired.p, c->stream);
  CUDA_TRY(cudaGetLastError(), "explosion launch");
  if (repaired) {
    unsigned long long r = 0;
    CUDA_TRY(cudaMemcpyAsync(&r, fl->il_repaired.p, sizeof r, cudaMemcpyDeviceToHost, c->stream), "counter");
    CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
    *repaired = (int64_t)r;
  }
  return ELBM_OK;
}

int elbm_average_down(elbm_ctx* c, int lvl) {
  Level* fl = get_level(c, lvl);
  Level* cl = lvl >= 1 ? get_level(c, lvl - 1) : nullptr;
  if (!fl || !cl) return fail(c, ELBM_E_ARG, "unknown levels");
  if (!fl->il_ready) return fail(c, ELBM_E_STATE, "call elbm_interlevel_setup first");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  if (fl->lattice == ELBM_D3Q39) {
    CUDA_TRY(views39(c, *fl, fl->il39_hfview, fl->il39_fview), "box views");
    for (size_t bi = 0; bi < cl->boxes.size(); ++bi) {
      const int64_t o = fl->il39_doff[bi], n = fl->il39_doff[bi + 1] - o;
      launch_d3q39_average_down(fl->il39_fview.p, view39(*cl->boxes[bi]), fl->il39_ddst.p + o, fl->il39_dsrc.p + o,
                                fl->il39_dbox.p + o, n, c->stream);
      CUDA_TRY(cudaGetLastError(), "average-down launch");
    }
    return ELBM_OK;
  }
  launch_average_down(fl->storage == ELBM_STORE_FP32_DEV, fl->pop[fl->cur].p, fl->plane, cl->pop[cl->cur].p, cl->plane,
                      fl->il_down_dst.p, fl->il_down_src.p, fl->il_ndown, c->stream);
  CUDA_TRY(cudaGetLastError(), "average-down launch");
  return ELBM_OK;
}

}  // extern "C"

namespace {

// Launches of one step of a D3Q27 level (no host synchronisation: capturable).
void enqueue_step27(elbm_ctx* c, Level& lv) {
  Step27Args a = level_args27(c, lv);
  a.check_dH = 0;
  enqueue_step27_args(c, lv, a);
}

// One step of level l with the 2:1 sub-cycle of the finer levels below it, in
// the reference's order (loop.f95:94-147, valid_levels): the level steps, then
// its finer level takes two steps, refilled from this level before its first
// (odd) step completes and averaged down onto this level after its second.
void enqueue_cycle(elbm_ctx* c, int l, int nlev) {
  enqueue_step27(c, c->levels[l]);
  if (l + 1 >= nlev) return;
  Level& fl = c->levels[l + 1];
  Level& cl = c->levels[l];
  for (int k = 0; k < 2; ++k) {
    enqueue_cycle(c, l + 1, nlev);
    if (k == 0)
      launch_explode(fl.storage == ELBM_STORE_FP32_DEV, cl.pop[cl.cur].p, cl.plane, fl.pop[fl.cur].p, fl.plane,
                     fl.il_ghost.p, fl.il_src.p, fl.il_cnt.p, fl.il_nghost, fl.il_repaired.p, c->stream);
  }
  launch_average_down(fl.storage == ELBM_STORE_FP32_DEV, fl.pop[fl.cur].p, fl.plane, cl.pop[cl.cur].p, cl.plane,
                      fl.il_down_dst.p, fl.il_down_src.p, fl.il_ndown, c->stream);
}

}  // namespace

extern "C" {

int elbm_amr_run(elbm_ctx* c, int nlev, int ncycles, elbm_stats* out) {
  if (!c || nlev < 1 || nlev > 8 || ncycles < 0) return fail(c, ELBM_E_ARG, "bad AMR run arguments");
  uint64_t key = 1469598103934665603ull;
  for (int l = 0; l < nlev; ++l) {
    Level* lv = get_level(c, l);
    if (!lv || lv->lattice != ELBM_D3Q27 || !lv->params_set || lv->p27.check_dH || lv->p27.record_alpha)
      return fail(c, ELBM_E_STATE, "level %d: a registered D3Q27 level without check mode or alpha recording", l);
    if (const int rc = ready27(c, *lv)) return rc;
    if (l > 0 && !lv->il_ready) return fail(c, ELBM_E_STATE, "level %d: call elbm_interlevel_setup first", l);
    // the graph bakes in buffer addresses and parameters
    const uintptr_t parts[5] = {(uintptr_t)lv->pop[0].p, (uintptr_t)lv->il_ghost.p, (uintptr_t)lv->p27.alpha_mode,
                                (uintptr_t)lv->variant, (uintptr_t)lv->p27.damp};
    for (uintptr_t v : parts) key = (key ^ (uint64_t)v) * 1099511628211ull;
    uint64_t pb;
    std::memcpy(&pb, &lv->p27.nu, sizeof pb);
    key = (key ^ pb) * 1099511628211ull;
    key = (key ^ (uint64_t)lv->cur) * 1099511628211ull;
  }
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  if (!c->amr_exec || c->amr_nlev != nlev || c->amr_key != key) {
    if (c->amr_exec) {
      cudaGraphExecDestroy(c->amr_exec);
      c->amr_exec = nullptr;
    }
    // capture two coarse cycles: every level then takes an even number of steps, so
    // its ping-pong buffers are back where they started and the graph can be replayed
    std::vector<int> cur0(nlev);
    for (int l = 0; l < nlev; ++l) cur0[l] = c->levels[l].cur;
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    for (int k = 0; k < 2; ++k) enqueue_cycle(c, 0, nlev);
    const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    for (int l = 0; l < nlev; ++l) c->levels[l].cur = cur0[l];
    if (ce != cudaSuccess) return cuda_fail(c, ce, "end capture");
    const cudaError_t ie = cudaGraphInstantiate(&c->amr_exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      c->amr_exec = nullptr;
      return cuda_fail(c, ie, "graph instantiate");
    }
    c->amr_nlev = nlev;
    c->amr_key = key;
  }
  CUDA_TRY(cudaMemsetAsync(c->stats.p, 0, kStatBytes, c->stream), "stats reset");
  CUDA_TRY(cudaEventRecord(c->ev0, c->stream), "event");
  for (int r = 0; r < ncycles / 2; ++r) CUDA_TRY(cudaGraphLaunch(c->amr_exec, c->stream), "graph launch");
  if (ncycles % 2) enqueue_cycle(c, 0, nlev);  // an odd count: the last cycle by plain launches
  CUDA_TRY(cudaGetLastError(), "AMR cycle");
  CUDA_TRY(cudaEventRecord(c->ev1, c->stream), "event");
  return finish_stats(c, out);
}

int elbm_damp_level(elbm_ctx* c, int lvl, int64_t* repaired) {
  Level* lv = get_level(c, lvl);
  if (!lv) return fail(c, ELBM_E_ARG, "unknown level %d", lvl);
  if (lv->lattice != ELBM_D3Q27) return fail(c, ELBM_E_UNSUPPORTED, "D3Q39 levels repair inside elbm_level_step");
  if (!lv->params_set) return fail(c, ELBM_E_STATE, "level parameters not set");
  if (const int rc = ready27(c, *lv)) return rc;
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  if (const int rc = damp_buffers(c, *lv)) return rc;
  Step27Args a = level_args27(c, *lv);
  a.neg_list = lv->damp_list.p;
  a.neg_count = lv->damp_count.p;
  a.neg_cap = kDampCap;
  const bool fp32 = lv->storage == ELBM_STORE_FP32_DEV;
  CUDA_TRY(cudaMemsetAsync(lv->damp_count.p, 0, sizeof(unsigned long long), c->stream), "memset");
  launch_damp27_scan(a, fp32, c->stream);
  CUDA_TRY(cudaGetLastError(), "repair scan");
  unsigned long long cnt = 0;
  CUDA_TRY(cudaMemcpyAsync(&cnt, lv->damp_count.p, sizeof cnt, cudaMemcpyDeviceToHost, c->stream), "count");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  if ((long long)cnt > kDampCap)
    return fail(c, ELBM_E_STATE, "%llu negative populations: more than the %lld one call repairs", cnt, kDampCap);
  launch_damp27_fix(a, fp32, lv->damp_vals.p, c->stream);
  CUDA_TRY(cudaGetLastError(), "repair");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  if (repaired) *repaired = (int64_t)cnt;
  return ELBM_OK;
}

int elbm_sync(elbm_ctx* c) {
  if (!c) return ELBM_E_ARG;
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  return ELBM_OK;
}

int elbm_set_d3q39_params(elbm_ctx* c, int lvl, const elbm_d3q39_params* p) {
  Level* lv = get_level(c, lvl);
  if (!lv || !p) return fail(c, ELBM_E_ARG, "unknown level or null params");
  if (lv->lattice != ELBM_D3Q39) return fail(c, ELBM_E_ARG, "level %d is not a D3Q39 level", lvl);
  if (p->periodic < 0 || p->periodic > 7) return fail(c, ELBM_E_ARG, "periodic is a 3-bit mask");
  if (p->primary_flow_dir < 1 || p->primary_flow_dir > 6 || p->max_lm_iters < 1 || p->startup_timesteps < 1 ||
      !(p->t_ref > 0) || !(p->mu_ref > 0) || !(p->kappa_ref > 0) || !(p->dt > 0))
    return fail(c, ELBM_E_ARG, "bad D3Q39 parameters");
  lv->p39 = *p;
  Lattice39 L;
  build_lattice39(p->shifted, p->primary_flow_dir, L);
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  upload_lattice39(L, c->stream);
  CUDA_TRY(cudaGetLastError(), "lattice upload");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  lv->params_set = true;
  return ELBM_OK;
}

namespace {
int set_links39_sheet(elbm_ctx* c, int lvl, Level* lv, Box* b, const int32_t* state, int ngrow_state,
                      const elbm_d3q39_bc* bc);
}

int elbm_set_links39(elbm_ctx* c, int lvl, int box, const int32_t* state, int ngrow_state, const elbm_d3q39_bc* bc) {
  Level* lv = nullptr;
  const Sub39 u = get_sub39(c, lvl, box, &lv);
  Box* b = u.b;
  if (!b || !state || !bc || ngrow_state < 0)
    return fail(c, ELBM_E_ARG, "unknown level/box, not a D3Q39 level, or null state/bc");
  if (!lv->params_set) return fail(c, ELBM_E_STATE, "set the level parameters before the links");
  if (u.whole) return set_links39_sheet(c, lvl, lv, b, state, ngrow_state, bc);
  // one box of a multi-box level: keep its state until every box has one, then decode the sheet
  const int g = ngrow_state;
  const int fx = u.n[0] + 2 * g, fy = u.n[1] + 2 * g, fz = u.n[2] + 2 * g;
  lv->sub39_state[box].assign(state, state + (size_t)39 * fx * fy * fz);
  lv->sub39_ngrow[box] = g;
  lv->sub39_bc = *bc;
  for (const auto& v : lv->sub39_state)
    if (v.empty()) return ELBM_OK;
  // the sheet's state: every box's valid nodes; a node outside every box takes the first code a
  // box's ghost layers give it (a coarse-fine ghost, a face code), else it stays inactive (-1)
  const int64_t N = b->N;
  std::vector<int32_t> sheet((size_t)39 * N, 0);
  std::vector<uint8_t> set(N, 0);
  for (int64_t n = 0; n < N; ++n) sheet[n] = -1;
  for (int pass = 0; pass < 2; ++pass)
    for (size_t k = 0; k < lv->sub39.size(); ++k) {
      const auto& bx = lv->sub39[k];
      const int gk = lv->sub39_ngrow[k];
      const int nx = bx[3] - bx[0] + 1, ny = bx[4] - bx[1] + 1, nz = bx[5] - bx[2] + 1;
      const int ex = nx + 2 * gk, ey = ny + 2 * gk, ez = nz + 2 * gk;
      const int64_t fplane = (int64_t)ex * ey * ez;
      const int32_t* st = lv->sub39_state[k].data();
      for (int z = -gk; z < nz + gk; ++z)
        for (int y = -gk; y < ny + gk; ++y)
          for (int x = -gk; x < nx + gk; ++x) {
            const bool valid = x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz;
            if (valid != (pass == 0)) continue;
            const int X = bx[0] + x - b->lo[0], Y = bx[1] + y - b->lo[1], Z = bx[2] + z - b->lo[2];
            if (X < 0 || X >= b->nx || Y < 0 || Y >= b->ny || Z < 0 || Z >= b->nz) continue;
            const int64_t n = ((int64_t)Z * b->ny + Y) * b->nx + X;
            if (set[n]) continue;
            const int64_t src = ((int64_t)(z + gk) * ey + (y + gk)) * ex + (x + gk);
            for (int q = 0; q < 39; ++q) sheet[(size_t)q * N + n] = st[(size_t)q * fplane + src];
            set[n] = valid ? 1 : 2;
          }
    }
  return set_links39_sheet(c, lvl, lv, b, sheet.data(), 0, bc);
}

namespace {
// Decode the link codes of an internal box (a single-box level's box, or a multi-box level's sheet)
// and upload its tables.
int set_links39_sheet(elbm_ctx* c, int lvl, Level* lv, Box* b, const int32_t* state, int ngrow_state,
                      const elbm_d3q39_bc* bc) {
  Links39 L;
  std::string why;
  const int rc = decode_links39(state, ngrow_state, b->nx, b->ny, b->nz, lv->p39.periodic, lv->p39.shifted,
                                lv->p39.primary_flow_dir, bc->inlet_type, bc->outlet_type, L, why);
  if (rc) return fail(c, rc, "%s", why.c_str());
  double tf[kEqTables][39], tg[kEqTables][39];
  for (int j = 0; j < 39; ++j) {
    tf[0][j] = bc->fs_fieq[j];
    tg[0][j] = bc->fs_gieq[j];
    for (int k = 0; k < 8; ++k) {
      tf[1 + k][j] = bc->inl_fieq[k][j];
      tg[1 + k][j] = bc->inl_gieq[k][j];
      tf[9 + k][j] = bc->outl_fieq[k][j];
      tg[9 + k][j] = bc->outl_gieq[k][j];
    }
  }
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  if (!lv->eq39f.p) CUDA_TRY(lv->eq39f.alloc(kEqTables * 39), "equilibria");
  if (!lv->eq39g.p) CUDA_TRY(lv->eq39g.alloc(kEqTables * 39), "equilibria");
  CUDA_TRY(cudaMemcpy(lv->eq39f.p, tf, sizeof tf, cudaMemcpyHostToDevice), "equilibria");
  CUDA_TRY(cudaMemcpy(lv->eq39g.p, tg, sizeof tg, cudaMemcpyHostToDevice), "equilibria");
  CUDA_TRY(b->ntype39.alloc(b->N), "node types");
  CUDA_TRY(cudaMemcpy(b->ntype39.p, L.ntype.data(), b->N, cudaMemcpyHostToDevice), "node types");
  CUDA_TRY(b->bidx39.alloc(b->N), "records");
  CUDA_TRY(cudaMemcpy(b->bidx39.p, L.bidx.data(), b->N * sizeof(int32_t), cudaMemcpyHostToDevice), "records");
  b->nrec39 = (int64_t)L.bnodes.size();
  const size_t nr = std::max<size_t>(L.bnodes.size(), 1);
  CUDA_TRY(b->bnodes39.alloc(nr), "records");
  CUDA_TRY(b->words39.alloc(nr * 39), "link words");
  CUDA_TRY(b->fprev39.alloc(nr * 39), "post-streaming f");
  CUDA_TRY(b->gprev39.alloc(nr * 39), "post-streaming g");
  if (!L.bnodes.empty()) {
    CUDA_TRY(cudaMemcpy(b->bnodes39.p, L.bnodes.data(), L.bnodes.size() * sizeof(int32_t), cudaMemcpyHostToDevice),
             "records");
    CUDA_TRY(cudaMemcpy(b->words39.p, L.words.data(), L.words.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
             "link words");
  }
  CUDA_TRY(b->gmask39.alloc(b->N), "ggm links");
  CUDA_TRY(cudaMemcpy(b->gmask39.p, L.gmask.data(), b->N * sizeof(uint16_t), cudaMemcpyHostToDevice), "ggm links");
  CUDA_TRY(b->dmask39.alloc(b->N), "repair classes");
  CUDA_TRY(cudaMemcpy(b->dmask39.p, L.dmask.data(), b->N * sizeof(uint64_t), cudaMemcpyHostToDevice), "repair classes");
  b->nwall39 = (int64_t)L.walls.size();
  const size_t nw = std::max<size_t>(L.walls.size(), 1);
  CUDA_TRY(b->recwall39.alloc(nr), "wall map");
  CUDA_TRY(b->walls39.alloc(nw), "wall records");
  CUDA_TRY(b->wallf39.alloc(nw * 39), "wall values");
  CUDA_TRY(b->wallg39.alloc(nw * 39), "wall values");
  if (!L.recwall.empty())
    CUDA_TRY(cudaMemcpy(b->recwall39.p, L.recwall.data(), L.recwall.size() * sizeof(int32_t), cudaMemcpyHostToDevice),
             "wall map");
  if (!L.walls.empty())
    CUDA_TRY(cudaMemcpy(b->walls39.p, L.walls.data(), L.walls.size() * sizeof(Wall39Rec), cudaMemcpyHostToDevice),
             "wall records");
  lv->fs39[0] = bc->fs_u;
  lv->fs39[1] = bc->fs_v;
  lv->fs39[2] = bc->fs_w;
  lv->fs39[3] = bc->fs_temp;
  // node types and fine ghost nodes (state 1e7 .. 1.1e9) for the coarse-fine transfer
  b->h_ntype = L.ntype;
  b->h_ghost.clear();
  {
    const int g = ngrow_state;
    const int fx = b->nx + 2 * g, fy = b->ny + 2 * g;
    for (int z = 0; z < b->nz; ++z)
      for (int y = 0; y < b->ny; ++y)
        for (int x = 0; x < b->nx; ++x) {
          const int64_t n = ((int64_t)z * b->ny + y) * b->nx + x;
          if (L.ntype[n] != 0 && node_is_ghost(state[((int64_t)(z + g) * fy + (y + g)) * fx + (x + g)]))
            b->h_ghost.push_back(n);
        }
  }
  lv->il_ready = false;
  if (lvl + 1 < (int)c->levels.size()) c->levels[lvl + 1].il_ready = false;
  b->links39 = true;
  // until a step has run, a slot that no rule writes holds the node's uploaded fout
  if (b->data_set) launch_stale39_init(*b, c->stream);
  CUDA_TRY(cudaGetLastError(), "stale init");
  return ELBM_OK;
}
}  // namespace

int elbm_upload_level39(elbm_ctx* c, int lvl, int box, const double* fout, const double* gout, const double* lm,
                        const double* w_vel) {
  Level* lv = nullptr;
  const Sub39 u = get_sub39(c, lvl, box, &lv);
  Box* b = u.b;
  if (!b || !fout || !gout || !lm || !w_vel)
    return fail(c, ELBM_E_ARG, "unknown level/box, not a D3Q39 level, or null data");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  if (!u.whole) {
    // one box of a multi-box level: its part of the sheet; the sheet is complete (both buffers,
    // the FP32 conversion, the slots that keep last step's values) once every box has arrived
    const int g = lv->ngrow;
    const bool f32 = lv->storage == ELBM_STORE_FP32_DEV;
    if (b->data_set) {
      // the level was complete: a new upload starts over, and the level steps again once every
      // box has arrived (a box not given again would keep a state of another time)
      std::fill(lv->sub39_have_pops.begin(), lv->sub39_have_pops.end(), 0);
      b->data_set = false;
    }
    if (f32) {
      if (!b->stage39.p) {
        CUDA_TRY(b->stage39.alloc((size_t)b->plane * 78), "FP64 staging");
        CUDA_TRY(cudaMemsetAsync(b->stage39.p, 0, b->stage39.n * sizeof(double), c->stream), "staging");
      }
      CUDA_TRY(sub39_copy(u, const_cast<double*>(fout), b->stage39.p, g, 39, b->plane, true, c->stream), "upload f");
      CUDA_TRY(sub39_copy(u, const_cast<double*>(gout), b->stage39.p + b->plane * 39, g, 39, b->plane, true,
                          c->stream), "upload g");
    } else {
      for (int s2 = 0; s2 < 2; ++s2) {
        CUDA_TRY(sub39_copy(u, const_cast<double*>(fout), (double*)b->buf[s2].p, g, 39, b->plane, true, c->stream),
                 "upload f");
        CUDA_TRY(sub39_copy(u, const_cast<double*>(gout), (double*)b->gbuf[s2].p, g, 39, b->plane, true, c->stream),
                 "upload g");
      }
    }
    CUDA_TRY(sub39_copy(u, const_cast<double*>(lm), b->lm.p, g, 13, b->plane, true, c->stream), "upload lm");
    CUDA_TRY(sub39_copy(u, const_cast<double*>(w_vel), b->w_vel.p, g, 1, b->plane, true, c->stream), "upload w");
    lv->sub39_have_pops[box] = 1;
    b->macro_set = false;
    std::fill(lv->sub39_have_macro.begin(), lv->sub39_have_macro.end(), 0);
    if (std::all_of(lv->sub39_have_pops.begin(), lv->sub39_have_pops.end(), [](uint8_t v) { return v; })) {
      if (f32) {
        CUDA_TRY(stage39_to_fp32(*b, c->stream), "FP32 conversion");
        CUDA_TRY(cudaMemcpyAsync(b->buf[1].p, b->buf[0].p, b->buf[0].n, cudaMemcpyDeviceToDevice, c->stream),
                 "copy f");
        CUDA_TRY(cudaMemcpyAsync(b->gbuf[1].p, b->gbuf[0].p, b->gbuf[0].n, cudaMemcpyDeviceToDevice, c->stream),
                 "copy g");
        b->cur = b->gcur = 0;
      }
      CUDA_TRY(cudaMemsetAsync(b->alpha64.p, 0, b->alpha64.n * sizeof(double), c->stream), "alpha");
      if (b->links39) launch_stale39_init(*b, c->stream);
      CUDA_TRY(cudaGetLastError(), "stale init");
      b->data_set = true;
    }
    CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
    return ELBM_OK;
  }
  if (lv->storage == ELBM_STORE_FP32_DEV) {
    if (!b->stage39.p) CUDA_TRY(b->stage39.alloc((size_t)b->plane * 78), "FP64 staging");
    CUDA_TRY(fab_to_packed(fout, b->stage39.p, *b, lv->ngrow, 39, b->plane, c->stream), "upload f");
    CUDA_TRY(fab_to_packed(gout, b->stage39.p + b->plane * 39, *b, lv->ngrow, 39, b->plane, c->stream), "upload g");
    CUDA_TRY(stage39_to_fp32(*b, c->stream), "FP32 conversion");
  } else {
    CUDA_TRY(fab_to_packed(fout, (double*)b->buf[0].p, *b, lv->ngrow, 39, b->plane, c->stream), "upload f");
    CUDA_TRY(fab_to_packed(gout, (double*)b->gbuf[0].p, *b, lv->ngrow, 39, b->plane, c->stream), "upload g");
  }
  CUDA_TRY(fab_to_packed(lm, b->lm.p, *b, lv->ngrow, 13, b->plane, c->stream), "upload lm");
  CUDA_TRY(fab_to_packed(w_vel, b->w_vel.p, *b, lv->ngrow, 1, b->plane, c->stream), "upload w");
  // both buffers start identical so that the nodes a step skips (solid) stay defined in either
  CUDA_TRY(cudaMemcpyAsync(b->buf[1].p, b->buf[0].p, b->buf[0].n, cudaMemcpyDeviceToDevice, c->stream), "copy f");
  CUDA_TRY(cudaMemcpyAsync(b->gbuf[1].p, b->gbuf[0].p, b->gbuf[0].n, cudaMemcpyDeviceToDevice, c->stream), "copy g");
  CUDA_TRY(cudaMemsetAsync(b->alpha64.p, 0, b->alpha64.n * sizeof(double), c->stream), "alpha");
  if (b->links39) launch_stale39_init(*b, c->stream);
  CUDA_TRY(cudaMemsetAsync(b->macro.p, 0, b->macro.n * sizeof(double), c->stream), "macro");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  b->cur = 0;
  b->gcur = 0;
  b->data_set = true;
  b->macro_set = false;
  return ELBM_OK;
}

// ---- level checkpoints: the dynamic state of a level in one file ----
// Layout: a 64-byte header (magic "ELBMCKP1", lattice, storage, box count,
// D3Q39 timestep, plane) and one record per array: an 8-byte byte count and
// the bytes, in a fixed order per lattice.  The link tables are not part of
// it: they come from the state FABs (elbm_set_links / elbm_set_links39).
namespace {
struct CkpHeader {
  char magic[8];
  int32_t lattice, storage, nbox, timestep;
  int64_t plane, nodes;
  int64_t reserved[3];
};
static_assert(sizeof(CkpHeader) == 64, "checkpoint header");

int ckp_arrays(Level& lv, std::vector<std::pair<void*, size_t>>& out) {
  out.clear();
  if (lv.lattice == ELBM_D3Q27) {
    out.push_back({lv.pop[lv.cur].p, lv.pop[lv.cur].n});
    return ELBM_OK;
  }
  for (auto& bp : lv.boxes) {
    Box& b = *bp;
    out.push_back({b.buf[b.cur].p, b.buf[b.cur].n});
    out.push_back({b.gbuf[b.gcur].p, b.gbuf[b.gcur].n});
    if (lv.storage == ELBM_STORE_FP32_DEV) out.push_back({b.ref39.p, 78 * sizeof(double)});
    out.push_back({b.lm.p, b.lm.n * sizeof(double)});
    out.push_back({b.w_vel.p, b.w_vel.n * sizeof(double)});
    out.push_back({b.macro.p, b.macro.n * sizeof(double)});
    if (b.links39) {
      out.push_back({b.fprev39.p, (size_t)b.nrec39 * 39 * sizeof(double)});
      out.push_back({b.gprev39.p, (size_t)b.nrec39 * 39 * sizeof(double)});
    }
  }
  return ELBM_OK;
}
}  // namespace

int elbm_checkpoint_write(elbm_ctx* c, int lvl, const char* path) {
  Level* lv = get_level(c, lvl);
  if (!lv || !path) return fail(c, ELBM_E_ARG, "unknown level or null path");
  for (auto& bp : lv->boxes)
    if (!bp->data_set) return fail(c, ELBM_E_STATE, "no state to write");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  std::vector<std::pair<void*, size_t>> arr;
  ckp_arrays(*lv, arr);
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return fail(c, ELBM_E_ARG, "cannot open %s for writing", path);
  CkpHeader h{};
  std::memcpy(h.magic, "ELBMCKP1", 8);
  h.lattice = lv->lattice;
  h.storage = lv->storage;
  h.nbox = (int32_t)lv->boxes.size();
  h.timestep = lv->lattice == ELBM_D3Q39 ? lv->p39.timestep : 0;
  h.plane = lv->plane;
  h.nodes = 0;
  for (auto& bp : lv->boxes) h.nodes += bp->N;
  bool ok = std::fwrite(&h, sizeof h, 1, fp) == 1;
  std::vector<char> host;
  for (auto& a : arr) {
    const int64_t n = (int64_t)a.second;
    host.resize(a.second);
    if (cudaMemcpy(host.data(), a.first, a.second, cudaMemcpyDeviceToHost) != cudaSuccess) ok = false;
    ok = ok && std::fwrite(&n, sizeof n, 1, fp) == 1 && std::fwrite(host.data(), 1, a.second, fp) == a.second;
  }
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) return fail(c, ELBM_E_ARG, "writing %s failed", path);
  return ELBM_OK;
}

int elbm_checkpoint_read(elbm_ctx* c, int lvl, const char* path) {
  Level* lv = get_level(c, lvl);
  if (!lv || !path) return fail(c, ELBM_E_ARG, "unknown level or null path");
  if (!lv->params_set) return fail(c, ELBM_E_STATE, "set the level parameters before reading a checkpoint");
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return fail(c, ELBM_E_ARG, "cannot open %s", path);
  CkpHeader h{};
  int64_t nodes = 0;
  for (auto& bp : lv->boxes) nodes += bp->N;
  if (std::fread(&h, sizeof h, 1, fp) != 1 || std::memcmp(h.magic, "ELBMCKP1", 8) != 0 || h.lattice != lv->lattice ||
      h.storage != lv->storage || h.nbox != (int32_t)lv->boxes.size() || h.plane != lv->plane || h.nodes != nodes) {
    std::fclose(fp);
    return fail(c, ELBM_E_ARG, "%s is not a checkpoint of this level's layout", path);
  }
  if (lv->lattice == ELBM_D3Q39)
    for (auto& bp : lv->boxes) {
      bp->cur = 0;
      bp->gcur = 0;
    }
  else
    lv->cur = 0;
  std::vector<std::pair<void*, size_t>> arr;
  ckp_arrays(*lv, arr);
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  std::vector<char> host;
  for (auto& a : arr) {
    int64_t n = 0;
    if (std::fread(&n, sizeof n, 1, fp) != 1 || n != (int64_t)a.second) {
      std::fclose(fp);
      return fail(c, ELBM_E_ARG, "%s: array sizes differ from this level's (were the links set the same way?)", path);
    }
    host.resize(a.second);
    if (std::fread(host.data(), 1, a.second, fp) != a.second) {
      std::fclose(fp);
      return fail(c, ELBM_E_ARG, "%s is truncated", path);
    }
    CUDA_TRY(cudaMemcpy(a.first, host.data(), a.second, cudaMemcpyHostToDevice), "checkpoint upload");
  }
  std::fclose(fp);
  // the second population buffer takes the same state, as after an upload: a step never
  // writes the nodes it skips (solid nodes), and reading them from either buffer must agree
  if (lv->lattice == ELBM_D3Q27) {
    CUDA_TRY(cudaMemcpy(lv->pop[1].p, lv->pop[0].p, lv->pop[0].n, cudaMemcpyDeviceToDevice), "checkpoint copy");
  } else {
    for (auto& bp : lv->boxes) {
      CUDA_TRY(cudaMemcpy(bp->buf[1].p, bp->buf[0].p, bp->buf[0].n, cudaMemcpyDeviceToDevice), "checkpoint copy f");
      CUDA_TRY(cudaMemcpy(bp->gbuf[1].p, bp->gbuf[0].p, bp->gbuf[0].n, cudaMemcpyDeviceToDevice), "checkpoint copy g");
    }
  }
  if (lv->lattice == ELBM_D3Q39) lv->p39.timestep = h.timestep;
  for (auto& bp : lv->boxes) {
    bp->data_set = true;
    bp->macro_set = true;
    bp->ref39_set = lv->lattice == ELBM_D3Q39 && lv->storage == ELBM_STORE_FP32_DEV;
  }
  return ELBM_OK;
}

// ---- output from the device buffers (output/plot3d_output.f95, output/mic_setup_stuff/mic_write.f95) ----
namespace {
// one Fortran unformatted sequential record: 4-byte length, payload, 4-byte length
bool f_record(FILE* fp, const std::vector<std::pair<const void*, size_t>>& parts) {
  size_t n = 0;
  for (auto& q : parts) n += q.second;
  if (n > 0x7fffffffu) return false;
  const int32_t m = (int32_t)n;
  bool ok = std::fwrite(&m, 4, 1, fp) == 1;
  for (auto& q : parts) ok = ok && (q.second == 0 || std::fwrite(q.first, 1, q.second, fp) == q.second);
  return ok && std::fwrite(&m, 4, 1, fp) == 1;
}
}  // namespace

int elbm_mark_triangles_gpu(elbm_ctx* c, int nx, int ny, int nz, const double* origin, double dx, int ntri,
                            const double* tri, int32_t* state) {
  if (!c || nx < 1 || ny < 1 || nz < 1 || !origin || !(dx > 0.0) || ntri < 1 || !tri || !state)
    return fail(c, ELBM_E_ARG, "bad arguments");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  std::string why;
  const int rc = mark_triangles_device(nx, ny, nz, origin, dx, ntri, tri, state, c->stream, why);
  if (rc) return fail(c, rc, "%s", why.c_str());
  return ELBM_OK;
}

int elbm_mark_triangles39_gpu(elbm_ctx* c, int nx, int ny, int nz, const double* origin, double dx, int ntri,
                              const double* tri, int shifted, int primary_flow_dir, int periodic, int32_t* state) {
  if (!c || nx < 1 || ny < 1 || nz < 1 || !origin || !(dx > 0.0) || ntri < 1 || !tri || !state || periodic < 0 ||
      periodic > 7 || primary_flow_dir < 1 || primary_flow_dir > 6)
    return fail(c, ELBM_E_ARG, "bad arguments");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  std::string why;
  const int rc = mark_triangles39_device(nx, ny, nz, origin, dx, ntri, tri, shifted, primary_flow_dir, periodic,
                                         state, c->stream, why);
  if (rc) return fail(c, rc, "%s", why.c_str());
  return ELBM_OK;
}

int elbm_write_plot3d(elbm_ctx* c, int lvl, const char* grid_path, const char* data_path, const double* origin,
                      double dx, const elbm_plot3d_header* hdr) {
  Level* lv = get_level(c, lvl);
  if (!lv || !grid_path || !data_path || !origin || !hdr || !(dx > 0)) return fail(c, ELBM_E_ARG, "bad arguments");
  if (lv->lattice != ELBM_D3Q39) return fail(c, ELBM_E_UNSUPPORTED, "Plot3D output writes the D3Q39 fields");
  for (auto& bp : lv->boxes)
    if (!bp->data_set) return fail(c, ELBM_E_STATE, "no state");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  FILE* g = std::fopen(grid_path, "wb");
  FILE* d = std::fopen(data_path, "wb");
  if (!g || !d) {
    if (g) std::fclose(g);
    if (d) std::fclose(d);
    return fail(c, ELBM_E_ARG, "cannot open the output files");
  }
  const int32_t nb = (int32_t)lv->boxes.size();
  std::vector<int32_t> dims, ddims;
  for (auto& bp : lv->boxes) {
    dims.insert(dims.end(), {bp->nx, bp->ny, bp->nz});
  }
  ddims = dims;
  ddims.push_back(6);  // rho, u, v, w, T, alpha
  ddims.push_back(0);
  bool ok = f_record(g, {{&nb, 4}}) && f_record(d, {{&nb, 4}}) && f_record(g, {{dims.data(), dims.size() * 4}}) &&
            f_record(d, {{ddims.data(), ddims.size() * 4}});
  const double zero = 0.0;
  const int32_t izero = 0, ts = lv->p39.timestep;
  std::vector<double> macro, alpha;
  std::vector<uint16_t> gm;
  std::vector<float> xyz;
  std::vector<int32_t> blank;
  for (auto& bp : lv->boxes) {
    Box& b = *bp;
    const size_t N = (size_t)b.N;
    macro.resize(5 * N);
    alpha.resize(N);
    for (int k = 0; k < 5; ++k)
      CUDA_TRY(cudaMemcpy(macro.data() + k * N, b.macro.p + (size_t)k * b.plane, N * sizeof(double),
                          cudaMemcpyDeviceToHost), "fields");
    CUDA_TRY(cudaMemcpy(alpha.data(), b.alpha64.p, N * sizeof(double), cudaMemcpyDeviceToHost), "alpha");
    gm.assign(N, (uint16_t)(1u << 12));
    if (b.gmask39.p) CUDA_TRY(cudaMemcpy(gm.data(), b.gmask39.p, N * 2, cudaMemcpyDeviceToHost), "node types");
    xyz.resize(3 * N);
    blank.resize(N);
    const double start[3] = {origin[0] + b.lo[0] * dx, origin[1] + b.lo[1] * dx, origin[2] + b.lo[2] * dx};
    for (int z = 0; z < b.nz; ++z)
      for (int y = 0; y < b.ny; ++y)
        for (int x = 0; x < b.nx; ++x) {
          const size_t n = ((size_t)z * b.ny + y) * b.nx + x;
          xyz[n] = (float)(start[0] + dx * x);
          xyz[N + n] = (float)(start[1] + dx * y);
          xyz[2 * N + n] = (float)(start[2] + dx * z);
          blank[n] = ((gm[n] >> 12) & 1u) ? 1 : ((gm[n] >> 13) & 1u) ? -1 : 0;
        }
    ok = ok && f_record(g, {{xyz.data(), 3 * N * 4}, {blank.data(), N * 4}});
    ok = ok && f_record(d, {{&hdr->mach, 8}, {&zero, 8}, {&hdr->reynolds, 8}, {&hdr->time, 8}, {&hdr->gama, 8},
                            {&zero, 8}, {&hdr->t_ref, 8}, {&izero, 4}, {&hdr->stag_temperature, 8},
                            {&hdr->const_vol, 8}, {&hdr->const_press, 8}, {&hdr->non_dim_R, 8},
                            {&hdr->non_dim_R, 8}, {&hdr->mach, 8}, {&hdr->time, 8}, {&ts, 4}});
    ok = ok && f_record(d, {{macro.data(), 5 * N * 8}, {alpha.data(), N * 8}});
  }
  ok = (std::fclose(g) == 0) && ok;
  ok = (std::fclose(d) == 0) && ok;
  if (!ok) return fail(c, ELBM_E_ARG, "writing the Plot3D files failed");
  return ELBM_OK;
}

int elbm_mic_sample(elbm_ctx* c, int lvl, int box, int nmic, const int32_t* nodes, const double* weights,
                    double* out) {
  Level* lv = get_level(c, lvl);
  if (lv && lv->lattice != ELBM_D3Q39) return fail(c, ELBM_E_UNSUPPORTED, "microphones read the D3Q39 fields");
  const Sub39 u = get_sub39(c, lvl, box, &lv);
  Box* b = u.b;
  if (!b || nmic < 0 || (nmic > 0 && (!nodes || !weights || !out))) return fail(c, ELBM_E_ARG, "bad arguments");
  const int64_t nbox = (int64_t)u.n[0] * u.n[1] * u.n[2];
  std::vector<int32_t> sn((size_t)8 * nmic);
  for (int k = 0; k < 8 * nmic; ++k) {
    if (nodes[k] < 0 || nodes[k] >= nbox) return fail(c, ELBM_E_ARG, "microphone node outside the box");
    // the node in the internal box (the sheet of a multi-box level)
    const int x = nodes[k] % u.n[0], y = (nodes[k] / u.n[0]) % u.n[1], z = nodes[k] / (u.n[0] * u.n[1]);
    sn[k] = (int32_t)(((int64_t)(z + u.off[2]) * b->ny + (y + u.off[1])) * b->nx + (x + u.off[0]));
  }
  if (nmic == 0) return ELBM_OK;
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  DevBuf<int32_t> dn;
  DevBuf<double> dw, dout;
  CUDA_TRY(dn.alloc((size_t)8 * nmic), "mic nodes");
  CUDA_TRY(dw.alloc((size_t)8 * nmic), "mic weights");
  CUDA_TRY(dout.alloc((size_t)6 * nmic), "mic values");
  CUDA_TRY(cudaMemcpyAsync(dn.p, sn.data(), (size_t)8 * nmic * 4, cudaMemcpyHostToDevice, c->stream), "mic nodes");
  CUDA_TRY(cudaMemcpyAsync(dw.p, weights, (size_t)8 * nmic * 8, cudaMemcpyHostToDevice, c->stream), "mic weights");
  launch_mic_sample(b->macro.p, b->plane, nmic, dn.p, dw.p, dout.p, c->stream);
  CUDA_TRY(cudaGetLastError(), "mic launch");
  CUDA_TRY(cudaMemcpyAsync(out, dout.p, (size_t)6 * nmic * 8, cudaMemcpyDeviceToHost, c->stream), "mic values");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  return ELBM_OK;
}

int elbm_ggm_tags(elbm_ctx* c, int lvl, int box, int variable, int scheme, double limit, uint8_t* tags, double* ggm,
                  int64_t* ntagged) {
  return elbm_ggm_tags_pgs(c, lvl, box, variable, scheme, limit, 0.0, -1, tags, ggm, ntagged);
}

int elbm_ggm_tags_pgs(elbm_ctx* c, int lvl, int box, int variable, int scheme, double limit, double pgs_sensitivity,
                      int pgs_reach, uint8_t* tags, double* ggm, int64_t* ntagged) {
  Level* lv = get_level(c, lvl);
  if (lv && lv->lattice != ELBM_D3Q39) return fail(c, ELBM_E_UNSUPPORTED, "GGM tagging reads the D3Q39 fields");
  const Sub39 u = get_sub39(c, lvl, box, &lv);
  Box* b = u.b;
  if (!b || !tags) return fail(c, ELBM_E_ARG, "unknown level/box or null tags");
  if (variable < 1 || variable > 8 || scheme < 0 || scheme > 2) return fail(c, ELBM_E_ARG, "bad variable or scheme");
  if (!b->data_set) return fail(c, ELBM_E_STATE, "no state");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  if (!b->links39 && !b->gmask39.p) {
    // a box without link codes (periodic on every axis): every link interior
    CUDA_TRY(b->gmask39.alloc(b->N), "ggm links");
    std::vector<uint16_t> all((size_t)b->N, (uint16_t)(((1u << 13) - 1u) | (1u << 14)));
    CUDA_TRY(cudaMemcpy(b->gmask39.p, all.data(), b->N * sizeof(uint16_t), cudaMemcpyHostToDevice), "ggm links");
  }
  DevBuf<double> gm, gg;
  DevBuf<uint8_t> tg;
  DevBuf<unsigned long long> cnt;
  CUDA_TRY(gm.alloc(b->N), "gm");
  CUDA_TRY(gg.alloc(b->N), "ggm");
  CUDA_TRY(tg.alloc(b->N), "tags");
  CUDA_TRY(cnt.alloc(1), "count");
  CUDA_TRY(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), c->stream), "count");
  const double fs[5] = {1.0, lv->fs39[0], lv->fs39[1], lv->fs39[2], lv->fs39[3]};  // rho_inf = 1 in lattice units
  launch_ggm(b->macro.p, b->plane, b->nx, b->ny, b->nz, lv->p39.periodic, b->gmask39.p, variable, scheme, fs, limit,
             gm.p, gg.p, tg.p, cnt.p, c->stream);
  CUDA_TRY(cudaGetLastError(), "ggm launch");
  if (pgs_reach >= 0) {
    launch_ggm_pgs(b->macro.p, b->plane, b->nx, b->ny, b->nz, b->gmask39.p, gg.p, pgs_sensitivity, pgs_reach, tg.p,
                   c->stream);
    CUDA_TRY(cudaGetLastError(), "pgs launch");
  }
  unsigned long long h = 0;
  if (!u.whole) {
    // one box of a multi-box level: the differences ran over the sheet (across box faces in place);
    // the box's part of the tags and ggm
    CUDA_TRY(sub_copy(tags, tg.p, *b, u.off, u.n, 0, 1, b->plane, false, c->stream), "tags");
    if (ggm) CUDA_TRY(sub_copy(ggm, gg.p, *b, u.off, u.n, 0, 1, b->plane, false, c->stream), "ggm");
    CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
    const int64_t nbox = (int64_t)u.n[0] * u.n[1] * u.n[2];
    for (int64_t k = 0; k < nbox; ++k) h += tags[k] != 0;
    if (ntagged) *ntagged = (int64_t)h;
    return ELBM_OK;
  }
  CUDA_TRY(cudaMemcpyAsync(tags, tg.p, b->N, cudaMemcpyDeviceToHost, c->stream), "tags");
  if (ggm) CUDA_TRY(cudaMemcpyAsync(ggm, gg.p, b->N * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "ggm");
  CUDA_TRY(cudaMemcpyAsync(&h, cnt.p, sizeof h, cudaMemcpyDeviceToHost, c->stream), "count");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  if (pgs_reach >= 0) {
    h = 0;  // predictive splitting adds tags: count them all
    for (int64_t k = 0; k < b->N; ++k) h += tags[k] != 0;
  }
  if (ntagged) *ntagged = (int64_t)h;
  return ELBM_OK;
}

int elbm_init_level39(elbm_ctx* c, int lvl, int box, const double* macro, const double* lm_start,
                      int64_t* capped) {
  Level* lv = nullptr;
  const Sub39 u = get_sub39(c, lvl, box, &lv);
  Box* b = u.b;
  if (!b || !macro || !lm_start) return fail(c, ELBM_E_ARG, "unknown level/box, not a D3Q39 level, or null data");
  if (!lv->params_set) return fail(c, ELBM_E_STATE, "set the level parameters first");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  CUDA_TRY(sub39_copy(u, const_cast<double*>(macro), b->macro.p, lv->ngrow, 5, b->plane, true, c->stream),
           "upload macro");
  if (capped) *capped = 0;
  if (!u.whole) {
    // one box of a multi-box level: the sheet's initial state is solved once every box's fields
    // have arrived (with the last call's start multipliers; its count covers the whole sheet);
    // on a complete level the first call starts over, as an upload does
    if (b->data_set) {
      std::fill(lv->sub39_have_pops.begin(), lv->sub39_have_pops.end(), 0);
      b->data_set = false;
    }
    lv->sub39_have_init[box] = 1;
    if (!std::all_of(lv->sub39_have_init.begin(), lv->sub39_have_init.end(), [](uint8_t v) { return v; })) {
      CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
      return ELBM_OK;
    }
    std::fill(lv->sub39_have_init.begin(), lv->sub39_have_init.end(), 0);
    std::fill(lv->sub39_have_pops.begin(), lv->sub39_have_pops.end(), 1);
    std::fill(lv->sub39_have_macro.begin(), lv->sub39_have_macro.end(), 1);
  }
  DevBuf<double> lm0;
  DevBuf<unsigned long long> cnt;
  CUDA_TRY(lm0.alloc(13), "start multipliers");
  CUDA_TRY(cnt.alloc(1), "counter");
  CUDA_TRY(cudaMemcpyAsync(lm0.p, lm_start, 13 * sizeof(double), cudaMemcpyHostToDevice, c->stream), "lm start");
  CUDA_TRY(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), c->stream), "counter");
  Step39Args a{};
  const bool f32 = lv->storage == ELBM_STORE_FP32_DEV;
  if (f32 && !b->stage39.p) CUDA_TRY(b->stage39.alloc((size_t)b->plane * 78), "FP64 staging");
  a.fdst = f32 ? b->stage39.p : (double*)b->buf[0].p;
  a.gdst = f32 ? b->stage39.p + b->plane * 39 : (double*)b->gbuf[0].p;
  a.lm = b->lm.p;
  a.w_vel = b->w_vel.p;
  a.macro = b->macro.p;
  a.plane = b->plane;
  a.nx = b->nx;
  a.ny = b->ny;
  a.nz = b->nz;
  a.N = b->N;
  a.k = dev39(lv->p39, *lv);
  launch_d3q39_init(a, lm0.p, cnt.p, c->stream);
  CUDA_TRY(cudaGetLastError(), "init launch");
  if (f32) CUDA_TRY(stage39_to_fp32(*b, c->stream), "FP32 conversion");
  // both buffers start identical so that the nodes a step skips (solid) stay defined in either
  CUDA_TRY(cudaMemcpyAsync(b->buf[1].p, b->buf[0].p, b->buf[0].n, cudaMemcpyDeviceToDevice, c->stream), "copy f");
  CUDA_TRY(cudaMemcpyAsync(b->gbuf[1].p, b->gbuf[0].p, b->gbuf[0].n, cudaMemcpyDeviceToDevice, c->stream), "copy g");
  CUDA_TRY(cudaMemsetAsync(b->alpha64.p, 0, b->alpha64.n * sizeof(double), c->stream), "alpha");
  b->cur = 0;
  b->gcur = 0;
  if (b->links39) launch_stale39_init(*b, c->stream);
  unsigned long long h = 0;
  CUDA_TRY(cudaMemcpyAsync(&h, cnt.p, sizeof h, cudaMemcpyDeviceToHost, c->stream), "counter");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  if (capped) *capped = (int64_t)h;
  b->data_set = true;
  b->macro_set = true;
  return ELBM_OK;
}

int elbm_d3q39_equilibrium(elbm_ctx* c, const elbm_d3q39_params* p, const double* macro, double* lm,
                           double* fieq, double* gieq) {
  if (!c || !p || !macro || !lm || !fieq || !gieq) return fail(c, ELBM_E_ARG, "null argument");
  if (p->primary_flow_dir < 1 || p->primary_flow_dir > 6 || p->max_lm_iters < 1)
    return fail(c, ELBM_E_ARG, "bad D3Q39 parameters");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  Lattice39 L;
  build_lattice39(p->shifted, p->primary_flow_dir, L);
  upload_lattice39(L, c->stream);
  // one node: macro (5), lm (13), f, g (39 each), w, counter
  DevBuf<double> buf;
  DevBuf<unsigned long long> cnt;
  CUDA_TRY(buf.alloc(5 + 13 + 13 + 39 + 39 + 1), "scratch");
  CUDA_TRY(cnt.alloc(1), "counter");
  double* d = buf.p;
  CUDA_TRY(cudaMemcpyAsync(d, macro, 5 * sizeof(double), cudaMemcpyHostToDevice, c->stream), "macro");
  CUDA_TRY(cudaMemcpyAsync(d + 5, lm, 13 * sizeof(double), cudaMemcpyHostToDevice, c->stream), "lm");
  CUDA_TRY(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), c->stream), "counter");
  Level none;
  Step39Args a{};
  a.macro = d;
  a.lm = d + 18;
  a.fdst = d + 31;
  a.gdst = d + 70;
  a.w_vel = d + 109;
  a.plane = 1;
  a.nx = a.ny = a.nz = 1;
  a.N = 1;
  a.k = dev39(*p, none);
  launch_d3q39_init(a, d + 5, cnt.p, c->stream);
  CUDA_TRY(cudaGetLastError(), "init launch");
  unsigned long long h = 0;
  CUDA_TRY(cudaMemcpyAsync(lm, d + 18, 13 * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "lm");
  CUDA_TRY(cudaMemcpyAsync(fieq, d + 31, 39 * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "fieq");
  CUDA_TRY(cudaMemcpyAsync(gieq, d + 70, 39 * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "gieq");
  CUDA_TRY(cudaMemcpyAsync(&h, cnt.p, sizeof h, cudaMemcpyDeviceToHost, c->stream), "counter");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  if (h) return fail(c, ELBM_E_NUMERIC, "the multiplier Newton did not converge within max_lm_iters");
  return ELBM_OK;
}

int elbm_upload_macro39(elbm_ctx* c, int lvl, int box, const double* macro) {
  Level* lv = nullptr;
  const Sub39 u = get_sub39(c, lvl, box, &lv);
  Box* b = u.b;
  if (!b || !macro) return fail(c, ELBM_E_ARG, "unknown level/box, not a D3Q39 level, or null data");
  if (!b->data_set) return fail(c, ELBM_E_STATE, "upload the populations (elbm_upload_level39) first");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  CUDA_TRY(sub39_copy(u, const_cast<double*>(macro), b->macro.p, lv->ngrow, 5, b->plane, true, c->stream),
           "upload macro");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  if (!u.whole) {
    lv->sub39_have_macro[box] = 1;
    b->macro_set = std::all_of(lv->sub39_have_macro.begin(), lv->sub39_have_macro.end(), [](uint8_t v) { return v; });
  } else {
    b->macro_set = true;
  }
  return ELBM_OK;
}

int elbm_download_level39(elbm_ctx* c, int lvl, int box, double* fout, double* gout, double* lm, double* w_vel,
                          double* alpha, double* macro) {
  Level* lv = nullptr;
  const Sub39 u = get_sub39(c, lvl, box, &lv);
  Box* b = u.b;
  if (!b) return fail(c, ELBM_E_ARG, "unknown level/box or not a D3Q39 level");
  if (!b->data_set) return fail(c, ELBM_E_STATE, "no populations uploaded");
  CUDA_TRY(cudaSetDevice(c->device), "cudaSetDevice");
  const int g = lv->ngrow;
  if (lv->storage == ELBM_STORE_FP32_DEV && (fout || gout)) {
    if (!b->stage39.p) CUDA_TRY(b->stage39.alloc((size_t)b->plane * 78), "FP64 staging");
    const dim3 grid((unsigned)((b->N + 255) / 256), 39);
    from_dev39_kernel<<<grid, 256, 0, c->stream>>>((const float*)b->buf[b->cur].p, b->stage39.p, b->N, b->plane,
                                                  b->ref39.p);
    from_dev39_kernel<<<grid, 256, 0, c->stream>>>((const float*)b->gbuf[b->gcur].p, b->stage39.p + b->plane * 39,
                                                  b->N, b->plane, b->ref39.p + 39);
    CUDA_TRY(cudaGetLastError(), "FP32 conversion");
    if (fout) CUDA_TRY(sub39_copy(u, fout, b->stage39.p, g, 39, b->plane, false, c->stream), "f");
    if (gout) CUDA_TRY(sub39_copy(u, gout, b->stage39.p + b->plane * 39, g, 39, b->plane, false, c->stream), "g");
  } else {
    if (fout) CUDA_TRY(sub39_copy(u, fout, (double*)b->buf[b->cur].p, g, 39, b->plane, false, c->stream), "f");
    if (gout) CUDA_TRY(sub39_copy(u, gout, (double*)b->gbuf[b->gcur].p, g, 39, b->plane, false, c->stream), "g");
  }
  if (lm) CUDA_TRY(sub39_copy(u, lm, b->lm.p, g, 13, b->plane, false, c->stream), "lm");
  if (w_vel) CUDA_TRY(sub39_copy(u, w_vel, b->w_vel.p, g, 1, b->plane, false, c->stream), "w");
  if (alpha) CUDA_TRY(sub39_copy(u, alpha, b->alpha64.p, g, 1, b->plane, false, c->stream), "alpha");
  if (macro) CUDA_TRY(sub39_copy(u, macro, b->macro.p, g, 5, b->plane, false, c->stream), "macro");
  CUDA_TRY(cudaStreamSynchronize(c->stream), "sync");
  return ELBM_OK;
}

}  // extern "C"


// Hooks for the allocation-free upload (csrc/noalloc.cu): expose the buffers of
// a registered D3Q27 FP32 box without allocating anything.
namespace elbm {

struct NoallocTarget {
  int device;
  cudaStream_t stream;
  float* pops;
  float* other;
  int nx, ny, nz, ngrow;
  int64_t N, plane;
};

int noalloc_fail(elbm_ctx* c, int code, const char* msg) { return fail(c, code, "%s", msg); }

int noalloc_target(elbm_ctx* c, int lvl, int box, NoallocTarget* t) {
  Level* lv = nullptr;
  Box* b = get_box(c, lvl, box, &lv);
  if (!b) return fail(c, ELBM_E_ARG, "unknown level/box");
  if (lv->lattice != ELBM_D3Q27 || lv->storage != ELBM_STORE_FP32_DEV)
    return fail(c, ELBM_E_UNSUPPORTED, "the allocation-free upload serves D3Q27 levels with FP32 deviation storage");
  t->device = c->device;
  t->stream = c->stream;
  t->pops = (float*)lv->pop[lv->cur].p + b->base;
  t->other = (float*)lv->pop[lv->cur ^ 1].p + b->base;
  t->nx = b->nx;
  t->ny = b->ny;
  t->nz = b->nz;
  t->ngrow = lv->ngrow;
  t->N = b->N;
  t->plane = lv->plane;
  return ELBM_OK;
}

void noalloc_mark_uploaded(elbm_ctx* c, int lvl, int box) {
  Box* b = get_box(c, lvl, box);
  if (b) b->data_set = true;
}

}  // namespace elbm
