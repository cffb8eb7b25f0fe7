// Allocation-free upload of a level's populations into FP32 deviation storage.
//
// elbm_upload_level stages the host FP64 FAB in a device buffer that the
// library allocates on first use, then converts it to FP32 deviations.  Some
// callers cannot let the library allocate device memory after set-up: an
// AMReX-based driver whose arena has already reserved the GPU's memory (a
// cudaMalloc then fails or steals from the arena), or a time loop that must
// not pay cudaMalloc's device-wide synchronisation while other streams run.
// For them this entry point stages through a fixed buffer that is part of the
// library image, and calls no cudaMalloc, cudaFree or allocating routine.
//
// The staging buffer is a file-scope __device__ array of kStageBytes (32 MiB):
// every GPU that loads the library holds it until the process exits.  Boxes
// whose FP64 populations (27 x nodes x 8 bytes) exceed it are rejected with
// ELBM_E_ARG.
//
// Set-up: this file's device code is a module of its own, and under CUDA's
// default lazy module loading the module -- and with it the 32 MiB array -- is
// only brought onto a device when one of its symbols or kernels is first
// used.  noalloc_setup() does that at context creation (elbm_create, with the
// context's device current): it looks the array's device address up
// (cudaGetSymbolAddress) and queries the conversion kernel, so the reservation
// happens before the caller's arena or time loop starts and no later call
// loads a module or synchronises the device.  Each context creation refreshes
// the per-device address; a cudaDeviceReset invalidates every context's
// device buffers as well, so contexts (and with them the address) are created
// anew after one.
//
// All calls share the buffer and it keeps the last call's contents; nothing in
// it needs to start at zero (each call overwrites the part it reads).  Calls
// that overlap on the GPU, e.g. from two host threads on two contexts of one
// device, race on the buffer.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/elbm_gb300.h"
#include "lattice.cuh"

namespace {

constexpr size_t kStageBytes = size_t(32) << 20;
constexpr size_t kStageDoubles = kStageBytes / sizeof(double);
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_stage[kStageDoubles];

// Device address of g_stage per device, looked up once with that device current.
double* g_stage_ptr[kMaxDevices] = {nullptr};
std::mutex g_stage_mu;

__global__ void stage_to_dev32_kernel(const double* __restrict__ f, float* __restrict__ d, int64_t N, int64_t plane) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (n >= N) return;
  d[(int64_t)j * plane + n] = (float)(f[(int64_t)j * N + n] - elbm::w27(j));
}

}  // namespace

namespace elbm {

// Loads this file's module on `device` (current) and records the staging
// buffer's device address; called by elbm_create.  Returns a CUDA error code.
cudaError_t noalloc_setup(int device) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  double* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress((void**)&p, g_stage);
  if (e != cudaSuccess) return e;
  if (!p) return cudaErrorInvalidSymbol;
  cudaFuncAttributes attr;
  e = cudaFuncGetAttributes(&attr, stage_to_dev32_kernel);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_stage_mu);
  g_stage_ptr[device] = p;
  return cudaSuccess;
}

// Internal hooks into the context (defined in capi.cu): target buffers of a
// registered D3Q27 FP32 box and its stream.
struct NoallocTarget {
  int device;
  cudaStream_t stream;
  float* pops;   // the box's nodes in the current population buffer (plane stride `plane`)
  float* other;  // the box's nodes in the second buffer (made identical)
  int nx, ny, nz, ngrow;
  int64_t N, plane;
};
int noalloc_target(elbm_ctx* ctx, int lvl, int box, NoallocTarget* t);
void noalloc_mark_uploaded(elbm_ctx* ctx, int lvl, int box);
int noalloc_fail(elbm_ctx* ctx, int code, const char* msg);

}  // namespace elbm

extern "C" int elbm_upload_level_noalloc(elbm_ctx* ctx, int lvl, int box, const double* fout) {
  using namespace elbm;
  if (!ctx || !fout) return noalloc_fail(ctx, ELBM_E_ARG, "null context or data");
  NoallocTarget t;
  const int rc = noalloc_target(ctx, lvl, box, &t);
  if (rc) return rc;
  const size_t need = (size_t)t.N * Q27 * sizeof(double);
  if (need > kStageBytes) {
    char msg[200];
    snprintf(msg, sizeof msg,
             "box of %lld nodes needs %zu bytes of FP64 staging; the allocation-free upload holds at most %zu bytes",
             (long long)t.N, need, kStageBytes);
    return noalloc_fail(ctx, ELBM_E_ARG, msg);
  }
  if (t.device < 0 || t.device >= kMaxDevices) return noalloc_fail(ctx, ELBM_E_ARG, "device ordinal out of range");
  if (cudaSetDevice(t.device) != cudaSuccess) return noalloc_fail(ctx, ELBM_E_CUDA, "cudaSetDevice failed");
  double* stage = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_stage_mu);
    stage = g_stage_ptr[t.device];
  }
  // elbm_create has set this device up; a context made otherwise is not supported
  if (!stage) return noalloc_fail(ctx, ELBM_E_STATE, "the staging buffer of this device was not set up");
  // host FAB (ghost width ngrow) -> packed staging: one 3-D copy per population
  const int g = t.ngrow;
  const int fx = t.nx + 2 * g, fy = t.ny + 2 * g, fz = t.nz + 2 * g;
  for (int q = 0; q < Q27; ++q) {
    cudaMemcpy3DParms p{};
    p.srcPtr = make_cudaPitchedPtr((void*)(fout + (int64_t)q * fx * fy * fz), fx * sizeof(double), fx, fy);
    p.srcPos = make_cudaPos(g * sizeof(double), g, g);
    p.dstPtr = make_cudaPitchedPtr((void*)(stage + (int64_t)q * t.N), t.nx * sizeof(double), t.nx, t.ny);
    p.dstPos = make_cudaPos(0, 0, 0);
    p.extent = make_cudaExtent(t.nx * sizeof(double), t.ny, t.nz);
    p.kind = cudaMemcpyHostToDevice;
    if (cudaMemcpy3DAsync(&p, t.stream) != cudaSuccess) return noalloc_fail(ctx, ELBM_E_CUDA, "staging copy failed");
  }
  dim3 grid((unsigned)((t.N + 255) / 256), Q27);
  stage_to_dev32_kernel<<<grid, 256, 0, t.stream>>>(stage, t.pops, t.N, t.plane);
  if (cudaGetLastError() != cudaSuccess) return noalloc_fail(ctx, ELBM_E_CUDA, "conversion launch failed");
  if (cudaMemcpy2DAsync(t.other, t.plane * sizeof(float), t.pops, t.plane * sizeof(float), t.N * sizeof(float), Q27,
                        cudaMemcpyDeviceToDevice, t.stream) != cudaSuccess)
    return noalloc_fail(ctx, ELBM_E_CUDA, "buffer copy failed");
  // the staging buffer is shared by every call: finish before returning so the next call may reuse it
  if (cudaStreamSynchronize(t.stream) != cudaSuccess) return noalloc_fail(ctx, ELBM_E_CUDA, "sync failed");
  noalloc_mark_uploaded(ctx, lvl, box);
  return ELBM_OK;
}
