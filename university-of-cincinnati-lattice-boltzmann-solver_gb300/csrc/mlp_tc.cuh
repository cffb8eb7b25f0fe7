// Tensor-core inference of the learned-alpha network for a tile of 128 nodes
// (one node per thread of a 128-thread block): tcgen05.mma with BF16 operands
// in shared memory and FP32 accumulators in tensor memory.
//
//   layer 1: H1[128 x 64] = X[128 x 32] W1[32 x 64]   (K = 27 padded to 32: 2 MMAs, K = 16 each)
//   layer 2: H2[128 x 64] = gelu(H1 + b1)[128 x 64] W2[64 x 64]   (4 MMAs)
//   output : out = gelu(H2 + b2) . w3 + b3   (per thread, from its own TMEM lane)
//
// Operands use the no-swizzle K-major canonical layout: 8 x 16-byte core
// matrices (8 rows x 8 BF16 along K, 128 contiguous bytes); the core matrices
// of one 8-row group follow each other along K (leading byte offset 128), the
// row groups follow at KG x 128 bytes (stride byte offset), KG = K / 8.
// D[m][n] lives in TMEM lane m, column n.  Warp w of the block reads lanes
// 32w .. 32w + 31, so thread t reads the row of its own node.
//
// Every wait on the MMA-completion mbarrier is bounded; a block whose MMA does
// not complete in time stops using the tensor cores (its guesses become 0,
// which the alpha solve's fallback absorbs) and reports ELBM_ST_COPY_TIMEOUT.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp.cuh"

namespace elbm {

constexpr int kTcRows = 128, kTcK1 = 32, kTcH = kMlpHidden;
constexpr uint32_t kTmemCols = 128;  // layer 1 in columns 0..63, layer 2 in 64..127

struct __align__(128) MlpTcSmem {
  __nv_bfloat16 a1[kTcRows * kTcK1];  // X tile           (8 KB)
  __nv_bfloat16 a2[kTcRows * kTcH];   // gelu(H1) tile    (16 KB)
  __nv_bfloat16 w1[kTcH * kTcK1];     // W1^T, [n][k]     (4 KB)
  __nv_bfloat16 w2[kTcH * kTcH];      // W2^T, [n][k]     (8 KB)
  float b1[kTcH], b2[kTcH], w3[kTcH], b3;
  unsigned long long bar;             // MMA completion
  uint32_t tmem;                      // TMEM base address from tcgen05.alloc
  int broken;                         // an MMA wait timed out: no more tensor-core use
};

// element offset of (row r, k) in a K-major no-swizzle operand with kg core matrices along K
__device__ __forceinline__ int tc_off(int r, int k, int kg) { return (((r >> 3) * kg + (k >> 3)) << 6) + ((r & 7) << 3) + (k & 7); }

__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t tc_desc(const void* p, uint32_t sbo) {
  const uint64_t a = (tc_smem(p) >> 4) & 0x3FFFu;
  return a | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major, N = 64, M = 128
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcH >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kTcIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Bounded wait on an mbarrier phase (2 s of the global timer at most).
__device__ __forceinline__ bool tc_wait(unsigned long long* bar, uint32_t parity) {
  unsigned long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (int i = 0; i < (1 << 20); ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(tc_smem(bar)), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 255) == 255) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      if (t - t0 > 2000000000ull) return false;
    }
  }
  return false;
}

__device__ __forceinline__ float tc_gelu(float z) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.7978845608028654f * fmaf(0.044715f * z * z, z, z)));
  return 0.5f * z * (1.0f + t);
}

// Block-wide set-up (all 128 threads): weights to BF16 operand layouts, the
// barrier, and (warp 0) the TMEM allocation.  Weights: FP32 master layout
// W1[27][64], b1[64], W2[64][64], b2[64], w3[64], b3.
__device__ __forceinline__ void mlp_tc_setup(MlpTcSmem& s, const float* __restrict__ w) {
  constexpr int OB1 = kMlpIn * kTcH, OW2 = OB1 + kTcH, OB2 = OW2 + kTcH * kTcH, OW3 = OB2 + kTcH, OB3 = OW3 + kTcH;
  for (int e = threadIdx.x; e < kTcH * kTcK1; e += blockDim.x) {
    const int n = e / kTcK1, k = e % kTcK1;
    s.w1[tc_off(n, k, kTcK1 / 8)] = __float2bfloat16_rn(k < kMlpIn ? w[k * kTcH + n] : 0.f);
  }
  for (int e = threadIdx.x; e < kTcH * kTcH; e += blockDim.x) {
    const int n = e / kTcH, k = e % kTcH;
    s.w2[tc_off(n, k, kTcH / 8)] = __float2bfloat16_rn(w[OW2 + k * kTcH + n]);
  }
  for (int e = threadIdx.x; e < kTcH; e += blockDim.x) {
    s.b1[e] = w[OB1 + e];
    s.b2[e] = w[OB2 + e];
    s.w3[e] = w[OW3 + e];
  }
  if (threadIdx.x == 0) {
    s.b3 = w[OB3];
    s.broken = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&s.bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&s.tmem)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic writes -> tensor-core reads
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}

// Block-wide tear-down (all 128 threads): TMEM back to the SM.  After a
// timed-out wait, first wait (bounded) for both completions of the tile whose
// MMAs may still be in flight.
__device__ __forceinline__ void mlp_tc_teardown(MlpTcSmem& s) {
  tc_fence_before();
  __syncthreads();
  if (s.broken && threadIdx.x == 0) {
    tc_wait(&s.bar, 0);
    tc_wait(&s.bar, 1);
  }
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(s.tmem), "r"(kTmemCols) : "memory");
}

// One tile (all 128 threads, block-uniform call): x = this thread's 27
// features (zeros for a thread without a node); returns the network output.
// Each call completes the barrier twice, so the parities are 0 then 1.
// Features k and k + 1 (k even) of this thread's row of the input tile.
__device__ __forceinline__ void mlp_tc_put(MlpTcSmem& s, int k, float v0, float v1) {
  __nv_bfloat162 v;
  v.x = __float2bfloat16_rn(v0);
  v.y = __float2bfloat16_rn(v1);
  *reinterpret_cast<__nv_bfloat162*>(&s.a1[tc_off(threadIdx.x, k, kTcK1 / 8)]) = v;
}

__device__ __forceinline__ float mlp_tc_run(MlpTcSmem& s, unsigned* status);

__device__ __forceinline__ float mlp_tc_tile(MlpTcSmem& s, const float (&x)[kMlpIn], unsigned* status) {
#pragma unroll
  for (int k = 0; k < kTcK1; k += 2) mlp_tc_put(s, k, k < kMlpIn ? x[k] : 0.f, k + 1 < kMlpIn ? x[k + 1] : 0.f);
  return mlp_tc_run(s, status);
}

// The network on the tile whose features every thread has put (mlp_tc_put).
__device__ __forceinline__ float mlp_tc_run(MlpTcSmem& s, unsigned* status) {
  const int r = threadIdx.x;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  const bool use_tc = !s.broken;
  const uint32_t lane_base = s.tmem + ((uint32_t)(threadIdx.x & ~31) << 16);
  if (use_tc && threadIdx.x == 0) {
    tc_fence_after();
#pragma unroll
    for (int ks = 0; ks < kTcK1 / 16; ++ks)
      tc_mma(s.tmem, tc_desc(s.a1 + ks * 128, (kTcK1 / 8) * 128), tc_desc(s.w1 + ks * 128, (kTcK1 / 8) * 128), ks > 0);
    tc_commit(&s.bar);
  }
  // block-uniform outcome: the tcgen05.ld below must be executed by whole warps
  bool ok = __syncthreads_and(use_tc && tc_wait(&s.bar, 0));
  tc_fence_after();
  if (ok) {
#pragma unroll
    for (int c = 0; c < kTcH; c += 16) {
      float v[16];
      tc_ld16(lane_base + c, v);
#pragma unroll
      for (int i = 0; i < 16; i += 2) {
        __nv_bfloat162 h;
        h.x = __float2bfloat16_rn(tc_gelu(v[i] + s.b1[c + i]));
        h.y = __float2bfloat16_rn(tc_gelu(v[i + 1] + s.b1[c + i + 1]));
        *reinterpret_cast<__nv_bfloat162*>(&s.a2[tc_off(r, c + i, kTcH / 8)]) = h;
      }
    }
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  ok = __syncthreads_and(ok);
  if (ok && threadIdx.x == 0) {
    tc_fence_after();
#pragma unroll
    for (int ks = 0; ks < kTcH / 16; ++ks)
      tc_mma(s.tmem + kTcH, tc_desc(s.a2 + ks * 128, (kTcH / 8) * 128), tc_desc(s.w2 + ks * 128, (kTcH / 8) * 128),
             ks > 0);
    tc_commit(&s.bar);
  }
  float out = 0.f;
  if (ok) {
    ok = __syncthreads_and(tc_wait(&s.bar, 1));
    tc_fence_after();
  }
  if (ok) {
    float acc = s.b3;
#pragma unroll
    for (int c = 0; c < kTcH; c += 16) {
      float v[16];
      tc_ld16(lane_base + kTcH + c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) acc = fmaf(tc_gelu(v[i] + s.b2[c + i]), s.w3[c + i], acc);
    }
    out = acc;
  }
  tc_fence_before();
  if (!__syncthreads_and(ok || !use_tc) && threadIdx.x == 0) {
    s.broken = 1;
    atomicOr(status, 0x10u);
  }
  return out;
}

}  // namespace elbm
