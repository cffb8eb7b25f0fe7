// Learned initial guess for the entropic alpha: a 27 -> 64 -> 64 -> 1 network
// with GELU, trained on (populations, alpha) pairs that the Newton solver
// harvests, by the kernels below (forward, backward, weight gradients, Adam).
// The reference has no counterpart (its Future Work.txt:34 proposes machine
// learning to shorten the Jacobian solves).
//
// Input: x_i = y_i / lambda, y_i = Delta_i / f_i, lambda = max_i |y_i|.
// Target: t = (alpha - 2) / lambda, so the guess is alpha = 2 + lambda * net(x)
// (alpha - 2 is, to leading order, homogeneous of degree one in y).
// Weights (FP32 master copy, 6017 floats): W1[27][64], b1[64], W2[64][64],
// b2[64], w3[64], b3.  Inference uses a BF16 copy.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "mlp.cuh"
#include "mlp_tc.cuh"

namespace elbm {
namespace {

constexpr int NI = kMlpIn, NH = kMlpHidden;
constexpr int OW1 = 0, OB1 = OW1 + NI * NH, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH, OB3 = OW3 + NH;

// tanh form of GELU and its derivative
__device__ __forceinline__ float gelu(float z, float& dg) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  const float u = k0 * fmaf(k1 * z * z, z, z);
  const float t = tanhf(u);
  dg = 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * k0 * fmaf(3.0f * k1, z * z, 1.0f);
  return 0.5f * z * (1.0f + t);
}

// One thread per sample: forward and per-sample backward; writes the vectors
// the weight gradients need.  Weights in shared memory.
__global__ void __launch_bounds__(128) mlp_fwd_bwd_kernel(const float* __restrict__ w, const float* __restrict__ rec,
                                                          int64_t n, float inv_b, float* __restrict__ scratch,
                                                          double* __restrict__ loss) {
  __shared__ float sw[kMlpParams];
  for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x) sw[k] = w[k];
  __syncthreads();
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (s < n) {
    const float* r = rec + s * kMlpRecord;
    float x[NI];
    for (int i = 0; i < NI; ++i) x[i] = r[i];
    const float target = r[NI + 1];
    float h1[NH], d1[NH];
    for (int j = 0; j < NH; ++j) {
      float z = sw[OB1 + j];
      for (int i = 0; i < NI; ++i) z = fmaf(x[i], sw[OW1 + i * NH + j], z);
      h1[j] = gelu(z, d1[j]);
    }
    float h2[NH], d2[NH];
    for (int k = 0; k < NH; ++k) {
      float z = sw[OB2 + k];
      for (int j = 0; j < NH; ++j) z = fmaf(h1[j], sw[OW2 + j * NH + k], z);
      h2[k] = gelu(z, d2[k]);
    }
    float out = sw[OB3];
    for (int k = 0; k < NH; ++k) out = fmaf(h2[k], sw[OW3 + k], out);
    const float err = out - target;
    l = (double)err * err;
    const float dout = 2.0f * err * inv_b;
    // dz2 = dout * w3 * gelu'(z2); dz1 = (W2 dz2) * gelu'(z1)
    float dz2[NH];
    for (int k = 0; k < NH; ++k) dz2[k] = dout * sw[OW3 + k] * d2[k];
    float* o = scratch + s * kMlpScratch;
    for (int j = 0; j < NH; ++j) {
      float a = 0.f;
      for (int k = 0; k < NH; ++k) a = fmaf(sw[OW2 + j * NH + k], dz2[k], a);
      o[NI + j] = a * d1[j];  // dz1
      o[NI + NH + j] = h1[j];
    }
    for (int i = 0; i < NI; ++i) o[i] = x[i];
    for (int k = 0; k < NH; ++k) {
      o[NI + 2 * NH + k] = dz2[k];
      o[NI + 3 * NH + k] = h2[k];
    }
    o[NI + 4 * NH] = dout;
  }
  // block sum of the loss
  for (int off = 16; off > 0; off >>= 1) l += __shfl_down_sync(0xffffffffu, l, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// Weight gradients: every parameter is a sum over the batch of a product of
// two scratch entries.  Each block reduces a chunk of samples for all
// parameters (thread k owns parameters k, k + blockDim, ...), then adds its
// partial sums to the gradient with one atomic per parameter.
__global__ void __launch_bounds__(256) mlp_wgrad_kernel(const float* __restrict__ scratch, int64_t n, int chunk,
                                                        float* __restrict__ grad) {
  constexpr int TS = 32;  // samples staged per round
  __shared__ float tile[TS][kMlpScratch + 1];
  const int64_t s0 = (int64_t)blockIdx.x * chunk;
  const int64_t s1 = (s0 + chunk < n) ? s0 + chunk : n;
  constexpr int PER = (kMlpParams + 255) / 256;
  float acc[PER];
  for (int k = 0; k < PER; ++k) acc[k] = 0.f;
  for (int64_t base = s0; base < s1; base += TS) {
    const int cnt = (int)((s1 - base < TS) ? s1 - base : TS);
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * kMlpScratch; e += blockDim.x)
      tile[e / kMlpScratch][e % kMlpScratch] = scratch[(base + e / kMlpScratch) * kMlpScratch + e % kMlpScratch];
    __syncthreads();
    for (int k = 0; k < PER; ++k) {
      const int p = threadIdx.x + k * 256;
      if (p >= kMlpParams) break;
      // (a, b) scratch columns whose product gives parameter p (b < 0: bias, a * 1)
      int ca, cb;
      if (p < OB1) {
        ca = p / NH;                    // x_i
        cb = NI + p % NH;               // dz1_j
      } else if (p < OW2) {
        ca = NI + (p - OB1);            // dz1_j
        cb = -1;
      } else if (p < OB2) {
        ca = NI + NH + (p - OW2) / NH;  // h1_j
        cb = NI + 2 * NH + (p - OW2) % NH;  // dz2_k
      } else if (p < OW3) {
        ca = NI + 2 * NH + (p - OB2);   // dz2_k
        cb = -1;
      } else if (p < OB3) {
        ca = NI + 3 * NH + (p - OW3);   // h2_k
        cb = NI + 4 * NH;               // dout
      } else {
        ca = NI + 4 * NH;
        cb = -1;
      }
      float a = acc[k];
      for (int t = 0; t < cnt; ++t) a = fmaf(tile[t][ca], cb >= 0 ? tile[t][cb] : 1.0f, a);
      acc[k] = a;
    }
  }
  for (int k = 0; k < PER; ++k) {
    const int p = threadIdx.x + k * 256;
    if (p < kMlpParams && acc[k] != 0.f) atomicAdd(grad + p, acc[k]);
  }
}

__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kMlpParams) return;
  const float gp = g[p];
  const float mp = fmaf(b1, m[p], (1.0f - b1) * gp);
  const float vp = fmaf(b2, v[p], (1.0f - b2) * gp * gp);
  m[p] = mp;
  v[p] = vp;
  w[p] -= lr * (mp / c1) / (sqrtf(vp / c2) + eps);
}

__global__ void gather_batch_kernel(const float* __restrict__ rec, const uint32_t* __restrict__ perm, int64_t off,
                                    int64_t b, float* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= b * kMlpRecord) return;
  const int64_t s = e / kMlpRecord, c = e % kMlpRecord;
  out[e] = rec[(int64_t)perm[off + s] * kMlpRecord + c];
}

// Tensor-core inference over n feature rows (27 floats each), 128 rows per tile.
__global__ void __launch_bounds__(128) mlp_tc_infer_kernel(const float* __restrict__ w, const float* __restrict__ x,
                                                           int64_t n, float* __restrict__ out, unsigned* status) {
  extern __shared__ __align__(128) unsigned char smraw[];
  MlpTcSmem& s = *reinterpret_cast<MlpTcSmem*>(smraw);
  mlp_tc_setup(s, w);
  for (int64_t t0 = (int64_t)blockIdx.x * kTcRows; t0 < n; t0 += (int64_t)gridDim.x * kTcRows) {
    const int64_t i = t0 + threadIdx.x;
    float xv[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) xv[k] = (i < n) ? x[i * kMlpIn + k] : 0.f;
    const float o = mlp_tc_tile(s, xv, status);
    if (i < n) out[i] = o;
  }
  mlp_tc_teardown(s);
}

}  // namespace

void mlp_tc_infer(const float* w, const float* x, int64_t n, float* out, unsigned* status, cudaStream_t s) {
  const int64_t tiles = (n + kTcRows - 1) / kTcRows;
  const unsigned grid = (unsigned)(tiles < 152 * 4 ? tiles : 152 * 4);
  mlp_tc_infer_kernel<<<grid, kTcRows, sizeof(MlpTcSmem), s>>>(w, x, n, out, status);
}

void mlp_batch_grad(const float* w, const float* rec, int64_t n, float* scratch, float* grad, double* loss,
                    cudaStream_t s) {
  const int threads = 128;
  mlp_fwd_bwd_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(w, rec, n, 1.0f / (float)n, scratch,
                                                                                   loss);
  const int chunk = 512;
  mlp_wgrad_kernel<<<(unsigned)((n + chunk - 1) / chunk), 256, 0, s>>>(scratch, n, chunk, grad);
}

void mlp_adam(float* w, const float* g, float* m, float* v, float lr, int t, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
  adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, s>>>(w, g, m, v, lr, b1, b2, 1e-8f, c1, c2);
}

void mlp_gather_batch(const float* rec, const uint32_t* perm, int64_t off, int64_t b, float* out, cudaStream_t s) {
  const int64_t e = b * kMlpRecord;
  gather_batch_kernel<<<(unsigned)((e + 255) / 256), 256, 0, s>>>(rec, perm, off, b, out);
}

}  // namespace elbm
