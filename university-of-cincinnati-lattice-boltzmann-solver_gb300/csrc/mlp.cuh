// Shapes and host launchers of the learned-alpha network (csrc/alpha_mlp.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace elbm {

constexpr int kMlpIn = 27;
constexpr int kMlpHidden = 64;
constexpr int kMlpParams = kMlpIn * kMlpHidden + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden + kMlpHidden + 1;
constexpr int kMlpRecord = kMlpIn + 2;                   // x[27], lambda, target (alpha - 2) / lambda
constexpr int kMlpScratch = kMlpIn + 4 * kMlpHidden + 1;  // x, dz1, h1, dz2, h2, dout per sample
static_assert(kMlpParams == 6017, "27-64-64-1 network");

void mlp_batch_grad(const float* w, const float* rec, int64_t n, float* scratch, float* grad, double* loss,
                    cudaStream_t s);
void mlp_adam(float* w, const float* g, float* m, float* v, float lr, int t, cudaStream_t s);
void mlp_tc_infer(const float* w, const float* x, int64_t n, float* out, unsigned* status, cudaStream_t s);
void mlp_gather_batch(const float* rec, const uint32_t* perm, int64_t off, int64_t b, float* out, cudaStream_t s);

}  // namespace elbm
