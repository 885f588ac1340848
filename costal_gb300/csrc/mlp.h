// The learned block-pruning model: an MLP that predicts each row's k-th-neighbour cosine.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "prune.h"

namespace costal {

constexpr int MLP_TOPC = 64;   // features: the row (d values) + its 64 largest centroid cosines, sorted
constexpr int MLP_H = 128;     // two hidden layers of 128 (ReLU), one linear output
constexpr int MLP_MAXF = 64 + MLP_TOPC;

// Parameter layout (float, contiguous): W1[H][F] b1[H] W2[H][H] b2[H] W3[H] b3.
__host__ __device__ inline size_t mlp_param_count(int F) { return (size_t)MLP_H * F + MLP_H + (size_t)MLP_H * MLP_H + MLP_H + MLP_H + 1; }

struct MlpState {
    bool ready = false;
    int d = 0, k = 0, F = 0;
    float quantile = 0.05f;
    float* params = nullptr;    // device, master weights (f32)
    float* params_bf = nullptr; // device, inference weights (f32 values rounded to bf16)
    size_t nparams = 0;
};

namespace mlp {

// Features of the rows `rows` (original indices; NULL = 0..m-1) from xsT and the unit centroids.
cudaError_t features(const float* xsT, int np, int d, const float* centroids, int K, const uint32_t* rows, int m,
                     float* feat, cudaStream_t st);
// Inference of m rows with the given parameter block: out[i] (tensor cores: bf16 weights, features and
// first-layer activations, FP32 accumulation).
cudaError_t forward(const float* params, int F, const float* feat, int m, float* out, cudaStream_t st);
// Loss gradient (pinball loss at `quantile`, mean over the m rows) with respect to every
// parameter, summed in a fixed order: grad[nparams]. `partial` holds ⌈m/32⌉ × nparams floats.
cudaError_t gradient(const float* params, int F, const float* feat, const float* y, int m, float quantile,
                     float* partial, float* grad, cudaStream_t st);
// One Adam step (β1 0.9, β2 0.999, ε 1e-8) on params with gradient grad, step count t ≥ 1.
cudaError_t adam(float* params, const float* grad, float* m1, float* m2, size_t np, float lr, int t, cudaStream_t st);
// params_bf = bf16-rounded copy of params (inference weights).
cudaError_t round_bf16(const float* params, float* params_bf, size_t np, cudaStream_t st);
// Per-query-block thresholds for the pruning lists: t_Q = min over the block's rows of the
// prediction (working order; rows past n ignored).
cudaError_t block_min(const float* pred_orig, const uint32_t* perm, int n, float* tq, cudaStream_t st);

}  // namespace mlp
}  // namespace costal
