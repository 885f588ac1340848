// The learned block-pruning model: features, forward, backward, Adam (all hand-written CUDA).
//
// Input of row i: its normalised coordinates (d values) and its 64 largest cosines to the 256
// k-means centroids, sorted descending (the "distances to the 64 nearest centroids"). Network:
// F = d + 64 → 128 (ReLU) → 128 (ReLU) → 1 (linear), predicting the row's k-th-neighbour cosine.
// Training (costal_mlp_train) uses the pinball loss at a low quantile, so the prediction sits below
// the true k-th score for most rows: it only sets a skip threshold, and every skip is certified
// after the fact (a query whose k-th score does not beat its skipped blocks' bound is rescanned).
// Training runs the FP32 forward of that definition; inference runs on the tensor cores with bf16
// operands (weights, features and first-layer activations) and FP32 accumulation. Gradients are
// summed over fixed 32-row groups and then over the groups in order, so training is deterministic.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "common.cuh"
#include "mlp.h"
#include "topk.cuh"

namespace costal {
namespace mlp {

constexpr int R = 32;    // rows per CTA
constexpr int T = MLP_H; // threads per CTA (one per hidden unit)

struct Off {
    size_t w1, b1, w2, b2, w3, b3;
};
__host__ __device__ inline Off offsets(int F) {
    Off o;
    o.w1 = 0;
    o.b1 = o.w1 + (size_t)MLP_H * F;
    o.w2 = o.b1 + MLP_H;
    o.b2 = o.w2 + (size_t)MLP_H * MLP_H;
    o.w3 = o.b2 + MLP_H;
    o.b3 = o.w3 + MLP_H;
    return o;
}

// ---- features ---------------------------------------------------------------------------------
// One warp per row (two rows at a time, interleaved): the row's (at most 64) coordinates loaded once, two per lane, and broadcast by
// shuffles; lane L takes the 8 consecutive centroids 8L … 8L + 7, read as two 16-byte words per
// dimension from a transposed shared copy laid out so that a warp's words are contiguous (no bank
// conflicts); then a branch-free warp bitonic sort of the 256 cosines (descending; only the values
// are kept, so ties need no order) in which strides below 8 stay in a lane's registers, and the first
// 64 (lanes 0-7) are kept. Each cosine is the same FMA chain over the dimensions in order.

// Bitonic sort of R warp-distributed arrays at once (independent sorts interleaved stage by stage, so
// that each stage's shuffles and compare-exchanges of one array hide the latencies of the other's),
// lane-major (position p = 8·lane + s), descending.
template <int R>
__device__ __forceinline__ void warp_sort_desc_lane8(float (&v)[R][8], int lane) {
#pragma unroll
    for (int size = 2; size <= 256; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride < 8) {
#pragma unroll
                for (int s = 0; s < 8; ++s) {
                    const int t = s ^ stride;
                    if (t > s) {
                        const bool desc = ((8 * lane + s) & size) == 0;
#pragma unroll
                        for (int r = 0; r < R; ++r) {
                            const float hi = fmaxf(v[r][s], v[r][t]), lo = fminf(v[r][s], v[r][t]);
                            v[r][s] = desc ? hi : lo;
                            v[r][t] = desc ? lo : hi;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int s = 0; s < 8; ++s) {
                    const int p = 8 * lane + s;
                    const bool keep_max = ((p & stride) == 0) == ((p & size) == 0);
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const float o = __shfl_xor_sync(COSTAL_FULL_MASK, v[r][s], stride >> 3);
                        v[r][s] = keep_max ? fmaxf(v[r][s], o) : fminf(v[r][s], o);
                    }
                }
            }
        }
    }
}

constexpr int FEAT_C = 256;  // centroid slots of the feature kernel (K ≤ 256)

__global__ void k_features(const float* __restrict__ xsT, int np, int d, const float* __restrict__ cent, int K,
                           const uint32_t* __restrict__ rows, int m, float* __restrict__ feat) {
    // [d][256]: for dimension t, word h (0, 1) of lane L sits at t·256 + 128·h + 4·L, holding centroids
    // 8L + 4h … 8L + 4h + 3 (zero past K)
    extern __shared__ float4 c_s4[];
    float* c_s = reinterpret_cast<float*>(c_s4);
    for (int e = threadIdx.x; e < d * FEAT_C; e += blockDim.x) {
        const int t = e / FEAT_C, q = e % FEAT_C;
        const int h = q >> 7, L = (q & 127) >> 2, j = q & 3;
        const int c = 8 * L + 4 * h + j;
        c_s[e] = c < K ? cent[(size_t)c * d + t] : 0.0f;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int F = d + MLP_TOPC;
    const int wpb = blockDim.x >> 5;
    // grid-stride over pairs of rows, one warp per pair (the two rows' chains interleave): the
    // centroids are loaded once per CTA. A pair's second row past m repeats the first and is not stored.
    constexpr int R2 = 2;
    const int stride = gridDim.x * wpb;
    for (int i0 = blockIdx.x * wpb + (threadIdx.x >> 5); i0 < m; i0 += R2 * stride) {
        int ii[R2];
        float x0[R2], x1[R2], dot[R2][8];
#pragma unroll
        for (int q = 0; q < R2; ++q) {
            ii[q] = i0 + q * stride;
            const int i = ii[q] < m ? ii[q] : i0;
            const uint32_t r = rows ? rows[i] : (uint32_t)i;
            x0[q] = lane < d ? xsT[(size_t)lane * np + r] : 0.0f;
            x1[q] = lane + 32 < d ? xsT[(size_t)(lane + 32) * np + r] : 0.0f;
#pragma unroll
            for (int s = 0; s < 8; ++s) dot[q][s] = 0.0f;
        }
        for (int t = 0; t < d; ++t) {
            const float4 w0 = c_s4[t * (FEAT_C / 4) + lane], w1 = c_s4[t * (FEAT_C / 4) + 32 + lane];
#pragma unroll
            for (int q = 0; q < R2; ++q) {
                const float a = __shfl_sync(COSTAL_FULL_MASK, t < 32 ? x0[q] : x1[q], t & 31);
                dot[q][0] = fmaf(a, w0.x, dot[q][0]);
                dot[q][1] = fmaf(a, w0.y, dot[q][1]);
                dot[q][2] = fmaf(a, w0.z, dot[q][2]);
                dot[q][3] = fmaf(a, w0.w, dot[q][3]);
                dot[q][4] = fmaf(a, w1.x, dot[q][4]);
                dot[q][5] = fmaf(a, w1.y, dot[q][5]);
                dot[q][6] = fmaf(a, w1.z, dot[q][6]);
                dot[q][7] = fmaf(a, w1.w, dot[q][7]);
            }
        }
#pragma unroll
        for (int q = 0; q < R2; ++q)
#pragma unroll
            for (int s = 0; s < 8; ++s)
                if (8 * lane + s >= K) dot[q][s] = -CUDART_INF_F;
        warp_sort_desc_lane8<R2>(dot, lane);
#pragma unroll
        for (int q = 0; q < R2; ++q) {
            if (ii[q] >= m) continue;
            float* f = feat + (size_t)ii[q] * F;
            if (lane < d) f[lane] = x0[q];
            if (lane + 32 < d) f[lane + 32] = x1[q];
            if (lane < MLP_TOPC / 8) {
#pragma unroll
                for (int s = 0; s < 8; ++s) f[d + 8 * lane + s] = dot[q][s];
            }
        }
    }
}

// ---- forward (shared by inference and training) ------------------------------------------------
// CTA: R rows × T hidden units. Leaves h1, h2 in shared memory and returns the outputs in out_s.
__device__ void forward_block(const float* __restrict__ P, int F, const float* __restrict__ feat, int m, int r0,
                              float* f_s, float* h1_s, float* h2_s, float* out_s) {
    const Off o = offsets(F);
    const int j = threadIdx.x;
    for (int e = j; e < R * F; e += T) {
        const int r = e / F, t = e % F;
        f_s[e] = r0 + r < m ? feat[(size_t)(r0 + r) * F + t] : 0.0f;
    }
    __syncthreads();
    {
        const float* w = P + o.w1 + (size_t)j * F;
        const float b = P[o.b1 + j];
        for (int r = 0; r < R; ++r) {
            float z = b;
            for (int t = 0; t < F; ++t) z = fmaf(w[t], f_s[r * F + t], z);
            h1_s[r * T + j] = fmaxf(z, 0.0f);
        }
    }
    __syncthreads();
    {
        const float* w = P + o.w2 + (size_t)j * MLP_H;
        const float b = P[o.b2 + j];
        for (int r = 0; r < R; ++r) {
            float z = b;
            for (int t = 0; t < MLP_H; ++t) z = fmaf(w[t], h1_s[r * T + t], z);
            h2_s[r * T + j] = fmaxf(z, 0.0f);
        }
    }
    __syncthreads();
    if (j < R) {
        float z = P[o.b3];
        for (int t = 0; t < MLP_H; ++t) z = fmaf(P[o.w3 + t], h2_s[j * T + t], z);
        out_s[j] = z;
    }
    __syncthreads();
}

// ---- inference ----------------------------------------------------------------------------------
// On the tensor cores (mma.sync m16n8k16, bf16 operands, FP32 accumulation): the weights, rounded to
// bf16, stay in shared memory ([unit][input], which is the MMA's column-major B) while persistent CTAs
// of 8 warps walk 128-row tiles, 16 rows a warp. Layer 1 multiplies the tile's features (rounded to
// bf16, row-major A in shared memory) by W1ᵀ into 16 accumulator fragments of 8 units; bias and ReLU
// are applied in registers, and the fragments, rounded to bf16, are layer 2's A operand as they stand
// (the accumulator layout of two adjacent 8-unit tiles is the A layout of one 16-wide K step), so the
// activations never leave the registers. Layer 2 likewise; the output is the dot of ReLU(layer 2) with
// w3 in FP32: each thread's 32 units, then the four threads of a row in a fixed tree, plus b3.
// Padded inputs (K up to the next multiple of 16) and rows past m are zero.
constexpr int IR = 128;           // rows per tile
constexpr int IT = 256;           // threads (8 warps × 16 rows)
constexpr int IKP = MLP_MAXF + 8;  // shared-memory row stride (bf16) of W1 and the features: conflict-free
constexpr int IHP = MLP_H + 8;     // row stride of W2

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (low half), .y = hi
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__global__ void __launch_bounds__(IT) k_infer(const float* __restrict__ P, int F, const float* __restrict__ feat,
                                              int m, float* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem_i[];
    __nv_bfloat16* w1s = reinterpret_cast<__nv_bfloat16*>(smem_i);  // [H][IKP]
    __nv_bfloat16* w2s = w1s + (size_t)MLP_H * IKP;                  // [H][IHP]
    __nv_bfloat16* xs = w2s + (size_t)MLP_H * IHP;                   // [IR][IKP] the tile's features
    float* b1 = reinterpret_cast<float*>(xs + (size_t)IR * IKP);     // [H]
    float* b2 = b1 + MLP_H;                                          // [H]
    float* w3 = b2 + MLP_H;                                          // [H]
    const Off o = offsets(F);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, tq = lane & 3;  // the fragment's row group and thread in group
    const int KS1 = (F + 15) >> 4;           // layer-1 K steps
    const int kp = KS1 * 16;
    for (int e = tid; e < MLP_H * kp; e += IT) {
        const int u = e / kp, t = e - u * kp;
        w1s[u * IKP + t] = __float2bfloat16_rn(t < F ? P[o.w1 + (size_t)u * F + t] : 0.0f);
    }
    for (int e = tid; e < MLP_H * MLP_H; e += IT) {
        const int u = e / MLP_H, t = e - u * MLP_H;
        w2s[u * IHP + t] = __float2bfloat16_rn(P[o.w2 + e]);
    }
    if (tid < MLP_H) {
        b1[tid] = P[o.b1 + tid];
        b2[tid] = P[o.b2 + tid];
        w3[tid] = P[o.w3 + tid];
    }
    const float b3 = P[o.b3];
    const int ntiles = (m + IR - 1) / IR;
    const int r_w = warp * 16;  // the warp's first row in the tile
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int r0 = tile * IR;
        __syncthreads();  // the previous tile's readers of xs are done (and the weights loaded)
        for (int e = tid; e < IR * kp; e += IT) {
            const int r = e / kp, t = e - r * kp;
            xs[r * IKP + t] = __float2bfloat16_rn(r0 + r < m && t < F ? feat[(size_t)(r0 + r) * F + t] : 0.0f);
        }
        __syncthreads();
        // layer 1: acc[j] = the 16 rows × units 8j … 8j+7
        float acc[16][4];
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
        for (int ks = 0; ks < KS1; ++ks) {
            const int k0 = ks * 16 + 2 * tq;
            uint32_t a[4];
            a[0] = *reinterpret_cast<const uint32_t*>(xs + (r_w + g) * IKP + k0);
            a[1] = *reinterpret_cast<const uint32_t*>(xs + (r_w + g + 8) * IKP + k0);
            a[2] = *reinterpret_cast<const uint32_t*>(xs + (r_w + g) * IKP + k0 + 8);
            a[3] = *reinterpret_cast<const uint32_t*>(xs + (r_w + g + 8) * IKP + k0 + 8);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const __nv_bfloat16* wr = w1s + (8 * j + g) * IKP + k0;
                mma_bf16_16816(acc[j], a, *reinterpret_cast<const uint32_t*>(wr),
                               *reinterpret_cast<const uint32_t*>(wr + 8));
            }
        }
        // bias + ReLU, rounded to bf16: layer 2's A fragments (K step s = units 16s … 16s+15)
        uint32_t h[8][4];
#pragma unroll
        for (int s2 = 0; s2 < 8; ++s2) {
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const int j = 2 * s2 + half, u = 8 * j + 2 * tq;
                const float bu = b1[u], bv = b1[u + 1];
                h[s2][2 * half] = pack_bf16(fmaxf(acc[j][0] + bu, 0.0f), fmaxf(acc[j][1] + bv, 0.0f));
                h[s2][2 * half + 1] = pack_bf16(fmaxf(acc[j][2] + bu, 0.0f), fmaxf(acc[j][3] + bv, 0.0f));
            }
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
        for (int s2 = 0; s2 < 8; ++s2) {
            // A fragment order: (row g, k lo), (row g + 8, k lo), (row g, k hi), (row g + 8, k hi)
            const uint32_t a[4] = {h[s2][0], h[s2][1], h[s2][2], h[s2][3]};
            const int k0 = s2 * 16 + 2 * tq;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const __nv_bfloat16* wr = w2s + (8 * j + g) * IHP + k0;
                mma_bf16_16816(acc[j], a, *reinterpret_cast<const uint32_t*>(wr),
                               *reinterpret_cast<const uint32_t*>(wr + 8));
            }
        }
        // output: Σ_u w3[u]·ReLU(layer 2 + b2) for rows g and g + 8, units 8j + 2tq, 8j + 2tq + 1
        float pg = 0.0f, pg8 = 0.0f;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int u = 8 * j + 2 * tq;
            pg = fmaf(w3[u], fmaxf(acc[j][0] + b2[u], 0.0f), pg);
            pg = fmaf(w3[u + 1], fmaxf(acc[j][1] + b2[u + 1], 0.0f), pg);
            pg8 = fmaf(w3[u], fmaxf(acc[j][2] + b2[u], 0.0f), pg8);
            pg8 = fmaf(w3[u + 1], fmaxf(acc[j][3] + b2[u + 1], 0.0f), pg8);
        }
#pragma unroll
        for (int off = 1; off < 4; off <<= 1) {
            pg += __shfl_xor_sync(COSTAL_FULL_MASK, pg, off);
            pg8 += __shfl_xor_sync(COSTAL_FULL_MASK, pg8, off);
        }
        if (tq == 0) {
            const int r = r0 + r_w + g;
            if (r < m) out[r] = b3 + pg;
            if (r + 8 < m) out[r + 8] = b3 + pg8;
        }
    }
}

// ---- backward ----------------------------------------------------------------------------------
// Per CTA: forward, the pinball-loss gradient of its rows (mean over all m rows), and the gradient
// of every parameter summed over the CTA's rows in row order → partial[blockIdx.x][nparams].
__global__ void __launch_bounds__(T) k_grad_partial(const float* __restrict__ P, int F, const float* __restrict__ feat,
                                                    const float* __restrict__ y, int m, float quantile,
                                                    float* __restrict__ partial) {
    extern __shared__ float sm[];
    float* f_s = sm;                  // [R][F]
    float* h1_s = f_s + R * F;        // [R][T]
    float* h2_s = h1_s + R * T;       // [R][T]
    float* out_s = h2_s + R * T;      // [R]
    float* g_s = out_s + R;           // [R] dL/dout
    float* dz2_s = g_s + R;           // [R][T]
    float* dz1_s = dz2_s + R * T;     // [R][T]
    const Off o = offsets(F);
    const int j = threadIdx.x;
    const int r0 = blockIdx.x * R;
    forward_block(P, F, feat, m, r0, f_s, h1_s, h2_s, out_s);
    if (j < R) {
        const int i = r0 + j;
        // pinball loss ρ(y − out): d/dout = (1 − α) when out > y, −α otherwise
        g_s[j] = i < m ? (out_s[j] > y[i] ? 1.0f - quantile : -quantile) / (float)m : 0.0f;
    }
    __syncthreads();
    float* G = partial + (size_t)blockIdx.x * mlp_param_count(F);
    const float w3j = P[o.w3 + j];
    {
        float gw3 = 0.0f;
        for (int r = 0; r < R; ++r) {
            gw3 = fmaf(g_s[r], h2_s[r * T + j], gw3);
            dz2_s[r * T + j] = h2_s[r * T + j] > 0.0f ? g_s[r] * w3j : 0.0f;
        }
        G[o.w3 + j] = gw3;
        if (j == 0) {
            float gb3 = 0.0f;
            for (int r = 0; r < R; ++r) gb3 += g_s[r];
            G[o.b3] = gb3;
        }
    }
    __syncthreads();
    {
        // layer 2: dW2[j][t] = Σ_r dz2[r][j] h1[r][t], db2[j] = Σ_r dz2[r][j]
        float gb = 0.0f;
        for (int r = 0; r < R; ++r) gb += dz2_s[r * T + j];
        G[o.b2 + j] = gb;
        for (int t = 0; t < MLP_H; ++t) {
            float s = 0.0f;
            for (int r = 0; r < R; ++r) s = fmaf(dz2_s[r * T + j], h1_s[r * T + t], s);
            G[o.w2 + (size_t)j * MLP_H + t] = s;
        }
        // dh1[r][j] = Σ_u dz2[r][u] W2[u][j], masked by the ReLU of layer 1
        for (int r = 0; r < R; ++r) {
            float s = 0.0f;
            for (int u = 0; u < MLP_H; ++u) s = fmaf(dz2_s[r * T + u], P[o.w2 + (size_t)u * MLP_H + j], s);
            dz1_s[r * T + j] = h1_s[r * T + j] > 0.0f ? s : 0.0f;
        }
    }
    __syncthreads();
    {
        float gb = 0.0f;
        for (int r = 0; r < R; ++r) gb += dz1_s[r * T + j];
        G[o.b1 + j] = gb;
        for (int t = 0; t < F; ++t) {
            float s = 0.0f;
            for (int r = 0; r < R; ++r) s = fmaf(dz1_s[r * T + j], f_s[r * F + t], s);
            G[o.w1 + (size_t)j * F + t] = s;
        }
    }
}

__global__ void k_grad_reduce(const float* __restrict__ partial, int groups, size_t np, float* __restrict__ grad) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < np; p += (size_t)gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int g = 0; g < groups; ++g) s += partial[(size_t)g * np + p];
        grad[p] = s;
    }
}

__global__ void k_adam(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m1, float* __restrict__ m2,
                       size_t np, float lr, float bc1, float bc2) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < np; p += (size_t)gridDim.x * blockDim.x) {
        const float gp = g[p];
        const float a = 0.9f * m1[p] + 0.1f * gp;
        const float b = 0.999f * m2[p] + 0.001f * gp * gp;
        m1[p] = a;
        m2[p] = b;
        P[p] -= lr * (a / bc1) / (sqrtf(b / bc2) + 1e-8f);
    }
}

__global__ void k_round_bf16(const float* __restrict__ P, float* __restrict__ Q, size_t np) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < np; p += (size_t)gridDim.x * blockDim.x)
        Q[p] = __bfloat162float(__float2bfloat16_rn(P[p]));
}

__global__ void k_block_min(const float* __restrict__ pred, const uint32_t* __restrict__ perm, int n,
                            float* __restrict__ tq) {
    const int Q = blockIdx.x;
    __shared__ float red[prune::QB];
    const int w = Q * prune::QB + threadIdx.x;
    red[threadIdx.x] = w < n ? pred[perm[w]] : CUDART_INF_F;
    __syncthreads();
    for (int s = prune::QB / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] = fminf(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) tq[Q] = red[0];
}

// ---- launchers ----------------------------------------------------------------------------------

static size_t grad_smem(int F) { return (size_t)(R * F + 4 * R * T + 2 * R) * 4; }

cudaError_t features(const float* xsT, int np, int d, const float* centroids, int K, const uint32_t* rows, int m,
                     float* feat, cudaStream_t st) {
    if (m == 0) return cudaSuccess;
    if (K > FEAT_C) return cudaErrorInvalidValue;
    const size_t smem = (size_t)d * FEAT_C * 4;
    cudaError_t e = cudaFuncSetAttribute(k_features, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const int blocks = (m + 7) / 8 < 4 * sms ? (m + 7) / 8 : 4 * sms;
    k_features<<<blocks, 256, smem, st>>>(xsT, np, d, centroids, K, rows, m, feat); note_launch();
    return cudaGetLastError();
}

static size_t infer_smem(int F) {
    (void)F;
    return ((size_t)MLP_H * IKP + (size_t)MLP_H * IHP + (size_t)IR * IKP) * 2 + 3 * MLP_H * 4;
}

cudaError_t forward(const float* params, int F, const float* feat, int m, float* out, cudaStream_t st) {
    if (m == 0) return cudaSuccess;
    const size_t smem = infer_smem(F);
    cudaError_t e = cudaFuncSetAttribute(k_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const int tiles = (m + IR - 1) / IR;
    k_infer<<<tiles < 2 * sms ? tiles : 2 * sms, IT, smem, st>>>(params, F, feat, m, out); note_launch();
    return cudaGetLastError();
}

cudaError_t gradient(const float* params, int F, const float* feat, const float* y, int m, float quantile,
                     float* partial, float* grad, cudaStream_t st) {
    const int groups = (m + R - 1) / R;
    const size_t smem = grad_smem(F);
    cudaError_t e = cudaFuncSetAttribute(k_grad_partial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_grad_partial<<<groups, T, smem, st>>>(params, F, feat, y, m, quantile, partial); note_launch();
    k_grad_reduce<<<128, 256, 0, st>>>(partial, groups, mlp_param_count(F), grad); note_launch();
    return cudaGetLastError();
}

cudaError_t adam(float* params, const float* grad, float* m1, float* m2, size_t np, float lr, int t, cudaStream_t st) {
    const float bc1 = 1.0f - powf(0.9f, (float)t), bc2 = 1.0f - powf(0.999f, (float)t);
    k_adam<<<128, 256, 0, st>>>(params, grad, m1, m2, np, lr, bc1, bc2); note_launch();
    return cudaGetLastError();
}

cudaError_t round_bf16(const float* params, float* params_bf, size_t np, cudaStream_t st) {
    k_round_bf16<<<64, 256, 0, st>>>(params, params_bf, np); note_launch();
    return cudaGetLastError();
}

cudaError_t block_min(const float* pred_orig, const uint32_t* perm, int n, float* tq, cudaStream_t st) {
    k_block_min<<<(n + prune::QB - 1) / prune::QB, prune::QB, 0, st>>>(pred_orig, perm, n, tq); note_launch();
    return cudaGetLastError();
}

}  // namespace mlp
}  // namespace costal
