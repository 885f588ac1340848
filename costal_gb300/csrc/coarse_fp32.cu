// The FP32 coarse pass: every (query block × column tile) dot product on the CUDA cores, fused with
// the per-query top-cap selection (crates/costal-core/src/knn.rs:603-660 tiles, :758-787 the
// threshold scan, :791-875 the per-row heaps).
//
// Layout: 256 threads per CTA own 128 query rows; each thread holds an 8 × 8 register tile (queries
// ty·4+i and 64+ty·4+i, columns tx·4+j and 64+tx·4+j), so all 128 columns of a query's tile row are
// computed inside ONE warp. The normalised rows are read transposed (xsT, d_pad × n_pad) so that a
// tile is d_pad contiguous 512-byte rows, staged by cp.async in a 3-stage shared-memory ring: one
// block barrier per tile, and the top-cap merges are warp-local (no block barrier).
//
// Selection: each query keeps its best `cap` columns by (score desc, index asc) in shared memory,
// with τ = the worst kept score (−∞ until full). A column is admitted when its score is strictly
// above the τ of the tile start; since every earlier tile holds smaller column indices, that is the
// reference's strict `v > th` test and the kept set is exactly the top-cap (knn.rs:774-780).
// Admissions go to a 16-entry buffer per query; a query whose buffer overflows (early tiles) has its
// tile row recomputed by its warp in the same FMA order and inserted column by column.

#include <cuda_runtime.h>

#include <algorithm>
#include <math_constants.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "topk.cuh"

namespace costal {
namespace plain {

constexpr int BM = 128;
constexpr int BN = 128;
constexpr int NT = 256;
constexpr int BUF = 16;
constexpr int STAGES = 3;

#ifndef COSTAL_FP32_PAIRED
#define COSTAL_FP32_PAIRED 1
#endif

__device__ __forceinline__ unsigned long long pack2(float x, float y) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
    return r;
}
__device__ __forceinline__ void unpack2(unsigned long long r, float& x, float& y) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(r));
}
__device__ __forceinline__ unsigned long long ffma2(unsigned long long a, unsigned long long b, unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// The CTA's lists out: by row (lstride per row), or, with column segments (part_stride > 0), by
// list slot into segment blockIdx.y's part of the output (cap per slot), for k_merge_parts.
template <class RowOf>
__device__ __forceinline__ void write_lists(const float* L_s, const uint32_t* L_i, const float* tau_s, int lcap, int cap,
                                            int lstride, int n, int nq, int q0, int part_stride, RowOf row_of,
                                            uint32_t* cand_idx, float* cand_score, float* tau_out) {
    const int tid = threadIdx.x;
    for (int e = tid; e < BM * cap; e += NT) {
        const int qi = e / cap, p = e % cap, q = row_of(qi);
        if (q < 0 || q >= n) continue;
        const size_t o = part_stride ? ((size_t)blockIdx.y * part_stride + q0 + qi) * cap + p : (size_t)q * lstride + p;
        cand_idx[o] = L_i[qi * lcap + p];
        cand_score[o] = L_s[qi * lcap + p];
    }
    for (int qi = tid; qi < BM; qi += NT) {
        const int q = row_of(qi);
        if (q < 0 || q >= n) continue;
        tau_out[part_stride ? (size_t)blockIdx.y * part_stride + q0 + qi : (size_t)q] = tau_s[qi];
    }
    (void)nq;
}

// The selection of one 128 × 128 tile, shared by both FP32 kernels: the admission test of the
// thread's 8 × 8 scores against each query's τ at the tile start, the per-query buffer, and the
// warp-local merges into the top-cap lists. τ is the worst kept score once cap are kept, before that
// the query's floor (−inf, or a bound from an earlier pass below which no column can be among the
// best cap). `recompute(qi, cl)` returns the score of query slot qi
// and tile column cl with the same FMA order as the main loop (used when a buffer overflows).
template <int SLOTS, class RowOf, class Recompute>
__device__ __forceinline__ void select_tile(const float (&acc)[8][8], int c0, int n, int cap, float* L_s, uint32_t* L_i,
                                            float* buf_s, uint32_t* buf_i, int* cnt_s, int* len_s, float* tau_s,
                                            const float* floor_s, int warp, int lane, int tx, int ty, RowOf row_of,
                                            Recompute recompute) {
    constexpr int LCAP = 32 * SLOTS;
    auto qi_of = [&](int i) { return i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4); };
    auto cj_of = [&](int j) { return j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4); };
    // Admission test against each query's τ at the tile start: a max-tree per register row.
    bool hit = false;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float m01 = fmaxf(acc[i][0], acc[i][1]), m23 = fmaxf(acc[i][2], acc[i][3]);
        const float m45 = fmaxf(acc[i][4], acc[i][5]), m67 = fmaxf(acc[i][6], acc[i][7]);
        hit |= fmaxf(fmaxf(m01, m23), fmaxf(m45, m67)) > tau_s[qi_of(i)];
    }
    if (hit) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const float th = tau_s[qi_of(i)];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (acc[i][j] > th) {
                    const int qi = qi_of(i), col = c0 + cj_of(j);
                    if (col < n && col != row_of(qi)) {
                        const int pos = atomicAdd(&cnt_s[qi], 1);
                        if (pos < BUF) {
                            buf_s[qi * BUF + pos] = acc[i][j];
                            buf_i[qi * BUF + pos] = (uint32_t)col;
                        }
                    }
                }
            }
        }
    }
    __syncwarp();
    if (__any_sync(COSTAL_FULL_MASK, hit)) {
        // Warp-local merge of this warp's 16 queries (8w..8w+7 and 64+8w..64+8w+7).
        for (int qq = 0; qq < 16; ++qq) {
            const int qi = qq < 8 ? 8 * warp + qq : 64 + 8 * warp + (qq - 8);
            const int c = cnt_s[qi];
            if (c == 0) continue;
            const int q = row_of(qi);
            float ls[SLOTS];
            uint32_t li[SLOTS];
#pragma unroll
            for (int s = 0; s < SLOTS; ++s) {
                ls[s] = L_s[qi * LCAP + s * 32 + lane];
                li[s] = L_i[qi * LCAP + s * 32 + lane];
            }
            int len = len_s[qi];
            if (c <= BUF) {
                for (int e = 0; e < c; ++e)
                    list_insert<SLOTS>(ls, li, len, cap, buf_s[qi * BUF + e], buf_i[qi * BUF + e], lane);
            } else {
                const float th0 = tau_s[qi];
                for (int cc = 0; cc < BN / 32; ++cc) {
                    const int cl = cc * 32 + lane, col = c0 + cl;
                    const float sv = recompute(qi, cl);
                    unsigned m = __ballot_sync(COSTAL_FULL_MASK, col < n && col != q && sv > th0);
                    while (m) {
                        const int src = __ffs(m) - 1;
                        m &= m - 1;
                        const float v = __shfl_sync(COSTAL_FULL_MASK, sv, src);
                        list_insert<SLOTS>(ls, li, len, cap, v, (uint32_t)(c0 + cc * 32 + src), lane);
                    }
                }
            }
#pragma unroll
            for (int s = 0; s < SLOTS; ++s) {
                L_s[qi * LCAP + s * 32 + lane] = ls[s];
                L_i[qi * LCAP + s * 32 + lane] = li[s];
            }
            const float worst = __shfl_sync(COSTAL_FULL_MASK, ls[(cap - 1) >> 5], (cap - 1) & 31);
            __syncwarp();
            if (lane == 0) {
                len_s[qi] = len;
                tau_s[qi] = len == cap ? worst : floor_s[qi];
                cnt_s[qi] = 0;
            }
        }
        __syncwarp();
    }
}

// The tile's 8 × 8 cosines → Tanimoto scores (rows qi_of(i), columns c0 + cj_of(j)).
__device__ __forceinline__ void tani_tile(float (&acc)[8][8], const float2* __restrict__ tnorm, int c0, int n, int tx,
                                          int ty, const int* rows8) {
    float2 cn[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int col = c0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
        cn[j] = col < n ? tnorm[col] : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float2 qn = rows8[i] >= 0 ? tnorm[rows8[i]] : make_float2(0.0f, 0.0f);
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = tani_coarse_f32(acc[i][j], qn, cn[j]);
    }
}

// The 8 × 8 register tile of one 128 × 128 tile: the FMA chains over the depth in dimension order
// (queries ty·4+i and 64+ty·4+i of A_s, columns tx·4+j and 64+tx·4+j of the stage Bst).
template <int DPC>
__device__ __forceinline__ void tile_fma(const float* A_s, const float* Bst, int dp, int tx, int ty, float (&acc)[8][8]) {
#if COSTAL_FP32_PAIRED
    // Blackwell's paired FP32 FMA: one instruction does two independent single-rounding FMAs,
    // so the values are those of the scalar fmaf chain below.
    unsigned long long acc2[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc2[i][j] = 0ull;
#pragma unroll(DPC ? DPC : 4)
    for (int t = 0; t < dp; ++t) {
        const float4 a0 = *reinterpret_cast<const float4*>(A_s + t * BM + ty * 4);
        const float4 a1 = *reinterpret_cast<const float4*>(A_s + t * BM + 64 + ty * 4);
        const float4 b0 = *reinterpret_cast<const float4*>(Bst + t * BN + tx * 4);
        const float4 b1 = *reinterpret_cast<const float4*>(Bst + t * BN + 64 + tx * 4);
        const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const unsigned long long bp[4] = {pack2(b0.x, b0.y), pack2(b0.z, b0.w), pack2(b1.x, b1.y), pack2(b1.z, b1.w)};
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const unsigned long long ap = pack2(a[i], a[i]);
#pragma unroll
            for (int j = 0; j < 4; ++j) acc2[i][j] = ffma2(ap, bp[j], acc2[i][j]);
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) unpack2(acc2[i][j], acc[i][2 * j], acc[i][2 * j + 1]);
#else
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
#pragma unroll(DPC ? DPC : 4)
    for (int t = 0; t < dp; ++t) {
        const float4 a0 = *reinterpret_cast<const float4*>(A_s + t * BM + ty * 4);
        const float4 a1 = *reinterpret_cast<const float4*>(A_s + t * BM + 64 + ty * 4);
        const float4 b0 = *reinterpret_cast<const float4*>(Bst + t * BN + tx * 4);
        const float4 b1 = *reinterpret_cast<const float4*>(Bst + t * BN + 64 + tx * 4);
        const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
#endif
}

template <int SLOTS, int DPC, bool TANI>
__global__ void __launch_bounds__(NT, 1)
    k_coarse_fp32(const float* __restrict__ xsT, int n, int np, int dp_rt, int cap, int lstride,
                  const uint32_t* __restrict__ qlist, const unsigned* __restrict__ qcount, int part_stride,
                  const float* __restrict__ tfloor, const float2* __restrict__ tnorm, uint32_t* __restrict__ cand_idx,
                  float* __restrict__ cand_score, float* __restrict__ tau_out) {
    constexpr int LCAP = 32 * SLOTS;
    const int dp = DPC ? DPC : dp_rt;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* A_s = reinterpret_cast<float*>(smem_raw);            // [dp][BM]
    float* B_s = A_s + (size_t)dp * BM;                          // [STAGES][dp][BN]
    float* L_s = B_s + (size_t)STAGES * dp * BN;                 // [BM][LCAP]
    uint32_t* L_i = reinterpret_cast<uint32_t*>(L_s + BM * LCAP);
    float* buf_s = reinterpret_cast<float*>(L_i + BM * LCAP);   // [BM][BUF]
    uint32_t* buf_i = reinterpret_cast<uint32_t*>(buf_s + BM * BUF);
    int* cnt_s = reinterpret_cast<int*>(buf_i + BM * BUF);       // [BM]
    int* len_s = cnt_s + BM;                                     // [BM]
    float* tau_s = reinterpret_cast<float*>(len_s + BM);         // [BM]
    float* floor_s = tau_s + BM;                                 // [BM]

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tx = tid & 15, ty = tid >> 4;
    // The block's 128 consecutive query rows, or 128 entries of a device-side row list.
    const int q0 = blockIdx.x * BM;
    const int nq = qlist ? min(BM, (int)*qcount - q0) : BM;
    if (nq <= 0) return;
    auto row_of = [&](int qi) -> int { return qlist ? (qi < nq ? (int)qlist[q0 + qi] : -1) : q0 + qi; };
    // Column segment blockIdx.y of gridDim.y (one segment: all tiles).
    const int all_tiles = np / BN, tps = (all_tiles + gridDim.y - 1) / gridDim.y;
    const int tile0 = blockIdx.y * tps, ntiles = max(0, min(all_tiles, tile0 + tps) - tile0);

    auto load_tile = [&](float* dst, int c0) {
        for (int ch = tid; ch < dp * (BN / 4); ch += NT) {
            const int t = ch / (BN / 4), c4 = ch % (BN / 4);
            cp_async16(dst + t * BN + c4 * 4, xsT + (size_t)t * np + c0 + c4 * 4);
        }
    };
    if (qlist) {
        for (int e = tid; e < dp * BM; e += NT) {
            const int t = e / BM, qi = e % BM;
            A_s[t * BM + qi] = qi < nq ? xsT[(size_t)t * np + qlist[q0 + qi]] : 0.0f;
        }
    } else {
        load_tile(A_s, q0);
    }
    if (ntiles > 0) load_tile(B_s, tile0 * BN);
    cp_async_commit();
    if (ntiles > 1) load_tile(B_s + (size_t)dp * BN, (tile0 + 1) * BN);
    cp_async_commit();
    for (int q = tid; q < BM; q += NT) {
        cnt_s[q] = 0;
        len_s[q] = 0;
        const int r = row_of(q);
        floor_s[q] = tfloor && r >= 0 ? tfloor[r] : -CUDART_INF_F;
        tau_s[q] = floor_s[q];
    }
    // Unfilled slots read back as index 0xffffffff with score −inf: an empty slot for the rescoring
    // (a list can stay short only with NaN input or a floor at a tie).
    for (int e = tid; e < BM * LCAP; e += NT) {
        L_s[e] = -CUDART_INF_F;
        L_i[e] = 0xffffffffu;
    }

    for (int tl = 0; tl < ntiles; ++tl) {
        cp_async_wait<1>();
        __syncthreads();  // tile's stage landed for every thread; stage (tl+2)%3 is free again
        if (tl + 2 < ntiles) load_tile(B_s + (size_t)((tl + 2) % STAGES) * dp * BN, (tile0 + tl + 2) * BN);
        cp_async_commit();
        const float* Bst = B_s + (size_t)(tl % STAGES) * dp * BN;
        const int c0 = (tile0 + tl) * BN;

        float acc[8][8];
        tile_fma<DPC>(A_s, Bst, dp, tx, ty, acc);
        if constexpr (TANI) {
            int rows8[8];  // this thread's 8 query rows (their norms enter the Tanimoto scores)
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int r = row_of(i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
                rows8[i] = r < n ? r : -1;
            }
            tani_tile(acc, tnorm, c0, n, tx, ty, rows8);
        }
        select_tile<SLOTS>(acc, c0, n, cap, L_s, L_i, buf_s, buf_i, cnt_s, len_s, tau_s, floor_s, warp, lane, tx, ty,
                           row_of,
                           [&](int qi, int cl) {
                               float sv = 0.0f;
#pragma unroll(DPC ? DPC : 4)
                               for (int t = 0; t < dp; ++t) sv = fmaf(A_s[t * BM + qi], Bst[t * BN + cl], sv);
                               if constexpr (TANI) {
                                   const int q = row_of(qi), col = c0 + cl;
                                   sv = tani_coarse_f32(sv, q >= 0 ? tnorm[q] : make_float2(0.0f, 0.0f),
                                                    col < n ? tnorm[col] : make_float2(0.0f, 0.0f));
                               }
                               return sv;
                           });
    }
    cp_async_wait<0>();
    __syncthreads();
    write_lists(L_s, L_i, tau_s, LCAP, cap, lstride, n, nq, q0, part_stride, row_of, cand_idx, cand_score, tau_out);
}

// Tanimoto selection with the norm window (knn.rs:197-284 `Tanimoto`, :595-644 `coarse_block`):
// the rows in norm order (the working order W; perm maps back), each CTA's 128 query rows scan the
// column tile of their own norms first and then walk outward, right (larger norms) and left
// (smaller), one tile each way in turn. With c = τ/(1+τ), a column of norm b can reach a row's
// threshold τ > 0 only if ρ = b/a lies in [ρ−, ρ+], the roots of ρ + 1/ρ = q with
// q = (1+τ)/τ·(1 + 1e-4) (knn.rs:270-283; cos ≤ 1); a side stops at the first tile whose norms all
// lie outside every row's window (every later tile of that side lies further out, and the windows
// only shrink as τ rises). A column left out this way has exact T < τ, so the certificate
// s_k > τ + E that the rescoring checks still covers it. Columns are not visited in index order,
// so ties at τ may be broken differently than in the unpruned pass; the certificate (or the
// regather) makes the answer the same.
template <int SLOTS>
__global__ void __launch_bounds__(NT, 1)
    k_coarse_tani_window(const float* __restrict__ xsW, int n, int np, int dp, int cap, const float2* __restrict__ tnW,
                         const double* __restrict__ normW, const double* __restrict__ tile_lo,
                         const double* __restrict__ tile_hi, const uint32_t* __restrict__ perm,
                         uint32_t* __restrict__ cand_idx, float* __restrict__ cand_score, float* __restrict__ tau_out,
                         unsigned long long* __restrict__ skipped_total) {
    constexpr int LCAP = 32 * SLOTS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* A_s = reinterpret_cast<float*>(smem_raw);            // [dp][BM]
    float* B_s = A_s + (size_t)dp * BM;                          // [STAGES][dp][BN]
    float* L_s = B_s + (size_t)STAGES * dp * BN;                 // [BM][LCAP]
    uint32_t* L_i = reinterpret_cast<uint32_t*>(L_s + BM * LCAP);
    float* buf_s = reinterpret_cast<float*>(L_i + BM * LCAP);   // [BM][BUF]
    uint32_t* buf_i = reinterpret_cast<uint32_t*>(buf_s + BM * BUF);
    int* cnt_s = reinterpret_cast<int*>(buf_i + BM * BUF);       // [BM]
    int* len_s = cnt_s + BM;                                     // [BM]
    float* tau_s = reinterpret_cast<float*>(len_s + BM);         // [BM]
    float* floor_s = tau_s + BM;                                 // [BM]
    __shared__ double win_lo_w[4], win_hi_w[4];
    __shared__ int win_ok_w[4];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tx = tid & 15, ty = tid >> 4;
    const int q0 = blockIdx.x * BM;  // working rows q0 .. q0 + 127
    auto row_of = [&](int qi) -> int { return q0 + qi; };
    const int all_tiles = np / BN;
    const int mid = min(all_tiles - 1, (q0 + BM / 2) / BN);  // the tile of the block's own norms
    auto load_tile = [&](float* dst, int c0) {
        for (int ch = tid; ch < dp * (BN / 4); ch += NT) {
            const int t = ch / (BN / 4), c4 = ch % (BN / 4);
            cp_async16(dst + t * BN + c4 * 4, xsW + (size_t)t * np + c0 + c4 * 4);
        }
    };
    // The visiting order, the same in every thread: mid, then right and left in turn; a stopped
    // side yields no more tiles.
    int right = mid + 1, left = mid - 1;
    bool rstop = false, lstop = false, take_right = true;
    auto next_tile = [&]() -> int {
        for (int tries = 0; tries < 2; ++tries) {
            const bool r = take_right;
            take_right = !take_right;
            if (r && !rstop && right < all_tiles) return right++;
            if (!r && !lstop && left >= 0) return left--;
        }
        return -1;
    };
    int stage_tile[STAGES];
    load_tile(A_s, q0);
    stage_tile[0] = mid;
    load_tile(B_s, mid * BN);
    cp_async_commit();
    stage_tile[1] = next_tile();
    if (stage_tile[1] >= 0) load_tile(B_s + (size_t)dp * BN, stage_tile[1] * BN);
    cp_async_commit();
    for (int q = tid; q < BM; q += NT) {
        cnt_s[q] = 0;
        len_s[q] = 0;
        floor_s[q] = -CUDART_INF_F;
        tau_s[q] = -CUDART_INF_F;
    }
    for (int e = tid; e < BM * LCAP; e += NT) {
        L_s[e] = -CUDART_INF_F;
        L_i[e] = 0xffffffffu;
    }
    // this thread's 8 query rows: f32 norm a and 1/a (constant over the tiles)
    float a8[8], ia8[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int r = row_of(i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
        a8[i] = r < n ? tnW[r].x : 0.0f;
        ia8[i] = a8[i] > 0.0f ? 1.0f / a8[i] : 0.0f;
    }
    bool win_ok = false;  // every row's window is defined (its list is full and τ > 0)
    double win_lo = 0.0, win_hi = 0.0;
    int scanned = 0;
    for (int it = 0;; ++it) {
        const int s = it % STAGES;
        const int tile = stage_tile[s];
        if (tile < 0) break;
        cp_async_wait<1>();
        __syncthreads();  // the stage landed for every thread; stage (it+2)%3 is free again
        const int nxt = next_tile();
        stage_tile[(it + 2) % STAGES] = nxt;
        if (nxt >= 0) load_tile(B_s + (size_t)((it + 2) % STAGES) * dp * BN, nxt * BN);
        cp_async_commit();
        if (tile != mid && win_ok) {
            // a side ends at its first tile outside every row's window (knn.rs:617-639)
            if (tile > mid && tile_lo[tile] > win_hi) {
                rstop = true;
                continue;
            }
            if (tile < mid && tile_hi[tile] < win_lo) {
                lstop = true;
                continue;
            }
        }
        ++scanned;
        const float* Bst = B_s + (size_t)s * dp * BN;
        const int c0 = tile * BN;
        float acc[8][8];
        tile_fma<0>(A_s, Bst, dp, tx, ty, acc);
        int rows8[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int r = row_of(i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
            rows8[i] = r < n ? r : -1;
        }
        // A cosine prefilter (knn.rs:239-252 `tile_threshold`): with c = τ/(1+τ) > 0, a column of norm b
        // can reach T > τ only if its cosine exceeds c·(b/a + a/b), and over this tile b/a + a/b is at
        // least m (2 when the tile's norm range holds a, else its nearer end). Below c·m·(1 − 2⁻¹⁶) no
        // entry of the row can be admitted (the margin covers every f32 rounding of T and of the
        // threshold), so the divisions of T are spent only on a thread whose tile rows have a hit.
        {
            const float blo = (float)tile_lo[tile], bhi = (float)tile_hi[tile];
            const float iblo = 1.0f / blo, ibhi = 1.0f / bhi;  // (+inf for a zero norm: unused then)
            bool hit = false;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const float tau = tau_s[i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4)];
                float thr = -CUDART_INF_F;
                if (tau > 0.0f && rows8[i] >= 0) {
                    if (a8[i] > 0.0f) {
                        // (few-ulp roundings and the fast quotient all sit inside the 2⁻¹⁶ margin)
                        const float rlo = blo * ia8[i], rhi = bhi * ia8[i];
                        const float m = (rlo <= 1.0f && rhi >= 1.0f) ? 2.0f
                                        : (rhi < 1.0f ? rhi + a8[i] * ibhi : rlo + a8[i] * iblo);
                        thr = __fdividef(tau, 1.0f + tau) * m * (1.0f - 0x1p-16f);
                    } else {
                        thr = CUDART_INF_F;  // a zero row: T = 0 ≤ τ with every column
                    }
                }
                const float m01 = fmaxf(acc[i][0], acc[i][1]), m23 = fmaxf(acc[i][2], acc[i][3]);
                const float m45 = fmaxf(acc[i][4], acc[i][5]), m67 = fmaxf(acc[i][6], acc[i][7]);
                hit |= fmaxf(fmaxf(m01, m23), fmaxf(m45, m67)) > thr;
            }
            if (hit) {
                tani_tile(acc, tnW, c0, n, tx, ty, rows8);
            } else {
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[i][j] = -CUDART_INF_F;
            }
        }
        select_tile<SLOTS>(acc, c0, n, cap, L_s, L_i, buf_s, buf_i, cnt_s, len_s, tau_s, floor_s, warp, lane, tx, ty,
                           row_of, [&](int qi, int cl) {
                               float sv = 0.0f;
                               for (int t = 0; t < dp; ++t) sv = fmaf(A_s[t * BM + qi], Bst[t * BN + cl], sv);
                               const int q = row_of(qi), col = c0 + cl;
                               return tani_coarse_f32(sv, q < n ? tnW[q] : make_float2(0.0f, 0.0f),
                                                      col < n ? tnW[col] : make_float2(0.0f, 0.0f));
                           });
        // The union of the rows' windows in absolute norms (knn.rs:668-678), in f64 (the GB300's slow
        // pipe): until every row has one, after each tile; then after every eighth tile scanned. In
        // between the tests use the last union, computed from lower thresholds, which only makes it
        // wider (the windows shrink as τ rises): the stops may come a few tiles later, never too early.
        const bool sides_open = (!rstop && right < all_tiles) || (!lstop && left >= 0);
        if (!sides_open || (win_ok && (scanned & 7) != 1)) continue;
        __syncthreads();  // every query's τ after this tile
        if (tid < BM) {
            const int w = q0 + tid;
            double lo = CUDART_INF, hi = -CUDART_INF;
            int ok = 1;
            if (w < n) {
                const float tf = tau_s[tid];
                if (!(tf > 0.0f)) {
                    ok = 0;
                } else {
                    const double tau = (double)tf;
                    const double q = (1.0 + tau) / tau * (1.0 + 1e-4);
                    const double disc = sqrt(fmax(q * q - 4.0, 0.0));
                    const double a = normW[w];
                    lo = (q - disc) / 2.0 * a;
                    hi = (q + disc) / 2.0 * a;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo = fmin(lo, __shfl_xor_sync(COSTAL_FULL_MASK, lo, o));
                hi = fmax(hi, __shfl_xor_sync(COSTAL_FULL_MASK, hi, o));
                ok &= __shfl_xor_sync(COSTAL_FULL_MASK, ok, o);
            }
            if (lane == 0) {
                win_lo_w[warp] = lo;
                win_hi_w[warp] = hi;
                win_ok_w[warp] = ok;
            }
        }
        __syncthreads();
        win_ok = win_ok_w[0] && win_ok_w[1] && win_ok_w[2] && win_ok_w[3];
        win_lo = fmin(fmin(win_lo_w[0], win_lo_w[1]), fmin(win_lo_w[2], win_lo_w[3]));
        win_hi = fmax(fmax(win_hi_w[0], win_hi_w[1]), fmax(win_hi_w[2], win_hi_w[3]));
    }
    cp_async_wait<0>();
    __syncthreads();
    // the lists out, in the input order: rows and columns mapped back through perm
    for (int e = tid; e < BM * cap; e += NT) {
        const int qi = e / cap, p = e % cap, w = q0 + qi;
        if (w >= n) continue;
        const uint32_t c = L_i[qi * LCAP + p];
        const size_t o = (size_t)perm[w] * cap + p;
        cand_idx[o] = c < (uint32_t)n ? perm[c] : 0xffffffffu;
        cand_score[o] = L_s[qi * LCAP + p];
    }
    for (int qi = tid; qi < BM; qi += NT)
        if (q0 + qi < n) tau_out[perm[q0 + qi]] = tau_s[qi];
    if (tid == 0 && skipped_total) atomicAdd(skipped_total, (unsigned long long)(all_tiles - scanned));
}

// The norm-ordered working copy for the windowed pass: xsW[t][w] = xsT[t][perm[w]] (zero for w ≥ n),
// the rows' f32 norm and squared norm, their f64 norms, and each 128-column tile's norm range.
__global__ void k_tani_gather(const float* __restrict__ xsT, int n, int np, int dp, const uint32_t* __restrict__ perm,
                              float* __restrict__ xsW) {
    const size_t total = (size_t)dp * np;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int t = (int)(e / np), w = (int)(e % np);
        xsW[e] = w < n ? xsT[(size_t)t * np + perm[w]] : 0.0f;
    }
}
__global__ void k_tani_norms_w(const double* __restrict__ norms, int n, const uint32_t* __restrict__ perm,
                               float2* __restrict__ tnW, double* __restrict__ normW) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= n) return;
    const double a = norms[perm[w]];
    tnW[w] = make_float2((float)a, (float)(a * a));  // knn.rs:207-212 rounds ‖x‖² to f32
    normW[w] = a;
}
__global__ void k_tile_norm_range(const double* __restrict__ normW, int n, int ntiles, double* __restrict__ lo,
                                  double* __restrict__ hi) {
    const int tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (tile >= ntiles) return;
    double a = CUDART_INF, b = -CUDART_INF;
    for (int j = lane; j < BN; j += 32) {
        const int w = tile * BN + j;
        if (w < n) {
            a = fmin(a, normW[w]);
            b = fmax(b, normW[w]);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a = fmin(a, __shfl_xor_sync(COSTAL_FULL_MASK, a, o));
        b = fmax(b, __shfl_xor_sync(COSTAL_FULL_MASK, b, o));
    }
    if (lane == 0) {
        lo[tile] = a;  // a tile of padding only: +inf / −inf, outside every window
        hi[tile] = b;
    }
}
// The ranges made monotone along the order (rows inside a norm bucket are not sorted, so a later
// tile may hold a smaller norm than an earlier one): lo[t] = the smallest norm of tiles t, t+1, …
// and hi[t] = the largest of tiles …, t−1, t. A side stopped at tile t then has every later tile of
// that side outside the window too. (One thread: a few thousand tiles.)
__global__ void k_tile_norm_envelope(int ntiles, double* __restrict__ lo, double* __restrict__ hi) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int t = ntiles - 2; t >= 0; --t) lo[t] = fmin(lo[t], lo[t + 1]);
    for (int t = 1; t < ntiles; ++t) hi[t] = fmax(hi[t], hi[t - 1]);
}

// The same pass for any depth: the dimensions stream through the 3-stage ring in chunks of KC rows
// of the transposed copy (query chunk and column chunk per stage), and the 8 × 8 register tile
// accumulates across the chunks of a tile in dimension order, so every score is the same FMA chain
// as in k_coarse_fp32. A query whose buffer overflows is recomputed from global memory.
template <int SLOTS, int KC, bool TANI>
__global__ void __launch_bounds__(NT, 1)
    k_coarse_fp32_kc(const float* __restrict__ xsT, int n, int np, int dp, int cap, int lstride,
                     const uint32_t* __restrict__ qlist, const unsigned* __restrict__ qcount, int part_stride,
                     const float* __restrict__ tfloor, const float2* __restrict__ tnorm, uint32_t* __restrict__ cand_idx,
                     float* __restrict__ cand_score, float* __restrict__ tau_out) {
    constexpr int LCAP = 32 * SLOTS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* S_s = reinterpret_cast<float*>(smem_raw);            // [STAGES][KC][BM + BN]
    float* L_s = S_s + (size_t)STAGES * KC * (BM + BN);          // [BM][LCAP]
    uint32_t* L_i = reinterpret_cast<uint32_t*>(L_s + BM * LCAP);
    float* buf_s = reinterpret_cast<float*>(L_i + BM * LCAP);   // [BM][BUF]
    uint32_t* buf_i = reinterpret_cast<uint32_t*>(buf_s + BM * BUF);
    int* cnt_s = reinterpret_cast<int*>(buf_i + BM * BUF);       // [BM]
    int* len_s = cnt_s + BM;                                     // [BM]
    float* tau_s = reinterpret_cast<float*>(len_s + BM);         // [BM]
    float* floor_s = tau_s + BM;                                 // [BM]

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tx = tid & 15, ty = tid >> 4;
    const int q0 = blockIdx.x * BM;
    const int nq = qlist ? min(BM, (int)*qcount - q0) : BM;
    if (nq <= 0) return;
    auto row_of = [&](int qi) -> int { return qlist ? (qi < nq ? (int)qlist[q0 + qi] : -1) : q0 + qi; };
    const int all_tiles = np / BN, tps = (all_tiles + gridDim.y - 1) / gridDim.y;
    const int tile0 = blockIdx.y * tps, ntiles = max(0, min(all_tiles, tile0 + tps) - tile0);
    const int nch = (dp + KC - 1) / KC;
    const int nsteps = ntiles * nch;

    // Stage of step s = (tile, chunk): rows [chunk·KC, +KC) of the queries' and the tile's columns.
    auto load_step = [&](int step) {
        float* A = S_s + (size_t)(step % STAGES) * KC * (BM + BN);
        float* B = A + KC * BM;
        const int tile = tile0 + step / nch, t0 = (step % nch) * KC;
        for (int ch = tid; ch < KC * (BM / 4); ch += NT) {
            const int t = ch / (BM / 4), c4 = ch % (BM / 4);
            if (t0 + t < dp) {
                if (qlist) {
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int qi = c4 * 4 + u;
                        A[t * BM + qi] = qi < nq ? xsT[(size_t)(t0 + t) * np + qlist[q0 + qi]] : 0.0f;
                    }
                } else {
                    cp_async16(A + t * BM + c4 * 4, xsT + (size_t)(t0 + t) * np + q0 + c4 * 4);
                }
                cp_async16(B + t * BN + c4 * 4, xsT + (size_t)(t0 + t) * np + tile * BN + c4 * 4);
            } else {
                *reinterpret_cast<float4*>(A + t * BM + c4 * 4) = make_float4(0.f, 0.f, 0.f, 0.f);
                *reinterpret_cast<float4*>(B + t * BN + c4 * 4) = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    };
    if (nsteps > 0) load_step(0);
    cp_async_commit();
    if (nsteps > 1) load_step(1);
    cp_async_commit();
    for (int q = tid; q < BM; q += NT) {
        cnt_s[q] = 0;
        len_s[q] = 0;
        const int r = row_of(q);
        floor_s[q] = tfloor && r >= 0 ? tfloor[r] : -CUDART_INF_F;
        tau_s[q] = floor_s[q];
    }
    // Unfilled slots read back as index 0xffffffff with score −inf: an empty slot for the rescoring
    // (a list can stay short only with NaN input or a floor at a tie).
    for (int e = tid; e < BM * LCAP; e += NT) {
        L_s[e] = -CUDART_INF_F;
        L_i[e] = 0xffffffffu;
    }

    for (int tl = 0; tl < ntiles; ++tl) {
        const int c0 = (tile0 + tl) * BN;
        unsigned long long acc2[8][4];
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc2[i][j] = 0ull;
        for (int ch = 0; ch < nch; ++ch) {
            const int step = tl * nch + ch;
            cp_async_wait<1>();
            __syncthreads();  // this step's stage landed for every thread; stage (step+2)%3 is free
            if (step + 2 < nsteps) load_step(step + 2);
            cp_async_commit();
            const float* A = S_s + (size_t)(step % STAGES) * KC * (BM + BN);
            const float* B = A + KC * BM;
#pragma unroll 4
            for (int t = 0; t < KC; ++t) {
                const float4 a0 = *reinterpret_cast<const float4*>(A + t * BM + ty * 4);
                const float4 a1 = *reinterpret_cast<const float4*>(A + t * BM + 64 + ty * 4);
                const float4 b0 = *reinterpret_cast<const float4*>(B + t * BN + tx * 4);
                const float4 b1 = *reinterpret_cast<const float4*>(B + t * BN + 64 + tx * 4);
                const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const unsigned long long bp[4] = {pack2(b0.x, b0.y), pack2(b0.z, b0.w), pack2(b1.x, b1.y),
                                                  pack2(b1.z, b1.w)};
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const unsigned long long ap = pack2(a[i], a[i]);
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc2[i][j] = ffma2(ap, bp[j], acc2[i][j]);
                }
            }
        }
        float acc[8][8];
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) unpack2(acc2[i][j], acc[i][2 * j], acc[i][2 * j + 1]);
        if constexpr (TANI) {
            int rows8[8];  // this thread's 8 query rows (their norms enter the Tanimoto scores)
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int r = row_of(i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
                rows8[i] = r < n ? r : -1;
            }
            tani_tile(acc, tnorm, c0, n, tx, ty, rows8);
        }
        select_tile<SLOTS>(acc, c0, n, cap, L_s, L_i, buf_s, buf_i, cnt_s, len_s, tau_s, floor_s, warp, lane, tx, ty,
                           row_of,
                           [&](int qi, int cl) {
                               // zero padding beyond dp adds exact zeros: the chain over dp is the same
                               const int q = row_of(qi);
                               float sv = 0.0f;
                               if (q >= 0)
                                   for (int t = 0; t < dp; ++t)
                                       sv = fmaf(xsT[(size_t)t * np + q], xsT[(size_t)t * np + c0 + cl], sv);
                               if constexpr (TANI) {
                                   const int col = c0 + cl;
                                   sv = tani_coarse_f32(sv, q >= 0 ? tnorm[q] : make_float2(0.0f, 0.0f),
                                                    col < n ? tnorm[col] : make_float2(0.0f, 0.0f));
                               }
                               return sv;
                           });
    }
    cp_async_wait<0>();
    __syncthreads();
    write_lists(L_s, L_i, tau_s, LCAP, cap, lstride, n, nq, q0, part_stride, row_of, cand_idx, cand_score, tau_out);
}

constexpr int kc_for(int slots) { return slots <= 2 ? 32 : 16; }

size_t coarse_smem_bytes_kc(int slots) {
    const size_t lcap = 32 * (size_t)slots;
    return (size_t)STAGES * kc_for(slots) * (BM + BN) * 4 + (size_t)BM * lcap * 8 + (size_t)BM * BUF * 8 + BM * 4 * 4;
}

template <int S>
cudaError_t launch_kc(const float* xsT, int n, int np, int dp, int cap, int lstride, const uint32_t* qlist,
                      const unsigned* qcount, int segs, int grid_rows, int part_stride, const float* tfloor, const float2* tnorm,
                      uint32_t* cand_idx, float* cand_score, float* tau, cudaStream_t st) {
    constexpr int KC = kc_for(S);
    const size_t smem = coarse_smem_bytes_kc(S);
    auto kern = tnorm ? k_coarse_fp32_kc<S, KC, true> : k_coarse_fp32_kc<S, KC, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<dim3(grid_rows ? (grid_rows + BM - 1) / BM : np / BM, segs), NT, smem, st>>>(
        xsT, n, np, dp, cap, lstride, qlist, qcount, part_stride, tfloor, tnorm, cand_idx, cand_score, tau);
    note_launch();
    return cudaGetLastError();
}

size_t coarse_smem_bytes(int dp, int slots) {
    const size_t lcap = 32 * (size_t)slots;
    return (size_t)dp * BM * 4 + (size_t)STAGES * dp * BN * 4 + (size_t)BM * lcap * 8 + (size_t)BM * BUF * 8 +
           BM * 4 * 4;
}

template <int S, int D>
cudaError_t launch_one(const float* xsT, int n, int np, int dp, int cap, int lstride, const uint32_t* qlist,
                       const unsigned* qcount, int segs, int grid_rows, int part_stride, const float* tfloor,
                       const float2* tnorm, uint32_t* cand_idx, float* cand_score, float* tau, cudaStream_t st) {
    const size_t smem = coarse_smem_bytes(dp, S);
    // (the Tanimoto variant is built only for a run-time depth: dispatch_d sends it there)
    auto kern = k_coarse_fp32<S, D, false>;
    if constexpr (D == 0)
        if (tnorm) kern = k_coarse_fp32<S, 0, true>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<dim3(grid_rows ? (grid_rows + BM - 1) / BM : np / BM, segs), NT, smem, st>>>(
        xsT, n, np, dp, cap, lstride, qlist, qcount, part_stride, tfloor, tnorm, cand_idx, cand_score, tau);
    note_launch();
    return cudaGetLastError();
}

template <int S>
cudaError_t dispatch_d(const float* xsT, int n, int np, int dp, int cap, int lstride, const uint32_t* qlist,
                       const unsigned* qcount, int segs, int grid_rows, int part_stride, const float* tfloor,
                       const float2* tnorm, uint32_t* cand_idx, float* cand_score, float* tau, cudaStream_t st) {
#define COSTAL_D(D)                                                                                            \
    case D:                                                                                                    \
        return launch_one<S, D>(xsT, n, np, dp, cap, lstride, qlist, qcount, segs, grid_rows, part_stride, tfloor, \
                                tnorm, cand_idx, cand_score, tau, st);
    if (tnorm)
        return launch_one<S, 0>(xsT, n, np, dp, cap, lstride, qlist, qcount, segs, grid_rows, part_stride, tfloor,
                                tnorm, cand_idx, cand_score, tau, st);
    switch (dp) {
        COSTAL_D(8) COSTAL_D(16) COSTAL_D(24) COSTAL_D(32) COSTAL_D(40) COSTAL_D(48) COSTAL_D(56) COSTAL_D(64)
        default:
            return launch_one<S, 0>(xsT, n, np, dp, cap, lstride, qlist, qcount, segs, grid_rows, part_stride,
                                    tfloor, tnorm, cand_idx, cand_score, tau, st);
    }
#undef COSTAL_D
}

cudaError_t launch_any(const float* xsT, int n, int np, int dp, int cap, int lstride, const uint32_t* qlist,
                       const unsigned* qcount, int segs, int grid_rows, int part_stride, const float* tfloor,
                       const float2* tnorm, uint32_t* cand_idx, float* cand_score, float* tau, cudaStream_t st) {
#define COSTAL_ARGS xsT, n, np, dp, cap, lstride, qlist, qcount, segs, grid_rows, part_stride, tfloor, tnorm, cand_idx, \
    cand_score, tau, st
    if (dp > 64) {  // deep rows: the chunked kernel
        switch (coarse_slots(cap)) {
            case 1: return launch_kc<1>(COSTAL_ARGS);
            case 2: return launch_kc<2>(COSTAL_ARGS);
            case 4: return launch_kc<4>(COSTAL_ARGS);
            default: return cudaErrorInvalidValue;
        }
    }
    switch (coarse_slots(cap)) {
        case 1: return dispatch_d<1>(COSTAL_ARGS);
        case 2: return dispatch_d<2>(COSTAL_ARGS);
        case 4: return launch_one<4, 0>(COSTAL_ARGS);
        default: return cudaErrorInvalidValue;
    }
#undef COSTAL_ARGS
}

// One warp per listed row: the union of its segments' lists (segs · cap entries) as (score desc,
// index asc) keys, 256 at a time: after each warp sort the first cap positions hold the best so far
// and the other 256 − cap take the next entries. The best cap go to the row's candidates, and τ is
// the cap-th score (≥ every segment's own τ, since a full segment list holds cap entries at or above
// it), or the row's floor when the segments hold fewer than cap together.
__global__ void k_merge_parts(const uint32_t* __restrict__ qlist, int count, int segs, int cap,
                              const uint32_t* __restrict__ part_idx, const float* __restrict__ part_score,
                              const float* __restrict__ tfloor, int lstride, uint32_t* __restrict__ cand_idx,
                              float* __restrict__ cand_score, float* __restrict__ tau_out) {
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= count) return;
    const int total = segs * cap;
    auto load = [&](int e) {
        if (e >= total) return PAD_KEY;
        const size_t o = ((size_t)(e / cap) * count + r) * cap + e % cap;
        return order_key(part_score[o], part_idx[o]);
    };
    uint64_t key[8];
#pragma unroll
    for (int s = 0; s < 8; ++s) key[s] = load(s * 32 + lane);
    warp_sort_keys<8>(key, lane);
    for (int next = 256; next < total; next += 256 - cap) {  // warp-uniform
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const int p = s * 32 + lane;
            if (p >= cap) key[s] = load(next + p - cap);
        }
        warp_sort_keys<8>(key, lane);
    }
    const uint32_t q = qlist[r];
    uint64_t kth = 0;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int p = s * 32 + lane;
        if (p < cap) {
            cand_idx[(size_t)q * lstride + p] = key_index(key[s]);
            cand_score[(size_t)q * lstride + p] = key_score(key[s]);
        }
        if (s == (cap - 1) >> 5) kth = key[s];
    }
    const uint64_t t = __shfl_sync(COSTAL_FULL_MASK, kth, (cap - 1) & 31);
    // with fewer than cap candidates in all segments together, the row's floor still bounds the rest
    if (lane == 0) tau_out[q] = fmaxf(key_score(t), tfloor ? tfloor[q] : -CUDART_INF_F);
}

}  // namespace plain

size_t coarse_fp32_smem(int dp, int cap) {
    return dp > 64 ? plain::coarse_smem_bytes_kc(coarse_slots(cap)) : plain::coarse_smem_bytes(dp, coarse_slots(cap));
}

int coarse_dpad(int d) { return d <= 64 ? ((d < 1 ? 1 : d) + 7) / 8 * 8 : (d + 3) / 4 * 4; }

cudaError_t launch_coarse_fp32(const float* xsT, int n, int np, int dp, int cap, int lstride, const uint32_t* qlist,
                               const unsigned* qcount, uint32_t* cand_idx, float* cand_score, float* tau,
                               cudaStream_t st) {
    return plain::launch_any(xsT, n, np, dp, cap, lstride, qlist, qcount, 1, 0, 0, nullptr, nullptr, cand_idx, cand_score,
                             tau, st);
}

// The rows' f32 norm and squared norm from the f64 norms (knn.rs:207-212 rounds ‖x‖² to f32).
__global__ void k_tani_norms(const double* __restrict__ norms, int n, float2* __restrict__ tnorm) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double a = norms[i];
        tnorm[i] = make_float2((float)a, (float)(a * a));
    }
}

cudaError_t launch_coarse_fp32_tanimoto(const float* xsT, int n, int np, int dp, int cap, const double* norms,
                                        float2* tnorm, uint32_t* cand_idx, float* cand_score, float* tau,
                                        cudaStream_t st) {
    k_tani_norms<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, st>>>(norms, n, tnorm); note_launch();
    return plain::launch_any(xsT, n, np, dp, cap, cap, nullptr, nullptr, 1, 0, 0, nullptr, tnorm, cand_idx, cand_score,
                             tau, st);
}

namespace {
inline size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }
}  // namespace

size_t tani_window_bytes(int n, int np, int dp) {
    const size_t ntiles = (size_t)np / plain::BN;
    return al256((size_t)dp * np * 4) + al256((size_t)n * 8) * 2 + al256(ntiles * 8) * 2 + 256;
}

cudaError_t launch_coarse_tani_window(const float* xsT, int n, int np, int dp, int cap, const double* norms,
                                      const uint32_t* perm, void* ws, uint32_t* cand_idx, float* cand_score,
                                      float* tau, unsigned long long* skipped_total, cudaStream_t st) {
    using namespace plain;
    if (dp > 64) return cudaErrorInvalidValue;
    const int ntiles = np / BN;
    char* p = static_cast<char*>(ws);
    float* xsW = reinterpret_cast<float*>(p);
    p += al256((size_t)dp * np * 4);
    float2* tnW = reinterpret_cast<float2*>(p);
    p += al256((size_t)n * 8);
    double* normW = reinterpret_cast<double*>(p);
    p += al256((size_t)n * 8);
    double* lo = reinterpret_cast<double*>(p);
    p += al256((size_t)ntiles * 8);
    double* hi = reinterpret_cast<double*>(p);
    const size_t total = (size_t)dp * np;
    k_tani_gather<<<(unsigned)std::min<size_t>((total + 255) / 256, 8192), 256, 0, st>>>(xsT, n, np, dp, perm, xsW);
    note_launch();
    k_tani_norms_w<<<(n + 255) / 256, 256, 0, st>>>(norms, n, perm, tnW, normW); note_launch();
    k_tile_norm_range<<<(ntiles + 7) / 8, 256, 0, st>>>(normW, n, ntiles, lo, hi); note_launch();
    k_tile_norm_envelope<<<1, 32, 0, st>>>(ntiles, lo, hi); note_launch();
    const int slots = coarse_slots(cap);
    const size_t smem = coarse_smem_bytes(dp, slots);
    auto kern = slots == 1 ? k_coarse_tani_window<1> : (slots == 2 ? k_coarse_tani_window<2> : k_coarse_tani_window<4>);
    if (slots == 0) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<np / BM, NT, smem, st>>>(xsW, n, np, dp, cap, tnW, normW, lo, hi, perm, cand_idx, cand_score, tau,
                                    skipped_total);
    note_launch();
    return cudaGetLastError();
}

int coarse_fp32_segments(int count, int np, int sm_count) {
    // enough CTAs for two per SM; the merge reads segs · cap entries per row, 256 − cap at a time
    const int qblocks = (count + plain::BM - 1) / plain::BM, all = np / plain::BN;
    int segs = (2 * sm_count + qblocks - 1) / qblocks;
    segs = std::min(segs, 64);
    segs = std::min(segs, all / 2);
    if (segs <= 1) return 1;
    const int tps = (all + segs - 1) / segs;
    return (all + tps - 1) / tps;  // no empty segment
}

cudaError_t launch_coarse_fp32_split(const float* xsT, int n, int np, int dp, int cap, int lstride,
                                     const uint32_t* qlist, const unsigned* qcount, int count, int segs,
                                     const float* tfloor, uint32_t* part_idx, float* part_score, float* part_tau,
                                     uint32_t* cand_idx, float* cand_score, float* tau, cudaStream_t st) {
    if (segs <= 1)
        return plain::launch_any(xsT, n, np, dp, cap, lstride, qlist, qcount, 1, count, 0, tfloor, nullptr, cand_idx,
                                 cand_score, tau, st);
    cudaError_t e = plain::launch_any(xsT, n, np, dp, cap, lstride, qlist, qcount, segs, count, count, tfloor, nullptr,
                                      part_idx, part_score, part_tau, st);
    if (e != cudaSuccess) return e;
    plain::k_merge_parts<<<(count + 7) / 8, 256, 0, st>>>(qlist, count, segs, cap, part_idx, part_score, tfloor,
                                                          lstride, cand_idx, cand_score, tau);
    note_launch();
    return cudaGetLastError();
}

// The re-run's floor for each listed row, from the tensor-core pass it follows: when that pass kept a
// full list of cap candidates above its threshold τ, their exact cosines are ≥ τ − E_i, so the row's
// cap-th FP32 score is ≥ τ − E_i − ε; below that no column can be among the best cap (rounded down).
__global__ void k_rerun_floor(const uint32_t* __restrict__ rows, const unsigned* __restrict__ count, int cap,
                              const float* __restrict__ tau, const float* __restrict__ cand_score,
                              const double* __restrict__ row_eps, double eps, float* __restrict__ tfloor) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (int)*count) return;
    const uint32_t i = rows[r];
    const bool full = cand_score[(size_t)i * cap + cap - 1] > -CUDART_INF_F;
    tfloor[i] = full ? __double2float_rd(__dsub_rd(__dsub_rd((double)tau[i], row_eps[i]), eps)) : -CUDART_INF_F;
}

cudaError_t launch_rerun_floor(const uint32_t* rows, const unsigned* count, int nmax, int cap, const float* tau,
                               const float* cand_score, const double* row_eps, double eps, float* tfloor,
                               cudaStream_t st) {
    if (nmax <= 0) return cudaSuccess;
    k_rerun_floor<<<(nmax + 255) / 256, 256, 0, st>>>(rows, count, cap, tau, cand_score, row_eps, eps, tfloor);
    note_launch();
    return cudaGetLastError();
}

}  // namespace costal
