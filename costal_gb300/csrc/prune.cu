// Locality order and block pruning for the tensor-core coarse pass.
//
// The reference visits column blocks in index order and prunes only for Tanimoto selection, by norm
// windows (crates/costal-core/src/knn.rs:603-644, :272-283). This file gives the cosine path the same
// two levers, with bounds that hold for the exact scores:
//
//   cells     spherical k-means (K = 256 centroids, a seeded sample of rows, a few Lloyd steps with
//             deterministic centroid sums) and the cell of every row;
//   order     a working order: rows stably sorted by cell (ties by original index). The tensor
//             operands are laid out in this order; candidates are mapped back to original indices.
//   geometry  for every 128-row query block Q and every column block B (128 working rows, or 256 for
//             lists longer than the sort takes; prune.h col_block) a
//             unit centre c and an angular radius r = max angle(row, c), in f64;
//   bound     for q ∈ Q, x ∈ B: angle(q, x) ≥ angle(c_Q, c_B) − r_Q − r_B (the angle is a metric on
//             the sphere), so cos(q, x) ≤ UB(Q, B) = cos(max(0, angle(c_Q, c_B) − r_Q − r_B − ξ)),
//             with ξ = 1e-6 rad covering the f32 rounding of the normalised rows (≤ 1e-7 rad); UB is
//             evaluated in f32 with directed roundings and margins for the f32 dot, acosf and cosf
//             (block_ub_f32), so it stays an upper bound;
//   row bound with M[Q][B] = the largest coarse score q·c_B over the rows q ∈ Q (tensor cores,
//             knn_tc.cu) and its margin δ: angle(q, c_B) ≥ acos(M + δ) for every q ∈ Q, so
//             cos(q, x) ≤ cos(max(0, acos(M + δ) − r_B − ξ)), evaluated like UB (row_ub_f32). It
//             drops the query block's radius, which the triangle inequality charges in full
//             although in d dimensions the rows spread mostly across the direction to c_B; the
//             lists use the smaller of the two bounds;
//   lists     for every Q, the column blocks with UB ≥ t_Q, sorted by UB descending (the closest
//             blocks first, so a query's threshold rises to its final value within the first tiles),
//             and ub_skip[Q] = the largest UB of a skipped block. A query is certified only if its
//             k-th exact score is strictly above ub_skip of its block; otherwise it is rescanned.

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "prune.h"

namespace costal {
namespace prune {

constexpr int KM_BLOCK = 128;

// ---- k-means ----------------------------------------------------------------------------------

// Rows of xsT (d × np, transposed) listed in `rows` → a row-major [m][d] copy.
__global__ void k_gather_rows(const float* __restrict__ xsT, int np, int d, const uint32_t* __restrict__ rows, int m,
                              float* __restrict__ out) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * d; e += gridDim.x * blockDim.x) {
        const int i = e / d, t = e % d;
        out[e] = xsT[(size_t)t * np + rows[i]];
    }
}

// Best centroid (largest dot with the unit centroid) of every row; rows are either a row-major
// [m][d] array (rows_rm) or the columns of xsT. Centroids live in shared memory, rows padded to a
// multiple of 4 with zeros, read 16 bytes at a time (every thread reads the same centroid: a
// broadcast); the dot keeps the dimension order.
__global__ void __launch_bounds__(KM_BLOCK) k_assign(const float* __restrict__ rows_rm, const float* __restrict__ xsT,
                                                     int np, int m, int d, const float* __restrict__ cent, int K,
                                                     uint32_t* __restrict__ assign) {
    extern __shared__ float4 c_s4[];  // [K][dq/4]
    float* c_s = reinterpret_cast<float*>(c_s4);
    const int dq = (d + 3) & ~3, q4 = dq >> 2;
    for (int e = threadIdx.x; e < K * dq; e += blockDim.x) {
        const int c = e / dq, t = e - c * dq;
        c_s[e] = t < d ? cent[c * d + t] : 0.0f;
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    float x[64];
#pragma unroll
    for (int t = 0; t < 64; ++t) x[t] = t < d ? (rows_rm ? rows_rm[(size_t)i * d + t] : xsT[(size_t)t * np + i]) : 0.0f;
    float best = -CUDART_INF_F;
    uint32_t arg = 0;
    for (int c = 0; c < K; ++c) {
        float s = 0.0f;
#pragma unroll
        for (int t4 = 0; t4 < 16; ++t4) {
            if (t4 < q4) {
                const float4 w = c_s4[c * q4 + t4];
                s = fmaf(x[4 * t4], w.x, s);
                s = fmaf(x[4 * t4 + 1], w.y, s);
                s = fmaf(x[4 * t4 + 2], w.z, s);
                s = fmaf(x[4 * t4 + 3], w.w, s);
            }
        }
        if (s > best) {
            best = s;
            arg = (uint32_t)c;
        }
    }
    assign[i] = arg;
}

// One CTA per centroid: the normalised sum of its rows, summed in a fixed order (deterministic): the
// rows fall into 128 classes by (row / 4) mod 128, each class adds its rows in row order, and the 128
// class sums are combined by a fixed pairwise tree. Warp w takes classes 16w … 16w+15 one after the
// other, lane t holding dimensions t and t + 32: the class's assignment words are loaded four per
// lane at once and its matches found by ballots, so the warp's branches are uniform and a row is read
// coalesced. An empty cluster keeps its previous centroid.
constexpr int UPD_T = 256;
constexpr int UPD_CLASSES = 128;
constexpr int UPD_GROUPS = 128;  // word groups of a class: m ≤ 4 · 128 · 128 rows
static_assert(4 * UPD_CLASSES * UPD_GROUPS >= SAMPLE, "the centroid update covers the k-means sample");
__global__ void __launch_bounds__(UPD_T) k_centroid_update(const float* __restrict__ rows, int m, int d,
                                                           const uint32_t* __restrict__ assign, float* __restrict__ cent) {
    constexpr int NW = UPD_T / 32, CPW = UPD_CLASSES / NW;
    __shared__ float part[UPD_CLASSES][65];
    __shared__ int cnt_s[UPD_CLASSES];
    __shared__ float nrm;
    const int c = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m4 = m & ~3;
    for (int k = 0; k < CPW; ++k) {
        const int cls = warp * CPW + k;
        float s0 = 0.0f, s1 = 0.0f;
        int cnt = 0;
        auto add_row = [&](int i) {
            ++cnt;
            if (lane < d) s0 += rows[(size_t)i * d + lane];
            if (lane + 32 < d) s1 += rows[(size_t)i * d + lane + 32];
        };
        // the class's word groups q = 0 … 127 (rows 4·cls + 512·q …+3), four per lane, all loaded at
        // once; then the matches are added in row order: group by group (ballot, lowest lane first)
        // and within a group by row
        uint32_t mask[UPD_GROUPS / 32];
#pragma unroll
        for (int r = 0; r < UPD_GROUPS / 32; ++r) {
            const int i4 = 4 * cls + 4 * UPD_CLASSES * (r * 32 + lane);
            mask[r] = 0u;
            if (i4 < m4) {
                const uint4 a = *reinterpret_cast<const uint4*>(assign + i4);  // (the array is 256-byte aligned)
                mask[r] = (a.x == (uint32_t)c ? 1u : 0u) | (a.y == (uint32_t)c ? 2u : 0u) |
                          (a.z == (uint32_t)c ? 4u : 0u) | (a.w == (uint32_t)c ? 8u : 0u);
            }
        }
#pragma unroll
        for (int r = 0; r < UPD_GROUPS / 32; ++r) {
            unsigned any = __ballot_sync(COSTAL_FULL_MASK, mask[r] != 0u);
            while (any) {
                const int L = __ffs(any) - 1;
                any &= any - 1;
                unsigned mk = __shfl_sync(COSTAL_FULL_MASK, mask[r], L);
                const int i4 = 4 * cls + 4 * UPD_CLASSES * (r * 32 + L);
                while (mk) {
                    add_row(i4 + __ffs(mk) - 1);
                    mk &= mk - 1;
                }
            }
        }
        if (m4 + cls < m && assign[m4 + cls] == (uint32_t)c) add_row(m4 + cls);  // the last m mod 4 rows
        if (lane < d) part[cls][lane] = s0;
        if (lane + 32 < d) part[cls][lane + 32] = s1;
        if (lane == 0) cnt_s[cls] = cnt;
    }
    __syncthreads();
    for (int s = UPD_CLASSES / 2; s > 0; s >>= 1) {
        for (int e = threadIdx.x; e < s * d; e += UPD_T) {
            const int cls = e / d, t = e - cls * d;
            part[cls][t] += part[cls + s][t];
        }
        if ((int)threadIdx.x < s) cnt_s[threadIdx.x] += cnt_s[threadIdx.x + s];
        __syncthreads();
    }
    if (cnt_s[0] == 0) return;
    if (threadIdx.x == 0) {
        double nn = 0.0;
        for (int t = 0; t < d; ++t) nn += (double)part[0][t] * part[0][t];
        nrm = (float)sqrt(nn);
    }
    __syncthreads();
    if ((int)threadIdx.x < d && nrm > 0.0f) cent[(size_t)c * d + threadIdx.x] = part[0][threadIdx.x] / nrm;
}

// ---- working order: stable counting sort of rows by cell -------------------------------------

constexpr int CHUNK = 1024;

__global__ void k_cell_hist(const uint32_t* __restrict__ cell, int n, int K, uint32_t* __restrict__ hist) {
    // one thread per chunk, sequential over its rows (deterministic)
    const int ch = blockIdx.x * blockDim.x + threadIdx.x;
    const int nch = (n + CHUNK - 1) / CHUNK;
    if (ch >= nch) return;
    uint32_t* h = hist + (size_t)ch * K;
    for (int c = 0; c < K; ++c) h[c] = 0;
    const int end = min(n, (ch + 1) * CHUNK);
    for (int i = ch * CHUNK; i < end; ++i) h[cell[i]] += 1;
}

// Exclusive offsets in (cell, chunk) order: thread c totals its cell over the chunks, one warp
// scans the K totals, then thread c rewrites its column of the histogram as offsets.
__global__ void k_cell_scan(uint32_t* __restrict__ hist, int nch, int K, uint32_t* __restrict__ cell_start) {
    __shared__ uint32_t tot[1024];
    const int c = threadIdx.x;
    uint32_t s = 0;
    if (c < K)
        for (int ch = 0; ch < nch; ++ch) s += hist[(size_t)ch * K + c];
    tot[c] = s;
    __syncthreads();
    if (c == 0) {
        uint32_t acc = 0;
        for (int j = 0; j < K; ++j) {
            const uint32_t v = tot[j];
            tot[j] = acc;
            acc += v;
        }
        cell_start[K] = acc;
    }
    __syncthreads();
    if (c < K) {
        uint32_t acc = tot[c];
        cell_start[c] = acc;
        for (int ch = 0; ch < nch; ++ch) {
            const uint32_t v = hist[(size_t)ch * K + c];
            hist[(size_t)ch * K + c] = acc;
            acc += v;
        }
    }
}

__global__ void k_cell_scatter(const uint32_t* __restrict__ cell, int n, int K, uint32_t* __restrict__ hist,
                               uint32_t* __restrict__ perm) {
    const int ch = blockIdx.x * blockDim.x + threadIdx.x;
    const int nch = (n + CHUNK - 1) / CHUNK;
    if (ch >= nch) return;
    uint32_t* h = hist + (size_t)ch * K;
    const int end = min(n, (ch + 1) * CHUNK);
    for (int i = ch * CHUNK; i < end; ++i) perm[h[cell[i]]++] = (uint32_t)i;
}

// ---- block geometry -------------------------------------------------------------------------------

// One CTA per block of `bs` consecutive working rows (wrows: the normalised rows in working order,
// row-major [n][d]): centre = normalised f64 sum (row order), radius = the largest angle between a row
// and the centre (f64). Rows past n are ignored.
__global__ void k_block_geom(const float* __restrict__ wrows, int d, int n, int bs, double* __restrict__ center,
                             double* __restrict__ radius, float* __restrict__ center_f, float* __restrict__ radius_f) {
    __shared__ double c_s[64];
    __shared__ double red[256];
    const int b = blockIdx.x;
    const int r0 = b * bs, r1 = min(n, r0 + bs);
    if (threadIdx.x < d) {
        double s = 0.0;
        for (int w = r0; w < r1; ++w) s += (double)wrows[(size_t)w * d + threadIdx.x];
        c_s[threadIdx.x] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double nn = 0.0;
        for (int t = 0; t < d; ++t) nn += c_s[t] * c_s[t];
        const double inv = nn > 0.0 ? 1.0 / sqrt(nn) : 0.0;
        for (int t = 0; t < d; ++t) c_s[t] *= inv;
    }
    __syncthreads();
    if (threadIdx.x < d) {
        center[(size_t)b * d + threadIdx.x] = c_s[threadIdx.x];
        if (center_f) center_f[(size_t)threadIdx.x * gridDim.x + b] = (float)c_s[threadIdx.x];  // [d][blocks]
    }
    // The radius in f32 with a rigorous margin: the rows are unit vectors to within (d + 2)·2⁻²⁴, the
    // f32 centre is the f64 one to 2⁻²⁴ per component, and the f32 dot and norm accumulate at most
    // d·2⁻²⁴ of relative error each, so the f32 cosine is within (2d + 8)·2⁻²⁴ of the exact one; twice
    // that is subtracted before acosf (itself within a few ulp, covered by 1e-6 rad), and every step
    // rounds up. A zero row has cosine 0 with everything: angle π/2 covers it.
    __shared__ float cf_s[64];
    if (threadIdx.x < d) cf_s[threadIdx.x] = (float)c_s[threadIdx.x];
    __syncthreads();
    const float margin = (float)(2 * d + 8) * 0x1p-23f;
    float worst = 0.0f;
    for (int w = r0 + threadIdx.x; w < r1; w += blockDim.x) {
        const float* row = wrows + (size_t)w * d;
        float dot = 0.0f, nn = 0.0f;
        for (int t = 0; t < d; ++t) {
            const float v = row[t];
            dot = fmaf(v, cf_s[t], dot);
            nn = fmaf(v, v, nn);
        }
        float ang = 1.57079637f;  // ≥ π/2
        if (nn > 0.0f) {
            const float cs = __fsub_rd(__fdiv_rd(dot, __fsqrt_ru(nn)), margin);
            ang = __fadd_ru(acosf(fminf(1.0f, fmaxf(-1.0f, cs))), 1e-6f);
        }
        worst = fmaxf(worst, ang);
    }
    red[threadIdx.x] = (double)worst;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        radius[b] = red[0];
        if (radius_f) {
            float rf = (float)red[0];
            if ((double)rf < red[0]) rf = nextafterf(rf, CUDART_INF_F);  // rounded up
            radius_f[b] = rf;
        }
    }
}

// ---- per-query-block lists ------------------------------------------------------------------------

constexpr int LIST_T = 512;
constexpr double XI = 1e-6;

// A list sort's shape: KPT keys per thread over LIST_T threads (16 → 8,192 column blocks, two CTAs
// per SM; 32 → 16,384, one CTA per SM with the keys in its registers). A key is 32 bits: a level of
// SBITS = 32 − ID_BITS bits above the complemented block id (ID_BITS bits). Levels [1, ONE) hold a
// bound u < 1 rounded up to a multiple of Q = 2 / ONE (u ≤ level·Q − 1 + Q); levels [ONE, 2·ONE) hold
// the blocks whose bound is 1, nearest centre first. Descending keys: larger bound first, then (at
// bound 1) smaller centre angle, then smaller block id.
template <int KPT>
struct ListShape {
    static constexpr int N = LIST_T * KPT;
    static constexpr int ID_BITS = KPT <= 16 ? 13 : 14;
    static constexpr uint32_t ID_MAX = (1u << ID_BITS) - 1u;
    static constexpr int SBITS = 32 - ID_BITS;
    static constexpr uint32_t ONE = 1u << (SBITS - 1);     // first level of the bound-1 range
    static constexpr float SCALE = (float)(1u << (SBITS - 2));  // levels per unit of (u + 1)
};

// The key of column block b with bound u (≤ 1) and centre angle φ (0 for a padding key never occurs:
// every key of a kept block is non-zero).
template <int KPT>
__device__ __forceinline__ uint32_t list_key(float u, float phi, int b) {
    using LS = ListShape<KPT>;
    uint32_t level;
    if (u >= 1.0f) {
        const float q = fmaxf(0.0f, phi) * ((float)LS::ONE / 3.14159265f);
        level = (2u * LS::ONE - 1u) - (uint32_t)fminf((float)(LS::ONE - 1u), q);
    } else {
        // ⌊(u + 1)·SCALE⌋ with u + 1 rounded up: level·Q − 1 + Q ≥ u holds for the level kept
        const float f = floorf(__fadd_ru(fmaxf(u, -1.0f), 1.0f) * LS::SCALE);
        level = (uint32_t)fminf((float)(LS::ONE - 1u), fmaxf(1.0f, f));
    }
    return (level << LS::ID_BITS) | (LS::ID_MAX - (uint32_t)b);
}

// The bound a key stands for: 1 in the bound-1 range, else the top of its level (exact in f32).
template <int KPT>
__device__ __forceinline__ float key_bound(uint32_t key) {
    using LS = ListShape<KPT>;
    const uint32_t level = key >> LS::ID_BITS;
    if (level >= LS::ONE) return 1.0f;
    return (float)(level + 1u) * (1.0f / LS::SCALE) - 1.0f;
}

// The bound in f32 for one (query block, column block) pair, rigorous for the f64 geometry: the
// f32 FMA dot of the two unit centres (each rounded to f32) is within (d + 2)·2⁻²⁴ of the f64 value,
// so acos(dot + δ) with δ = (d + 4)·2⁻²³, the sum rounded up, never exceeds the centres' angle;
// acosf and cosf are within a few ulp, covered by 1e-6 on each side; every subtraction rounds down
// and the final addition up. Radii arrive rounded up to f32.
// Also returns (in *phi_out) the centres' angle, used only to order blocks of equal bound.
__device__ __forceinline__ float block_ub_f32(const float* cq, float rq, const float* cb, int cstride, float rb, int d,
                                             float* phi_out = nullptr) {
    float dot = 0.0f;
    for (int t = 0; t < d; ++t) dot = fmaf(cq[t], cb[(size_t)t * cstride], dot);
    const float delta = (float)(d + 4) * 0x1p-23f;
    const float c = fminf(1.0f, __fadd_ru(dot, delta));
    const float phi = __fsub_rd(acosf(c), 1e-6f);
    if (phi_out) *phi_out = phi;
    const float th = __fsub_rd(__fsub_rd(__fsub_rd(phi, rq), rb), (float)XI);
    if (th <= 0.0f) return 1.0f;
    return fminf(1.0f, __fadd_ru(cosf(th), 1e-6f));
}

// The per-row bound in f32 from M = max over the query block's rows of the coarse q·c_B and its
// margin δ (M + δ ≥ the largest exact cosine of a row with c_B); radii arrive rounded up to f32,
// acosf and cosf are covered by 1e-6 on each side, subtractions round down, the last addition up.
__device__ __forceinline__ float row_ub_f32(float m, float delta, float rb) {
    const float c = fmaxf(-1.0f, fminf(1.0f, __fadd_ru(m, delta)));
    const float th = __fsub_rd(__fsub_rd(__fsub_rd(acosf(c), 1e-6f), rb), (float)XI);
    if (th <= 0.0f) return 1.0f;
    return fminf(1.0f, __fadd_ru(cosf(th), 1e-6f));
}

// Compare-exchange of list keys (descending) at a register distance S within a thread's run.
template <int S, int KPT>
__device__ __forceinline__ void cx_regs(uint32_t (&v)[KPT], int base, int size) {
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        const int p = j ^ S;
        if (p > j) {
            const bool desc = ((base + j) & size) == 0;
            const uint32_t a = v[j], b = v[p];
            const uint32_t hi = max(a, b), lo = min(a, b);
            v[j] = desc ? hi : lo;
            v[p] = desc ? lo : hi;
        }
    }
}

// Bitonic sort (descending) of the CTA's LIST_T·KPT keys, KPT per thread at positions base..base+KPT−1:
// compare-exchanges in registers, by warp shuffles, or through shared memory (xk) by distance.
template <int KPT>
__device__ __forceinline__ void block_sort_keys(uint32_t (&v)[KPT], uint32_t* xk, int base, int lane) {
    constexpr int N = LIST_T * KPT;
    for (int size = 2; size <= N; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= KPT * 32) {  // across warps
                __syncthreads();
#pragma unroll
                for (int j = 0; j < KPT; ++j) xk[base + j] = v[j];
                __syncthreads();
#pragma unroll
                for (int j = 0; j < KPT; ++j) {
                    const int e = base + j;
                    const uint32_t o = xk[e ^ stride];
                    const bool keep_max = ((e & stride) == 0) == ((e & size) == 0);
                    const uint32_t hi = max(v[j], o), lo = min(v[j], o);
                    v[j] = keep_max ? hi : lo;
                }
            } else if (stride >= KPT) {  // within the warp
                const int lstride = stride / KPT;
#pragma unroll
                for (int j = 0; j < KPT; ++j) {
                    const int e = base + j;
                    const uint32_t o = __shfl_xor_sync(COSTAL_FULL_MASK, v[j], lstride);
                    const bool keep_max = ((lane & lstride) == 0) == ((e & size) == 0);
                    const uint32_t hi = max(v[j], o), lo = min(v[j], o);
                    v[j] = keep_max ? hi : lo;
                }
            } else if (stride == 16) {
                if constexpr (KPT > 16) cx_regs<16>(v, base, size);
            } else if (stride == 8) {
                if constexpr (KPT > 8) cx_regs<8>(v, base, size);
            } else if (stride == 4) {
                if constexpr (KPT > 4) cx_regs<4>(v, base, size);
            } else if (stride == 2) {
                cx_regs<2>(v, base, size);
            } else {
                cx_regs<1>(v, base, size);
            }
        }
    }
}

// The sorted keys out (keys of ListShape<KPT_ALL>, KPT per thread): list position e holds block
// ID_MAX − (low ID_BITS bits) and the bound its level stands for.
template <int KPT, int KPT_ALL>
__device__ __forceinline__ void write_keys(const uint32_t (&v)[KPT], int base, unsigned nk, uint32_t* out, float* out_ub) {
    using LS = ListShape<KPT_ALL>;
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        const unsigned e = (unsigned)(base + j);
        if (e < nk) {
            out[e] = LS::ID_MAX - (v[j] & LS::ID_MAX);
            out_ub[e] = key_bound<KPT_ALL>(v[j]);
        }
    }
}

// Compact the kept keys (non-zero) of every thread into xk[0 .. kept) in any order, zero-fill up to
// LIST_T·KPT, and load KPT of them per thread.
template <int KPT, int KPT_ALL>
__device__ __forceinline__ void compact_keys(const uint32_t (&all)[KPT_ALL], uint32_t (&v)[KPT], uint32_t* xk,
                                             unsigned* slot, unsigned nk, int base) {
    constexpr int N = LIST_T * KPT;
    for (int e = threadIdx.x + (int)nk; e < N; e += LIST_T) xk[e] = 0u;
#pragma unroll
    for (int j = 0; j < KPT_ALL; ++j)
        if (all[j]) xk[atomicAdd(slot, 1u)] = all[j];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < KPT; ++j) v[j] = xk[base + j];
    __syncthreads();  // every thread has its keys before the sort reuses xk
}

// One CTA per query block: the upper bound against every column block; the blocks kept (UB ≥ t_Q)
// sorted by (UB desc, centre angle asc at UB = 1, block asc) with their bounds rounded up to the keys'
// levels — a bitonic sort of 32-bit keys, 16 per thread, exchanged in registers, by warp shuffles or
// through shared memory by distance — and the largest UB of a skipped block. Lists longer than the
// shape's N stay in block order with bounds +inf.
template <int KPT_ALL>
__global__ void __launch_bounds__(LIST_T, KPT_ALL <= 16 ? 2 : 1)
    k_block_lists(const double* __restrict__ qcenter, const double* __restrict__ qradius,
                  const float* __restrict__ ccenter_f, const float* __restrict__ cradius_f, int nqb, int ncb, int d,
                  const float* __restrict__ tq, const float* __restrict__ rowmax, const float* __restrict__ rm_delta,
                  uint32_t* __restrict__ lists, float* __restrict__ list_ub, uint32_t* __restrict__ counts,
                  float* __restrict__ ub_skip, unsigned long long* __restrict__ skipped_total) {
    using LS = ListShape<KPT_ALL>;
    extern __shared__ uint32_t xk[];  // [LS::N] exchange buffer
    __shared__ float cq[64];
    __shared__ unsigned kept, slot;
    __shared__ int skip_max_bits;
    const int Q = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
    if (tid < d) cq[tid] = (float)qcenter[(size_t)Q * d + tid];
    if (tid == 0) {
        kept = 0;
        slot = 0;
        skip_max_bits = __float_as_int(-CUDART_INF_F);
    }
    __syncthreads();
    float rq = (float)qradius[Q];
    if ((double)rq < qradius[Q]) rq = nextafterf(rq, CUDART_INF_F);
    const float t = tq ? tq[Q] : -CUDART_INF_F;
    const float* rm = rowmax ? rowmax + (size_t)Q * ncb : nullptr;
    const float delta = rowmax ? *rm_delta : 0.0f;
    // the smaller of the cone bound and the per-row bound
    auto bound = [&](int b, float* phi) {
        const float u = block_ub_f32(cq, rq, ccenter_f + b, ncb, cradius_f[b], d, phi);
        return rm ? fminf(u, row_ub_f32(rm[b], delta, cradius_f[b])) : u;
    };
    uint32_t* out = lists + (size_t)Q * ncb;
    float* out_ub = list_ub + (size_t)Q * ncb;
    if (ncb > LS::N) {
        if (tid == 0) {
            unsigned c = 0;
            for (int b = 0; b < ncb; ++b) {
                const float u = bound(b, nullptr);
                if (u >= t) {
                    out_ub[c] = CUDART_INF_F;  // block order: the bounds do not decrease along the list
                    out[c++] = (uint32_t)b;
                } else {
                    skip_max_bits = max(skip_max_bits, __float_as_int(fmaxf(u, 0.0f)));
                }
            }
            kept = c;
        }
    } else {
        const int base = tid * KPT_ALL;
        uint32_t v[KPT_ALL];
        unsigned my_kept = 0;
        int my_skip = __float_as_int(-CUDART_INF_F);
        // keys are computed for blocks j·LIST_T + tid (coalesced reads of the transposed centres); the
        // sort does not care where each key starts
#pragma unroll
        for (int j = 0; j < KPT_ALL; ++j) {
            const int b = j * LIST_T + tid;
            v[j] = 0u;  // absent or skipped: sorts last
            if (b < ncb) {
                float phi;
                const float u = bound(b, &phi);
                if (u >= t) {
                    ++my_kept;
                    // ties of the bound at 1 (e.g. every block of the query's own cluster) go nearest
                    // centre first, then by block
                    v[j] = list_key<KPT_ALL>(u, phi, b);
                } else {
                    // a skipped block's bound, clamped at 0 so that the int order of the bits is the float order
                    my_skip = max(my_skip, __float_as_int(fmaxf(u, 0.0f)));
                }
            }
        }
        atomicAdd(&kept, my_kept);
        atomicMax(&skip_max_bits, my_skip);
        __syncthreads();  // kept is final
        const unsigned nk = kept;
        // Short lists (a learned threshold skips most blocks) sort only their kept keys, compacted.
        if (nk <= (unsigned)(LIST_T * 4)) {
            uint32_t w[4];
            compact_keys<4>(v, w, xk, &slot, nk, tid * 4);
            block_sort_keys<4>(w, xk, tid * 4, lane);
            write_keys<4, KPT_ALL>(w, tid * 4, nk, out, out_ub);
        } else if (nk <= (unsigned)(LIST_T * 8)) {
            uint32_t w[8];
            compact_keys<8>(v, w, xk, &slot, nk, tid * 8);
            block_sort_keys<8>(w, xk, tid * 8, lane);
            write_keys<8, KPT_ALL>(w, tid * 8, nk, out, out_ub);
        } else if (KPT_ALL > 16 && nk <= (unsigned)(LIST_T * 16)) {
            uint32_t w[16];
            compact_keys<16>(v, w, xk, &slot, nk, tid * 16);
            block_sort_keys<16>(w, xk, tid * 16, lane);
            write_keys<16, KPT_ALL>(w, tid * 16, nk, out, out_ub);
        } else {
            // the keys start interleaved over all N positions, so the sort covers all of them
            block_sort_keys<KPT_ALL>(v, xk, base, lane);
            write_keys<KPT_ALL, KPT_ALL>(v, base, nk, out, out_ub);
        }
    }
    __syncthreads();
    if (tid == 0) {
        counts[Q] = kept;
        ub_skip[Q] = __int_as_float(skip_max_bits);
        if (skipped_total) atomicAdd(skipped_total, (unsigned long long)(ncb - (int)kept));
    }
}

// The per-row certificate floor from pruning: ub_skip of the row's query block, or −∞.
__global__ void k_row_ub(const uint32_t* __restrict__ perm, int n, const float* __restrict__ ub_skip,
                         double* __restrict__ row_ub) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= n) return;
    const float u = ub_skip[w / 128];
    row_ub[perm[w]] = u == -CUDART_INF_F ? -CUDART_INF : (double)u;
}

}  // namespace prune
}  // namespace costal

namespace costal {
namespace prune {

namespace {
inline size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }
}  // namespace

bool supported(int d) { return d >= 1 && d <= 64; }

size_t workspace_bytes(int n, int d) {
    const int cb = col_block(n);
    const size_t nqb = (size_t)(n + QB - 1) / QB, ncb = (size_t)(n + cb - 1) / cb;
    const size_t m = (size_t)(n < SAMPLE ? n : SAMPLE), nch = (size_t)(n + CHUNK - 1) / CHUNK;
    return a256(n * 4ull) * 2 + a256((size_t)K_CENTROIDS * d * 4) + a256(nqb * d * 8) + a256(nqb * 8) +
           a256(ncb * d * 8) + a256(ncb * 8) + a256(ncb * d * 4) + a256(ncb * 4) + 2 * a256(nqb * ncb * 4) +
           a256(nqb * 4) + a256(nqb * 4) + a256(n * 8ull) + a256(nqb * 4) + a256(m * d * 4) + a256(m * 4) + a256(nch * K_CENTROIDS * 4) + a256((K_CENTROIDS + 1) * 4) +
           a256(m * 4) + a256((size_t)n * d * 4) + 4096;
}

namespace {
struct Scratch {
    float* sample_rows;
    uint32_t* sample_assign;
    uint32_t* hist;
    uint32_t* cell_start;
    uint32_t* sample_idx;
};

__global__ void k_sample_idx(uint32_t* idx, int m, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) idx[j] = (uint32_t)(((unsigned long long)j * (unsigned long long)n) / (unsigned long long)m);
}

// Initial centroids: K evenly spaced sample rows (deterministic).
__global__ void k_init_centroids(const float* rows, int m, int d, int K, float* cent) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= K * d) return;
    const int c = e / d, t = e % d;
    const int i = (int)(((long long)c * m) / K);
    cent[e] = rows[(size_t)i * d + t];
}
}  // namespace

cudaError_t build_order(void* ws, const float* xsT, int n, int np, int d, cudaStream_t st, Plan& P) {
    const int K = K_CENTROIDS;
    const int cb = col_block(n);
    const int nqb = (n + QB - 1) / QB, ncb = (n + cb - 1) / cb;
    const int m = n < SAMPLE ? n : SAMPLE, nch = (n + CHUNK - 1) / CHUNK;
    char* p = static_cast<char*>(ws);
    auto take = [&](size_t bytes) {
        char* r = p;
        p += a256(bytes);
        return r;
    };
    P.n = n;
    P.d = d;
    P.K = K;
    P.nqb = nqb;
    P.ncb = ncb;
    P.cb = cb;
    P.perm = reinterpret_cast<uint32_t*>(take(n * 4ull));
    P.cell = reinterpret_cast<uint32_t*>(take(n * 4ull));
    P.centroids = reinterpret_cast<float*>(take((size_t)K * d * 4));
    P.qcenter = reinterpret_cast<double*>(take((size_t)nqb * d * 8));
    P.qradius = reinterpret_cast<double*>(take((size_t)nqb * 8));
    P.ccenter = reinterpret_cast<double*>(take((size_t)ncb * d * 8));
    P.cradius = reinterpret_cast<double*>(take((size_t)ncb * 8));
    P.ccenter_f = reinterpret_cast<float*>(take((size_t)ncb * d * 4));
    P.cradius_f = reinterpret_cast<float*>(take((size_t)ncb * 4));
    P.lists = reinterpret_cast<uint32_t*>(take((size_t)nqb * ncb * 4));
    P.list_ub = reinterpret_cast<float*>(take((size_t)nqb * ncb * 4));
    P.counts = reinterpret_cast<uint32_t*>(take((size_t)nqb * 4));
    P.ub_skip = reinterpret_cast<float*>(take((size_t)nqb * 4));
    P.row_ub = reinterpret_cast<double*>(take(n * 8ull));
    P.tq = reinterpret_cast<float*>(take((size_t)nqb * 4));
    Scratch S;
    S.sample_rows = reinterpret_cast<float*>(take((size_t)m * d * 4));
    S.sample_assign = reinterpret_cast<uint32_t*>(take((size_t)m * 4));
    S.hist = reinterpret_cast<uint32_t*>(take((size_t)nch * K * 4));
    S.cell_start = reinterpret_cast<uint32_t*>(take((size_t)(K + 1) * 4));
    S.sample_idx = reinterpret_cast<uint32_t*>(take((size_t)m * 4));
    P.wrows = reinterpret_cast<float*>(take((size_t)n * d * 4));
    P.scratch = S.sample_rows;

    const size_t csm = (size_t)K * ((d + 3) & ~3) * 4;
    cudaError_t e = cudaFuncSetAttribute(k_assign, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm);
    if (e != cudaSuccess) return e;
    k_sample_idx<<<(m + 255) / 256, 256, 0, st>>>(S.sample_idx, m, n); note_launch();
    k_gather_rows<<<1024, 256, 0, st>>>(xsT, np, d, S.sample_idx, m, S.sample_rows); note_launch();
    k_init_centroids<<<(K * d + 255) / 256, 256, 0, st>>>(S.sample_rows, m, d, K, P.centroids); note_launch();
    for (int it = 0; it < LLOYD_STEPS; ++it) {
        k_assign<<<(m + KM_BLOCK - 1) / KM_BLOCK, KM_BLOCK, csm, st>>>(S.sample_rows, nullptr, np, m, d, P.centroids, K,
                                                                         S.sample_assign); note_launch();
        k_centroid_update<<<K, UPD_T, 0, st>>>(S.sample_rows, m, d, S.sample_assign, P.centroids); note_launch();
    }
    k_assign<<<(n + KM_BLOCK - 1) / KM_BLOCK, KM_BLOCK, csm, st>>>(nullptr, xsT, np, n, d, P.centroids, K, P.cell); note_launch();
    k_cell_hist<<<(nch + 127) / 128, 128, 0, st>>>(P.cell, n, K, S.hist); note_launch();
    k_cell_scan<<<1, K, 0, st>>>(S.hist, nch, K, S.cell_start); note_launch();
    k_cell_scatter<<<(nch + 127) / 128, 128, 0, st>>>(P.cell, n, K, S.hist, P.perm); note_launch();
    // the rows in working order, row-major, for the block geometry's contiguous reads
    k_gather_rows<<<std::min((n * d + 255) / 256, 8 * 1024), 256, 0, st>>>(xsT, np, d, P.perm, n, P.wrows); note_launch();
    k_block_geom<<<nqb, 256, 0, st>>>(P.wrows, d, n, QB, P.qcenter, P.qradius, nullptr, nullptr); note_launch();
    k_block_geom<<<ncb, 256, 0, st>>>(P.wrows, d, n, cb, P.ccenter, P.cradius, P.ccenter_f, P.cradius_f); note_launch();
    return cudaGetLastError();
}

// The smallest and largest positive norm (order-preserving u64 bits of positive doubles).
__global__ void k_norm_range(const double* __restrict__ norms, int n, unsigned long long* __restrict__ range) {
    unsigned long long lo = ~0ull, hi = 0ull;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double a = norms[i];
        if (a > 0.0) {
            const unsigned long long b = (unsigned long long)__double_as_longlong(a);
            lo = min(lo, b);
            hi = max(hi, b);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(COSTAL_FULL_MASK, lo, o));
        hi = max(hi, __shfl_xor_sync(COSTAL_FULL_MASK, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&range[0], lo);
        atomicMax(&range[1], hi);
    }
}

// Bucket of every row: 0 for a zero row, else 1 + ⌊(NORM_BUCKETS − 2)·log(a/lo)/log(hi/lo)⌋.
__global__ void k_norm_bucket(const double* __restrict__ norms, int n, const unsigned long long* __restrict__ range,
                              uint32_t* __restrict__ cell) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = norms[i];
    const double lo = __longlong_as_double((long long)range[0]), hi = __longlong_as_double((long long)range[1]);
    uint32_t b = 0;
    if (a > 0.0) {
        const double span = hi > lo ? log(hi / lo) : 1.0;
        const double f = log(a / lo) / span * (double)(NORM_BUCKETS - 2);
        b = 1u + (uint32_t)fmin(fmax(f, 0.0), (double)(NORM_BUCKETS - 2));
    }
    cell[i] = b;
}

size_t norm_order_bytes(int n) {
    const size_t nch = (size_t)(n + CHUNK - 1) / CHUNK;
    return a256((size_t)n * 4) + a256(nch * NORM_BUCKETS * 4) + a256((NORM_BUCKETS + 1) * 4) + 256;
}

cudaError_t norm_order(const double* norms, int n, void* ws, uint32_t* perm, cudaStream_t st) {
    char* p = static_cast<char*>(ws);
    const int nch = (n + CHUNK - 1) / CHUNK;
    uint32_t* cell = reinterpret_cast<uint32_t*>(p);
    p += a256((size_t)n * 4);
    uint32_t* hist = reinterpret_cast<uint32_t*>(p);
    p += a256((size_t)nch * NORM_BUCKETS * 4);
    uint32_t* start = reinterpret_cast<uint32_t*>(p);
    p += a256((NORM_BUCKETS + 1) * 4);
    unsigned long long* range = reinterpret_cast<unsigned long long*>(p);
    cudaError_t e = cudaMemsetAsync(range, 0xff, 8, st);  // smallest: all ones
    if (e == cudaSuccess) e = cudaMemsetAsync(range + 1, 0, 8, st);  // largest: zero
    if (e != cudaSuccess) return e;
    k_norm_range<<<std::min((n + 255) / 256, 1024), 256, 0, st>>>(norms, n, range); note_launch();
    k_norm_bucket<<<(n + 255) / 256, 256, 0, st>>>(norms, n, range, cell); note_launch();
    k_cell_hist<<<(nch + 127) / 128, 128, 0, st>>>(cell, n, NORM_BUCKETS, hist); note_launch();
    k_cell_scan<<<1, NORM_BUCKETS, 0, st>>>(hist, nch, NORM_BUCKETS, start); note_launch();
    k_cell_scatter<<<(nch + 127) / 128, 128, 0, st>>>(cell, n, NORM_BUCKETS, hist, perm); note_launch();
    return cudaGetLastError();
}

cudaError_t build_lists(Plan& P, unsigned long long* skipped_total, cudaStream_t st) {
    // up to 8,192 column blocks: 16 keys a thread, two CTAs per SM; up to 16,384: 32 keys a thread;
    // beyond that (n > 4,194,304 with blocks of 256) the lists stay in block order (no early stop)
    const bool wide = P.ncb > ListShape<16>::N;
    auto kern = wide ? k_block_lists<32> : k_block_lists<16>;
    const size_t smem = (size_t)(wide ? ListShape<32>::N : ListShape<16>::N) * 4;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<P.nqb, LIST_T, smem, st>>>(P.qcenter, P.qradius, P.ccenter_f, P.cradius_f, P.nqb, P.ncb, P.d, P.tq,
                                      P.rowmax, P.rm_delta, P.lists, P.list_ub, P.counts, P.ub_skip, skipped_total);
    note_launch();
    k_row_ub<<<(P.n + 255) / 256, 256, 0, st>>>(P.perm, P.n, P.ub_skip, P.row_ub); note_launch();
    return cudaGetLastError();
}

}  // namespace prune
}  // namespace costal
