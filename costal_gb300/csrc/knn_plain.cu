// Plain FP32 exact kNN on GB300: the correctness-defining form of the hot path.
//
// Restates the algorithm of crates/costal-core/src/knn.rs (CosTaL 2.1.0) for one GPU:
//   k_prep      — knn.rs:315-323 row_norms64 (f64, dimension order) and knn.rs:420-436 the
//                 L2-normalised f32 working copy, written transposed (d_pad × n_pad) for the tiles;
//                 also knn.rs:325-342's non-finite check (first bad row).
//   (the FP32 coarse kernel, knn.rs:603-660 + 758-875, lives in coarse_fp32.cu)
//   k_rescore   — knn.rs:688-720 + 746-753: f64 rescoring of the cap candidates, the sort, the
//                 ε-certificate s_k > τ + (d+4)·2⁻²³, and (fused) the Tanimoto edge weight of
//                 weight.rs:30-37 for the k survivors.
//   k_gather    — knn.rs:723-743: the full-row regather for rows that fail the certificate; with
//                 min_sim = −∞ over every row it is knn.rs:884-924's brute force.
//
// The output does not depend on how the coarse pass orders its sums: every candidate left out has
// an FP32 score ≤ τ, its exact score is within ε of it, and the certificate (or the regather)
// makes the final ranking a function of the f64 rescoring alone (knn.rs:682-687).

#include <algorithm>

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"

namespace costal {

// =================================================================================================
// k_prep: norms, non-finite check, transposed normalised copy
// =================================================================================================

constexpr int PREP_ROWS = 128;
constexpr int PREP_TCHUNK = 64;

// Block = PREP_ROWS threads = PREP_ROWS rows. Rows are staged through shared memory in chunks of
// PREP_TCHUNK dimensions (coalesced loads), then each thread walks its own row in dimension order,
// so the f64 sum has exactly the reference's order.
__global__ void __launch_bounds__(PREP_ROWS) k_prep(const float* __restrict__ x, int n, int d, int np, int dp,
                                                    double* __restrict__ norms, float* __restrict__ xsT,
                                                    unsigned long long* __restrict__ bad_row) {
    __shared__ float tile[PREP_ROWS * (PREP_TCHUNK + 1)];
    const int r0 = blockIdx.x * PREP_ROWS;
    const int r = r0 + threadIdx.x;
    const int rows = min(PREP_ROWS, n - r0);
    double s = 0.0;
    bool bad = false;
    for (int t0 = 0; t0 < d; t0 += PREP_TCHUNK) {
        const int tc = min(PREP_TCHUNK, d - t0);
        __syncthreads();
        for (int e = threadIdx.x; e < rows * tc; e += PREP_ROWS) {
            const int rr = e / tc, tt = e % tc;
            tile[rr * (PREP_TCHUNK + 1) + tt] = x[(size_t)(r0 + rr) * d + t0 + tt];
        }
        __syncthreads();
        if (r < n) {
            for (int tt = 0; tt < tc; ++tt) {
                const float v = tile[threadIdx.x * (PREP_TCHUNK + 1) + tt];
                bad |= !isfinite(v);
                s = dot64_step(s, v, v);
            }
        }
    }
    double nrm = __dsqrt_rn(s);
    if (r < n) {
        norms[r] = nrm;
        if (bad) atomicMin(bad_row, (unsigned long long)r);
    }
    // xs = f32(x / ‖x‖) through the f64 reciprocal: ≤ 2⁻²⁴(1 + 2⁻²⁸) relative error per entry,
    // inside the (d+4)·2⁻²³ coarse bound the certificate uses. Zero rows stay zero (knn.rs:430-435).
    const double inv = (r < n && nrm > 0.0) ? __drcp_rn(nrm) : 0.0;
    for (int t0 = 0; t0 < dp; t0 += PREP_TCHUNK) {
        const int tc = min(PREP_TCHUNK, d - t0);
        if (tc > 0) {
            __syncthreads();
            for (int e = threadIdx.x; e < rows * tc; e += PREP_ROWS) {
                const int rr = e / tc, tt = e % tc;
                tile[rr * (PREP_TCHUNK + 1) + tt] = x[(size_t)(r0 + rr) * d + t0 + tt];
            }
            __syncthreads();
        }
        const int tend = min(PREP_TCHUNK, dp - t0);
        if (r < np) {
            for (int tt = 0; tt < tend; ++tt) {
                float v = 0.0f;
                if (r < n && t0 + tt < d) v = (float)(f64_of(tile[threadIdx.x * (PREP_TCHUNK + 1) + tt]) * inv);
                xsT[(size_t)(t0 + tt) * np + r] = v;
            }
        }
    }
}

// Rows of the padded range [n, np) in a block that has no real row still need zero columns.
__global__ void k_zero_pad_cols(float* __restrict__ xsT, int n, int np, int dp) {
    const int pad = np - n;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < pad * dp; e += gridDim.x * blockDim.x) {
        const int t = e / pad, c = n + e % pad;
        xsT[(size_t)t * np + c] = 0.0f;
    }
}

// lib.rs:94-102 / crates/costal-core/src/lib.rs:34-47: f32 row norms, sequential f32 sum.
__global__ void k_row_l2_norms_f32(const float* __restrict__ x, int n, int d, float* __restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    float s = 0.0f;
    for (int t = 0; t < d; ++t) {
        const float v = x[(size_t)r * d + t];
        s = __fadd_rn(s, __fmul_rn(v, v));
    }
    out[r] = sqrtf(s);
}

// =================================================================================================
// k_rescore: f64 rescoring, sort, certificate, fused Tanimoto weight
// =================================================================================================

// before64 without short-circuit evaluation: a predicate, never a branch.
__device__ __forceinline__ bool before64_p(double sa, uint32_t ia, double sb, uint32_t ib) {
    const long long ka = total_key(sa), kb = total_key(sb);
    return (ka > kb) | ((ka == kb) & (ia < ib));
}

// Bitonic sort of a warp-distributed array (position p = s·32 + lane) into (score desc, idx asc).
// Every compare-exchange is a predicate and selects, so the warp never diverges between shuffles.
template <int SLOTS>
__device__ __forceinline__ void warp_sort(double (&sc)[SLOTS], double (&cs)[SLOTS], uint32_t (&id)[SLOTS],
                                          int lane) {
    constexpr int N = 32 * SLOTS;
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= 32) {
                const int ss = stride >> 5;
#pragma unroll
                for (int s = 0; s < SLOTS; ++s) {
                    const int t = s ^ ss;
                    if (t > s) {
                        const bool asc = ((s * 32 + lane) & size) == 0;
                        const bool sw = asc ? before64_p(sc[t], id[t], sc[s], id[s])
                                            : before64_p(sc[s], id[s], sc[t], id[t]);
                        const double a = sc[s], b = cs[s];
                        const uint32_t c = id[s];
                        sc[s] = sw ? sc[t] : a;
                        cs[s] = sw ? cs[t] : b;
                        id[s] = sw ? id[t] : c;
                        sc[t] = sw ? a : sc[t];
                        cs[t] = sw ? b : cs[t];
                        id[t] = sw ? c : id[t];
                    }
                }
            } else {
#pragma unroll
                for (int s = 0; s < SLOTS; ++s) {
                    const double osc = __shfl_xor_sync(COSTAL_FULL_MASK, sc[s], stride);
                    const double ocs = __shfl_xor_sync(COSTAL_FULL_MASK, cs[s], stride);
                    const uint32_t oid = __shfl_xor_sync(COSTAL_FULL_MASK, id[s], stride);
                    const bool lower = (lane & stride) == 0;
                    const bool asc = ((s * 32 + lane) & size) == 0;
                    const bool take = (lower == asc) ? before64_p(osc, oid, sc[s], id[s])
                                                     : before64_p(sc[s], id[s], osc, oid);
                    sc[s] = take ? osc : sc[s];
                    cs[s] = take ? ocs : cs[s];
                    id[s] = take ? oid : id[s];
                }
            }
        }
    }
}

// The k-th largest of a warp's 32·SLOTS order keys (ballot counts, bit by bit from the top).
template <int SLOTS>
__device__ __forceinline__ uint32_t warp_kth_key(const uint32_t (&key)[SLOTS], int k) {
    uint32_t prefix = 0;
    int need = k;
#pragma unroll 1
    for (int b = 31; b >= 0; --b) {
        const uint32_t hmask = ~0u << b, want = prefix | (1u << b);
        int c = 0;
#pragma unroll
        for (int s = 0; s < SLOTS; ++s) c += __popc(__ballot_sync(COSTAL_FULL_MASK, (key[s] & hmask) == want));
        if (c >= need) prefix = want;
        else need -= c;
    }
    return prefix;
}

// Three phases per CTA of 8 rows.
// (0) One warp per row finds the k-th largest coarse score c_k among the row's candidates. At least k
//     candidates score ≥ c_k coarse, so ≥ c_k − E exact, so the row's exact k-th score s_k ≥ c_k − E;
//     a candidate whose coarse score is below c_k − 2E scores below s_k exactly and can neither enter
//     the top-k nor change s_k. Only the others are rescored (cosine selection; E the row's coarse
//     error bound); they are packed into one list for the CTA.
// (1) Every thread rescores entries of that list — all lanes of a warp on real work, since the f64
//     dot products are the kernel's cost on the GB300's narrow FP64 pipe — into shared memory.
// (2) One warp per row sorts its cap results (skipped and empty slots as −∞), certifies and writes
//     the row.
constexpr int RS_ROWS = 8;
constexpr int RS_MAXCAP = 128;

template <int SLOTS>
__device__ __forceinline__ void rescore_group(int g, const float* __restrict__ x, int n, int d, int k, int cap, int lstride,
              const uint32_t* __restrict__ cand_idx, const float* __restrict__ cand_score,
              const float* __restrict__ tau, const double* __restrict__ norms, const double* __restrict__ row_eps,
              const double* __restrict__ row_ub, unsigned* __restrict__ ub_fail, double eps, int certify, int select,
              const uint32_t* __restrict__ rlist,
              const unsigned* __restrict__ rcount, uint32_t* __restrict__ out_idx, double* __restrict__ out_cos,
              double* __restrict__ out_w, uint32_t* __restrict__ fb_rows, double* __restrict__ fb_minsim,
              unsigned* __restrict__ fb_count, unsigned long long* __restrict__ max_err_bits) {
    __shared__ double sc_s[RS_ROWS * RS_MAXCAP], cs_s[RS_ROWS * RS_MAXCAP];
    __shared__ uint32_t id_s[RS_ROWS * RS_MAXCAP];
    __shared__ uint16_t work_s[RS_ROWS * RS_MAXCAP];  // packed (row, slot) entries to rescore
    __shared__ int row_s[RS_ROWS], cnt_s[RS_ROWS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nrows = rlist ? (int)*rcount : n;
    const int w0 = g * RS_ROWS;
    if (w0 >= nrows) return;
    const int nr = min(RS_ROWS, nrows - w0);
    if (tid < RS_ROWS) row_s[tid] = tid < nr ? (rlist ? (int)rlist[w0 + tid] : w0 + tid) : 0;
    __syncthreads();
    // phase 0: which slots need the f64 score
    unsigned keep[SLOTS] = {};
    if (warp < nr) {
        const int i = row_s[warp];
        uint32_t key[SLOTS];
        int valid = 0;
#pragma unroll
        for (int s = 0; s < SLOTS; ++s) {
            const int p = s * 32 + lane;
            key[s] = 0;  // below every real score's key
            if (p < cap && cand_idx[(size_t)i * lstride + p] < (uint32_t)n) {
                const uint32_t u = __float_as_uint(cand_score[(size_t)i * lstride + p]);
                key[s] = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
            }
            valid += __popc(__ballot_sync(COSTAL_FULL_MASK, key[s] != 0));
        }
        double thr = -CUDART_INF;
        if (select == 0 && valid >= k) {
            const uint32_t h = warp_kth_key<SLOTS>(key, k);
            const float ck = __uint_as_float((h & 0x80000000u) ? (h & 0x7fffffffu) : ~h);
            const double e = row_eps ? row_eps[i] : eps;
            thr = __dsub_rd((double)ck, __dadd_ru(e, e));
        }
        int n_keep = 0;
#pragma unroll
        for (int s = 0; s < SLOTS; ++s) {
            const int p = s * 32 + lane;
            bool kp = false;
            if (key[s] != 0) {
                const float cf = __uint_as_float((key[s] & 0x80000000u) ? (key[s] & 0x7fffffffu) : ~key[s]);
                kp = !((double)cf < thr);
            }
            keep[s] = __ballot_sync(COSTAL_FULL_MASK, kp);
            if (!kp && p < cap) {
                sc_s[warp * cap + p] = -CUDART_INF;
                cs_s[warp * cap + p] = 0.0;
                id_s[warp * cap + p] = 0xffffffffu;
            }
            n_keep += __popc(keep[s]);
        }
        if (lane == 0) cnt_s[warp] = n_keep;
    } else if (lane == 0) {
        cnt_s[warp] = 0;  // (blockDim = 32·RS_ROWS: one warp per row slot)
    }
    __syncthreads();
    int total = 0, base = 0;
#pragma unroll
    for (int r = 0; r < RS_ROWS; ++r) {
        base += r < warp ? cnt_s[r] : 0;
        total += cnt_s[r];
    }
    if (warp < nr) {
        int off = base;
#pragma unroll
        for (int s = 0; s < SLOTS; ++s) {
            if (keep[s] >> lane & 1u)
                work_s[off + __popc(keep[s] & ((1u << lane) - 1u))] = (uint16_t)(warp * RS_MAXCAP + s * 32 + lane);
            off += __popc(keep[s]);
        }
    }
    __syncthreads();
    // phase 1: the f64 rescoring of the packed entries
    const bool vec4 = (d & 3) == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0;
    double err = 0.0, ratio = 0.0;
    for (int w = tid; w < total; w += blockDim.x) {
        const int code = work_s[w], r = code / RS_MAXCAP, p = code - r * RS_MAXCAP, e = r * cap + p;
        const int i = row_s[r];
        const uint32_t j = cand_idx[(size_t)i * lstride + p];
        const float* xi = x + (size_t)i * d;
        const float* xj = x + (size_t)j * d;
        double dot = 0.0;
        if (vec4) {  // the same dimension order, 16-byte loads
            for (int t = 0; t < d; t += 4) {
                const float4 a = __ldg(reinterpret_cast<const float4*>(xi + t));
                const float4 b = __ldg(reinterpret_cast<const float4*>(xj + t));
                dot = dot64_step(dot, a.x, b.x);
                dot = dot64_step(dot, a.y, b.y);
                dot = dot64_step(dot, a.z, b.z);
                dot = dot64_step(dot, a.w, b.w);
            }
        } else {
            for (int t = 0; t < d; ++t) dot = dot64_step(dot, __ldg(xi + t), __ldg(xj + t));
        }
        const double ni = norms[i], nj = norms[j];
        const double c = cos64(dot, ni, nj);
        const double score = select == 0 ? c : tani_from_cos(ni, nj, c);
        const double diff = fabs((double)cand_score[(size_t)i * lstride + p] - score);
        err = fmax(err, diff);
        ratio = fmax(ratio, diff / (row_eps ? row_eps[i] : eps));  // against the bound the certificate used
        sc_s[e] = score;
        cs_s[e] = c;
        id_s[e] = j;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        err = fmax(err, __shfl_xor_sync(COSTAL_FULL_MASK, err, o));
        ratio = fmax(ratio, __shfl_xor_sync(COSTAL_FULL_MASK, ratio, o));
    }
    // max_err_bits[0]: the largest |coarse − rescored|, [1]: the largest ratio of it to the row's bound
    // (non-negative doubles order like their bits). One address for the whole grid: read it first,
    // so that only a new maximum pays for the atomic.
    if (lane == 0 && max_err_bits && err > 0.0) {
        const unsigned long long eb = (unsigned long long)__double_as_longlong(err);
        if (eb > *reinterpret_cast<volatile unsigned long long*>(max_err_bits)) atomicMax(max_err_bits, eb);
        const unsigned long long rb = (unsigned long long)__double_as_longlong(ratio);
        if (rb > *reinterpret_cast<volatile unsigned long long*>(max_err_bits + 1)) atomicMax(max_err_bits + 1, rb);
    }
    __syncthreads();
    if (warp >= nr) return;  // no barrier below
    const int i = row_s[warp];
    const double ni = norms[i];
    double sc[SLOTS], cs[SLOTS];
    uint32_t id[SLOTS];
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
        const int p = s * 32 + lane;
        const bool v = p < cap;
        sc[s] = v ? sc_s[warp * cap + p] : -CUDART_INF;
        cs[s] = v ? cs_s[warp * cap + p] : 0.0;
        id[s] = v ? id_s[warp * cap + p] : 0xffffffffu;
    }
    warp_sort<SLOTS>(sc, cs, id, lane);
    const double s_k = __shfl_sync(COSTAL_FULL_MASK, sc[(k - 1) >> 5], (k - 1) & 31);
    const double e = row_eps ? row_eps[i] : eps;
    // knn.rs:704-714: with cap == n−1 nothing was left out; otherwise exact iff s_k > τ + ε. With
    // block pruning, every column of a skipped block scores at most row_ub: s_k must also beat it.
    const bool ub_bad = row_ub && s_k <= row_ub[i];
    if (ub_bad && lane == 0 && ub_fail) atomicAdd(ub_fail, 1u);
    // fewer than k candidates kept (possible only when a coarse threshold cut the list): regather
    const bool short_list = s_k == -CUDART_INF;
    if ((certify && s_k <= __dadd_rn((double)tau[i], e)) || ub_bad || short_list) {
        if (lane == 0) {
            const unsigned slot = atomicAdd(fb_count, 1u);
            fb_rows[slot] = (uint32_t)i;
            fb_minsim[slot] = __dsub_rn(s_k, e);
        }
        return;
    }
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
        const int p = s * 32 + lane;
        if (p < k) {
            out_idx[(size_t)i * k + p] = id[s];
            out_cos[(size_t)i * k + p] = cs[s];
            if (out_w) out_w[(size_t)i * k + p] = tani_from_cos(ni, norms[id[s]], cs[s]);
        }
    }
}

// Row groups of RS_ROWS, grid-stride: one group per CTA, or (deep rows) a few CTAs per SM walking
// many groups, so that the rows each thread streams through stay in L1.
template <int SLOTS>
__global__ void __launch_bounds__(256)
    k_rescore(const float* __restrict__ x, int n, int d, int k, int cap, int lstride,
              const uint32_t* __restrict__ cand_idx, const float* __restrict__ cand_score,
              const float* __restrict__ tau, const double* __restrict__ norms, const double* __restrict__ row_eps,
              const double* __restrict__ row_ub, unsigned* __restrict__ ub_fail, double eps, int certify, int select,
              const uint32_t* __restrict__ rlist,
              const unsigned* __restrict__ rcount, uint32_t* __restrict__ out_idx, double* __restrict__ out_cos,
              double* __restrict__ out_w, uint32_t* __restrict__ fb_rows, double* __restrict__ fb_minsim,
              unsigned* __restrict__ fb_count, unsigned long long* __restrict__ max_err_bits) {
    const int nrows = rlist ? (int)*rcount : n;
    for (int g = blockIdx.x; g * RS_ROWS < nrows; g += gridDim.x) {
        rescore_group<SLOTS>(g, x, n, d, k, cap, lstride, cand_idx, cand_score, tau, norms, row_eps, row_ub, ub_fail,
                             eps, certify, select, rlist, rcount, out_idx, out_cos, out_w, fb_rows, fb_minsim, fb_count,
                             max_err_bits);
        __syncthreads();  // the group's shared arrays are free again
    }
}

// =================================================================================================
// k_gather: full-row regather (fallback) and brute force
// =================================================================================================

constexpr int GT = 256;

struct GatherSmem {
    double* sc;
    double* cs;
    uint32_t* id;
};

__device__ void block_sort(double* sc, double* cs, uint32_t* id, int cnt, int capb) {
    for (int p = cnt + threadIdx.x; p < capb; p += GT) {
        sc[p] = -CUDART_INF;
        cs[p] = 0.0;
        id[p] = 0xffffffffu;
    }
    __syncthreads();
    for (int size = 2; size <= capb; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int e = threadIdx.x; e < capb / 2; e += GT) {
                const int lo = 2 * e - (e & (stride - 1));
                const int hi = lo + stride;
                const bool asc = (lo & size) == 0;
                const bool sw = asc ? before64(sc[hi], id[hi], sc[lo], id[lo]) : before64(sc[lo], id[lo], sc[hi], id[hi]);
                if (sw) {
                    double a = sc[lo]; sc[lo] = sc[hi]; sc[hi] = a;
                    double b = cs[lo]; cs[lo] = cs[hi]; cs[hi] = b;
                    uint32_t c = id[lo]; id[lo] = id[hi]; id[hi] = c;
                }
            }
            __syncthreads();
        }
    }
}

// One CTA per row (grid-stride over the fallback list, whose length stays on the device). Keeps a
// shared-memory buffer of rescored candidates; when it could overflow, sorts it and keeps the best
// k (at least k candidates always qualify: the k rescored ones that defined s_k).
__global__ void __launch_bounds__(GT)
    k_gather(const float* __restrict__ x, const float* __restrict__ xsT, int n, int np, int d, int dp, int k,
             const double* __restrict__ norms, const uint32_t* __restrict__ rows, const double* __restrict__ minsim,
             const unsigned* __restrict__ count, int all_rows, int select, int capb, uint32_t* __restrict__ out_idx,
             double* __restrict__ out_cos, double* __restrict__ out_w) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* sc = reinterpret_cast<double*>(smem_raw);
    double* cs = sc + capb;
    uint32_t* id = reinterpret_cast<uint32_t*>(cs + capb);
    float* q_s = reinterpret_cast<float*>(id + capb);  // [dp] normalised query
    float* xi_s = q_s + dp;                             // [d] raw query
    __shared__ int cnt;
    const int nrows = all_rows ? n : (int)*count;
    for (int r = blockIdx.x; r < nrows; r += gridDim.x) {
        const int i = all_rows ? r : (int)rows[r];
        const double ms = all_rows ? -CUDART_INF : minsim[r];
        for (int t = threadIdx.x; t < dp; t += GT) q_s[t] = all_rows ? 0.0f : xsT[(size_t)t * np + i];
        for (int t = threadIdx.x; t < d; t += GT) xi_s[t] = x[(size_t)i * d + t];
        if (threadIdx.x == 0) cnt = 0;
        __syncthreads();
        const double ni = norms[i];
        for (int c0 = 0; c0 < n; c0 += GT) {
            const int c = c0 + threadIdx.x;
            if (c < n && c != i) {
                bool take = true;
                if (!all_rows) {
                    float s = 0.0f;
                    for (int t = 0; t < dp; ++t) s = fmaf(q_s[t], xsT[(size_t)t * np + c], s);
                    if (select != 0) {  // minsim is a Tanimoto score: compare the coarse T
                        const double nj = norms[c];
                        s = tani_coarse_f32(s, make_float2((float)ni, (float)(ni * ni)),
                                            make_float2((float)nj, (float)(nj * nj)));
                    }
                    take = (double)s >= ms;
                }
                if (take) {
                    double dot = 0.0;
                    const float* xc = x + (size_t)c * d;
                    for (int t = 0; t < d; ++t) dot = dot64_step(dot, xi_s[t], __ldg(xc + t));
                    const double nj = norms[c];
                    const double cv = cos64(dot, ni, nj);
                    const int pos = atomicAdd(&cnt, 1);
                    sc[pos] = select == 0 ? cv : tani_from_cos(ni, nj, cv);
                    cs[pos] = cv;
                    id[pos] = (uint32_t)c;
                }
            }
            __syncthreads();
            if (cnt > capb - GT) {
                block_sort(sc, cs, id, cnt, capb);
                if (threadIdx.x == 0) cnt = k;
                __syncthreads();
            }
        }
        block_sort(sc, cs, id, cnt, capb);
        for (int p = threadIdx.x; p < k; p += GT) {
            out_idx[(size_t)i * k + p] = id[p];
            out_cos[(size_t)i * k + p] = cs[p];
            if (out_w) out_w[(size_t)i * k + p] = tani_from_cos(ni, norms[id[p]], cs[p]);
        }
        __syncthreads();
    }
}

// =================================================================================================
// launchers
// =================================================================================================

cudaError_t launch_prep(const float* x, int n, int d, int np, int dp, double* norms, float* xsT,
                        unsigned long long* bad_row, cudaStream_t st) {
    const int blocks = (np + PREP_ROWS - 1) / PREP_ROWS;
    k_prep<<<blocks, PREP_ROWS, 0, st>>>(x, n, d, np, dp, norms, xsT, bad_row); note_launch();
    return cudaGetLastError();
}

cudaError_t launch_row_l2_norms_f32(const float* x, int n, int d, float* out, cudaStream_t st) {
    k_row_l2_norms_f32<<<(n + 255) / 256, 256, 0, st>>>(x, n, d, out); note_launch();
    return cudaGetLastError();
}

// Every finite f32 bit pattern: f64_of against the conversion instruction; counts the mismatches.
__global__ void k_check_f64_of(unsigned long long* __restrict__ mismatches) {
    unsigned long long bad = 0;
    for (unsigned long long b = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; b < (1ull << 32);
         b += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t u = (uint32_t)b;
        if ((u & 0x7f800000u) == 0x7f800000u) continue;  // inf / NaN
        const float f = __uint_as_float(u);
        bad += __double_as_longlong(f64_of(f)) != __double_as_longlong((double)f);
    }
    if (bad) atomicAdd(mismatches, bad);
}

cudaError_t launch_check_f64_of(unsigned long long* mismatches, int sm_count, cudaStream_t st) {
    k_check_f64_of<<<8 * sm_count, 256, 0, st>>>(mismatches); note_launch();
    return cudaGetLastError();
}

int coarse_slots(int cap) { return cap <= 32 ? 1 : (cap <= 64 ? 2 : (cap <= 128 ? 4 : 0)); }

cudaError_t launch_rescore(const float* x, int n, int d, int k, int cap, int lstride, const uint32_t* cand_idx,
                           const float* cand_score, const float* tau, const double* norms, const double* row_eps,
                           const double* row_ub, unsigned* ub_fail, double eps, int certify, int select,
                           const uint32_t* rlist, const unsigned* rcount,
                           uint32_t* out_idx, double* out_cos, double* out_w, uint32_t* fb_rows, double* fb_minsim,
                           unsigned* fb_count, unsigned long long* max_err_bits, cudaStream_t st) {
    const int slots = coarse_slots(cap);
    // deep rows: three CTAs per SM (their streamed rows fit L1); otherwise one CTA per group
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                       cudaSuccess)
            sms = 148;
    }
    const int groups = (n + RS_ROWS - 1) / RS_ROWS;
    const int blocks = d >= 256 ? std::min(groups, 3 * sms) : groups;
#define COSTAL_RESCORE(S)                                                                                   \
    k_rescore<S><<<blocks, 256, 0, st>>>(x, n, d, k, cap, lstride, cand_idx, cand_score, tau, norms, row_eps, \
                                         row_ub, ub_fail, eps, certify, select, rlist, rcount, out_idx, out_cos, \
                                         out_w, fb_rows, \
                                         fb_minsim,                                                           \
                                         fb_count, max_err_bits); note_launch();
    if (slots == 1) {
        COSTAL_RESCORE(1)
    } else if (slots == 2) {
        COSTAL_RESCORE(2)
    } else {
        COSTAL_RESCORE(4)
    }
#undef COSTAL_RESCORE
    return cudaGetLastError();
}

int gather_capb(int k) {
    int c = 512;
    while (c < k + GT) c <<= 1;
    return c;
}

size_t gather_smem(int k, int d, int dp) { return (size_t)gather_capb(k) * 20 + (size_t)(dp + d) * 4 + 16; }

cudaError_t launch_gather(const float* x, const float* xsT, int n, int np, int d, int dp, int k, const double* norms,
                          const uint32_t* rows, const double* minsim, const unsigned* count, int all_rows, int select,
                          int grid, uint32_t* out_idx, double* out_cos, double* out_w, cudaStream_t st) {
    const int capb = gather_capb(k);
    const size_t smem = gather_smem(k, d, dp);
    cudaError_t e = cudaFuncSetAttribute(k_gather, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_gather<<<grid, GT, smem, st>>>(x, xsT, n, np, d, dp, k, norms, rows, minsim, count, all_rows, select, capb,
                                     out_idx, out_cos, out_w); note_launch();
    return cudaGetLastError();
}

cudaError_t launch_zero_pad(float* xsT, int n, int np, int dp, cudaStream_t st) {
    if (np == n) return cudaSuccess;
    k_zero_pad_cols<<<64, 256, 0, st>>>(xsT, n, np, dp); note_launch();
    return cudaGetLastError();
}

}  // namespace costal
