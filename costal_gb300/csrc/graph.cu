// Edge weights and the fuzzy-union symmetrisation on GB300.
//
//   k_tanimoto_w   — weight.rs:30-37, 52-57: T = d / (a² + b² − d), d = a·b·cos (non-contracted f64).
//   k_sort_rows +
//   k_jaccard      — weight.rs:64-93: s = |N(i) ∩ N(j)| by a merge of two sorted rows (integer
//                    exact), w = s / (2k − s).
//   fuzzy union    — graph.rs:24-68: S + Sᵀ − S∘Sᵀ, self-loops and exact zeros dropped, upper
//                    triangle in ascending (row, col). Instead of a global sort of n·k 64-bit keys,
//                    each directed edge i→j looks up its reverse in row j (k entries), the pair is
//                    emitted once (from its lower endpoint when both directions exist) with weight
//                    (a + b) − a·b, edges are bucketed by their lower endpoint (count, scan,
//                    scatter) and each bucket is sorted by its upper endpoint. The result is the
//                    same sorted, de-duplicated list; (a + b) − a·b is commutative, so which
//                    direction supplies a never changes a bit (graph.rs:20-23).

#include <algorithm>

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"

namespace costal {

// ---- index check (lib.rs:65-78 `neighbours`): first flat position of an index outside [0, n) ---
__global__ void k_check_idx(const int32_t* __restrict__ idx, uint64_t nk, int n, unsigned long long* first_bad) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nk; e += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t j = idx[e];
        if (j < 0 || j >= n) atomicMin(first_bad, (unsigned long long)e);
    }
}

cudaError_t launch_check_idx(const int32_t* idx, uint64_t nk, int n, unsigned long long* first_bad, cudaStream_t st) {
    if (nk == 0) return cudaSuccess;
    k_check_idx<<<1024, 256, 0, st>>>(idx, nk, n, first_bad); note_launch();
    return cudaGetLastError();
}

// ---- small utilities ------------------------------------------------------------------------------
__global__ void k_iota(uint32_t* __restrict__ out, int start, int m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) out[i] = (uint32_t)(start + i);
}
cudaError_t launch_iota(uint32_t* out, int start, int m, cudaStream_t st) {
    if (m > 0) { k_iota<<<(m + 255) / 256, 256, 0, st>>>(out, start, m); note_launch(); }
    return cudaGetLastError();
}
// A shard's outputs packed: packed row r takes row rows[r] of the (n, k) idx / cos / w (w optional).
// One thread per output entry; rows[] holds valid row ids (the shard's own list).
__global__ void k_take_rows(const uint32_t* __restrict__ rows, int nrows, int k, const uint32_t* __restrict__ idx,
                            const double* __restrict__ cos, const double* __restrict__ w, uint32_t* __restrict__ oidx,
                            double* __restrict__ ocos, double* __restrict__ ow) {
    const uint64_t total = (uint64_t)nrows * k;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = e / k, t = e - r * k;
        const uint64_t src = (uint64_t)rows[r] * k + t;
        oidx[e] = idx[src];
        ocos[e] = cos[src];
        if (w) ow[e] = w[src];
    }
}
cudaError_t launch_take_rows(const uint32_t* rows, int nrows, int k, const uint32_t* idx, const double* cos,
                             const double* w, uint32_t* oidx, double* ocos, double* ow, cudaStream_t st) {
    const uint64_t total = (uint64_t)nrows * k;
    if (total == 0) return cudaGetLastError();
    const unsigned grid = (unsigned)std::min<uint64_t>((total + 255) / 256, 4096);
    k_take_rows<<<grid, 256, 0, st>>>(rows, nrows, k, idx, cos, w, oidx, ocos, ow); note_launch();
    return cudaGetLastError();
}

// Evenly spaced sample rows: out[j] = ⌊j·n/m⌋.
__global__ void k_stride_rows(uint32_t* __restrict__ out, int m, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) out[j] = (uint32_t)(((unsigned long long)j * (unsigned long long)n) / (unsigned long long)m);
}
cudaError_t launch_stride_rows(uint32_t* out, int m, int n, cudaStream_t st) {
    if (m > 0) { k_stride_rows<<<(m + 255) / 256, 256, 0, st>>>(out, m, n); note_launch(); }
    return cudaGetLastError();
}
// y[j] = cos[rows[j]·k + k − 1]: the k-th neighbour cosine of each listed row.
__global__ void k_kth(const double* __restrict__ cos, const uint32_t* __restrict__ rows, int m, int k,
                      float* __restrict__ y) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) y[j] = (float)cos[(size_t)rows[j] * k + k - 1];
}
cudaError_t launch_kth(const double* cos, const uint32_t* rows, int m, int k, float* y, cudaStream_t st) {
    if (m > 0) { k_kth<<<(m + 255) / 256, 256, 0, st>>>(cos, rows, m, k, y); note_launch(); }
    return cudaGetLastError();
}
// Deterministic He-uniform initialisation from a counter-based hash (SplitMix64 of seed + index).
__global__ void k_init_params(float* __restrict__ P, int F, unsigned long long seed) {
    const size_t np = (size_t)128 * F + 128 + (size_t)128 * 128 + 128 + 128 + 1;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < np; p += (size_t)gridDim.x * blockDim.x) {
        unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (p + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const float u = (float)(z >> 40) / (float)(1ull << 24) * 2.0f - 1.0f;  // [-1, 1)
        const size_t w1 = (size_t)128 * F, b1 = w1 + 128, w2 = b1 + (size_t)128 * 128, b2 = w2 + 128, w3 = b2 + 128;
        float v = 0.0f;
        if (p < w1) v = u * sqrtf(6.0f / (float)F);
        else if (p >= b1 && p < w2) v = u * sqrtf(6.0f / 128.0f);
        else if (p >= b2 && p < w3) v = u * sqrtf(6.0f / 128.0f);
        P[p] = v;
    }
}
cudaError_t launch_init_params(float* P, int F, unsigned long long seed, cudaStream_t st) {
    k_init_params<<<64, 256, 0, st>>>(P, F, seed); note_launch();
    return cudaGetLastError();
}

// ---- Tanimoto weights --------------------------------------------------------------------------
__global__ void k_tanimoto_w(const uint32_t* __restrict__ idx, const double* __restrict__ cos,
                             const double* __restrict__ norms, uint64_t nk, int k, double* __restrict__ out) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nk; e += (uint64_t)gridDim.x * blockDim.x)
        out[e] = tani_from_cos(norms[e / k], norms[idx[e]], cos[e]);
}

cudaError_t launch_tanimoto_w(const uint32_t* idx, const double* cos, const double* norms, uint64_t nk, int k,
                              double* out, cudaStream_t st) {
    if (nk == 0) return cudaSuccess;
    k_tanimoto_w<<<2048, 256, 0, st>>>(idx, cos, norms, nk, k, out); note_launch();
    return cudaGetLastError();
}

// ---- Jaccard -----------------------------------------------------------------------------------
__global__ void k_sort_rows(const uint32_t* __restrict__ idx, int n, int k, uint32_t* __restrict__ sorted) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t* row = sorted + (size_t)i * k;
    for (int t = 0; t < k; ++t) {  // insertion sort into the output row (k is small)
        const uint32_t v = idx[(size_t)i * k + t];
        int p = t;
        while (p > 0 && row[p - 1] > v) {
            row[p] = row[p - 1];
            --p;
        }
        row[p] = v;
    }
}

__global__ void k_jaccard(const uint32_t* __restrict__ idx, const uint32_t* __restrict__ sorted, uint64_t nk, int k,
                          double* __restrict__ out) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nk; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t* a = sorted + (e / k) * k;
        const uint32_t* b = sorted + (size_t)idx[e] * k;
        int p = 0, q = 0, c = 0;
        while (p < k && q < k) {
            const uint32_t x = a[p], y = b[q];
            p += x <= y;
            q += y <= x;
            c += x == y;
        }
        const double s = (double)c;
        out[e] = __ddiv_rn(s, __dsub_rn(__dmul_rn(2.0, (double)k), s));
    }
}

cudaError_t launch_jaccard(const uint32_t* idx, int n, int k, uint32_t* sorted_scratch, double* out, cudaStream_t st) {
    if (n == 0 || k == 0) return cudaSuccess;
    k_sort_rows<<<(n + 127) / 128, 128, 0, st>>>(idx, n, k, sorted_scratch); note_launch();
    k_jaccard<<<2048, 256, 0, st>>>(idx, sorted_scratch, (uint64_t)n * k, k, out); note_launch();
    return cudaGetLastError();
}

// =================================================================================================
// fuzzy union
// =================================================================================================

namespace fu {

constexpr uint32_t NONE = 0xffffffffu;
constexpr int SCAN_B = 1024;
constexpr int WARP_MAX = 128;   // buckets up to this size are sorted by one warp in registers
constexpr int SMEM_MAX = 4096;  // larger buckets: one CTA, shared-memory runs of this size + merges

struct Scratch {
    uint32_t* cnt;       // [n + 1] counts, then exclusive offsets
    uint32_t* cursor;    // [n]
    uint32_t* lo;        // [nk] lower endpoint of each emitted edge, NONE if not emitted
    uint32_t* hi;        // [nk]
    double* v;           // [nk]
    uint32_t* bsum;      // [ceil((n+1)/SCAN_B) + 1]
    uint32_t* big;       // [n] buckets larger than WARP_MAX
    uint32_t* nbig;      // [1]
    uint32_t* tmp_hi;    // [nk] merge ping-pong for the largest buckets
    double* tmp_v;       // [nk]
};

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

inline Scratch carve(void* base, int n, int k) {
    const size_t nk = (size_t)n * k;
    const size_t nb = (size_t)(n + 1 + SCAN_B - 1) / SCAN_B + 1;
    char* p = static_cast<char*>(base);
    Scratch s;
    s.cnt = reinterpret_cast<uint32_t*>(p);    p += align256((n + 1) * 4ull);
    s.cursor = reinterpret_cast<uint32_t*>(p); p += align256(n * 4ull);
    s.lo = reinterpret_cast<uint32_t*>(p);     p += align256(nk * 4);
    s.hi = reinterpret_cast<uint32_t*>(p);     p += align256(nk * 4);
    s.v = reinterpret_cast<double*>(p);        p += align256(nk * 8);
    s.bsum = reinterpret_cast<uint32_t*>(p);   p += align256(nb * 4);
    s.big = reinterpret_cast<uint32_t*>(p);    p += align256(n * 4ull);
    s.nbig = reinterpret_cast<uint32_t*>(p);   p += align256(4);
    s.tmp_hi = reinterpret_cast<uint32_t*>(p); p += align256(nk * 4);
    s.tmp_v = reinterpret_cast<double*>(p);    p += align256(nk * 8);
    return s;
}

inline size_t scratch_bytes(int n, int k) {
    const size_t nk = (size_t)n * k;
    const size_t nb = (size_t)(n + 1 + SCAN_B - 1) / SCAN_B + 1;
    return align256((n + 1) * 4ull) + align256(n * 4ull) + 2 * align256(nk * 4) + align256(nk * 8) + align256(nb * 4) +
           align256(n * 4ull) + align256(4) + align256(nk * 4) + align256(nk * 8);
}

// One thread per directed edge i→j (row i, slot t): find the reverse edge j→i in row j, then
// emit the unordered pair once with its combined weight, or drop it (self-loop, zero, or the upper
// side of a two-way pair).
__global__ void k_emit(const uint32_t* __restrict__ idx, const double* __restrict__ w, int n, int k, Scratch s) {
    const uint64_t nk = (uint64_t)n * k;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nk; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(e / k), j = idx[e];
        uint32_t lo = NONE;
        if (j != i) {
            const uint32_t* rj = idx + (size_t)j * k;
            int u = 0;
            while (u < k && rj[u] != i) ++u;
            const bool rev = u < k;
            if (!(rev && i > j)) {
                const double a = w[e];
                double v = a;
                if (rev) {
                    const double b = w[(size_t)j * k + u];
                    v = __dsub_rn(__dadd_rn(a, b), __dmul_rn(a, b));  // graph.rs:49
                }
                if (v != 0.0) {  // graph.rs:54
                    lo = i < j ? i : j;
                    s.hi[e] = i < j ? j : i;
                    s.v[e] = v;
                    atomicAdd(&s.cnt[lo], 1u);
                }
            }
        }
        s.lo[e] = lo;
    }
}

// Exclusive scan of cnt[0..len) in place (cnt[len] receives the total): per-block scans, a scan
// of the block totals by one block, then the add.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* warp_tot, uint32_t* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(COSTAL_FULL_MASK, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(COSTAL_FULL_MASK, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;  // inclusive prefix of warp totals
    }
    __syncthreads();
    const uint32_t before_warp = wid > 0 ? warp_tot[wid - 1] : 0;
    if (total) *total = warp_tot[(blockDim.x >> 5) - 1];
    return before_warp + x - v;
}

__global__ void __launch_bounds__(SCAN_B) k_scan_blocks(uint32_t* __restrict__ a, int len, uint32_t* __restrict__ bsum) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t tot;
    const int e = blockIdx.x * SCAN_B + threadIdx.x;
    const uint32_t v = e < len ? a[e] : 0;
    const uint32_t ex = block_excl_scan(v, warp_tot, threadIdx.x == 0 ? &tot : nullptr);
    if (e < len) a[e] = ex;
    __syncthreads();
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_B) k_scan_sums(uint32_t* __restrict__ bsum, int nb, uint32_t* __restrict__ total_out) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t tot;
    uint32_t carry = 0;
    for (int b0 = 0; b0 < nb; b0 += SCAN_B) {
        const int e = b0 + threadIdx.x;
        const uint32_t v = e < nb ? bsum[e] : 0;
        const uint32_t ex = block_excl_scan(v, warp_tot, threadIdx.x == 0 ? &tot : nullptr);
        __syncthreads();
        if (e < nb) bsum[e] = carry + ex;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total_out = carry;
}

__global__ void k_scan_add(uint32_t* __restrict__ a, int len, const uint32_t* __restrict__ bsum) {
    const int e = blockIdx.x * SCAN_B + threadIdx.x;
    if (e < len) a[e] += bsum[blockIdx.x];
}

__global__ void k_scatter(int n, int k, Scratch s) {
    const uint64_t nk = (uint64_t)n * k;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nk; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t lo = s.lo[e];
        if (lo == NONE) continue;
        const uint32_t pos = s.cnt[lo] + atomicAdd(&s.cursor[lo], 1u);
        s.tmp_hi[pos] = s.hi[e];
        s.tmp_v[pos] = s.v[e];
    }
}

// Warp-register bitonic sort of one bucket by its (unique) upper endpoints.
template <int SLOTS>
__device__ void warp_sort_bucket(uint32_t* hi, double* v, int len, int lane) {
    uint32_t key[SLOTS];
    double val[SLOTS];
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
        const int p = s * 32 + lane;
        key[s] = p < len ? hi[p] : NONE;
        val[s] = p < len ? v[p] : 0.0;
    }
    constexpr int N = 32 * SLOTS;
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= 32) {
#pragma unroll
                for (int s = 0; s < SLOTS; ++s) {
                    const int t = s ^ (stride >> 5);
                    if (t > s) {
                        const bool asc = ((s * 32 + lane) & size) == 0;
                        if (asc ? key[t] < key[s] : key[s] < key[t]) {
                            uint32_t a = key[s]; key[s] = key[t]; key[t] = a;
                            double b = val[s]; val[s] = val[t]; val[t] = b;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int s = 0; s < SLOTS; ++s) {
                    const uint32_t ok = __shfl_xor_sync(COSTAL_FULL_MASK, key[s], stride);
                    const double ov = __shfl_xor_sync(COSTAL_FULL_MASK, val[s], stride);
                    const bool lower = (lane & stride) == 0;
                    const bool asc = ((s * 32 + lane) & size) == 0;
                    const bool take = (lower == asc) ? ok < key[s] : key[s] < ok;
                    if (take) {
                        key[s] = ok;
                        val[s] = ov;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
        const int p = s * 32 + lane;
        if (p < len) {
            hi[p] = key[s];
            v[p] = val[s];
        }
    }
}

// One warp per bucket of ≤ WARP_MAX entries; larger buckets are queued for k_sort_big. Also writes
// the output row/col/weight arrays.
__global__ void k_sort_small(int n, Scratch s, int32_t* __restrict__ rows, int32_t* __restrict__ cols,
                             double* __restrict__ wout) {
    const int lane = threadIdx.x & 31;
    const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= n) return;
    const uint32_t off = s.cnt[b], len = s.cnt[b + 1] - off;
    if (len == 0) return;
    uint32_t* hi = s.tmp_hi + off;
    double* v = s.tmp_v + off;
    if (len > (uint32_t)WARP_MAX) {
        if (lane == 0) s.big[atomicAdd(s.nbig, 1u)] = (uint32_t)b;
        return;
    }
    if (len <= 32) warp_sort_bucket<1>(hi, v, (int)len, lane);
    else if (len <= 64) warp_sort_bucket<2>(hi, v, (int)len, lane);
    else warp_sort_bucket<4>(hi, v, (int)len, lane);
    __syncwarp();
    for (uint32_t p = lane; p < len; p += 32) {
        rows[off + p] = b;
        cols[off + p] = (int32_t)hi[p];
        wout[off + p] = v[p];
    }
}

// One CTA per large bucket: shared-memory bitonic runs of SMEM_MAX, then pairwise merges of runs
// (each element's output position is its rank in its own run plus its rank in the other run; keys
// are unique) between the bucket's two ping-pong copies.
__global__ void __launch_bounds__(512) k_sort_big(Scratch s, int32_t* __restrict__ rows, int32_t* __restrict__ cols,
                                                 double* __restrict__ wout) {
    __shared__ uint32_t sk[SMEM_MAX];
    __shared__ double sv[SMEM_MAX];
    const uint32_t nbig = *s.nbig;
    for (uint32_t q = blockIdx.x; q < nbig; q += gridDim.x) {
        const uint32_t b = s.big[q];
        const uint32_t off = s.cnt[b], len = s.cnt[b + 1] - off;
        uint32_t* A = s.tmp_hi + off;
        double* Av = s.tmp_v + off;
        uint32_t* B = s.hi + off;  // s.hi / s.v are free after the scatter: the ping-pong copy
        double* Bv = s.v + off;
        for (uint32_t r0 = 0; r0 < len; r0 += SMEM_MAX) {
            const uint32_t rl = min((uint32_t)SMEM_MAX, len - r0);
            uint32_t np2 = 1;
            while (np2 < rl) np2 <<= 1;
            for (uint32_t p = threadIdx.x; p < np2; p += blockDim.x) {
                sk[p] = p < rl ? A[r0 + p] : NONE;
                sv[p] = p < rl ? Av[r0 + p] : 0.0;
            }
            __syncthreads();
            for (uint32_t size = 2; size <= np2; size <<= 1) {
                for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                    for (uint32_t e = threadIdx.x; e < np2 / 2; e += blockDim.x) {
                        const uint32_t lo = 2 * e - (e & (stride - 1)), hi = lo + stride;
                        const bool asc = (lo & size) == 0;
                        if (asc ? sk[hi] < sk[lo] : sk[lo] < sk[hi]) {
                            uint32_t a = sk[lo]; sk[lo] = sk[hi]; sk[hi] = a;
                            double c = sv[lo]; sv[lo] = sv[hi]; sv[hi] = c;
                        }
                    }
                    __syncthreads();
                }
            }
            for (uint32_t p = threadIdx.x; p < rl; p += blockDim.x) {
                A[r0 + p] = sk[p];
                Av[r0 + p] = sv[p];
            }
            __syncthreads();
        }
        for (uint32_t width = SMEM_MAX; width < len; width <<= 1) {
            for (uint32_t p = threadIdx.x; p < len; p += blockDim.x) {
                const uint32_t run = p / (2 * width), base = run * 2 * width;
                const uint32_t a0 = base, a1 = min(base + width, len), b1 = min(base + 2 * width, len);
                const bool in_a = p < a1;
                const uint32_t o0 = in_a ? a1 : a0, o1 = in_a ? b1 : a1;  // the other run
                const uint32_t key = A[p];
                uint32_t lo = o0, hi = o1;  // first position in the other run with a larger key
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (A[mid] < key) lo = mid + 1;
                    else hi = mid;
                }
                const uint32_t own = in_a ? p - a0 : p - a1;
                const uint32_t dst = base + own + (lo - o0);
                B[dst] = key;
                Bv[dst] = Av[p];
            }
            __syncthreads();
            uint32_t* t = A; A = B; B = t;
            double* tv = Av; Av = Bv; Bv = tv;
        }
        for (uint32_t p = threadIdx.x; p < len; p += blockDim.x) {
            rows[off + p] = (int32_t)b;
            cols[off + p] = (int32_t)A[p];
            wout[off + p] = Av[p];
        }
        __syncthreads();
    }
}

// ---- the Leiden graph (CSR) from the fuzzy-union edge list ---------------------------------------
// leiden.rs:52-101 `Csr::from_edges` walks the edges in order and appends j to row i and i to row j.
// On the union's list (unique pairs i < j, ascending (i, j), no zero weights) that puts, in every
// row v, first the lower neighbours u < v in ascending order (their edges come in the blocks of rows
// u < v, in order of u), then the upper ones in ascending order (v's own block): every row ascending.
// So the same bucket machinery builds it: both directions of each edge emitted (slot 2e: i → j,
// slot 2e + 1: j → i), bucketed by source, each bucket sorted by destination (unique in a row).
__global__ void k_csr_emit(const int32_t* __restrict__ rows, const int32_t* __restrict__ cols,
                           const double* __restrict__ w, const uint32_t* __restrict__ m_dev, uint64_t slots, Scratch s) {
    const uint64_t m = *m_dev;
    for (uint64_t e2 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e2 < slots;
         e2 += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t e = e2 >> 1;
        uint32_t src = NONE;
        if (e < m) {
            const uint32_t i = (uint32_t)rows[e], j = (uint32_t)cols[e];
            src = (e2 & 1) ? j : i;
            s.hi[e2] = (e2 & 1) ? i : j;
            s.v[e2] = w[e];
            atomicAdd(&s.cnt[src], 1u);
        }
        s.lo[e2] = src;
    }
}

__global__ void k_widen(const uint32_t* __restrict__ a, int len, uint64_t* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) out[i] = a[i];
}

}  // namespace fu

size_t fuzzy_union_scratch_bytes(int n, int k) { return fu::scratch_bytes(n, k); }

size_t csr_scratch_bytes(int n, int k) { return fu::scratch_bytes(n, 2 * k); }

cudaError_t launch_csr_from_union(const int32_t* rows, const int32_t* cols, const double* w, const uint32_t* m_dev,
                                  int n, int k, void* scratch, uint64_t* indptr, int32_t* src_out, int32_t* nbr,
                                  double* w_out, uint32_t* nnz_dev, cudaStream_t st) {
    using namespace fu;
    const int k2 = 2 * k;  // two directed slots per union edge (at most n·k edges)
    Scratch s = carve(scratch, n, k2);
    cudaError_t e;
    if ((e = cudaMemsetAsync(s.cnt, 0, (n + 1) * 4ull, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(s.cursor, 0, n * 4ull, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(s.nbig, 0, 4, st)) != cudaSuccess) return e;
    k_csr_emit<<<2048, 256, 0, st>>>(rows, cols, w, m_dev, (uint64_t)n * k2, s); note_launch();
    const int len = n + 1;
    const int nb = (len + SCAN_B - 1) / SCAN_B;
    k_scan_blocks<<<nb, SCAN_B, 0, st>>>(s.cnt, len, s.bsum); note_launch();
    k_scan_sums<<<1, SCAN_B, 0, st>>>(s.bsum, nb, nnz_dev); note_launch();
    k_scan_add<<<nb, SCAN_B, 0, st>>>(s.cnt, len, s.bsum); note_launch();
    k_scatter<<<2048, 256, 0, st>>>(n, k2, s); note_launch();
    k_sort_small<<<(n + 7) / 8, 256, 0, st>>>(n, s, src_out, nbr, w_out); note_launch();
    k_sort_big<<<256, 512, 0, st>>>(s, src_out, nbr, w_out); note_launch();
    k_widen<<<(len + 255) / 256 < 4096 ? (len + 255) / 256 : 4096, 256, 0, st>>>(s.cnt, len, indptr); note_launch();
    return cudaGetLastError();
}

cudaError_t launch_fuzzy_union(const uint32_t* idx, const double* w, int n, int k, void* scratch, int32_t* rows,
                               int32_t* cols, double* w_out, uint32_t* m_dev, cudaStream_t st) {
    using namespace fu;
    Scratch s = carve(scratch, n, k);
    cudaError_t e;
    if ((e = cudaMemsetAsync(s.cnt, 0, (n + 1) * 4ull, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(s.cursor, 0, n * 4ull, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(s.nbig, 0, 4, st)) != cudaSuccess) return e;
    k_emit<<<2048, 256, 0, st>>>(idx, w, n, k, s); note_launch();
    const int len = n + 1;
    const int nb = (len + SCAN_B - 1) / SCAN_B;
    k_scan_blocks<<<nb, SCAN_B, 0, st>>>(s.cnt, len, s.bsum); note_launch();
    k_scan_sums<<<1, SCAN_B, 0, st>>>(s.bsum, nb, m_dev); note_launch();
    k_scan_add<<<nb, SCAN_B, 0, st>>>(s.cnt, len, s.bsum); note_launch();
    k_scatter<<<2048, 256, 0, st>>>(n, k, s); note_launch();
    k_sort_small<<<(n + 7) / 8, 256, 0, st>>>(n, s, rows, cols, w_out); note_launch();
    k_sort_big<<<256, 512, 0, st>>>(s, rows, cols, w_out); note_launch();
    return cudaGetLastError();
}

}  // namespace costal
