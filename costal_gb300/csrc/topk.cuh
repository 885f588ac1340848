// Warp-cooperative top-cap list shared by the FP32 and tensor-core coarse kernels.
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace costal {

// (score desc, index asc) on coarse f32 scores: the heap order of knn.rs:798-801, reversed.
__device__ __forceinline__ bool better(float sa, uint32_t ia, float sb, uint32_t ib) {
    return sa > sb || (sa == sb && ia < ib);
}

// Insert (sv, cv) into the warp-distributed sorted list (position p = s·32 + lane), keeping the best
// `cap`. `len` is warp-uniform.
template <int SLOTS>
__device__ __forceinline__ void list_insert(float (&ls)[SLOTS], uint32_t (&li)[SLOTS], int& len, int cap, float sv,
                                            uint32_t cv, int lane) {
    if (len == cap) {
        const float ws = __shfl_sync(COSTAL_FULL_MASK, ls[(cap - 1) >> 5], (cap - 1) & 31);
        const uint32_t wi = __shfl_sync(COSTAL_FULL_MASK, li[(cap - 1) >> 5], (cap - 1) & 31);
        if (!better(sv, cv, ws, wi)) return;
    }
    int pos = 0;
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
        const int p = s * 32 + lane;
        pos += __popc(__ballot_sync(COSTAL_FULL_MASK, p < len && better(ls[s], li[s], sv, cv)));
    }
    float ns[SLOTS];
    uint32_t ni[SLOTS];
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
        float up_s = __shfl_up_sync(COSTAL_FULL_MASK, ls[s], 1);
        uint32_t up_i = __shfl_up_sync(COSTAL_FULL_MASK, li[s], 1);
        if (s > 0) {
            const float cs = __shfl_sync(COSTAL_FULL_MASK, ls[s > 0 ? s - 1 : 0], 31);
            const uint32_t ci = __shfl_sync(COSTAL_FULL_MASK, li[s > 0 ? s - 1 : 0], 31);
            if (lane == 0) {
                up_s = cs;
                up_i = ci;
            }
        }
        const int p = s * 32 + lane;
        ns[s] = p > pos ? up_s : (p == pos ? sv : ls[s]);
        ni[s] = p > pos ? up_i : (p == pos ? cv : li[s]);
    }
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
        ls[s] = ns[s];
        li[s] = ni[s];
    }
    len = len + 1 < cap ? len + 1 : cap;
}


// (score, index) as one 64-bit key whose unsigned order is `better`: the f32 score mapped to an
// order-preserving u32 in the high word, the complemented index in the low word (smaller index →
// larger key). Padding (−inf, 0xffffffff) maps to the smallest keys.
__device__ __forceinline__ uint64_t order_key(float s, uint32_t i) {
    const uint32_t u = __float_as_uint(s);
    const uint32_t h = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return ((uint64_t)h << 32) | (uint64_t)(~i);
}
__device__ __forceinline__ float key_score(uint64_t k) {
    const uint32_t h = (uint32_t)(k >> 32);
    return __uint_as_float((h & 0x80000000u) ? (h & 0x7fffffffu) : ~h);
}
__device__ __forceinline__ uint32_t key_index(uint64_t k) { return ~(uint32_t)k; }
constexpr uint64_t PAD_KEY = 0x007fffff00000000ull;  // order_key(−inf, 0xffffffff)

// Bitonic sort of warp-distributed 64-bit keys (position p = s·32 + lane) into descending order.
// Every compare-exchange is a max/min pair and a select: no branch, so the warp never diverges
// between its shuffles.
template <int SL>
__device__ __forceinline__ void warp_sort_keys(uint64_t (&v)[SL], int lane) {
    constexpr int N = 32 * SL;
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= 32) {
#pragma unroll
                for (int s = 0; s < SL; ++s) {
                    const int t = s ^ (stride >> 5);
                    if (t > s) {
                        const bool desc = ((s * 32 + lane) & size) == 0;
                        const uint64_t a = v[s], b = v[t];
                        const uint64_t hi = a > b ? a : b, lo = a > b ? b : a;
                        v[s] = desc ? hi : lo;
                        v[t] = desc ? lo : hi;
                    }
                }
            } else {
#pragma unroll
                for (int s = 0; s < SL; ++s) {
                    const uint64_t o = __shfl_xor_sync(COSTAL_FULL_MASK, v[s], stride);
                    const bool keep_max = ((lane & stride) == 0) == (((s * 32 + lane) & size) == 0);
                    const uint64_t hi = v[s] > o ? v[s] : o, lo = v[s] > o ? o : v[s];
                    v[s] = keep_max ? hi : lo;
                }
            }
        }
    }
}

}  // namespace costal
