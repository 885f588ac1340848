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


// Bitonic sort of a warp-distributed array (position p = s·32 + lane) into (score desc, index asc).
template <int SL>
__device__ __forceinline__ void warp_sort_f32(float (&sc)[SL], uint32_t (&id)[SL], int lane) {
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
                        const bool asc = ((s * 32 + lane) & size) == 0;
                        const bool sw = asc ? better(sc[t], id[t], sc[s], id[s]) : better(sc[s], id[s], sc[t], id[t]);
                        if (sw) {
                            const float a = sc[s];
                            sc[s] = sc[t];
                            sc[t] = a;
                            const uint32_t b = id[s];
                            id[s] = id[t];
                            id[t] = b;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int s = 0; s < SL; ++s) {
                    const float os = __shfl_xor_sync(COSTAL_FULL_MASK, sc[s], stride);
                    const uint32_t oi = __shfl_xor_sync(COSTAL_FULL_MASK, id[s], stride);
                    const bool lower = (lane & stride) == 0;
                    const bool asc = ((s * 32 + lane) & size) == 0;
                    const bool take = (lower == asc) ? better(os, oi, sc[s], id[s]) : better(sc[s], id[s], os, oi);
                    if (take) {
                        sc[s] = os;
                        id[s] = oi;
                    }
                }
            }
        }
    }
}

}  // namespace costal
