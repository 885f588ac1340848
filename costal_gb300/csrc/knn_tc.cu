// The certified split-BF16 coarse pass on the 5th-generation tensor cores (tcgen05 + TMEM + TMA).
//
// Same job as the FP32 coarse kernel (crates/costal-core/src/knn.rs:603-660 tiles, :758-875
// threshold scan and per-row heaps), with the dot products on the tensor cores:
//
//   split     Every normalised row a (f32) is written as a = a_hi + a_lo + r with a_hi = bf16(a),
//             a_lo = bf16(a − a_hi); |r| ≤ 2⁻¹⁶|a|. The tensor cores compute a_hi·b_hi + a_lo·b_hi +
//             a_hi·b_lo with FP32 accumulation in TMEM. Plain BF16 would put ~2⁻⁸ of error on every
//             cosine, far wider than the gap between the k-th and (k+m)-th neighbour; the split keeps
//             the bound near 5e-5. Usually A = [a_hi | a_lo | a_hi], B = [b_hi | b_hi | b_lo] (K = 3d,
//             zero-padded to a multiple of 64) and one MMA chain; the query tile stays resident for
//             3d ≤ 128, deeper rows stream both operands by K block. Compact operands (22 ≤ d ≤ 32,
//             where they save a column K block): A = [a_hi | a_hi | 0 | a_lo | 0] resident, a column
//             row is only B = [b_hi | b_lo] (2d bf16), and two chains run into one accumulator: A's
//             [hi | hi] × B's [hi | lo], then A's [lo] × B's leading [hi].
//   kernel    One CTA per 128 query rows (M = 128, one TMEM lane per query), column tiles of N = 256.
//             Warp 4 streams B tiles with TMA (128-byte swizzle) into a ring of shared-memory
//             stages; warp 5 issues the MMAs (one elected thread) into two 256-column TMEM
//             accumulators; warps 0-3 read the accumulators back (tcgen05.ld, 64 columns at a time,
//             the next load in flight while one is scanned), reject whole slices with a 3-input max
//             tree against the query's threshold, and append the rare survivors to per-query buffers
//             that the warp shrinks cooperatively to the best cap (strict `v > τ` admission,
//             knn.rs:774-780).
//   bound     Every query row i gets a rigorous bound E_i on |coarse − exact cosine| (k_row_eps):
//             split remainder ‖a_lo‖·max‖b_lo‖ + ‖a_hi+a_lo‖·max‖r_b‖ + ‖r_a‖·max‖b_hi+b_lo‖ + ‖r_a‖·max‖r_b‖
//             (Cauchy–Schwarz), plus the tensor-core accumulation (K + 16)·2⁻²¹·Σ|products| (four
//             times the error of an FP32 accumulation that truncates instead of rounding: the
//             hardware's internal order and rounding are not documented, so the bound is generous),
//             plus the f32 normalisation 2.0001·2⁻²⁴ and the f64 rescoring (d + 8)·2⁻⁵². The
//             certificate s_k > τ + E_i (k_rescore) then proves the row exact; rows that fail it are
//             re-run by the FP32 kernel, and those the FP32 certificate fails take the regather.
//
// Every mbarrier wait is bounded: after 2²² polls a thread raises `timeout_flag` and its role stops
// (and every other wait of the launch then returns at once); the host reports COSTAL_ETIMEOUT.

#include <algorithm>

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "knn_tc.h"
#include "topk.cuh"

namespace costal {
namespace tc {

constexpr int KB = 64;                 // bf16 elements per 128-byte swizzle row (one K block)
constexpr int A_KB_BYTES = BLOCK_M * 128;  // 16 KB per K block of the query tile
constexpr int B_KB_BYTES = BLOCK_N * 128;  // 32 KB per K block of a column tile
constexpr int HALF_N = BLOCK_N / 2;            // columns of one TMA box of a column tile
constexpr int B_HALF_BYTES = HALF_N * 128;     // 16 KB: the second half of a K block
constexpr int EPI_WARPS = 4;
constexpr int NTHREADS = (EPI_WARPS + 2) * 32;  // 4 epilogue warps, 1 TMA warp, 1 MMA warp
constexpr uint32_t TMEM_COLS = 512;    // two 256-column FP32 accumulators
constexpr long long WAIT_LIMIT = 1ll << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- mbarrier --------------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false (and the flag raised) if the phase never completes. Every 1024 polls the wait
// also checks the global flag, so once any thread of any CTA has given up, every later wait of the
// launch returns at once and the kernel drains in microseconds.
// Roles that are not the bottleneck (TMA, MMA issue) sleep between polls so that they do not take
// issue slots from the epilogue warps that share their schedulers.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned long long* timeout_flag,
                                          bool sleep) {
    for (long long i = 0; i < WAIT_LIMIT; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if (sleep) __nanosleep(64);
        if ((i & 1023) == 1023 && *reinterpret_cast<volatile unsigned long long*>(timeout_flag)) return false;
    }
    atomicExch(timeout_flag, 1ull);
    return false;
}

// ---- TMA ---------------------------------------------------------------------------------------
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

// ---- tcgen05 -----------------------------------------------------------------------------------
// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;               // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;     // stride byte offset: 8 rows × 128 B
    d |= (uint64_t)1 << 46;               // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;               // SWIZZLE_128B
    return d;
}
// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major, N = 256, M = 128.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BLOCK_N >> 3) << 17) |
                           ((uint32_t)(BLOCK_M >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate)
        : "memory");
}
// kind::f8f6f4 with both operands e4m3 (format code 0) and an F32 accumulator: 32 elements (bytes)
// of K per instruction, so the shared-memory descriptors advance by the same 32 bytes per step.
constexpr uint32_t IDESC_E4M3 = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(BLOCK_N >> 3) << 17) |
                                ((uint32_t)(BLOCK_M >> 4) << 24);
__device__ __forceinline__ void mma_e4m3(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(IDESC_E4M3), "r"(accumulate)
        : "memory");
}
template <bool FP8>
__device__ __forceinline__ void mma_kind(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    if constexpr (FP8)
        mma_e4m3(tmem_d, adesc, bdesc, accumulate);
    else
        mma_bf16(tmem_d, adesc, bdesc, accumulate);
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 64 consecutive TMEM columns of this thread's lane (32x32b shape, 64 repetitions). The load is
// asynchronous: the values may be read only after tmem_wait on the same registers.
#define COSTAL_R8(i) "=r"(r[i]), "=r"(r[i + 1]), "=r"(r[i + 2]), "=r"(r[i + 3]), "=r"(r[i + 4]), "=r"(r[i + 5]), \
                     "=r"(r[i + 6]), "=r"(r[i + 7])
#define COSTAL_W8(i) "+r"(r[i]), "+r"(r[i + 1]), "+r"(r[i + 2]), "+r"(r[i + 3]), "+r"(r[i + 4]), "+r"(r[i + 5]), \
                     "+r"(r[i + 6]), "+r"(r[i + 7])
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t (&r)[64]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,"
        "%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
        : COSTAL_R8(0), COSTAL_R8(8), COSTAL_R8(16), COSTAL_R8(24), COSTAL_R8(32), COSTAL_R8(40), COSTAL_R8(48),
          COSTAL_R8(56)
        : "r"(taddr)
        : "memory");
}
// Wait for this thread's outstanding TMEM loads. The registers are in/out operands, so no use of
// them can be scheduled before the wait.
__device__ __forceinline__ void tmem_wait(uint32_t (&r)[64]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : COSTAL_W8(0), COSTAL_W8(8), COSTAL_W8(16), COSTAL_W8(24), COSTAL_W8(32), COSTAL_W8(40),
                   COSTAL_W8(48), COSTAL_W8(56)
                 :
                 : "memory");
}
#undef COSTAL_R8
#undef COSTAL_W8

// 8 TMEM columns at a run-time column offset, loaded and waited for.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

struct __align__(8) Barriers {
    uint64_t a_full;
    uint64_t b_full[4];
    uint64_t b_empty[4];
    uint64_t t_full[2];
    uint64_t t_empty[2];
    uint32_t tmem_base;
    int stop_tile;         // the list position at which the CTA stops (set by the TMA warp)
    float warp_floor[4];   // per epilogue warp: min over its rows of τ − E (never decreases)
};

// Per-query candidate buffer: BCAP = 2·LCAP entries in shared memory, [entry][query] with a row
// stride of BLOCK_M + 1 words (appends of 32 lanes and the warp's reads of one query are both free
// of bank conflicts). Survivors are appended with predicated stores; when a buffer could overflow,
// the warp selects its best `cap` cooperatively (radix select, no sort) and raises τ to the cap-th
// score. Every candidate outside a buffer scored ≤ τ when it was seen or evicted, and τ only grows.
constexpr int BSTRIDE = BLOCK_M + 1;

// f32 score → u32 with the same order (every admitted score is finite).
__device__ __forceinline__ uint32_t fkey(float v) {
    const uint32_t u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Shrink one query's buffer (cntL entries, all above its threshold tauL) to `cap` entries and return
// the new threshold: T = the cap-th largest score, found by a warp-wide radix select on the order
// keys (bit by bit from the highest bit where the buffer's keys differ, one ballot per slot a bit);
// the entries above T and enough of those equal to T are compacted to positions 0..cap-1 in buffer
// order. Entries dropped score ≤ T, so "everything outside the buffer scores ≤ τ" still holds. With
// cntL ≤ cap nothing changes.
template <int SL>
__device__ __noinline__ float flush_one(float* B_s, uint32_t* B_i, int qL, int cntL, int cap, int lane, float tauL) {
    if (cntL <= cap) return tauL;
    float sc[SL];
    uint32_t id[SL], key[SL];
    uint32_t kmin = 0xffffffffu, kmax = 0u;
#pragma unroll
    for (int s = 0; s < SL; ++s) {
        const int p = s * 32 + lane;
        const bool v = p < cntL;
        sc[s] = v ? B_s[p * BSTRIDE + qL] : 0.0f;
        id[s] = v ? B_i[p * BSTRIDE + qL] : 0u;
        key[s] = v ? fkey(sc[s]) : 0u;  // 0: below every valid key
        if (v) {
            kmin = min(kmin, key[s]);
            kmax = max(kmax, key[s]);
        }
    }
    kmin = __reduce_min_sync(COSTAL_FULL_MASK, kmin);
    kmax = __reduce_max_sync(COSTAL_FULL_MASK, kmax);
    // T lies in [kmin, kmax]: its bits above the highest differing bit are theirs
    const uint32_t diff = kmin ^ kmax;
    const int top = diff ? 31 - __clz(diff) : -1;
    uint32_t T = top >= 0 ? (kmax & ~((2u << top) - 1u)) : kmax;
    for (int b = top; b >= 0; --b) {
        const uint32_t c = T | (1u << b);
        int n_ge = 0;
#pragma unroll
        for (int s = 0; s < SL; ++s) n_ge += __popc(__ballot_sync(COSTAL_FULL_MASK, key[s] >= c));
        if (n_ge >= cap) T = c;
    }
    // keep key > T, and the first (cap − #{key > T}) entries with key == T
    int n_gt = 0;
#pragma unroll
    for (int s = 0; s < SL; ++s) n_gt += __popc(__ballot_sync(COSTAL_FULL_MASK, key[s] > T));
    const unsigned below = (1u << lane) - 1u;
    int eq_before = 0, kept_before = 0;
    bool keep[SL];
    int pos[SL];
#pragma unroll
    for (int s = 0; s < SL; ++s) {
        const unsigned meq = __ballot_sync(COSTAL_FULL_MASK, key[s] == T);
        const bool k = key[s] > T || (key[s] == T && eq_before + __popc(meq & below) < cap - n_gt);
        const unsigned mk = __ballot_sync(COSTAL_FULL_MASK, k);
        keep[s] = k;
        pos[s] = kept_before + __popc(mk & below);
        eq_before += __popc(meq);
        kept_before += __popc(mk);
    }
    __syncwarp();  // every lane has read its entries before any is overwritten
#pragma unroll
    for (int s = 0; s < SL; ++s) {
        if (keep[s]) {
            B_s[pos[s] * BSTRIDE + qL] = sc[s];
            B_i[pos[s] * BSTRIDE + qL] = id[s];
        }
    }
    __syncwarp();
    return fkey_inv(T);
}

// Flush every lane whose buffer holds more than `limit` entries.
template <int SL>
__device__ __forceinline__ void flush_full(float* B_s, uint32_t* B_i, int qbase, int lane, int cap, int limit, int& cnt,
                                           float& tau) {
    unsigned pend = __ballot_sync(COSTAL_FULL_MASK, cnt > limit);
    if (!pend) return;
    __syncwarp();  // the lanes' appends are visible to the whole warp
    while (pend) {
        const int L = __ffs(pend) - 1;
        pend &= pend - 1;
        const float t = flush_one<SL>(B_s, B_i, qbase + L, __shfl_sync(COSTAL_FULL_MASK, cnt, L), cap, lane,
                                      __shfl_sync(COSTAL_FULL_MASK, tau, L));
        if (lane == L) {
            cnt = min(cnt, cap);
            tau = t;
        }
    }
}

__device__ __forceinline__ float max8(const uint32_t* r) {
    const float a = max3f(__uint_as_float(r[0]), __uint_as_float(r[1]), __uint_as_float(r[2]));
    const float b = max3f(__uint_as_float(r[3]), __uint_as_float(r[4]), __uint_as_float(r[5]));
    return max3f(a, b, fmaxf(__uint_as_float(r[6]), __uint_as_float(r[7])));
}

// The 8 group maxima of a 64-column slice.
__device__ __forceinline__ void group_max8(const uint32_t (&r)[64], float* gm) {
#pragma unroll
    for (int g = 0; g < 8; ++g) gm[g] = max8(r + 8 * g);
}

// The cap-th largest of N values (cap ≤ N, N a power of two): a bitonic sorting network in registers.
template <int N>
__device__ __forceinline__ float kth_of(float (&v)[N], int cap) {
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const int j = i ^ stride;
                if (j > i) {
                    const float a = v[i], b = v[j];
                    const bool desc = (i & size) == 0;  // descending runs first
                    v[i] = desc ? fmaxf(a, b) : fminf(a, b);
                    v[j] = desc ? fminf(a, b) : fmaxf(a, b);
                }
            }
        }
    }
    float t = v[0];
#pragma unroll
    for (int i = 0; i < N; ++i)
        if (i == cap - 1) t = v[i];
    return t;
}

// The 16 four-column group maxima of a 64-column slice.
__device__ __forceinline__ void group_max4(const uint32_t (&r)[64], float* gm) {
#pragma unroll
    for (int g = 0; g < 16; ++g)
        gm[g] = fmaxf(max3f(__uint_as_float(r[4 * g]), __uint_as_float(r[4 * g + 1]), __uint_as_float(r[4 * g + 2])),
                      __uint_as_float(r[4 * g + 3]));
}

// One 64-column slice held in registers: a per-lane 8-bit mask of the 8-column groups whose maximum
// is above the lane's threshold, OR-ed over the warp. Returns the warp's mask.
__device__ __forceinline__ unsigned slice_mask(const uint32_t (&r)[64], float tau) {
    unsigned m = 0;
#pragma unroll
    for (int g = 0; g < 8; ++g) m |= (max8(r + 8 * g) > tau ? 1u : 0u) << g;
    return __reduce_or_sync(COSTAL_FULL_MASK, m);
}

// The 8-column groups of a slice that some lane of the warp needs: re-read each from TMEM (at a
// run-time column) and append each lane's survivors (strictly above τ, in range, not the query
// itself). Kept out of line: the rare path stays off the hot loop's instruction footprint.
template <int SL>
__device__ __noinline__ void admit_groups(unsigned gmask, uint32_t taddr, int cb, int n, int q, int qi, int qbase,
                                          int lane, int cap, int q_lo, float* B_s, uint32_t* B_i,
                                          int* cnt_io, float* tau_io) {
    constexpr int BCAP = 32 * SL;
    int cnt = *cnt_io;
    float tau = *tau_io;
    while (gmask) {
        const int g = __ffs(gmask) - 1;
        gmask &= gmask - 1;
        float v[8];
        tmem_ld8(taddr + (uint32_t)(8 * g), v);
        const int c = cb + 8 * g;
        const bool clean = c + 8 <= n && (c + 8 <= q_lo || c >= q_lo + 32);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int col = c + j;
            if (v[j] > tau && (clean || (col < n && col != q))) {
                B_s[cnt * BSTRIDE + qi] = v[j];
                B_i[cnt * BSTRIDE + qi] = (uint32_t)col;
                ++cnt;
            }
        }
        flush_full<SL>(B_s, B_i, qbase, lane, cap, BCAP - 8, cnt, tau);
    }
    *cnt_io = cnt;
    *tau_io = tau;
}

template <int SLOTS, bool KLOOP, bool FP8 = false, bool PAIR = false>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_coarse_tc(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                const __grid_constant__ CUtensorMap map_bw, int n, int np,
                int nkb, int nkb_b, int ksteps, int k1s, int stages, int cap, const uint32_t* __restrict__ perm,
                const uint32_t* __restrict__ lists, const float* __restrict__ list_ub,
                const uint32_t* __restrict__ counts, int ncb, const double* __restrict__ row_eps,
                uint32_t* __restrict__ cand_idx, float* __restrict__ cand_score, float* __restrict__ tau_out,
                unsigned long long* __restrict__ stopped_total, unsigned long long* __restrict__ timeout_flag,
                int qb0) {
    constexpr int SL = 2 * SLOTS;  // buffer slots per lane in a flush: BCAP = 2·LCAP entries
    // The split-FP8 kind computes on the rows scaled by 2^8, so its accumulators hold 2^16 × the
    // coarse score: thresholds and admissions stay in those units, the lists and floors are scaled
    // back exactly.
    constexpr float OSCALE = FP8 ? 0x1p-16f : 1.0f;
    constexpr int KBE = FP8 ? 128 : KB;  // elements in one 128-byte K block (the TMA x coordinate step)
    constexpr int BCAP = 32 * SL;
    extern __shared__ unsigned char smem_raw[];
    // 1024-byte alignment for the swizzled tiles
    const uint32_t base_u32 = smem_u32(smem_raw);
    unsigned char* smem = smem_raw + ((1024 - (base_u32 & 1023)) & 1023);
    // Resident A: the query tile (nkb K blocks) once, then `stages` column tiles of nkb_b K blocks. K loop (deep rows, KLOOP): every stage holds one K block of the query tile
    // and of the column tile, and a tile's MMA chain runs over nkb stages.
    const uint32_t stage_bytes = KLOOP ? (uint32_t)(A_KB_BYTES + B_KB_BYTES) : (uint32_t)nkb_b * B_KB_BYTES;
    unsigned char* a_tile = smem;                                            // nkb × 16 KB (resident A)
    unsigned char* b_tiles = KLOOP ? smem : a_tile + (size_t)nkb * A_KB_BYTES;  // stages × stage_bytes
    float* B_s = reinterpret_cast<float*>(b_tiles + (size_t)stages * stage_bytes);  // [BCAP][BSTRIDE]
    uint32_t* B_i = reinterpret_cast<uint32_t*>(B_s + BCAP * BSTRIDE);
    Barriers* bars = reinterpret_cast<Barriers*>(B_i + BCAP * BSTRIDE);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Rows and columns are in the working order (rows sorted by locality cell; perm maps back to the
    // original index). A CTA visits the column blocks of its list, nearest first, or all of them.
    // CTA b takes query block qb0 + b (a launch over a contiguous range of query blocks: one shard).
    const int qb = qb0 + (int)blockIdx.x;
    const int q0 = qb * BLOCK_M;
    // A tile's 256 columns are two halves of HALF_N. PAIR (lists of 128-column blocks): the halves are
    // two consecutive list entries, each loaded by its own TMA box unless they are adjacent; an odd
    // list's last tile has one entry, its second half repeats the first and the epilogue leaves it out.
    // Otherwise one list entry of 256 columns, or without lists 256 consecutive columns. (The pairing
    // is a compile-time choice: the epilogue is latency-bound, and its runtime tests cost 3 % of the
    // kernel when the lists hold 256-column blocks.)
    constexpr int EPC = PAIR ? 2 : 1;  // list entries per tile
    const int nentries = lists ? (int)counts[qb] : 0;
    const int ntiles = lists ? (nentries + EPC - 1) / EPC : np / BLOCK_N;
    const uint32_t* my_list = lists ? lists + (size_t)qb * ncb : nullptr;
    auto tile_cols = [&](int t, int& c0, int& c1) -> bool {
        if constexpr (PAIR) {
            const bool two = 2 * t + 1 < nentries;
            c0 = (int)my_list[2 * t] * HALF_N;
            c1 = two ? (int)my_list[2 * t + 1] * HALF_N : c0;
            return two;
        } else {
            c0 = (my_list ? (int)my_list[t] : t) * BLOCK_N;
            c1 = c0 + HALF_N;
            return true;
        }
    };
    // the list entries of tile t lie inside the operands (the list kernel never writes others)
    auto tile_ok = [&](int t) -> bool {
        if (!my_list) return true;
        if constexpr (PAIR) {
            const unsigned lim = (unsigned)(np / HALF_N);
            return my_list[2 * t] < lim && (2 * t + 1 >= nentries || my_list[2 * t + 1] < lim);
        } else {
            return my_list[t] < (unsigned)(np / BLOCK_N);
        }
    };
    const uint32_t a_bytes = (uint32_t)nkb * A_KB_BYTES, b_bytes = (uint32_t)nkb_b * B_KB_BYTES;
    (void)a_bytes;

    if (threadIdx.x == 0) {
        mbar_init(&bars->a_full, 1);
        for (int s = 0; s < stages; ++s) {
            mbar_init(&bars->b_full[s], 1);
            mbar_init(&bars->b_empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&bars->t_full[b], 1);
            mbar_init(&bars->t_empty[b], EPI_WARPS);
        }
        bars->stop_tile = ntiles;
        for (int w = 0; w < EPI_WARPS; ++w) bars->warp_floor[w] = -CUDART_INF_F;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == EPI_WARPS + 1) {  // the MMA warp owns the TMEM allocation
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&bars->tmem_base)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = bars->tmem_base;

    if (warp == EPI_WARPS) {
        // ------------------------------------------------------------------ TMA producer
        if (KLOOP && lane == 0) {
            const float* my_ub = list_ub ? list_ub + (size_t)qb * ncb : nullptr;
            bool go = true;
            for (int t = 0; go && t < ntiles; ++t) {
                const bool ok = tile_ok(t);
                int c0 = 0, c1 = 0;
                if (ok) tile_cols(t, c0, c1);
                for (int kb = 0; kb < nkb; ++kb) {
                    const int g = t * nkb + kb, s = g % stages;
                    const uint32_t ph = (uint32_t)(g / stages) & 1u;
                    if (!mbar_wait(&bars->b_empty[s], ph ^ 1u, timeout_flag, true)) {
                        go = false;
                        break;
                    }
                    if (kb == 0) {
                        bool stop = false;
                        if (!ok) {
                            atomicExch(timeout_flag, 2ull);  // never produced by the list kernel
                            stop = true;
                        } else if (t > 0 && my_ub) {
                            volatile float* wf = bars->warp_floor;
                            const float fl = fminf(fminf(wf[0], wf[1]), fminf(wf[2], wf[3]));
                            if (my_ub[t * EPC] < fl) {
                                stop = true;
                                if (stopped_total)
                                    atomicAdd(stopped_total, (unsigned long long)(nentries - t * EPC));
                            }
                        }
                        if (stop) {
                            *reinterpret_cast<volatile int*>(&bars->stop_tile) = t;
                            mbar_arrive(&bars->b_full[s]);
                            go = false;
                            break;
                        }
                    }
                    mbar_expect_tx(&bars->b_full[s], (uint32_t)(A_KB_BYTES + B_KB_BYTES));
                    unsigned char* dst = b_tiles + (size_t)s * stage_bytes;
                    tma_load_2d(dst, &map_a, kb * KBE, q0, &bars->b_full[s]);
                    if (c1 == c0 + HALF_N) {  // adjacent halves: one 256-row box
                        tma_load_2d(dst + A_KB_BYTES, &map_bw, kb * KBE, c0, &bars->b_full[s]);
                    } else {
                        tma_load_2d(dst + A_KB_BYTES, &map_b, kb * KBE, c0, &bars->b_full[s]);
                        tma_load_2d(dst + A_KB_BYTES + B_HALF_BYTES, &map_b, kb * KBE, c1, &bars->b_full[s]);
                    }
                }
            }
        }
        if (!KLOOP && lane == 0) {
            mbar_expect_tx(&bars->a_full, a_bytes);
            for (int kb = 0; kb < nkb; ++kb) tma_load_2d(a_tile + kb * A_KB_BYTES, &map_a, kb * KBE, q0, &bars->a_full);
            const float* my_ub = list_ub ? list_ub + (size_t)qb * ncb : nullptr;
            for (int t = 0; t < ntiles; ++t) {
                const int s = t % stages;
                const uint32_t ph = (uint32_t)(t / stages) & 1u;
                if (!mbar_wait(&bars->b_empty[s], ph ^ 1u, timeout_flag, true)) break;
                if (!tile_ok(t)) {
                    // a list entry outside the operands (never produced by the list kernel): report it
                    // and stop the CTA here like an early stop, so no role reads past the operands
                    atomicExch(timeout_flag, 2ull);
                    *reinterpret_cast<volatile int*>(&bars->stop_tile) = t;
                    mbar_arrive(&bars->b_full[s]);
                    break;
                }
                if (t > 0 && my_ub) {
                    // Every column of the tile's first list entry (and of all later ones: the bounds do
                    // not increase) has cosine ≤ its bound; its coarse score is ≤ bound + E_i. When that
                    // is below every row's threshold τ_i, none of them can be admitted: stop here. The
                    // floors read may be stale, i.e. lower, which only delays the stop.
                    volatile float* wf = bars->warp_floor;
                    const float fl = fminf(fminf(wf[0], wf[1]), fminf(wf[2], wf[3]));
                    if (my_ub[t * EPC] < fl) {
                        *reinterpret_cast<volatile int*>(&bars->stop_tile) = t;
                        if (stopped_total) atomicAdd(stopped_total, (unsigned long long)(nentries - t * EPC));
                        mbar_arrive(&bars->b_full[s]);  // completes the phase without data (release)
                        break;
                    }
                }
                mbar_expect_tx(&bars->b_full[s], b_bytes);
                unsigned char* dst = b_tiles + (size_t)s * b_bytes;
                int c0, c1;
                tile_cols(t, c0, c1);
                // (the last K block may reach past the operand's row: TMA fills those columns with zeros
                // and reads nothing for them)
                if (c1 == c0 + HALF_N) {  // adjacent halves: one 256-row box per K block
                    for (int kb = 0; kb < nkb_b; ++kb)
                        tma_load_2d(dst + kb * B_KB_BYTES, &map_bw, kb * KBE, c0, &bars->b_full[s]);
                } else {
                    for (int kb = 0; kb < nkb_b; ++kb) {
                        tma_load_2d(dst + kb * B_KB_BYTES, &map_b, kb * KBE, c0, &bars->b_full[s]);
                        tma_load_2d(dst + kb * B_KB_BYTES + B_HALF_BYTES, &map_b, kb * KBE, c1, &bars->b_full[s]);
                    }
                }
            }
        }
    } else if (warp == EPI_WARPS + 1) {
        // ------------------------------------------------------------------ MMA issuer
        if (KLOOP && lane == 0) {
            bool go = true;
            for (int t = 0; go && t < ntiles; ++t) {
                const int buf = t & 1;
                const uint32_t bph = (uint32_t)(t >> 1) & 1u;
                if (!mbar_wait(&bars->t_empty[buf], bph ^ 1u, timeout_flag, true)) break;
                const uint32_t d = tmem + (uint32_t)(buf * BLOCK_N);
                for (int kb = 0; kb < nkb; ++kb) {
                    const int g = t * nkb + kb, s = g % stages;
                    const uint32_t ph = (uint32_t)(g / stages) & 1u;
                    if (!mbar_wait(&bars->b_full[s], ph, timeout_flag, true)) {
                        go = false;
                        break;
                    }
                    tc_fence_after();
                    if (kb == 0 && *reinterpret_cast<volatile int*>(&bars->stop_tile) == t) {
                        mbar_arrive(&bars->t_full[buf]);  // pass the stop on to the epilogue warps
                        go = false;
                        break;
                    }
                    const uint32_t a_base = smem_u32(b_tiles + (size_t)s * stage_bytes);
                    const uint32_t b_base = a_base + A_KB_BYTES;
                    const int nks = min(4, ksteps - 4 * kb);
                    for (int ks = 0; ks < nks; ++ks) {
                        const uint32_t koff = (uint32_t)(ks * 32);  // 16 bf16 = 32 bytes inside the swizzle row
                        mma_kind<FP8>(d, sw128_desc(a_base + koff), sw128_desc(b_base + koff), (kb | ks) ? 1u : 0u);
                    }
                    mma_commit(&bars->b_empty[s]);
                }
                if (!go) break;
                mma_commit(&bars->t_full[buf]);
            }
        }
        if (!KLOOP && lane == 0) {
            bool ok = mbar_wait(&bars->a_full, 0, timeout_flag, true);
            tc_fence_after();
            const uint32_t a_base = smem_u32(a_tile);
            for (int t = 0; ok && t < ntiles; ++t) {
                const int s = t % stages, buf = t & 1;
                const uint32_t ph = (uint32_t)(t / stages) & 1u, bph = (uint32_t)(t >> 1) & 1u;
                if (!mbar_wait(&bars->t_empty[buf], bph ^ 1u, timeout_flag, true)) break;
                if (!mbar_wait(&bars->b_full[s], ph, timeout_flag, true)) break;
                tc_fence_after();
                if (*reinterpret_cast<volatile int*>(&bars->stop_tile) == t) {
                    mbar_arrive(&bars->t_full[buf]);  // pass the stop on to the epilogue warps
                    break;
                }
                const uint32_t b_base = smem_u32(b_tiles + (size_t)s * b_bytes);
                const uint32_t d = tmem + (uint32_t)(buf * BLOCK_N);
                // Two chains into one accumulator: steps [0, k1s) pair A's [hi | hi] with B's [hi | lo];
                // steps [k1s, ksteps) pair A's [lo] with B's leading [hi] (A's zero padding cancels
                // whatever of B's lo those steps also cover). 16 bf16 = 32 bytes inside a swizzle row.
                for (int ks = 0; ks < ksteps; ++ks) {
                    const int kb = ks < k1s ? ks : ks - k1s;
                    const uint64_t ad = sw128_desc(a_base + (uint32_t)(ks >> 2) * A_KB_BYTES + (uint32_t)((ks & 3) * 32));
                    const uint64_t bd = sw128_desc(b_base + (uint32_t)(kb >> 2) * B_KB_BYTES + (uint32_t)((kb & 3) * 32));
                    mma_kind<FP8>(d, ad, bd, ks > 0 ? 1u : 0u);
                }
                mma_commit(&bars->b_empty[s]);
                mma_commit(&bars->t_full[buf]);
            }
        }
    } else {
        // ------------------------------------------------------------------ epilogue (warps 0-3)
        const int qbase = warp * 32;
        const int qi = qbase + lane;  // TMEM lane = query row within the block
        const int q = q0 + qi, q_lo = q0 + qbase;
        // this row's coarse-error bound, rounded up to f32 (rows past n never hold the CTA back)
        const float row_e = q < n ? __double2float_ru(row_eps[perm ? perm[q] : (uint32_t)q]) : 0.0f;
        float tau = -CUDART_INF_F;
        int cnt = 0;
        const uint32_t lane_addr = tmem + ((uint32_t)qbase << 16);
        uint32_t ra[64], rb[64];
        int cnt_m = 0;  // cnt and tau round-trip through these when the rare path runs
        float tau_m = tau;
        for (int t = 0; t < ntiles; ++t) {
            const int buf = t & 1;
            const uint32_t bph = (uint32_t)(t >> 1) & 1u;
            if (!mbar_wait(&bars->t_full[buf], bph, timeout_flag, false)) break;
            tc_fence_after();
            if (*reinterpret_cast<volatile int*>(&bars->stop_tile) == t) break;
            int c0, c1;
            const bool two = tile_cols(t, c0, c1);  // false: the tile's second half has no list entry
            const uint32_t tb = lane_addr + (uint32_t)(buf * BLOCK_N);
            if (t == 0) {
                // A starting threshold from the first tiles: the cap-th largest of their column-group
                // maxima (64 groups of 8 columns over tiles 0 and 1, 32 over tile 0 alone, or 64 of 4
                // when cap > 32) is reached by cap distinct columns, so no other column below it can
                // be among the query's best cap. (When the
                // query's own column or padding supplies one of those maxima, τ₀ can be a little too
                // high; that only costs the certificate, since τ never falls and everything left out
                // stays below it.) A half without a list entry counts as −∞. The first tile itself is
                // admitted at ≥ τ₀ (one below in the strict test), later tiles at > τ as usual.
                if (cap <= 32 && ntiles >= 2) {
                    // both accumulators hold a tile by now (tiles 0 and 1): 64 groups of 512 columns
                    if (!mbar_wait(&bars->t_full[1], 0, timeout_flag, false)) break;
                    tc_fence_after();
                    // (no stop can fall on tile 1: the warps' floors are still −inf when it is issued)
                    int d0, d1;
                    const bool two1 = tile_cols(1, d0, d1);
                    float gmax[64];
#pragma unroll
                    for (int h = 0; h < 8; ++h) {
                        tmem_ld64(lane_addr + (uint32_t)((h >> 2) * BLOCK_N + 64 * (h & 3)), ra);
                        tmem_wait(ra);
                        group_max8(ra, gmax + 8 * h);
                        if ((h & 3) >= 2 && !((h >> 2) ? two1 : two))
#pragma unroll
                            for (int g = 0; g < 8; ++g) gmax[8 * h + g] = -CUDART_INF_F;
                    }
                    tau = nextafterf(kth_of<64>(gmax, cap), -CUDART_INF_F);
                } else if (cap <= 32) {
                    float gmax[32];
#pragma unroll
                    for (int h = 0; h < 4; ++h) {
                        tmem_ld64(tb + (uint32_t)(64 * h), ra);
                        tmem_wait(ra);
                        group_max8(ra, gmax + 8 * h);
                        if (h >= 2 && !two)
#pragma unroll
                            for (int g = 0; g < 8; ++g) gmax[8 * h + g] = -CUDART_INF_F;
                    }
                    tau = nextafterf(kth_of<32>(gmax, cap), -CUDART_INF_F);
                } else {
                    float gmax[64];
#pragma unroll
                    for (int h = 0; h < 4; ++h) {
                        tmem_ld64(tb + (uint32_t)(64 * h), ra);
                        tmem_wait(ra);
                        group_max4(ra, gmax + 16 * h);
                        if (h >= 2 && !two)
#pragma unroll
                            for (int g = 0; g < 16; ++g) gmax[16 * h + g] = -CUDART_INF_F;
                    }
                    tau = nextafterf(kth_of<64>(gmax, cap), -CUDART_INF_F);
                }
            }
            // Four 64-column slices (two per half), as a two-step software pipeline: the next
            // slice's TMEM load is in flight while one is scanned. A slice costs a max tree and a warp
            // OR; only the 8-column groups some lane needs are re-read and scanned.
            tmem_ld64(tb, ra);
            tmem_wait(ra);
#pragma unroll 1
            for (int h = 0; h < 2; ++h) {
                const int ch = h ? c1 : c0;  // the half's first column
                tmem_ld64(tb + (uint32_t)(HALF_N * h + 64), rb);
                unsigned gm = slice_mask(ra, tau);
                if (gm) {
                    cnt_m = cnt;
                    tau_m = tau;
                    admit_groups<SL>(gm, tb + (uint32_t)(HALF_N * h), ch, n, q, qi, qbase, lane, cap, q_lo, B_s, B_i,
                                     &cnt_m, &tau_m);
                    cnt = cnt_m;
                    tau = tau_m;
                }
                tmem_wait(rb);
                if (h == 0 && two) tmem_ld64(tb + HALF_N, ra);
                gm = slice_mask(rb, tau);
                if (gm) {
                    cnt_m = cnt;
                    tau_m = tau;
                    admit_groups<SL>(gm, tb + (uint32_t)(HALF_N * h + 64), ch + 64, n, q, qi, qbase, lane, cap, q_lo,
                                     B_s, B_i, &cnt_m, &tau_m);
                    cnt = cnt_m;
                    tau = tau_m;
                }
                if (h == 0) {
                    if (!two) break;
                    tmem_wait(ra);
                }
            }
            // every TMEM read of this accumulator is complete: hand it back to the MMA warp
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&bars->t_empty[buf]);
            // the warp's floor min(τ − E) for the TMA warp's stop test (signed-int order of the f32)
            if (list_ub) {
                const float f = q < n ? __fsub_rd(tau * OSCALE, row_e) : CUDART_INF_F;
                int key = __float_as_int(f);
                key = __reduce_min_sync(COSTAL_FULL_MASK, key >= 0 ? key : key ^ 0x7fffffff);
                if (lane == 0)
                    *reinterpret_cast<volatile float*>(&bars->warp_floor[warp]) =
                        __int_as_float(key >= 0 ? key : key ^ 0x7fffffff);
            }
        }
        // final selection: every buffer down to its best `cap` entries (in buffer order)
        flush_full<SL>(B_s, B_i, qbase, lane, cap, cap, cnt, tau);
        __syncwarp();
        if (q < n) {
            const uint32_t qo = perm ? perm[q] : (uint32_t)q;
            for (int p = 0; p < cap; ++p) {
                // an empty slot (fewer than cap candidates) carries index 0xffffffff and score −inf
                const uint32_t cw = p < cnt ? B_i[p * BSTRIDE + qi] : 0xffffffffu;
                cand_idx[(size_t)qo * cap + p] = cw < (uint32_t)n ? (perm ? perm[cw] : cw) : 0xffffffffu;
                cand_score[(size_t)qo * cap + p] = p < cnt ? B_s[p * BSTRIDE + qi] * OSCALE : -CUDART_INF_F;
            }
            tau_out[qo] = tau * OSCALE;
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == EPI_WARPS + 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// ---- per-row block bounds --------------------------------------------------------------------------
//
// Every row x of column block B lies within angle r_B of B's unit centre c_B, so for a query row q,
// cos(q, x) ≤ cos(max(0, angle(q, c_B) − r_B)). Over a query block Q the bound is loosest for the
// row nearest c_B, so the block needs only M[Q][B] = max over q ∈ Q of q·c_B: a (centres × query
// rows) product, run here with the coarse pass's split-BF16 operands. The centres take the A layout
// (M = 128 centres per tile, one TMEM lane each) and the query block's rows the B layout (N = 128),
// so every epilogue thread reduces its own centre's 128 accumulators in registers. One CTA per query
// block: warp 4 loads the block's rows once and streams centre tiles into a ring of stages, warp 5
// issues the MMAs into two 128-column accumulators, warps 0-3 reduce and write M[Q][·].
constexpr int RM_N = 128;                       // query rows per tile (the MMA's N)
constexpr int RM_KB_BYTES = 128 * 128;          // one 128-byte K block of 128 operand rows
constexpr uint32_t RM_TMEM_COLS = 2 * RM_N;     // two accumulators
constexpr uint32_t IDESC_RM = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(RM_N >> 3) << 17) |
                              ((uint32_t)(BLOCK_M >> 4) << 24);

struct __align__(8) RmBars {
    uint64_t q_full;
    uint64_t c_full[4];
    uint64_t c_empty[4];
    uint64_t t_full[2];
    uint64_t t_empty[2];
    uint32_t tmem_base;
};

__device__ __forceinline__ void mma_rm(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(IDESC_RM), "r"(accumulate)
        : "memory");
}

__global__ void __launch_bounds__(NTHREADS, 1)
    k_block_rowmax(const __grid_constant__ CUtensorMap map_c, const __grid_constant__ CUtensorMap map_q, int n, int ncb,
                   int nkb_c, int nkb_q, int ksteps, int k1s, int stages, float* __restrict__ rowmax,
                   unsigned long long* __restrict__ timeout_flag) {
    extern __shared__ unsigned char smem_raw[];
    const uint32_t base_u32 = smem_u32(smem_raw);
    unsigned char* smem = smem_raw + ((1024 - (base_u32 & 1023)) & 1023);  // 1024-byte aligned tiles
    const uint32_t q_bytes = (uint32_t)nkb_q * RM_KB_BYTES, c_bytes = (uint32_t)nkb_c * RM_KB_BYTES;
    unsigned char* q_tile = smem;                 // the query block's rows, resident
    unsigned char* c_tiles = smem + q_bytes;      // stages × one centre tile
    RmBars* bars = reinterpret_cast<RmBars*>(c_tiles + (size_t)stages * c_bytes);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int Q = (int)blockIdx.x, q0 = Q * RM_N;
    const int ntiles = (ncb + BLOCK_M - 1) / BLOCK_M;

    if (threadIdx.x == 0) {
        mbar_init(&bars->q_full, 1);
        for (int s = 0; s < stages; ++s) {
            mbar_init(&bars->c_full[s], 1);
            mbar_init(&bars->c_empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&bars->t_full[b], 1);
            mbar_init(&bars->t_empty[b], EPI_WARPS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == EPI_WARPS + 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&bars->tmem_base)),
                     "r"(RM_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = bars->tmem_base;

    if (warp == EPI_WARPS) {
        if (lane == 0) {
            mbar_expect_tx(&bars->q_full, q_bytes);
            for (int kb = 0; kb < nkb_q; ++kb)
                tma_load_2d(q_tile + (size_t)kb * RM_KB_BYTES, &map_q, kb * KB, q0, &bars->q_full);
            for (int t = 0; t < ntiles; ++t) {
                const int s = t % stages;
                const uint32_t ph = (uint32_t)(t / stages) & 1u;
                if (!mbar_wait(&bars->c_empty[s], ph ^ 1u, timeout_flag, true)) break;
                mbar_expect_tx(&bars->c_full[s], c_bytes);
                unsigned char* dst = c_tiles + (size_t)s * c_bytes;
                for (int kb = 0; kb < nkb_c; ++kb)
                    tma_load_2d(dst + (size_t)kb * RM_KB_BYTES, &map_c, kb * KB, t * BLOCK_M, &bars->c_full[s]);
            }
        }
    } else if (warp == EPI_WARPS + 1) {
        if (lane == 0) {
            const bool ok = mbar_wait(&bars->q_full, 0, timeout_flag, true);
            tc_fence_after();
            const uint32_t q_base = smem_u32(q_tile);
            for (int t = 0; ok && t < ntiles; ++t) {
                const int s = t % stages, buf = t & 1;
                const uint32_t ph = (uint32_t)(t / stages) & 1u, bph = (uint32_t)(t >> 1) & 1u;
                if (!mbar_wait(&bars->t_empty[buf], bph ^ 1u, timeout_flag, true)) break;
                if (!mbar_wait(&bars->c_full[s], ph, timeout_flag, true)) break;
                tc_fence_after();
                const uint32_t c_base = smem_u32(c_tiles + (size_t)s * c_bytes);
                const uint32_t dt = tmem + (uint32_t)(buf * RM_N);
                // the coarse pass's chains with the operands' roles swapped: the products are the
                // same three pieces (hi·hi, hi·lo, lo·hi) of every (centre, row) pair
                for (int ks = 0; ks < ksteps; ++ks) {
                    const int kb = ks < k1s ? ks : ks - k1s;
                    const uint64_t ad = sw128_desc(c_base + (uint32_t)(ks >> 2) * RM_KB_BYTES + (uint32_t)((ks & 3) * 32));
                    const uint64_t bd = sw128_desc(q_base + (uint32_t)(kb >> 2) * RM_KB_BYTES + (uint32_t)((kb & 3) * 32));
                    mma_rm(dt, ad, bd, ks > 0 ? 1u : 0u);
                }
                mma_commit(&bars->c_empty[s]);
                mma_commit(&bars->t_full[buf]);
            }
        }
    } else {
        const int nv = min(RM_N, n - q0);  // live query rows of the block (the rest are zero rows)
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        uint32_t ra[64], rb[64];
        for (int t = 0; t < ntiles; ++t) {
            const int buf = t & 1;
            const uint32_t bph = (uint32_t)(t >> 1) & 1u;
            if (!mbar_wait(&bars->t_full[buf], bph, timeout_flag, false)) break;
            tc_fence_after();
            const uint32_t tb = lane_addr + (uint32_t)(buf * RM_N);
            tmem_ld64(tb, ra);
            tmem_ld64(tb + 64, rb);
            tmem_wait(ra);
            tmem_wait(rb);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&bars->t_empty[buf]);
            if (nv < RM_N) {  // the last block: rows past n do not count
#pragma unroll
                for (int j = 0; j < 64; ++j) {
                    if (j >= nv) ra[j] = __float_as_uint(-CUDART_INF_F);
                    if (64 + j >= nv) rb[j] = __float_as_uint(-CUDART_INF_F);
                }
            }
            float m0 = -CUDART_INF_F, m1 = -CUDART_INF_F, m2 = -CUDART_INF_F, m3 = -CUDART_INF_F;
#pragma unroll
            for (int j = 0; j < 64; j += 4) {
                m0 = max3f(m0, __uint_as_float(ra[j]), __uint_as_float(rb[j]));
                m1 = max3f(m1, __uint_as_float(ra[j + 1]), __uint_as_float(rb[j + 1]));
                m2 = max3f(m2, __uint_as_float(ra[j + 2]), __uint_as_float(rb[j + 2]));
                m3 = max3f(m3, __uint_as_float(ra[j + 3]), __uint_as_float(rb[j + 3]));
            }
            const int c = t * BLOCK_M + warp * 32 + lane;
            if (c < ncb) rowmax[(size_t)Q * ncb + c] = fmaxf(fmaxf(m0, m1), fmaxf(m2, m3));
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == EPI_WARPS + 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(RM_TMEM_COLS) : "memory");
    }
}

// ---- operand preparation ----------------------------------------------------------------------

// One CTA per 128 working rows: each thread splits its row (read from xsT at the original index, or
// from wrows, the rows already in working order, row-major: a row's values are then contiguous instead
// of one cache line each) into the two operands in shared memory and records the f64 norms of the pieces: [0] ‖a_hi‖,
// [1] ‖a_lo‖, [2] ‖r‖, [3] ‖a_hi + a_lo‖; then the CTA writes the 128 operand rows with coalesced
// word stores. Rows in [n, rows) are written as zeros. The maxima over rows go to colmax through one
// atomic per warp. Two layouts: compact (k1 > 0) A = [hi | hi | 0 … k1 | lo | 0 … kpa] and
// B = [hi | lo | 0 … kpb]; otherwise A = [hi | lo | hi | 0 … kp], B = [hi | hi | lo | 0 … kp].
constexpr int SPLIT_ROWS = 128;
__global__ void __launch_bounds__(SPLIT_ROWS)
    k_split(const float* __restrict__ xsT, const float* __restrict__ wrows, int n, int np_x, int rows, int d, int kpa,
            int kpb, int k1, const uint32_t* __restrict__ perm, __nv_bfloat16* __restrict__ opa,
            __nv_bfloat16* __restrict__ opb, double* __restrict__ pnorm, unsigned long long* __restrict__ colmax) {
    extern __shared__ uint32_t sw[];  // [SPLIT_ROWS][kpa/2 + 1] then [SPLIT_ROWS][kpb/2 + 1] words
    const int wsa = kpa / 2 + 1, wsb = kpb / 2 + 1;  // odd word strides: the 32 lanes' rows fall in 32 banks
    __nv_bfloat16* ta = reinterpret_cast<__nv_bfloat16*>(sw);
    __nv_bfloat16* tb = reinterpret_cast<__nv_bfloat16*>(sw + SPLIT_ROWS * wsa);
    const int lr = threadIdx.x, r = blockIdx.x * SPLIT_ROWS + lr;  // working row
    const bool live = r < n;
    const int o = live ? (perm ? (int)perm[r] : r) : 0;  // its original row
    __nv_bfloat16* ra = ta + (size_t)lr * 2 * wsa;
    __nv_bfloat16* rb = tb + (size_t)lr * 2 * wsb;
    double sh = 0.0, sl = 0.0, sr = 0.0, sp = 0.0;
    const __nv_bfloat16 zero = __float2bfloat16_rn(0.0f);
    for (int t = 0; t < kpa; ++t) ra[t] = zero;
    for (int t = 0; t < kpb; ++t) rb[t] = zero;
    for (int t = 0; t < d; ++t) {
        const float a = live ? (wrows ? wrows[(size_t)r * d + t] : xsT[(size_t)t * np_x + o]) : 0.0f;
        const __nv_bfloat16 hb = __float2bfloat16_rn(a);
        const float h = __bfloat162float(hb);
        const float e = a - h;  // exact in f32
        const __nv_bfloat16 lb = __float2bfloat16_rn(e);
        const float l = __bfloat162float(lb);
        const float rem = e - l;  // exact in f32
        if (k1 > 0) {
            ra[t] = hb;
            ra[d + t] = hb;
            ra[k1 + t] = lb;
            rb[t] = hb;
            rb[d + t] = lb;
        } else {
            ra[t] = hb;
            ra[d + t] = lb;
            ra[2 * d + t] = hb;
            rb[t] = hb;
            rb[d + t] = hb;
            rb[2 * d + t] = lb;
        }
        const double h64 = f64_of(h), l64 = f64_of(l), r64 = f64_of(rem);  // exact widenings
        sh = __fma_rn(h64, h64, sh);
        sl = __fma_rn(l64, l64, sl);
        sr = __fma_rn(r64, r64, sr);
        const double p = h64 + l64;
        sp = __fma_rn(p, p, sp);
    }
    const double v[4] = {sqrt(sh), sqrt(sl), sqrt(sr), sqrt(sp)};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (live) pnorm[(size_t)j * n + o] = v[j];
        // non-negative doubles order like their bit patterns
        unsigned long long b = live ? (unsigned long long)__double_as_longlong(v[j]) : 0ull;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const unsigned long long ob = __shfl_xor_sync(COSTAL_FULL_MASK, b, off);
            b = ob > b ? ob : b;
        }
        if ((threadIdx.x & 31) == 0 && b > *reinterpret_cast<volatile unsigned long long*>(&colmax[j]))
            atomicMax(&colmax[j], b);
    }
    __syncthreads();
    const int wpa = kpa / 2, wpb = kpb / 2;  // words per operand row
    uint32_t* ga = reinterpret_cast<uint32_t*>(opa) + (size_t)blockIdx.x * SPLIT_ROWS * wpa;
    uint32_t* gb = reinterpret_cast<uint32_t*>(opb) + (size_t)blockIdx.x * SPLIT_ROWS * wpb;
    for (int e = threadIdx.x; e < SPLIT_ROWS * wpa; e += SPLIT_ROWS) {
        const int row = e / wpa, w = e % wpa;
        if (blockIdx.x * SPLIT_ROWS + row < rows) ga[e] = sw[row * wsa + w];
    }
    for (int e = threadIdx.x; e < SPLIT_ROWS * wpb; e += SPLIT_ROWS) {
        const int row = e / wpb, w = e % wpb;
        if (blockIdx.x * SPLIT_ROWS + row < rows) gb[e] = sw[SPLIT_ROWS * wsa + row * wsb + w];
    }
}

// The same split for deep rows (operands too wide for k_split's shared-memory staging): one CTA
// per working row, 256 threads over its dimensions, the four f64 piece norms by a fixed-order tree.
__global__ void __launch_bounds__(256)
    k_split_wide(const float* __restrict__ xsT, int n, int np_x, int d, int kp, const uint32_t* __restrict__ perm,
                 __nv_bfloat16* __restrict__ opa, __nv_bfloat16* __restrict__ opb, double* __restrict__ pnorm,
                 unsigned long long* __restrict__ colmax) {
    __shared__ double red[4][256];
    const int r = blockIdx.x, tid = threadIdx.x;
    const bool live = r < n;
    const int o = live ? (perm ? (int)perm[r] : r) : 0;
    __nv_bfloat16* ra = opa + (size_t)r * kp;
    __nv_bfloat16* rb = opb + (size_t)r * kp;
    double sh = 0.0, sl = 0.0, sr = 0.0, sp = 0.0;
    for (int t = tid; t < d; t += 256) {
        const float a = live ? xsT[(size_t)t * np_x + o] : 0.0f;
        const __nv_bfloat16 hb = __float2bfloat16_rn(a);
        const float h = __bfloat162float(hb);
        const float e = a - h;  // exact in f32
        const __nv_bfloat16 lb = __float2bfloat16_rn(e);
        const float l = __bfloat162float(lb);
        const float rem = e - l;  // exact in f32
        ra[t] = hb;
        ra[d + t] = lb;
        ra[2 * d + t] = hb;
        rb[t] = hb;
        rb[d + t] = hb;
        rb[2 * d + t] = lb;
        const double h64 = f64_of(h), l64 = f64_of(l), r64 = f64_of(rem);  // exact widenings
        sh = __fma_rn(h64, h64, sh);
        sl = __fma_rn(l64, l64, sl);
        sr = __fma_rn(r64, r64, sr);
        const double p = h64 + l64;
        sp = __fma_rn(p, p, sp);
    }
    const __nv_bfloat16 zero = __float2bfloat16_rn(0.0f);
    for (int t = 3 * d + tid; t < kp; t += 256) {
        ra[t] = zero;
        rb[t] = zero;
    }
    red[0][tid] = sh;
    red[1][tid] = sl;
    red[2][tid] = sr;
    red[3][tid] = sp;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (tid < h)
            for (int j = 0; j < 4; ++j) red[j][tid] += red[j][tid + h];
        __syncthreads();
    }
    if (tid < 4 && live) {
        const double v = sqrt(red[tid][0]);
        pnorm[(size_t)tid * n + o] = v;
        const unsigned long long b = (unsigned long long)__double_as_longlong(v);
        if (b > *reinterpret_cast<volatile unsigned long long*>(&colmax[tid])) atomicMax(&colmax[tid], b);
    }
}

// e4m3 bits → value (exact): sign, 4-bit exponent biased by 7, 3-bit significand; exponent 0 is
// subnormal (m · 2⁻⁹). 0x7f / 0xff (NaN) never occur: the inputs are finite and well inside ±448.
__device__ __forceinline__ float e4m3_value(uint8_t b) {
    const int e = (b >> 3) & 15, m = b & 7;
    const float mag = e ? ldexpf((float)(8 + m), e - 10) : ldexpf((float)m, -9);
    return (b & 0x80) ? -mag : mag;
}

// The split-FP8 operands: a row a (normalised f32) becomes u = 2⁸·a (exact; |u| ≤ 256 < 448, so
// e4m3's normal range covers every entry above 2⁻¹⁴) split into e4m3 pieces u = hi + lo + r', written
// as A = [hi | lo | hi], B = [hi | hi | lo] (bytes, zero-padded to kp), one CTA per working row. The
// piece norms are those of the unscaled pieces h = hi/2⁸, l = lo/2⁸, r = a − h − l (each difference
// exact in f32: the pieces round to nearest, so each is within a factor two of what it approximates),
// so the certificate bound of k_row_eps applies unchanged.
constexpr float FP8_SCALE = 256.0f;
__global__ void __launch_bounds__(256)
    k_split_wide_fp8(const float* __restrict__ xsT, int n, int np_x, int d, int kp, const uint32_t* __restrict__ perm,
                     uint8_t* __restrict__ opa, uint8_t* __restrict__ opb, double* __restrict__ pnorm,
                     unsigned long long* __restrict__ colmax) {
    __shared__ double red[4][256];
    const int r = blockIdx.x, tid = threadIdx.x;
    const bool live = r < n;
    const int o = live ? (perm ? (int)perm[r] : r) : 0;
    uint8_t* ra = opa + (size_t)r * kp;
    uint8_t* rb = opb + (size_t)r * kp;
    double sh = 0.0, sl = 0.0, sr = 0.0, sp = 0.0;
    for (int t = tid; t < d; t += 256) {
        const float a = live ? xsT[(size_t)t * np_x + o] : 0.0f;
        const uint8_t hb = (uint8_t)__nv_cvt_float_to_fp8(a * FP8_SCALE, __NV_SATFINITE, __NV_E4M3);
        const float h = e4m3_value(hb) * (1.0f / FP8_SCALE);
        const float e = a - h;  // exact in f32
        const uint8_t lb = (uint8_t)__nv_cvt_float_to_fp8(e * FP8_SCALE, __NV_SATFINITE, __NV_E4M3);
        const float l = e4m3_value(lb) * (1.0f / FP8_SCALE);
        const float rem = e - l;  // exact in f32
        ra[t] = hb;
        ra[d + t] = lb;
        ra[2 * d + t] = hb;
        rb[t] = hb;
        rb[d + t] = hb;
        rb[2 * d + t] = lb;
        const double h64 = f64_of(h), l64 = f64_of(l), r64 = f64_of(rem);  // exact widenings
        sh = __fma_rn(h64, h64, sh);
        sl = __fma_rn(l64, l64, sl);
        sr = __fma_rn(r64, r64, sr);
        const double p = h64 + l64;
        sp = __fma_rn(p, p, sp);
    }
    for (int t = 3 * d + tid; t < kp; t += 256) {
        ra[t] = 0;
        rb[t] = 0;
    }
    red[0][tid] = sh;
    red[1][tid] = sl;
    red[2][tid] = sr;
    red[3][tid] = sp;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (tid < h)
            for (int j = 0; j < 4; ++j) red[j][tid] += red[j][tid + h];
        __syncthreads();
    }
    if (tid < 4 && live) {
        const double v = sqrt(red[tid][0]);
        pnorm[(size_t)tid * n + o] = v;
        const unsigned long long b = (unsigned long long)__double_as_longlong(v);
        if (b > *reinterpret_cast<volatile unsigned long long*>(&colmax[tid])) atomicMax(&colmax[tid], b);
    }
}

__global__ void k_row_eps(const double* __restrict__ pnorm, const unsigned long long* __restrict__ colmax, int n,
                          int d, int keff, double* __restrict__ row_eps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double up = 1.0 + 1e-12;  // the f64 norms themselves are rounded
    const double h = pnorm[i] * up, l = pnorm[(size_t)n + i] * up, r = pnorm[(size_t)2 * n + i] * up,
                 p = pnorm[(size_t)3 * n + i] * up;
    const double Mh = __longlong_as_double((long long)colmax[0]) * up, Ml = __longlong_as_double((long long)colmax[1]) * up,
                 Mr = __longlong_as_double((long long)colmax[2]) * up, Mp = __longlong_as_double((long long)colmax[3]) * up;
    const double split = l * Ml + p * Mr + r * Mp + r * Mr;
    const double acc = (double)(keff + 16) * 0x1p-21 * (h * Mh + l * Mh + h * Ml);
    const double norm = 2.0001 * 0x1p-24;
    const double resc = (double)(d + 8) * 0x1p-52;
    row_eps[i] = (split + acc + norm + resc) * (1.0 + 1e-9) + 1e-30;
}

// ---- host side -----------------------------------------------------------------------------------

static int kpad(int d) { return (3 * d + KB - 1) / KB * KB; }

// The operand shape for d. Three forms:
//   resident, 3d-wide (3d ≤ 128): A = [hi | lo | hi] stays in shared memory for the whole CTA, each
//     stage holds one column tile B = [hi | hi | lo], one MMA chain;
//   resident, compact (when it needs fewer column K blocks than the 3d-wide form, 22 ≤ d ≤ 32):
//     A = [hi | hi | 0 | lo | 0] resident, a column row is only B = [hi | lo] (2d bf16, ≥ 64), two
//     chains into one accumulator — the column tile, streamed for every tile, is one K block;
//   K loop (3d > 128): both 3d-wide operands streamed one K block per stage.
struct Shape {
    bool resident;  // the query tile stays in shared memory (else the K loop)
    bool compact;   // [hi | hi | lo] × [hi | lo] operands (else [hi | lo | hi] × [hi | hi | lo])
    int kpa, kpb;   // operand row lengths (bf16) of A and B
    int nkb_a;      // K blocks of A (resident) or of both operands (K loop)
    int nkb_b;      // K blocks of B per stage (resident)
    int ksteps;     // MMA steps of 16 per tile
    int k1s;        // steps of the first chain (compact: A [hi | hi] × B [hi | lo]; else all of them)
    int keff;       // products per dot product, for the accumulation term of the bound
};
static Shape shape_of(int d) {
    Shape s{};
    const int kp = kpad(d);
    const int k1 = (2 * d + 15) / 16 * 16, k2 = (d + 15) / 16 * 16;
    if (k1 + k2 <= 2 * KB && (k1 + KB - 1) / KB < kp / KB) {
        s.resident = s.compact = true;
        s.kpa = (k1 + k2 + KB - 1) / KB * KB;
        s.kpb = std::max(KB, (2 * d + 7) / 8 * 8);
        s.nkb_a = s.kpa / KB;
        s.nkb_b = (k1 + KB - 1) / KB;
        s.ksteps = (k1 + k2) / 16;
        s.k1s = k1 / 16;
        s.keff = k1 + k2;
    } else {
        s.resident = kp <= 2 * KB;
        s.compact = false;
        s.kpa = s.kpb = kp;
        s.nkb_a = s.nkb_b = kp / KB;
        s.ksteps = (3 * d + 15) / 16;
        s.k1s = s.ksteps;
        s.keff = 3 * d;
    }
    return s;
}

// The split-FP8 shape: K loop over 128-byte K blocks of e4m3 (A = [hi | lo | hi], B = [hi | hi | lo]),
// 32 elements per MMA step.
static Shape shape_fp8(int d) {
    Shape s{};
    const int kp = (3 * d + 127) / 128 * 128;
    s.resident = false;
    s.compact = false;
    s.kpa = s.kpb = kp;
    s.nkb_a = s.nkb_b = kp / 128;
    s.ksteps = (3 * d + 31) / 32;
    s.k1s = s.ksteps;
    s.keff = 3 * d;
    return s;
}

static size_t fixed_smem(const Shape& sh, int cap) {
    const int bcap = cap <= 32 ? 64 : 128;
    return 1024 + (sh.resident ? (size_t)sh.nkb_a * A_KB_BYTES : 0) + (size_t)(BLOCK_M + 1) * bcap * 8 + sizeof(Barriers);
}
static size_t stage_smem(const Shape& sh) {
    return sh.resident ? (size_t)sh.nkb_b * B_KB_BYTES : (size_t)(A_KB_BYTES + B_KB_BYTES);
}

bool supported(int d, int cap) {
    if (d < 1 || cap < 1 || cap > 64) return false;
    const Shape sh = shape_of(d);
    return fixed_smem(sh, cap) + stage_smem(sh) <= 227 * 1024;  // at least one stage
}

bool supported_fp8(int d, int cap) {
    if (d < 1 || cap < 1 || cap > 64 || 3 * d <= 128) return false;
    const Shape sh = shape_fp8(d);
    return fixed_smem(sh, cap) + stage_smem(sh) <= 227 * 1024;
}

size_t workspace_bytes(int n, int d, bool fp8) {
    const size_t np = (size_t)(n + 255) / 256 * 256;
    const Shape sh = fp8 ? shape_fp8(d) : shape_of(d);
    return np * (size_t)(sh.kpa + sh.kpb) * (fp8 ? 1 : 2) + 4 * (size_t)n * 8 + (size_t)n * 8 + 4 * 8 + 4096;
}

namespace {
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// A 2-D map of an operand ([rows][kp] elements of bf16 or e4m3 bytes) with 128-byte boxes of
// box_rows rows (one K block: 64 bf16 or 128 e4m3).
bool make_map(CUtensorMap* m, const void* base, int kp, int rows, int box_rows, bool fp8 = false) {
    auto fn = encode_fn();
    if (!fn) return false;
    const int esize = fp8 ? 1 : 2;
    cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)kp * esize};
    cuuint32_t box[2] = {(cuuint32_t)(128 / esize), (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(m, fp8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base),
              dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct Layout {
    void *opa, *opb;
    double *pnorm, *row_eps;
    unsigned long long* colmax;
};

Layout carve(void* ws, int n, int d, bool fp8) {
    const size_t np = (size_t)(n + 255) / 256 * 256;
    const Shape sh = fp8 ? shape_fp8(d) : shape_of(d);
    const size_t esize = fp8 ? 1 : 2;
    char* p = static_cast<char*>(ws);
    Layout L;
    L.opa = p;
    p += np * (size_t)sh.kpa * esize;
    L.opb = p;
    p += np * (size_t)sh.kpb * esize;
    L.pnorm = reinterpret_cast<double*>(p);
    p += 4 * (size_t)n * 8;
    L.row_eps = reinterpret_cast<double*>(p);
    p += (size_t)n * 8;
    L.colmax = reinterpret_cast<unsigned long long*>(p);
    return L;
}
}  // namespace

cudaError_t prepare(void* ws, const float* xsT, int n, int np_x, int dp, int d, const uint32_t* perm, cudaStream_t st,
                    Plan& plan, bool fp8, const float* wrows) {
    (void)dp;
    const int np = (n + 255) / 256 * 256;  // the tensor tiles are 256 columns wide
    const Shape sh = fp8 ? shape_fp8(d) : shape_of(d);
    Layout L = carve(ws, n, d, fp8);
    cudaError_t e = cudaMemsetAsync(L.colmax, 0, 4 * 8, st);
    if (e != cudaSuccess) return e;
    // xsT has ⌈n/128⌉·128 columns; operand rows in [n, np) are zero-filled by k_split itself.
    const size_t smem = (size_t)SPLIT_ROWS * (sh.kpa / 2 + 1 + sh.kpb / 2 + 1) * 4;
    if (fp8) {
        k_split_wide_fp8<<<np, 256, 0, st>>>(xsT, n, np_x, d, sh.kpa, perm, static_cast<uint8_t*>(L.opa),
                                              static_cast<uint8_t*>(L.opb), L.pnorm, L.colmax);
    } else if (smem <= 227 * 1024) {
        e = cudaFuncSetAttribute(k_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_split<<<np / SPLIT_ROWS, SPLIT_ROWS, smem, st>>>(xsT, wrows, n, np_x, np, d, sh.kpa, sh.kpb,
                                                            sh.compact ? sh.k1s * 16 : 0, perm,
                                                            static_cast<__nv_bfloat16*>(L.opa),
                                                            static_cast<__nv_bfloat16*>(L.opb), L.pnorm, L.colmax);
    } else {  // (deep rows: never the compact shape)
        k_split_wide<<<np, 256, 0, st>>>(xsT, n, np_x, d, sh.kpa, perm, static_cast<__nv_bfloat16*>(L.opa),
                                         static_cast<__nv_bfloat16*>(L.opb), L.pnorm, L.colmax);
    }
    note_launch();
    k_row_eps<<<(n + 255) / 256, 256, 0, st>>>(L.pnorm, L.colmax, n, d, sh.keff, L.row_eps); note_launch();
    plan.n = n;
    plan.d = d;
    plan.np = np;
    plan.fp8 = fp8;
    plan.kpa = sh.kpa;
    plan.kpb = sh.kpb;
    plan.ops_a = L.opa;
    plan.ops_b = L.opb;
    plan.row_eps = L.row_eps;
    plan.col_max = reinterpret_cast<const double*>(L.colmax);
    plan.perm = perm;
    return cudaGetLastError();
}

cudaError_t launch_coarse(const Plan& plan, int cap, const uint32_t* lists, const float* list_ub,
                          const uint32_t* counts, int ncb, int list_cb, uint32_t* cand_idx, float* cand_score,
                          float* tau, unsigned long long* stopped_total, unsigned long long* timeout_flag,
                          int sm_count, cudaStream_t st, int qb0, int qb1) {
    (void)sm_count;
    if (lists && list_cb != HALF_N && list_cb != BLOCK_N) return cudaErrorInvalidValue;
    const bool pair = lists && list_cb == HALF_N;  // two list entries per tile
    CUtensorMap ma, mb, mbw;  // the column operand in boxes of one half tile and of a whole tile
    if (!make_map(&ma, plan.ops_a, plan.kpa, plan.np, BLOCK_M, plan.fp8) ||
        !make_map(&mb, plan.ops_b, plan.kpb, plan.np, HALF_N, plan.fp8) ||
        !make_map(&mbw, plan.ops_b, plan.kpb, plan.np, BLOCK_N, plan.fp8))
        return cudaErrorInvalidValue;
    const Shape sh = plan.fp8 ? shape_fp8(plan.d) : shape_of(plan.d);
    const size_t fixed = fixed_smem(sh, cap), per = stage_smem(sh);
    int stages = 4;
    while (stages > 1 && fixed + (size_t)stages * per > 227 * 1024) --stages;
    const size_t smem = fixed + (size_t)stages * per;
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    const int qblocks = (plan.n + BLOCK_M - 1) / BLOCK_M;
    if (qb1 < 0) qb1 = qblocks;
    if (qb0 < 0 || qb1 > qblocks || qb0 >= qb1) return cudaErrorInvalidValue;
    auto kern = plan.fp8 ? (cap <= 32 ? k_coarse_tc<1, true, true> : k_coarse_tc<2, true, true>)
                : !sh.resident ? (pair ? (cap <= 32 ? k_coarse_tc<1, true, false, true> : k_coarse_tc<2, true, false, true>)
                                       : (cap <= 32 ? k_coarse_tc<1, true> : k_coarse_tc<2, true>))
                               : (pair ? (cap <= 32 ? k_coarse_tc<1, false, false, true> : k_coarse_tc<2, false, false, true>)
                                       : (cap <= 32 ? k_coarse_tc<1, false> : k_coarse_tc<2, false>));
    if (plan.fp8 && pair) return cudaErrorInvalidValue;  // (deep rows never get lists)
    if (plan.fp8 && sh.resident) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<qb1 - qb0, NTHREADS, smem, st>>>(ma, mb, mbw, plan.n, plan.np, sh.nkb_a, sh.nkb_b, sh.ksteps, sh.k1s, stages,
                                            cap, plan.perm, lists, lists ? list_ub : nullptr, counts, ncb, plan.row_eps, cand_idx, cand_score, tau, stopped_total, timeout_flag, qb0);
    note_launch();
    return cudaGetLastError();
}

// The margin of the row bounds' coarse scores, in cosine: k_row_eps's split-remainder and
// accumulation terms with the maxima of both sides' piece norms (the centres and the rows; the bound
// is symmetric in the two operands), plus (2d + 8)·2⁻²³ for the f32 rows' norms (within (d + 2)·2⁻²⁴
// of 1) and the centres' rounding to f32 (2⁻²⁴), rounded up to f32.
__global__ void k_rowmax_delta(const unsigned long long* __restrict__ cm_c, const unsigned long long* __restrict__ cm_r,
                               int d, int keff, float* __restrict__ delta) {
    if (threadIdx.x != 0) return;
    const double up = 1.0 + 1e-12;
    double c[4], r[4];
    for (int j = 0; j < 4; ++j) {
        c[j] = __longlong_as_double((long long)cm_c[j]) * up;
        r[j] = __longlong_as_double((long long)cm_r[j]) * up;
    }
    // [0] ‖hi‖, [1] ‖lo‖, [2] ‖remainder‖, [3] ‖hi + lo‖
    const double split = c[1] * r[1] + c[3] * r[2] + c[2] * r[3] + c[2] * r[2];
    const double acc = (double)(keff + 16) * 0x1p-21 * (c[0] * r[0] + c[1] * r[0] + c[0] * r[1]);
    const double rnd = (double)(2 * d + 8) * 0x1p-23;
    *delta = __double2float_ru((split + acc + rnd) * (1.0 + 1e-9));
}

namespace {
struct RmLayout {
    void *opa, *opb;
    double* pnorm;
    unsigned long long* colmax;
    float* delta;
};
RmLayout rm_carve(void* ws, int ncb, int d) {
    const Shape sh = shape_of(d);
    const size_t rows = (size_t)(ncb + BLOCK_M - 1) / BLOCK_M * BLOCK_M;
    char* p = static_cast<char*>(ws);
    RmLayout L;
    L.opa = p;
    p += rows * (size_t)sh.kpa * 2;
    L.opb = p;
    p += rows * (size_t)sh.kpb * 2;
    L.pnorm = reinterpret_cast<double*>(p);
    p += 4 * (size_t)ncb * 8;
    L.colmax = reinterpret_cast<unsigned long long*>(p);
    p += 4 * 8;
    L.delta = reinterpret_cast<float*>(p);
    return L;
}
}  // namespace

size_t rowmax_bytes(int ncb, int d) {
    const Shape sh = shape_of(d);
    const size_t rows = (size_t)(ncb + BLOCK_M - 1) / BLOCK_M * BLOCK_M;
    return rows * (size_t)(sh.kpa + sh.kpb) * 2 + 4 * (size_t)ncb * 8 + 4 * 8 + 16 + 256;
}

bool rowmax_supported(const Plan& plan) {
    const Shape sh = shape_of(plan.d);
    return !plan.fp8 && sh.kpa <= 4 * KB && sh.kpb <= 4 * KB;
}

cudaError_t launch_rowmax(const Plan& plan, const float* centers_fT, int ncb, void* ws, float* rowmax,
                          const float** delta, unsigned long long* timeout_flag, cudaStream_t st) {
    if (!rowmax_supported(plan) || ncb < 1) return cudaErrorInvalidValue;
    const Shape sh = shape_of(plan.d);
    const int rows = (ncb + BLOCK_M - 1) / BLOCK_M * BLOCK_M;
    RmLayout L = rm_carve(ws, ncb, plan.d);
    cudaError_t e = cudaMemsetAsync(L.colmax, 0, 4 * 8, st);
    if (e != cudaSuccess) return e;
    // the centres in the operands' split form (the same k_split as the rows, identity order)
    const size_t ssm = (size_t)SPLIT_ROWS * (sh.kpa / 2 + 1 + sh.kpb / 2 + 1) * 4;
    if ((e = cudaFuncSetAttribute(k_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm)) != cudaSuccess)
        return e;
    k_split<<<rows / SPLIT_ROWS, SPLIT_ROWS, ssm, st>>>(centers_fT, nullptr, ncb, ncb, rows, plan.d, sh.kpa, sh.kpb,
                                                         sh.compact ? sh.k1s * 16 : 0, nullptr,
                                                         static_cast<__nv_bfloat16*>(L.opa),
                                                         static_cast<__nv_bfloat16*>(L.opb), L.pnorm, L.colmax);
    note_launch();
    k_rowmax_delta<<<1, 32, 0, st>>>(L.colmax, reinterpret_cast<const unsigned long long*>(plan.col_max), plan.d,
                                     sh.keff, L.delta);
    note_launch();
    CUtensorMap mc, mq;
    if (!make_map(&mc, L.opa, sh.kpa, rows, BLOCK_M) || !make_map(&mq, plan.ops_b, plan.kpb, plan.np, RM_N))
        return cudaErrorInvalidValue;
    const int nkb_c = sh.kpa / KB, nkb_q = (sh.kpb + KB - 1) / KB;
    const size_t fixed = 1024 + (size_t)nkb_q * RM_KB_BYTES + sizeof(RmBars), per = (size_t)nkb_c * RM_KB_BYTES;
    // two CTAs per SM (their accumulators fill the 512 TMEM columns), and never a third
    int stages = (int)std::min<size_t>(4, (112 * 1024 - std::min<size_t>(fixed, 112 * 1024)) / per);
    if (stages < 1) stages = 1;
    const size_t smem = std::max<size_t>(fixed + (size_t)stages * per, 80 * 1024);
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    if ((e = cudaFuncSetAttribute(k_block_rowmax, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
        return e;
    const int nqb = (plan.n + RM_N - 1) / RM_N;
    k_block_rowmax<<<nqb, NTHREADS, smem, st>>>(mc, mq, plan.n, ncb, nkb_c, nkb_q, sh.ksteps, sh.k1s, stages, rowmax,
                                                timeout_flag);
    note_launch();
    *delta = L.delta;
    return cudaGetLastError();
}

}  // namespace tc
}  // namespace costal

