// The certified split-BF16 coarse pass on the 5th-generation tensor cores (tcgen05 + TMEM + TMA).
//
// Same job as the FP32 coarse kernel (crates/costal-core/src/knn.rs:603-660 tiles, :758-875
// threshold scan and per-row heaps), with the dot products on the tensor cores:
//
//   split     Every normalised row a (f32) is written as a = a_hi + a_lo + r with a_hi = bf16(a),
//             a_lo = bf16(a − a_hi); |r| ≤ 2⁻¹⁶|a|. The query operand is A = [a_hi | a_lo | a_hi] and
//             the column operand B = [b_hi | b_hi | b_lo] (K = 3d, zero-padded to a multiple of 64), so
//             ONE tcgen05.mma chain computes a_hi·b_hi + a_lo·b_hi + a_hi·b_lo with FP32 accumulation
//             in TMEM. Plain BF16 would put ~2⁻⁸ of error on every cosine, far wider than the gap
//             between the k-th and (k+m)-th neighbour; the split keeps the bound near 5e-5.
//   kernel    One CTA per 128 query rows (M = 128, one TMEM lane per query), column tiles of N = 256.
//             Warp 4 streams B tiles with TMA (128-byte swizzle) into a ring of shared-memory
//             stages; warp 5 issues the MMAs (one elected thread) into two 256-column TMEM
//             accumulators; warps 0-3 read the accumulators back (tcgen05.ld, 32 columns at a time),
//             reject whole 32-column chunks with a 3-input max tree against the query's threshold,
//             and push the rare survivors into a per-query heap in shared memory (the reference's
//             BlockHeaps order: score desc, index asc; strict `v > τ` admission, knn.rs:774-780).
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

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "knn_tc.h"

namespace costal {
namespace tc {

constexpr int KB = 64;                 // bf16 elements per 128-byte swizzle row (one K block)
constexpr int A_KB_BYTES = BLOCK_M * 128;  // 16 KB per K block of the query tile
constexpr int B_KB_BYTES = BLOCK_N * 128;  // 32 KB per K block of a column tile
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
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned long long* timeout_flag) {
    for (long long i = 0; i < WAIT_LIMIT; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
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
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// ---- the per-query heap (knn.rs:791-875), one per epilogue thread, [slot][query] in smem --------
__device__ __forceinline__ bool worse(float sa, uint32_t ia, float sb, uint32_t ib) {
    return sa < sb || (sa == sb && ia > ib);
}

__device__ __noinline__ void heap_push(float* hs, uint32_t* hi, int q, int cap, int& len, float score, uint32_t id) {
#define HS(p) hs[(p) * BLOCK_M + q]
#define HI(p) hi[(p) * BLOCK_M + q]
    if (len < cap) {
        int pos = len;
        while (pos > 0) {
            const int parent = (pos - 1) >> 1;
            const float ps = HS(parent);
            const uint32_t pi = HI(parent);
            if (!worse(score, id, ps, pi)) break;
            HS(pos) = ps;
            HI(pos) = pi;
            pos = parent;
        }
        HS(pos) = score;
        HI(pos) = id;
        ++len;
        return;
    }
    if (!worse(HS(0), HI(0), score, id)) return;
    int pos = 0;
    for (;;) {
        const int left = 2 * pos + 1;
        if (left >= cap) break;
        int w = left;
        if (left + 1 < cap && worse(HS(left + 1), HI(left + 1), HS(left), HI(left))) w = left + 1;
        if (!worse(HS(w), HI(w), score, id)) break;
        HS(pos) = HS(w);
        HI(pos) = HI(w);
        pos = w;
    }
    HS(pos) = score;
    HI(pos) = id;
#undef HS
#undef HI
}

struct __align__(8) Barriers {
    uint64_t a_full;
    uint64_t b_full[4];
    uint64_t b_empty[4];
    uint64_t t_full[2];
    uint64_t t_empty[2];
    uint32_t tmem_base;
};

__global__ void __launch_bounds__(NTHREADS, 1)
    k_coarse_tc(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, int n, int np,
                int nkb, int ksteps, int stages, int cap, uint32_t* __restrict__ cand_idx, float* __restrict__ cand_score,
                float* __restrict__ tau_out, unsigned long long* __restrict__ timeout_flag) {
    extern __shared__ unsigned char smem_raw[];
    // 1024-byte alignment for the swizzled tiles
    const uint32_t base_u32 = smem_u32(smem_raw);
    unsigned char* smem = smem_raw + ((1024 - (base_u32 & 1023)) & 1023);
    unsigned char* a_tile = smem;                                   // nkb × 16 KB
    unsigned char* b_tiles = a_tile + (size_t)nkb * A_KB_BYTES;     // stages × nkb × 32 KB
    float* heap_s = reinterpret_cast<float*>(b_tiles + (size_t)stages * nkb * B_KB_BYTES);  // [cap][128]
    uint32_t* heap_i = reinterpret_cast<uint32_t*>(heap_s + (size_t)cap * BLOCK_M);
    Barriers* bars = reinterpret_cast<Barriers*>(heap_i + (size_t)cap * BLOCK_M);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int q0 = blockIdx.x * BLOCK_M;
    const int ntiles = np / BLOCK_N;
    const uint32_t a_bytes = (uint32_t)nkb * A_KB_BYTES, b_bytes = (uint32_t)nkb * B_KB_BYTES;

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
        if (lane == 0) {
            mbar_expect_tx(&bars->a_full, a_bytes);
            for (int kb = 0; kb < nkb; ++kb) tma_load_2d(a_tile + kb * A_KB_BYTES, &map_a, kb * KB, q0, &bars->a_full);
            for (int t = 0; t < ntiles; ++t) {
                const int s = t % stages;
                const uint32_t ph = (uint32_t)(t / stages) & 1u;
                if (!mbar_wait(&bars->b_empty[s], ph ^ 1u, timeout_flag)) break;
                mbar_expect_tx(&bars->b_full[s], b_bytes);
                unsigned char* dst = b_tiles + (size_t)s * b_bytes;
                for (int kb = 0; kb < nkb; ++kb)
                    tma_load_2d(dst + kb * B_KB_BYTES, &map_b, kb * KB, t * BLOCK_N, &bars->b_full[s]);
            }
        }
    } else if (warp == EPI_WARPS + 1) {
        // ------------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            bool ok = mbar_wait(&bars->a_full, 0, timeout_flag);
            tc_fence_after();
            const uint32_t a_base = smem_u32(a_tile);
            for (int t = 0; ok && t < ntiles; ++t) {
                const int s = t % stages, buf = t & 1;
                const uint32_t ph = (uint32_t)(t / stages) & 1u, bph = (uint32_t)(t >> 1) & 1u;
                if (!mbar_wait(&bars->t_empty[buf], bph ^ 1u, timeout_flag)) break;
                if (!mbar_wait(&bars->b_full[s], ph, timeout_flag)) break;
                tc_fence_after();
                const uint32_t b_base = smem_u32(b_tiles + (size_t)s * b_bytes);
                const uint32_t d = tmem + (uint32_t)(buf * BLOCK_N);
                for (int ks = 0; ks < ksteps; ++ks) {
                    const uint32_t koff = (uint32_t)((ks & 3) * 32);  // 16 bf16 = 32 bytes inside the swizzle row
                    const uint64_t ad = sw128_desc(a_base + (uint32_t)(ks >> 2) * A_KB_BYTES + koff);
                    const uint64_t bd = sw128_desc(b_base + (uint32_t)(ks >> 2) * B_KB_BYTES + koff);
                    mma_bf16(d, ad, bd, ks > 0 ? 1u : 0u);
                }
                mma_commit(&bars->b_empty[s]);
                mma_commit(&bars->t_full[buf]);
            }
        }
    } else {
        // ------------------------------------------------------------------ epilogue (warps 0-3)
        const int qi = warp * 32 + lane;  // TMEM lane = query row within the block
        const int q = q0 + qi;
        float tau = -CUDART_INF_F;
        int len = 0;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        for (int t = 0; t < ntiles; ++t) {
            const int buf = t & 1;
            const uint32_t bph = (uint32_t)(t >> 1) & 1u;
            if (!mbar_wait(&bars->t_full[buf], bph, timeout_flag)) break;
            tc_fence_after();
            const int c0 = t * BLOCK_N;
#pragma unroll 1
            for (int ch = 0; ch < BLOCK_N / 32; ++ch) {
                float v[32];
                tmem_ld32(lane_addr + (uint32_t)(buf * BLOCK_N + ch * 32), v);
                float m[11];
#pragma unroll
                for (int j = 0; j < 10; ++j) m[j] = max3f(v[3 * j], v[3 * j + 1], v[3 * j + 2]);
                m[10] = fmaxf(v[30], v[31]);
                const float mm = max3f(max3f(m[0], m[1], m[2]), max3f(m[3], m[4], m[5]),
                                       max3f(max3f(m[6], m[7], m[8]), m[9], m[10]));
                if (mm > tau) {
                    const int cb = c0 + ch * 32;
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        if (v[j] > tau) {
                            const int col = cb + j;
                            if (col < n && col != q) {
                                heap_push(heap_s, heap_i, qi, cap, len, v[j], (uint32_t)col);
                                tau = len < cap ? -CUDART_INF_F : heap_s[qi];
                            }
                        }
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&bars->t_empty[buf]);
        }
        if (q < n) {
            for (int p = 0; p < cap; ++p) {
                cand_idx[(size_t)q * cap + p] = p < len ? heap_i[p * BLOCK_M + qi] : 0u;
                cand_score[(size_t)q * cap + p] = p < len ? heap_s[p * BLOCK_M + qi] : -CUDART_INF_F;
            }
            tau_out[q] = tau;
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == EPI_WARPS + 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// ---- operand preparation ----------------------------------------------------------------------

// One thread per padded row: split the normalised row (read from xsT) into the two operands and
// record the f64 norms of its pieces: [0] ‖a_hi‖, [1] ‖a_lo‖, [2] ‖r‖, [3] ‖a_hi + a_lo‖.
__global__ void k_split(const float* __restrict__ xsT, int n, int np, int d, int kp, __nv_bfloat16* __restrict__ opa,
                        __nv_bfloat16* __restrict__ opb, double* __restrict__ pnorm,
                        unsigned long long* __restrict__ colmax) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= np) return;
    __nv_bfloat16* ra = opa + (size_t)r * kp;
    __nv_bfloat16* rb = opb + (size_t)r * kp;
    double sh = 0.0, sl = 0.0, sr = 0.0, sp = 0.0;
    const __nv_bfloat16 zero = __float2bfloat16_rn(0.0f);
    for (int t = 0; t < d; ++t) {
        const float a = r < n ? xsT[(size_t)t * np + r] : 0.0f;
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
        sh = __fma_rn((double)h, (double)h, sh);
        sl = __fma_rn((double)l, (double)l, sl);
        sr = __fma_rn((double)rem, (double)rem, sr);
        const double p = (double)h + (double)l;
        sp = __fma_rn(p, p, sp);
    }
    for (int t = 3 * d; t < kp; ++t) {
        ra[t] = zero;
        rb[t] = zero;
    }
    if (r < n) {
        const double v[4] = {sqrt(sh), sqrt(sl), sqrt(sr), sqrt(sp)};
        for (int j = 0; j < 4; ++j) {
            pnorm[(size_t)j * n + r] = v[j];
            atomicMax(&colmax[j], (unsigned long long)__double_as_longlong(v[j]));
        }
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

bool supported(int d, int cap) {
    if (d < 1 || 3 * d > 128 || cap < 1) return false;
    const int nkb = kpad(d) / KB;
    const size_t fixed = 1024 + (size_t)nkb * A_KB_BYTES + (size_t)cap * BLOCK_M * 8 + sizeof(Barriers);
    return fixed + 2ull * nkb * B_KB_BYTES <= 227 * 1024;
}

size_t workspace_bytes(int n, int d) {
    const size_t np = (size_t)(n + 255) / 256 * 256;
    const size_t kp = (size_t)kpad(d);
    return 2 * np * kp * 2 + 4 * (size_t)n * 8 + (size_t)n * 8 + 4 * 8 + 4096;
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

bool make_map(CUtensorMap* m, const void* base, int kp, int rows, int box_rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
    cuuint32_t box[2] = {(cuuint32_t)KB, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct Layout {
    __nv_bfloat16 *opa, *opb;
    double *pnorm, *row_eps;
    unsigned long long* colmax;
};

Layout carve(void* ws, int n, int d) {
    const size_t np = (size_t)(n + 255) / 256 * 256, kp = (size_t)kpad(d);
    char* p = static_cast<char*>(ws);
    Layout L;
    L.opa = reinterpret_cast<__nv_bfloat16*>(p);
    p += np * kp * 2;
    L.opb = reinterpret_cast<__nv_bfloat16*>(p);
    p += np * kp * 2;
    L.pnorm = reinterpret_cast<double*>(p);
    p += 4 * (size_t)n * 8;
    L.row_eps = reinterpret_cast<double*>(p);
    p += (size_t)n * 8;
    L.colmax = reinterpret_cast<unsigned long long*>(p);
    return L;
}
}  // namespace

cudaError_t prepare(void* ws, const float* xsT, int n, int np_x, int dp, int d, cudaStream_t st, Plan& plan) {
    (void)dp;
    const int np = (n + 255) / 256 * 256;  // the tensor tiles are 256 columns wide
    const int kp = kpad(d);
    Layout L = carve(ws, n, d);
    cudaError_t e = cudaMemsetAsync(L.colmax, 0, 4 * 8, st);
    if (e != cudaSuccess) return e;
    // xsT has n_pad = ⌈n/128⌉·128 columns; rows in [n, np) are zero-filled by k_split itself.
    k_split<<<(np + 127) / 128, 128, 0, st>>>(xsT, n, np_x, d, kp, L.opa, L.opb, L.pnorm, L.colmax);
    k_row_eps<<<(n + 255) / 256, 256, 0, st>>>(L.pnorm, L.colmax, n, d, 3 * d, L.row_eps);
    plan.n = n;
    plan.d = d;
    plan.np = np;
    plan.kp = kp;
    plan.ops_a = L.opa;
    plan.ops_b = L.opb;
    plan.row_eps = L.row_eps;
    plan.col_max = reinterpret_cast<const double*>(L.colmax);
    return cudaGetLastError();
}

cudaError_t launch_coarse(const Plan& plan, int cap, uint32_t* cand_idx, float* cand_score, float* tau,
                          unsigned long long* timeout_flag, int sm_count, cudaStream_t st) {
    (void)sm_count;
    CUtensorMap ma, mb;
    if (!make_map(&ma, plan.ops_a, plan.kp, plan.np, BLOCK_M) || !make_map(&mb, plan.ops_b, plan.kp, plan.np, BLOCK_N))
        return cudaErrorInvalidValue;
    const int nkb = plan.kp / KB;
    const int ksteps = (3 * plan.d + 15) / 16;
    const size_t fixed = 1024 + (size_t)nkb * A_KB_BYTES + (size_t)cap * BLOCK_M * 8 + sizeof(Barriers);
    int stages = 4;
    while (stages > 2 && fixed + (size_t)stages * nkb * B_KB_BYTES > 227 * 1024) --stages;
    const size_t smem = fixed + (size_t)stages * nkb * B_KB_BYTES;
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_coarse_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int qblocks = (plan.n + BLOCK_M - 1) / BLOCK_M;
    k_coarse_tc<<<qblocks, NTHREADS, smem, st>>>(ma, mb, plan.n, plan.np, nkb, ksteps, stages, cap, cand_idx, cand_score,
                                                 tau, timeout_flag);
    return cudaGetLastError();
}

}  // namespace tc
}  // namespace costal
