// Shared device helpers of the GB300 kNN-graph kernels (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define COSTAL_FULL_MASK 0xffffffffu

namespace costal {

// Counts every kernel launch this library issues (host side, relaxed atomic); read through
// costal_launch_count().
void note_launch();

// ---- exact f64 arithmetic in the reference's order of operations ---------------------------------
//
// Each helper names the rounding of every operation, so nvcc can never contract a multiply and an
// add into one FMA where the reference (Rust, which never contracts) rounds twice.

// The exact f64 value of a finite f32, built with integer operations. f32 → f64 is exact, so this is
// the same value as the conversion instruction; it is written out because the conversion issues to
// the FP64 pipe, which the GB300 has only a narrow one of, and the rescoring's dot products would
// otherwise spend two conversions per multiply-add there. Normal numbers move their exponent from
// bias 127 to bias 1023 (+896 = 0x380) and their 23-bit significand to the top of the 52-bit one;
// zero keeps its sign; a subnormal m·2⁻¹⁴⁹ is normalised from its leading bit. Not for inf/NaN
// (the path's inputs are checked finite).
__device__ __forceinline__ double f64_of(float f) {
    const uint32_t u = __float_as_uint(f), v = u & 0x7fffffffu, sgn = u & 0x80000000u;
    uint32_t hi = sgn | ((v >> 3) + 0x38000000u), lo = v << 29;
    if (v < 0x00800000u) {
        if (v == 0u) {
            hi = sgn;
        } else {  // subnormal: leading bit p in [0, 22], value 2^(p−149)·(1.f)
            const int p = 31 - __clz(v);
            const unsigned long long b = ((unsigned long long)(p + 874) << 52) |
                                         (((unsigned long long)v << (52 - p)) & 0x000fffffffffffffull);
            hi = sgn | (uint32_t)(b >> 32);
            lo = (uint32_t)b;
        }
    }
    return __hiloint2double((int)hi, (int)lo);
}

// knn.rs:290-296 `dot64`: Σ_t f64(a_t)·f64(b_t) in dimension order. An f32×f32 product is exact
// in f64, so fma(a, b, s) rounds exactly like s + a·b: the FMA is bit-identical here.
__device__ __forceinline__ double dot64_step(double s, float a, float b) {
    return __fma_rn(f64_of(a), f64_of(b), s);
}

// knn.rs:301-312 `cos64`: 0 for a zero row, dot / (n_i·n_j), −0 → +0.
__device__ __forceinline__ double cos64(double dot, double ni, double nj) {
    if (ni == 0.0 || nj == 0.0) return 0.0;
    double c = __ddiv_rn(dot, __dmul_rn(ni, nj));
    return c == 0.0 ? 0.0 : c;
}

// weight.rs:30-37 `tani_from_cos`: d = a·b·cos; 0 when d == 0, else d / (a² + b² − d).
__device__ __forceinline__ double tani_from_cos(double a, double b, double c) {
    double d = __dmul_rn(__dmul_rn(a, b), c);
    if (d == 0.0) return 0.0;
    double den = __dsub_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), d);
    return __ddiv_rn(d, den);
}

// Tanimoto selection (knn.rs:197-284): the coarse score of a pair from an f32 cosine ĉ of the
// normalised rows and the rows' f32 norms (x) and squared norms (y): T = dot / (A + B − dot) with
// dot = a·b·ĉ, 0 when dot is 0 or the denominator is not positive (knn.rs:254-262). Within
// 2(d+12)·2⁻²³ of the exact T: ∂T/∂dot ≤ 4/(A+B) and a·b ≤ (A+B)/2 turn ĉ's (d+4)·2⁻²³ into
// 2(d+4)·2⁻²³, and the f32 norms and the four roundings add at most 8·2⁻²³ more (the argument of
// knn.rs:270-274).
__device__ __forceinline__ float tani_coarse_f32(float c, float2 qn, float2 cn) {
    const float dn = qn.x * cn.x * c;
    const float den = qn.y + cn.y - dn;
    return (dn == 0.0f || den <= 0.0f) ? 0.0f : __fdiv_rn(dn, den);
}

// Rust's f64::total_cmp as a signed integer key (knn.rs:589-591 sorts with it).
__device__ __forceinline__ long long total_key(double v) {
    long long b = __double_as_longlong(v);
    return b ^ (long long)(((unsigned long long)(b >> 63)) >> 1);
}

// (score desc, index asc): the final order of a row (knn.rs:589-591).
__device__ __forceinline__ bool before64(double sa, uint32_t ia, double sb, uint32_t ib) {
    long long ka = total_key(sa), kb = total_key(sb);
    return ka > kb || (ka == kb && ia < ib);
}

// ---- cp.async (Ampere-style asynchronous global→shared copies; no spin-waits) -------------------

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

}  // namespace costal
