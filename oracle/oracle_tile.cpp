// TEST INFRASTRUCTURE ONLY — the coarse f32 tile product of the CPU oracle.
//
// Restates the contract of crates/costal-core/src/matmul.rs:56-106 (`tile_nt`):
// out[r·cols + c] = Σ_t a[r·d + t] · b[c·d + t] in f32, row-major. The reference says the backend
// (and so the summation order) changes speed only, never the kNN output (matmul.rs:1-6,
// knn.rs:8-10): the f64 rescoring and the (d+4)·2⁻²³ coarse-error bound make the result
// independent of it. This file is compiled with contraction allowed; the rest of the oracle is not.

#include <cstddef>
#include <cstring>

extern "C" void oracle_tile_nt(const float* a, size_t rows, const float* b, size_t cols, size_t d,
                               float* out, float* bt) {
    // Pack B transposed (d × cols) so the inner loop runs over contiguous columns.
    for (size_t c = 0; c < cols; ++c)
        for (size_t t = 0; t < d; ++t) bt[t * cols + c] = b[c * d + t];
    constexpr size_t RB = 4, CB = 16;
    size_t r = 0;
    for (; r + RB <= rows; r += RB) {
        size_t c = 0;
        for (; c + CB <= cols; c += CB) {
            float acc[RB][CB] = {};
            for (size_t t = 0; t < d; ++t) {
                const float* bv = bt + t * cols + c;
                for (size_t i = 0; i < RB; ++i) {
                    float av = a[(r + i) * d + t];
                    for (size_t j = 0; j < CB; ++j) acc[i][j] += av * bv[j];
                }
            }
            for (size_t i = 0; i < RB; ++i) std::memcpy(out + (r + i) * cols + c, acc[i], sizeof acc[i]);
        }
        for (; c < cols; ++c)
            for (size_t i = 0; i < RB; ++i) {
                float s = 0.0f;
                for (size_t t = 0; t < d; ++t) s += a[(r + i) * d + t] * bt[t * cols + c];
                out[(r + i) * cols + c] = s;
            }
    }
    for (; r < rows; ++r) {
        for (size_t c = 0; c < cols; ++c) out[r * cols + c] = 0.0f;
        for (size_t t = 0; t < d; ++t) {
            float av = a[r * d + t];
            const float* bv = bt + t * cols;
            float* o = out + r * cols;
            for (size_t c = 0; c < cols; ++c) o[c] += av * bv[c];
        }
    }
}
