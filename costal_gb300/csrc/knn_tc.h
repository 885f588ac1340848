// Certified split-BF16 coarse pass on the 5th-generation tensor cores (tcgen05, TMEM accumulators).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace costal {
namespace tc {

constexpr int BLOCK_M = 128;  // query rows per CTA tile (the MMA's M; one TMEM lane per query)
constexpr int BLOCK_N = 256;  // columns per tile (the MMA's N)

struct Plan {
    int n, d, np;           // rows, features, padded rows
    bool fp8;               // e4m3 operands (the split-FP8 kind) instead of bf16
    int kpa, kpb;           // row lengths (elements: bf16, or e4m3 bytes) of the split operands
    const void* ops_a;      // [np][kpa] bf16 query operand  (hi | hi | lo, or hi | lo | hi for deep rows)
    const void* ops_b;      // [np][kpb] bf16 column operand (hi | lo, or hi | hi | lo for deep rows)
    const double* row_eps;  // [n] certificate bound of each query row
    const double* col_max;  // [4] maxima over all rows of the split-residual norms
    const uint32_t* perm;   // working -> original row (NULL: identity); operands are in working order
};

bool supported(int d, int cap);
// The split-FP8 kind (e4m3 pieces of the rows scaled by 2^8, three products per pair, K loop): for
// rows deep enough that the query tile is streamed (3d > 128), cap ≤ 64.
bool supported_fp8(int d, int cap);
size_t workspace_bytes(int n, int d, bool fp8 = false);
// Split the normalised rows (xsT, d_pad × n_pad) into BF16 operands and per-row error norms, and
// derive each row's certificate bound. wrows (optional, split BF16 only): the same rows already in the
// working order, row-major [n][d] (prune::Plan::wrows), read instead of gathering xsT through perm.
cudaError_t prepare(void* ws, const float* xsT, int n, int np, int dp, int d, const uint32_t* perm, cudaStream_t st,
                    Plan& plan, bool fp8 = false, const float* wrows = nullptr);
// All (query tile × column tile) products on tcgen05, fused with the per-query top-cap selection.
// With lists/counts (prune.cu), CTA Q visits only the column blocks lists[Q·ncb .. + counts[Q]) of
// list_cb working rows each (128: two list entries fill one 256-column tile; 256: one); with list_ub
// (their bounds, non-increasing) it stops once no later block can hold an admissible column for any
// of its rows. [qb0, qb1) restricts the launch to those query blocks (one shard of the rows); qb1 = -1
// means all of them.
cudaError_t launch_coarse(const Plan& plan, int cap, const uint32_t* lists, const float* list_ub,
                          const uint32_t* counts, int ncb, int list_cb, uint32_t* cand_idx, float* cand_score,
                          float* tau, unsigned long long* stopped_total, unsigned long long* timeout_flag,
                          int sm_count, cudaStream_t st, int qb0 = 0, int qb1 = -1);

// Per-row block bounds for the column lists (prune.cu): for every query block Q (128 working rows)
// and column block B with unit centre c_B (centers_fT: [d][ncb] f32), rowmax[Q·ncb + B] = the largest
// coarse score q·c_B over the rows q of Q, on the tensor cores with the split operands of `plan`;
// *delta (device) receives its error margin in cosine. BF16 operands only (not the split-FP8 kind).
bool rowmax_supported(const Plan& plan);
size_t rowmax_bytes(int ncb, int d);
cudaError_t launch_rowmax(const Plan& plan, const float* centers_fT, int ncb, void* ws, float* rowmax,
                          const float** delta, unsigned long long* timeout_flag, cudaStream_t st);

}  // namespace tc
}  // namespace costal
