// Locality order and block pruning for the tensor-core coarse pass (prune.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace costal {
namespace prune {

constexpr int K_CENTROIDS = 256;  // spherical k-means cells
constexpr int QB = 128;           // query block (rows of one tensor-core CTA)
constexpr int CB = 256;           // column block (one tensor-core tile)
constexpr int SAMPLE = 65536;     // rows of the k-means sample
constexpr int LLOYD_STEPS = 8;

struct Plan {
    int n, d, K, nqb, ncb;
    uint32_t* perm;      // working -> original [n]
    uint32_t* cell;      // cell of every original row [n]
    float* centroids;    // [K][d] unit centroids
    double* qcenter;     // [nqb][d]
    double* qradius;     // [nqb]
    double* ccenter;     // [ncb][d]
    double* cradius;     // [ncb]
    float* ccenter_f;    // [d][ncb] the centres rounded to f32, transposed (for the f32 bound)
    float* cradius_f;    // [ncb] the radii rounded up to f32
    uint32_t* lists;     // [nqb][ncb] kept column blocks, nearest first
    float* list_ub;      // [nqb][ncb] the bound of each list entry (non-increasing; +inf when unsorted)
    uint32_t* counts;    // [nqb]
    float* ub_skip;      // [nqb]
    double* row_ub;      // [n] (original order) pruning floor of the certificate
    float* tq;           // [nqb] per-query-block thresholds (NULL = keep every block)
    void* scratch;       // k-means sample, histograms
};

size_t workspace_bytes(int n, int d);
bool supported(int d);
// Cells, working order and block geometry from the normalised rows (xsT, d_pad × np).
cudaError_t build_order(void* ws, const float* xsT, int n, int np, int d, cudaStream_t st, Plan& plan);
// Per-query-block column lists with the thresholds in plan.tq (NULL: keep all, nearest first).
cudaError_t build_lists(Plan& plan, unsigned long long* skipped_total, cudaStream_t st);

}  // namespace prune
}  // namespace costal
