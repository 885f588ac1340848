// Locality order and block pruning for the tensor-core coarse pass (prune.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace costal {
namespace prune {

constexpr int K_CENTROIDS = 256;  // spherical k-means cells
constexpr int QB = 128;           // query block (rows of one tensor-core CTA)
// Column blocks: 128 working rows (half a tensor-core tile; the coarse kernel fills a tile from two
// list entries) while a query block's list fits the 16-keys-a-thread sort (≤ 8,192 blocks, n ≤
// 1,048,576), else 256 (one tile per entry). Blocks of 128 straddle fewer k-means cells, so their
// bounds skip more columns (visited pairs 25 % instead of 36 % at 200,000 rows of the Zipf mixture, 14.1
// instead of 15.1 % at 2,000,000), but twice as many list entries cost more to bound and sort: measured
// per step they win up to 1,000,000 rows (−6.6 % at 200,000, −1.9 % at 1,000,000) and lose at
// 2,000,000 (+5.5 %), where the lists need the 32-keys-a-thread sort.
constexpr int CB_FINE = 128, CB_WIDE = 256;
constexpr int LIST_FAST = 8192;  // the widest list of the 16-keys-a-thread sort
inline int col_block(int n) { return (n + CB_FINE - 1) / CB_FINE <= LIST_FAST ? CB_FINE : CB_WIDE; }
constexpr int SAMPLE = 65536;     // rows of the k-means sample
constexpr int LLOYD_STEPS = 8;

struct Plan {
    int n, d, K, nqb, ncb;
    int cb;              // rows of a column block (col_block(n))
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
    float* wrows;        // [n][d] the normalised rows in working order, row-major
    const float* rowmax;    // [nqb][ncb] per-row bound data (tc::launch_rowmax), or NULL: cone bound only
    const float* rm_delta;  // its error margin (device scalar)
    void* scratch;       // k-means sample, histograms
};

size_t workspace_bytes(int n, int d);
bool supported(int d);
// Cells, working order and block geometry from the normalised rows (xsT, d_pad × np).
cudaError_t build_order(void* ws, const float* xsT, int n, int np, int d, cudaStream_t st, Plan& plan);
// Per-query-block column lists with the thresholds in plan.tq (NULL: keep all, nearest first).
cudaError_t build_lists(Plan& plan, unsigned long long* skipped_total, cudaStream_t st);

// Rows grouped by norm for Tanimoto selection's norm window (knn.rs:413-418 sorts by norm): a stable
// counting sort into NORM_BUCKETS buckets spaced evenly in log(norm) between the smallest and the
// largest positive norm (zero rows first). Within a bucket rows keep their input order; the window
// test only needs each column tile's exact norm range, so the order inside a bucket does not matter.
constexpr int NORM_BUCKETS = 1024;
size_t norm_order_bytes(int n);
cudaError_t norm_order(const double* norms, int n, void* ws, uint32_t* perm, cudaStream_t st);

}  // namespace prune
}  // namespace costal
