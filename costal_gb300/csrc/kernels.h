// Internal launcher declarations shared by the .cu files of libcostal_gb300 (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace costal {

// ---- knn_plain.cu ------------------------------------------------------------------------------
cudaError_t launch_prep(const float* x, int n, int d, int np, int dp, double* norms, float* xsT,
                        unsigned long long* bad_row, cudaStream_t st);
cudaError_t launch_row_l2_norms_f32(const float* x, int n, int d, float* out, cudaStream_t st);
int coarse_slots(int cap);
// d_pad of the working copy: a multiple of 8 up to 64 (compile-time tile depths), else of 4.
int coarse_dpad(int d);
size_t coarse_fp32_smem(int dp, int cap);
// qlist/qcount (optional): run only the rows listed on the device (128 per CTA, grid sized for n).
cudaError_t launch_coarse_fp32(const float* xsT, int n, int np, int dp, int cap, int lstride, const uint32_t* qlist,
                               const unsigned* qcount, uint32_t* cand_idx, float* cand_score, float* tau,
                               cudaStream_t st);
// Few listed rows: the columns split into `segs` segments (one CTA per 128 rows per segment), their
// lists merged per row. part_* hold segs × count × cap entries (τ: segs × count).
int coarse_fp32_segments(int count, int np, int sm_count);
// tfloor (optional, by row): a per-row threshold below which no column can be among the best cap.
cudaError_t launch_coarse_fp32_split(const float* xsT, int n, int np, int dp, int cap, int lstride,
                                     const uint32_t* qlist, const unsigned* qcount, int count, int segs,
                                     const float* tfloor, uint32_t* part_idx, float* part_score, float* part_tau,
                                     uint32_t* cand_idx, float* cand_score, float* tau, cudaStream_t st);
// Tanimoto selection (knn.rs:197-284): the same FP32 pass over all columns with the coarse score
// T = a·b·ĉ / (A + B − a·b·ĉ) from the normalised tile and the rows' norms (tnorm: n entries of
// scratch, filled here); within 2(d+12)·2⁻²³ of the exact T.
cudaError_t launch_coarse_fp32_tanimoto(const float* xsT, int n, int np, int dp, int cap, const double* norms,
                                        float2* tnorm, uint32_t* cand_idx, float* cand_score, float* tau,
                                        cudaStream_t st);
// Tanimoto selection with the norm window (knn.rs:595-644): rows in the norm order `perm` (working →
// original, prune::norm_order), each query block walking outward from its own norms and stopping a
// side once its norms leave every row's window; d_pad ≤ 64. ws holds tani_window_bytes(n, np, dp)
// (the norm-ordered working copy, norms and tile ranges); the lists are written in input order.
size_t tani_window_bytes(int n, int np, int dp);
cudaError_t launch_coarse_tani_window(const float* xsT, int n, int np, int dp, int cap, const double* norms,
                                      const uint32_t* perm, void* ws, uint32_t* cand_idx, float* cand_score,
                                      float* tau, unsigned long long* skipped_total, cudaStream_t st);
// The floor of rows re-run after the tensor-core pass (rows[0..*count), cand_* and tau of that pass).
cudaError_t launch_rerun_floor(const uint32_t* rows, const unsigned* count, int nmax, int cap, const float* tau,
                               const float* cand_score, const double* row_eps, double eps, float* tfloor,
                               cudaStream_t st);
// Self-check of the integer f32 → f64 conversion used by the f64 dot products (all 2³² patterns).
cudaError_t launch_check_f64_of(unsigned long long* mismatches, int sm_count, cudaStream_t st);
cudaError_t launch_rescore(const float* x, int n, int d, int k, int cap, int lstride, const uint32_t* cand_idx,
                           const float* cand_score, const float* tau, const double* norms, const double* row_eps,
                           const double* row_ub, unsigned* ub_fail, double eps, int certify, int select,
                           const uint32_t* rlist, const unsigned* rcount,
                           uint32_t* out_idx, double* out_cos, double* out_w, uint32_t* fb_rows, double* fb_minsim,
                           unsigned* fb_count, unsigned long long* max_err_bits, cudaStream_t st);
int gather_capb(int k);
size_t gather_smem(int k, int d, int dp);
cudaError_t launch_gather(const float* x, const float* xsT, int n, int np, int d, int dp, int k, const double* norms,
                          const uint32_t* rows, const double* minsim, const unsigned* count, int all_rows, int select,
                          int grid, uint32_t* out_idx, double* out_cos, double* out_w, cudaStream_t st);

// ---- graph.cu ----------------------------------------------------------------------------------
cudaError_t launch_iota(uint32_t* out, int start, int m, cudaStream_t st);
// Pack the rows `rows[0..nrows)` of (n, k) neighbour arrays into (nrows, k) ones (w may be NULL).
cudaError_t launch_take_rows(const uint32_t* rows, int nrows, int k, const uint32_t* idx, const double* cos,
                             const double* w, uint32_t* oidx, double* ocos, double* ow, cudaStream_t st);
cudaError_t launch_stride_rows(uint32_t* out, int m, int n, cudaStream_t st);
cudaError_t launch_kth(const double* cos, const uint32_t* rows, int m, int k, float* y, cudaStream_t st);
cudaError_t launch_init_params(float* P, int F, unsigned long long seed, cudaStream_t st);
cudaError_t launch_check_idx(const int32_t* idx, uint64_t nk, int n, unsigned long long* first_bad, cudaStream_t st);
cudaError_t launch_tanimoto_w(const uint32_t* idx, const double* cos, const double* norms, uint64_t nk, int k,
                              double* out, cudaStream_t st);
cudaError_t launch_jaccard(const uint32_t* idx, int n, int k, uint32_t* sorted_scratch, double* out, cudaStream_t st);
// Fuzzy union S + Sᵀ − S∘Sᵀ on the device. Scratch sizes in fuzzy_union_scratch_bytes.
size_t fuzzy_union_scratch_bytes(int n, int k);
// The Leiden CSR (leiden.rs:52-101 layout: indptr, both directions, rows in edge-list order, which
// for the union's sorted list is ascending) from the union's edges rows/cols/w (m at m_dev on the
// device): indptr[n + 1] (u64), nbr/w_out[2m], src_out[2m] the row of each entry; nnz at nnz_dev.
size_t csr_scratch_bytes(int n, int k);
cudaError_t launch_csr_from_union(const int32_t* rows, const int32_t* cols, const double* w, const uint32_t* m_dev,
                                  int n, int k, void* scratch, uint64_t* indptr, int32_t* src_out, int32_t* nbr,
                                  double* w_out, uint32_t* nnz_dev, cudaStream_t st);
cudaError_t launch_fuzzy_union(const uint32_t* idx, const double* w, int n, int k, void* scratch, int32_t* rows,
                               int32_t* cols, double* w_out, uint32_t* m_dev, cudaStream_t st);

}  // namespace costal
