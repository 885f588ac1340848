/* costal_gb300 — C ABI of the GB300 (sm_103a) exact cosine kNN graph.
 *
 * Drop-in boundary for CosTaL 2.1.0's `costal._costal` extension (crates/costal-py/src/lib.rs). Each
 * entry point replaces the reference function named beside it; the Python module
 * costal_gb300/_costal.py binds them with the reference's exact signatures.
 *
 * Conventions:
 *  - plain pointers and sizes only; arrays are row-major and C-contiguous;
 *  - entry points whose name does not end in `_device` take HOST pointers and do their own
 *    host<->device copies; `_device` entry points take DEVICE pointers and a cudaStream_t (as void*);
 *  - every entry point returns a status (COSTAL_OK = 0) and, on failure, writes a NUL-terminated
 *    message into `err` (at most `errlen` bytes). Nothing aborts or exits the process;
 *  - calls are serialised on one cached per-process device context (a mutex), so they are re-entrant
 *    from several host threads.
 */
#ifndef COSTAL_GB300_H
#define COSTAL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define COSTAL_OK 0
#define COSTAL_EINVAL 2     /* invalid input: the reference raises ValueError (lib.rs:31-33) */
#define COSTAL_ECUDA 3      /* a CUDA call failed, or no usable GB300 device */
#define COSTAL_ENOMEM 4     /* a device allocation failed */
#define COSTAL_ETIMEOUT 5   /* a bounded device-side wait gave up; the context stays usable */
#define COSTAL_EUNSUPPORTED 6 /* valid input outside what the GPU kernels support (e.g. k + margin > 128) */

/* Coarse-pass backends. Like the reference's `matmul` knob (crates/costal-core/src/matmul.rs:10-50)
 * they change speed only, never the output. */
#define COSTAL_BACKEND_FP32 0    /* plain FP32 CUDA-core tiles: the default drop-in */
#define COSTAL_BACKEND_BF16 1    /* certified tcgen05 tiles, FP32 accumulate in TMEM: split BF16, or split
                                    FP8 e4m3 for d >= 512 */
#define COSTAL_BACKEND_BF16X3 2  /* certified split-BF16 tcgen05 tiles at every depth */
#define COSTAL_BACKEND_FP8 3     /* certified split-FP8 (e4m3) tcgen05 tiles wherever the query tile is
                                    streamed (3d > 128); split BF16 below that */

#define COSTAL_SELECT_COSINE 0
#define COSTAL_SELECT_TANIMOTO 1

#define COSTAL_WEIGHT_TANIMOTO 0
#define COSTAL_WEIGHT_COSINE 1
#define COSTAL_WEIGHT_JACCARD 2

/* Options of an exact kNN call: KnnParams (crates/costal-core/src/knn.rs:27-60) plus the backend. */
typedef struct costal_knn_opts {
    uint32_t margin;       /* over-selection m; UINT32_MAX = the reference default m = k (knn.rs:52) */
    uint32_t select;       /* COSTAL_SELECT_*; knn.rs:64-69 */
    uint32_t backend;      /* COSTAL_BACKEND_* */
    uint32_t row_block;    /* accepted for compatibility (knn.rs:35-37); speed-only, 0 = derive */
    uint32_t col_block;    /* idem */
    int32_t sort_by_norm;  /* idem (knn.rs:41): output-independent */
    int32_t prune;         /* idem (knn.rs:44): output-independent; on the bf16 backend it enables the
                              exact early stop of each query block's column list */
    int32_t learned_prune; /* 1 = use the trained block-pruning model if one is loaded (bf16 backend) */
} costal_knn_opts;

/* KnnStats (knn.rs:346-357) plus the GPU path's own counters. */
typedef struct costal_knn_stats {
    uint64_t fallback_rows;    /* rows that took the full-row regather (knn.rs:704-714) */
    uint64_t row_block;        /* query rows per CTA tile */
    uint64_t col_block;        /* columns per tile */
    uint64_t blocks_skipped;   /* (row block, column block) tiles skipped by pruning */
    uint64_t blocks_total;     /* row blocks x column blocks */
    uint64_t margin;           /* the m in effect */
    uint64_t recomputed_rows;  /* bf16 backend: rows whose certificate failed, redone in FP32 */
    uint64_t pruned_fallback_rows; /* learned pruning: rows whose skip was not certified, rescanned */
    double max_coarse_err;     /* max |coarse score - f64 rescored score| over all kept candidates */
    double ms_prep, ms_coarse, ms_rescore, ms_fallback, ms_total; /* CUDA-event times of the stages */
    double ms_order;           /* bf16 backend: locality order, block bounds and lists (inside ms_total) */
    double ms_kernel;          /* the coarse tile + selection kernel alone (inside ms_coarse) */
    uint64_t blocks_stopped;   /* bf16 backend: list blocks left out because every row's threshold
                                  already exceeded their bound (exact; no certificate needed) */
    double max_err_ratio;      /* max over the rescored candidates of |coarse - f64 score| divided by the
                                  bound the row's certificate used (E_i on the bf16 backend, the FP32
                                  epsilon otherwise): the certificate is sound while this stays below 1 */
    uint64_t coarse_kind;      /* the coarse pass that ran: 0 FP32 tiles, 1 split BF16, 2 split FP8 */
} costal_knn_stats;

/* ---- module surface (crates/costal-py/src/lib.rs:80-102, 430-446) ---------------------------- */
const char* costal_version(void);   /* replaces env!("CARGO_PKG_VERSION") of lib.rs:450 */
/* GB300 addition, no reference counterpart: the number of CUDA kernels this library has launched
   in this process (a monotone counter; take differences around a call). */
unsigned long long costal_launch_count(void);
int costal_device_ok(char* err, size_t errlen);  /* 0 when a usable sm_103 device is present */
/* GB300 addition, no reference counterpart: a self-check of the integer f32 -> f64 conversion that
   the f64 rescoring uses in place of the conversion instruction; compares the two over every finite
   f32 bit pattern on the device and stores the number of mismatches (0 expected). */
int costal_check_f64_conversion(uint64_t* mismatches, char* err, size_t errlen);
/* lib.rs:94-102 (costal_core::row_l2_norms, crates/costal-core/src/lib.rs:34-47): f32 row norms. */
int costal_row_l2_norms(const float* x, uint64_t n, uint32_t d, float* out, char* err, size_t errlen);

/* ---- the hot path ------------------------------------------------------------------------------ */
/* lib.rs:114-167 `_knn_exact` -> knn.rs:365 knn_exact_with_stats. Host buffers: x n*d f32;
 * idx n*k, cos n*k, norms n. */
int costal_knn_exact(const float* x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts,
                     uint32_t* idx, double* cos, double* norms, costal_knn_stats* stats, char* err,
                     size_t errlen);
/* The same on device buffers, on `stream` (a cudaStream_t; NULL = the library's stream). */
int costal_knn_exact_device(const float* d_x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts,
                            uint32_t* d_idx, double* d_cos, double* d_norms, costal_knn_stats* stats,
                            void* stream, char* err, size_t errlen);
/* lib.rs:172-191 `_knn_bruteforce` -> knn.rs:884 knn_bruteforce_select: every candidate in f64. */
int costal_knn_bruteforce(const float* x, uint64_t n, uint32_t d, uint32_t k, uint32_t select, uint32_t* idx,
                          double* cos, double* norms, char* err, size_t errlen);
/* lib.rs:195-214 `_reweight` -> weight.rs:41 reweight. idx values are checked to be in [0, n). */
int costal_reweight(uint64_t n, uint32_t k, const int32_t* idx, const double* cos, const double* norms,
                    uint32_t weight, double* out, char* err, size_t errlen);
/* lib.rs:219-239 `_fuzzy_union` -> graph.rs:24 fuzzy_union. rows/cols/w hold up to n*k edges;
 * *m receives the edge count. */
int costal_fuzzy_union(uint64_t n, uint32_t k, const int32_t* idx, const double* w, int32_t* rows,
                       int32_t* cols, double* w_out, uint64_t* m, char* err, size_t errlen);
/* The fused device pipeline of _api.py:460-462 (knn -> reweight -> _fuzzy_union): X goes up once,
 * the kNN stays on the device, and only the edge list (and the kNN, if idx/cos/norms are not
 * NULL) comes back. rows/cols/w hold up to n*k edges. */
int costal_build_graph(const float* x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts,
                       uint32_t weight, int32_t* rows, int32_t* cols, double* w, uint64_t* m, uint32_t* idx,
                       double* cos, double* norms, costal_knn_stats* stats, char* err, size_t errlen);
/* GB300 addition: the same pipeline, with the graph handed back in the CSR layout the Leiden uses
 * (leiden.rs:52-101 `Csr::from_edges` of the edge list: rows ascending; see costal_leiden_csr), built
 * on the device. indptr holds n+1 u64; nbr/w hold up to 2*n*k entries; *nnz = 2 * edges. */
int costal_build_graph_csr(const float* x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts,
                           uint32_t weight, uint64_t* indptr, uint32_t* nbr, double* w, uint64_t* nnz,
                           costal_knn_stats* stats, char* err, size_t errlen);
/* The same from device-resident X, with device outputs (capacity n*k edges); *m is written on the host. */
int costal_build_graph_device(const float* d_x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts,
                              uint32_t weight, int32_t* d_rows, int32_t* d_cols, double* d_w, uint64_t* m,
                              costal_knn_stats* stats, void* stream, char* err, size_t errlen);

/* ---- row shards: the path split across GPUs (knn.rs:403-512 `run_blocked`'s unit of work, a
 * block of query rows against all columns) -------------------------------------------------------
 * The query rows are cut into blocks of 128 in the order the coarse pass processes them (the input
 * order; on the bf16 backend for d <= 64, the locality order, which every rank derives identically
 * from the same X); shard s of S takes the contiguous blocks [s*B/S, (s+1)*B/S) of the B blocks, so
 * the S shards hold every row exactly once. Each rank keeps all of X and computes its shard against
 * every column: the only exchange is gathering the shards' rows afterwards. */
/* The most rows any of n_shards shards holds (the capacity of the packed outputs). */
uint64_t costal_shard_rows_max(uint64_t n, uint32_t n_shards);
/* The kNN of shard `shard` of `n_shards` on device buffers: d_rows receives the shard's rows (original
 * ids, *count of them), d_idx/d_cos (and d_w, the Tanimoto weight, unless NULL) their neighbours
 * packed row by row (*count x k); d_norms the norms of all n rows. Cosine selection only. Output
 * equals the same rows of costal_knn_exact_device. */
int costal_knn_shard_device(const float* d_x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts,
                            uint32_t shard, uint32_t n_shards, uint32_t* d_rows, uint64_t* count, uint32_t* d_idx,
                            double* d_cos, double* d_w, double* d_norms, costal_knn_stats* stats, void* stream,
                            char* err, size_t errlen);
/* lib.rs:219-239 `_fuzzy_union` on device buffers (the gathered kNN of a sharded run): rows/cols/w_out
 * hold up to n*k edges; *m is written on the host. */
int costal_fuzzy_union_device(const int32_t* d_idx, const double* d_w, uint64_t n, uint32_t k, int32_t* d_rows,
                              int32_t* d_cols, double* d_w_out, uint64_t* m, void* stream, char* err, size_t errlen);

/* Jaccard weights (the computation of costal_reweight with COSTAL_WEIGHT_JACCARD) on DEVICE buffers,
 * for callers that may not allocate device memory: it has no counterpart in the reference. Its scratch is
 * a fixed 16 MiB array compiled into the library (reserved on every GPU that loads it, until the process
 * exits), so n*k is limited to 4,194,304 neighbour entries; larger inputs return COSTAL_EINVAL before any
 * device work. The first call on a device looks up that array's address (make it before any stream
 * capture); under CUDA's lazy module loading that first call may also be when the 16 MiB is reserved,
 * and it fails with COSTAL_ECUDA on a device without that much free, so a caller with a fixed budget
 * makes it at start-up. All calls share the array: calls that overlap on the GPU race and must be
 * serialised. */
int costal_reweight_jaccard_device_noalloc(const int32_t* d_idx, uint64_t n, uint32_t k, double* d_out, void* stream,
                                           char* err, size_t errlen);

/* ---- the learned block-pruning model (GB300 addition; no counterpart in the reference) -------------
 * An MLP (d + 64 centroid cosines -> 128 -> 128 -> 1) predicts each row's k-th-neighbour cosine; with
 * costal_knn_opts.learned_prune = 1 and the bf16 backend, column blocks whose rigorous upper bound is
 * below a query block's smallest prediction are skipped, and every skip is certified afterwards (a row
 * whose k-th score does not beat its skipped blocks' bound is rescanned in full). */
typedef struct costal_mlp_opts {
    uint32_t sample;    /* rows used for training (evenly spaced); 0 = all rows; default 200,000 */
    uint32_t epochs;    /* passes over the sample (default 30) */
    uint32_t batch;     /* rows per Adam step (default 2048) */
    uint32_t margin;    /* over-selection of the FP32 label pass; UINT32_MAX = k */
    float lr;           /* Adam learning rate (default 2e-3) */
    float quantile;     /* pinball-loss quantile (default 0.05: predictions below the truth for ~95% of rows) */
    uint64_t seed;      /* parameter initialisation */
} costal_mlp_opts;

typedef struct costal_mlp_stats {
    uint64_t samples, steps, params;
    double loss;        /* final mean pinball loss on the training rows (bf16 weights) */
    double mae;         /* mean |prediction - exact k-th cosine| */
    double coverage;    /* fraction of training rows whose prediction is <= their exact k-th cosine */
    double ms_labels;   /* exact labels (plain FP32 path) and features */
    double ms_train;    /* forward/backward/Adam kernels */
} costal_mlp_stats;

/* Train the model on X (host, n x d): labels are the exact k-th-neighbour cosines of the sampled rows
 * from the plain FP32 path, features use the same k-means cells as the pruned kNN. The model stays
 * loaded in the library's context. mo may be NULL (defaults). */
int costal_mlp_train(const float* x, uint64_t n, uint32_t d, uint32_t k, const costal_mlp_opts* mo,
                     costal_mlp_stats* stats, char* err, size_t errlen);
/* Checkpointing: read (params may be NULL to query *count) or load the f32 master weights. */
int costal_mlp_get(float* params, uint64_t capacity, uint64_t* count, uint32_t* d, uint32_t* k, float* quantile,
                   char* err, size_t errlen);
int costal_mlp_set(const float* params, uint64_t count, uint32_t d, uint32_t k, float quantile, char* err,
                   size_t errlen);
int costal_mlp_clear(char* err, size_t errlen);
/* Test hooks: the inference pass (bf16 operands on the tensor cores, FP32 accumulation) and the loss
 * gradient (FP32) for given weights and features (host buffers). */
int costal_mlp_forward(const float* params, uint32_t F, const float* feat, uint64_t m, float* out, char* err,
                       size_t errlen);
int costal_mlp_gradient(const float* params, uint32_t F, const float* feat, const float* y, uint64_t m,
                        float quantile, float* grad, char* err, size_t errlen);
/* Test hook: the per-row block bound data of the tensor-core path for X (host, n x d, 1 <= d <= 64):
 * the working order perm[n] (working -> original row), the column blocks' unit centres ccenter[ncb][d]
 * and angular radii cradius[ncb] (f64, blocks of cb working rows: 128 while ceil(n/128) <= 8192, else
 * 256), rowmax[nqb][ncb] = the largest split-BF16 coarse score of a query block's rows (blocks of 128)
 * with each centre, and *delta, its error margin in cosine; nqb = ceil(n/128), ncb = ceil(n/cb). */
int costal_block_bounds(const float* x, uint64_t n, uint32_t d, uint32_t* perm, double* ccenter, double* cradius,
                        float* rowmax, float* delta, char* err, size_t errlen);

/* ---- the host consumer: Leiden (leiden="fast"), crates/costal-core/src/leiden.rs ------------- */
/* lib.rs:275-306 `_leiden` (from_coo = 0, objective = 0) and lib.rs:356-412 `_leiden_coo`
 * (from_coo = 1). objective: 0 modularity, 1 CPM. initial may be NULL. quality may be NULL. */
int costal_leiden(uint64_t n, const uint32_t* rows, const uint32_t* cols, const double* weights, uint64_t m,
                  int objective, int from_coo, double resolution, double beta, int32_t n_iterations,
                  uint64_t seed, const uint32_t* initial, uint32_t* membership, uint64_t* n_clusters,
                  uint64_t* iterations, int* converged, double* quality, char* err, size_t errlen);
/* GB300 addition (the first "next" item of the path): the same Leiden on a graph given directly in
   the CSR layout of leiden.rs:52-101 `Csr::from_edges` (indptr n+1 u64 from 0; for every row its
   neighbours and weights, both directions of every edge), as costal_build_graph_csr produces it;
   used in place, without building a CSR from an edge list. Weights must be finite and positive. */
int costal_leiden_csr(uint64_t n, const uint64_t* indptr, const uint32_t* nbr, const double* weights, int objective,
                      double resolution, double beta, int32_t n_iterations, uint64_t seed, const uint32_t* initial,
                      uint32_t* membership, uint64_t* n_clusters, uint64_t* iterations, int* converged,
                      double* quality, char* err, size_t errlen);
/* lib.rs:311-350 `_leiden_many`: out is (n_resolutions * n_seeds) x n, resolutions outer. */
int costal_leiden_many(uint64_t n, const uint32_t* rows, const uint32_t* cols, const double* weights, uint64_t m,
                       const double* resolutions, uint64_t n_resolutions, const uint64_t* seeds, uint64_t n_seeds,
                       double beta, int32_t n_iterations, int n_threads, uint32_t* out, char* err, size_t errlen);
/* GB300 addition: lib.rs:311-350 `_leiden_many` on a graph given in the CSR layout of costal_leiden_csr
   (as costal_build_graph_csr produces it), used in place: the same labels as on its edge list. */
int costal_leiden_many_csr(uint64_t n, const uint64_t* indptr, const uint32_t* nbr, const double* weights,
                           const double* resolutions, uint64_t n_resolutions, const uint64_t* seeds, uint64_t n_seeds,
                           double beta, int32_t n_iterations, int n_threads, uint32_t* out, char* err, size_t errlen);
/* lib.rs:416-428 `_modularity`. */
int costal_modularity(uint64_t n, const uint32_t* rows, const uint32_t* cols, const double* weights, uint64_t m,
                      const uint32_t* membership, double resolution, double* q, char* err, size_t errlen);

#ifdef __cplusplus
}
#endif

#endif /* COSTAL_GB300_H */
