// The C ABI of libcostal_gb300: validation, the cached device context and the orchestration of the
// kernels of knn_plain.cu, knn_tc.cu and graph.cu. Mirrors crates/costal-py/src/lib.rs (the PyO3
// boundary) and the knn.rs/weight.rs/graph.rs entry points behind it; see include/costal_gb300.h.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "costal_gb300.h"
#include "kernels.h"
#include "knn_tc.h"
#include "mlp.h"
#include "prune.h"

namespace {
std::atomic<unsigned long long> g_launches{0};
}  // namespace

namespace costal {
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
}  // namespace costal

namespace {

using namespace costal;

constexpr double F32_EPS = 1.1920928955078125e-07;  // 2^-23

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

struct Misc {  // small device-side results read back at the end of a call
    unsigned long long bad_row;
    unsigned long long max_err_bits[2];  // max |coarse − rescored|, and its max ratio to the row's bound
    unsigned long long first_bad_idx;
    unsigned fb_count;
    unsigned m;
    unsigned tc_fail_count;
    unsigned prune_fail_count;
    unsigned long long blocks_skipped;
    unsigned long long timeout_flag;
    unsigned long long blocks_stopped;
    unsigned long long conv_mismatches;
    unsigned nnz;
    unsigned shard_rows;  // rows of the shard being computed (the rescoring's device-side row count)
};

struct Context {
    std::mutex mu;
    bool inited = false;
    int init_rc = COSTAL_OK;
    std::string init_err;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    Misc* h_misc = nullptr;
    DevBuf x, norms, xsT, cand_idx, cand_score, tau, out_idx, out_cos, out_w, fb_rows, fb_minsim, misc;
    DevBuf fu_scratch, rows, cols, wout, idx_in, cos_in, norms_in, w_in, jac, f32out, tc_ws, tc_rows, prune_ws;
    DevBuf mlp_params, mlp_params_bf, mlp_m1, mlp_m2, mlp_feat, mlp_y, mlp_pred, mlp_partial, mlp_grad, mlp_rows;
    DevBuf part_idx, part_score, part_tau, tfloor;
    DevBuf csr_ws, csr_indptr, csr_src, csr_nbr, csr_w, tnorm, shard_rows, tani_perm, tani_ws, rm_ws, rm_out;
    MlpState mlp;
};

Context& ctx() {
    static Context c;
    return c;
}

void put_err(char* err, size_t errlen, const std::string& msg) {
    if (err && errlen) std::snprintf(err, errlen, "%s", msg.c_str());
}

cudaError_t ensure(DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 256;
    if (b.bytes >= bytes) return cudaSuccess;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return e;
    }
    b.bytes = bytes;
    return cudaSuccess;
}

struct Fail {
    int rc;
    std::string msg;
};

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e__ = (call);                                                                       \
        if (e__ != cudaSuccess) {                                                                       \
            throw Fail{e__ == cudaErrorMemoryAllocation ? COSTAL_ENOMEM : COSTAL_ECUDA,                 \
                       std::string(#call) + ": " + cudaGetErrorString(e__)};                            \
        }                                                                                               \
    } while (0)

int init_locked(Context& c) {
    if (c.inited) return c.init_rc;
    c.inited = true;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        c.init_rc = COSTAL_ECUDA;
        c.init_err = std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
        return c.init_rc;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp p{};
    cudaGetDeviceProperties(&p, dev);
    if (!(p.major == 10 && p.minor == 3)) {
        c.init_rc = COSTAL_ECUDA;
        c.init_err = std::string("libcostal_gb300 is built for sm_103a (GB300); device 0 is ") + p.name + " sm_" +
                     std::to_string(p.major) + std::to_string(p.minor);
        return c.init_rc;
    }
    c.sm_count = p.multiProcessorCount;
    if ((e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMallocHost(&c.h_misc, sizeof(Misc))) != cudaSuccess) {
        c.init_rc = COSTAL_ECUDA;
        c.init_err = std::string("context set-up failed: ") + cudaGetErrorString(e);
        return c.init_rc;
    }
    for (auto& ev : c.ev) cudaEventCreate(&ev);
    c.init_rc = COSTAL_OK;
    return COSTAL_OK;
}

std::string knn_arg_error(uint64_t n, uint32_t k) {
    if (n > 0xFFFFFFFFull) return "n=" + std::to_string(n) + " exceeds the u32 index range";  // knn.rs:118
    if (k == 0 || (uint64_t)k >= n)
        return "invalid k=" + std::to_string(k) + ": need 1 <= k <= n-1 (n=" + std::to_string(n) + ")";  // knn.rs:117
    return "";
}

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

constexpr int MLP_CHUNK = 262144;  // rows per feature/forward chunk at inference

// Learned thresholds: the model's prediction for every row, then t_Q = min over each query block.
cudaError_t mlp_predict_thresholds(Context& c, prune::Plan& pp, cudaStream_t s) {
    const int n = pp.n, d = pp.d, F = c.mlp.F;
    const int np = (n + 127) / 128 * 128;
    cudaError_t e;
    if ((e = ensure(c.mlp_feat, (size_t)std::min(n, MLP_CHUNK) * F * 4)) != cudaSuccess) return e;
    if ((e = ensure(c.mlp_pred, (size_t)n * 4)) != cudaSuccess) return e;
    if ((e = ensure(c.mlp_rows, (size_t)std::min(n, MLP_CHUNK) * 4)) != cudaSuccess) return e;
    for (int r0 = 0; r0 < n; r0 += MLP_CHUNK) {
        const int m = std::min(MLP_CHUNK, n - r0);
        if ((e = launch_iota(c.mlp_rows.as<uint32_t>(), r0, m, s)) != cudaSuccess) return e;
        if ((e = mlp::features(c.xsT.as<float>(), np, d, pp.centroids, pp.K, c.mlp_rows.as<uint32_t>(), m,
                               c.mlp_feat.as<float>(), s)) != cudaSuccess)
            return e;
        if ((e = mlp::forward(c.mlp.params_bf, F, c.mlp_feat.as<float>(), m, c.mlp_pred.as<float>() + r0, s)) !=
            cudaSuccess)
            return e;
    }
    return mlp::block_min(c.mlp_pred.as<float>(), pp.perm, n, pp.tq, s);
}

// One shard of the query rows (a multi-GPU run gives each rank one): the rows are cut into query
// blocks of 128 in the order the coarse pass processes them (the input order, or the locality order
// of the tensor-core path), and shard `index` of `count` takes the contiguous blocks
// [index·B/count, (index+1)·B/count) of the B blocks. Every column stays in the computation.
struct Shard {
    int index = 0, count = 1;
    int nrows = 0;  // filled: the shard's rows, listed (original ids) in Context::shard_rows
};

// The query-block range of a shard.
void shard_blocks(int n, const Shard& sh, int& qb0, int& qb1) {
    const long long nqb = (n + 127) / 128;
    qb0 = (int)(nqb * sh.index / sh.count);
    qb1 = (int)(nqb * (sh.index + 1) / sh.count);
}

// The kNN on device buffers. Everything is asynchronous on `s` except the final read of Misc.
// d_w (optional): the Tanimoto weight of every output edge, fused into the rescoring.
// shard (optional): compute only that shard's rows (their outputs are written at their rows of
// d_idx/d_cos/d_w; the norms of all rows are written).
void run_knn(Context& c, const float* d_x, int n, int d, int k, const costal_knn_opts& o, uint32_t* d_idx,
             double* d_cos, double* d_norms, double* d_w, costal_knn_stats* st, cudaStream_t s,
             Shard* shard = nullptr) {
    uint64_t margin = o.margin == UINT32_MAX ? (uint64_t)k : (uint64_t)o.margin;
    int cap = (int)std::min<uint64_t>((uint64_t)k + margin, (uint64_t)n - 1);
    const int dp = coarse_dpad(d);
    const int np = round_up(n, 128);
    // The coarse passes keep at most 128 candidates a row (fewer for 40 < d ≤ 64, where the query
    // tile shares the shared memory). The over-selection m changes only how often the certificate
    // holds, never the output (knn.rs:45-52), so a larger k + m runs with the largest candidate count
    // the FP32 kernel holds that still exceeds k (rows the certificate then fails take the regather);
    // when none does, every candidate is scanned exactly in f64 (knn.rs:884-924).
    bool scan_all = false;
    auto fits = [&](int c) { return coarse_slots(c) != 0 && coarse_fp32_smem(dp, c) <= 227 * 1024; };
    if (!fits(cap)) {
        int smaller = 0;
        for (int c : {128, 64, 32})
            if (c < cap && c > k && fits(c)) {
                smaller = c;
                break;
            }
        if (smaller) {
            cap = smaller;
            margin = (uint64_t)(cap - k);
        } else {
            scan_all = true;
        }
    }
    if (shard && o.select == COSTAL_SELECT_TANIMOTO)
        throw Fail{COSTAL_EUNSUPPORTED, "row shards support cosine selection only"};
    CK(ensure(c.misc, sizeof(Misc)));
    Misc* dm = c.misc.as<Misc>();
    CK(cudaMemsetAsync(dm, 0, sizeof(Misc), s));
    CK(cudaMemsetAsync(&dm->bad_row, 0xff, 8, s));
    int qb0 = 0, qb1 = (n + 127) / 128;
    uint32_t* srows = nullptr;        // the shard's rows (original ids), on the device
    const unsigned* scount = nullptr;  // their number, on the device
    if (shard) {
        shard_blocks(n, *shard, qb0, qb1);
        shard->nrows = std::max(0, std::min(n, qb1 * 128) - qb0 * 128);
        CK(ensure(c.shard_rows, (size_t)n * 4));
        srows = c.shard_rows.as<uint32_t>();
        c.h_misc->shard_rows = (unsigned)shard->nrows;
        CK(cudaMemcpyAsync(&dm->shard_rows, &c.h_misc->shard_rows, 4, cudaMemcpyHostToDevice, s));
        scount = &dm->shard_rows;
    }
    const int nrows = shard ? shard->nrows : n;
    CK(ensure(c.xsT, (size_t)dp * np * 4));
    CK(ensure(c.fb_rows, (size_t)n * 4));
    CK(ensure(c.fb_minsim, (size_t)n * 8));
    CK(cudaEventRecord(c.ev[0], s));
    CK(launch_prep(d_x, n, d, np, dp, d_norms, c.xsT.as<float>(), &dm->bad_row, s));
    CK(cudaEventRecord(c.ev[1], s));
    CK(cudaEventRecord(c.ev[5], s));
    const bool tanimoto = o.select == COSTAL_SELECT_TANIMOTO;
    bool used_tc = false;
    int list_cb = 0;  // rows of a column block of the tensor-core path's lists (0: no lists)
    // The split-FP8 kind: its coarse scores are ~2⁻⁸ coarser than split BF16's, so it keeps 64
    // candidates a row whatever the margin (the output does not depend on it) to let the certificate
    // hold for nearly every row.
    const bool tc_backend = o.backend == COSTAL_BACKEND_BF16 || o.backend == COSTAL_BACKEND_BF16X3 ||
                            o.backend == COSTAL_BACKEND_FP8;
    bool fp8 = !tanimoto && !scan_all && (o.backend == COSTAL_BACKEND_FP8 || (o.backend == COSTAL_BACKEND_BF16 && d >= 512));
    if (fp8) {
        const int cap8 = std::max(cap, std::min(64, n - 1));
        if (tc::supported_fp8(d, cap8) && coarse_slots(cap8) != 0 && coarse_fp32_smem(dp, cap8) <= 227 * 1024) {
            cap = cap8;
            margin = (uint64_t)(cap - k);
        } else {
            fp8 = false;
        }
    }
    if (scan_all) {
        if (shard) throw Fail{COSTAL_EUNSUPPORTED, "row shards need k + margin within the coarse pass's 128 candidates"};
        if (gather_smem(k, d, dp) > 227 * 1024) throw Fail{COSTAL_EUNSUPPORTED, "k too large for the GPU scan kernel"};
        // (no candidate count the coarse kernel holds exceeds k) the exact f64 scan of every
        // candidate on the GPU (knn.rs:884-924's brute force), exact by construction
        CK(cudaEventRecord(c.ev[2], s));
        CK(cudaEventRecord(c.ev[3], s));
        CK(launch_gather(d_x, c.xsT.as<float>(), n, np, d, dp, k, d_norms, nullptr, nullptr, nullptr, 1,
                         tanimoto ? 1 : 0, std::min(n, 8 * c.sm_count), d_idx, d_cos, d_w, s));
    } else if (tanimoto) {
        // Tanimoto selection (knn.rs:197-284): the FP32 pass over all columns with the coarse
        // Tanimoto score, the f64 rescoring of the cap candidates by T with the certificate
        // s_k > τ + 2(d+12)·2⁻²³, and the regather (filtered by the coarse T) for rows that fail it.
        CK(ensure(c.cand_idx, (size_t)n * cap * 4));
        CK(ensure(c.cand_score, (size_t)n * cap * 4));
        CK(ensure(c.tau, (size_t)n * 4));
        CK(ensure(c.tnorm, (size_t)n * 8));
        const double eps_t = 2.0 * ((double)d + 12.0) * F32_EPS;
        if (o.prune && cap < n - 1 && dp <= 64) {
            // the norm window (knn.rs:595-644): rows in norm order, each query block walking outward
            CK(ensure(c.tani_perm, (size_t)n * 4));
            CK(ensure(c.tani_ws, std::max(prune::norm_order_bytes(n), tani_window_bytes(n, np, dp))));
            CK(prune::norm_order(d_norms, n, c.tani_ws.p, c.tani_perm.as<uint32_t>(), s));
            CK(launch_coarse_tani_window(c.xsT.as<float>(), n, np, dp, cap, d_norms, c.tani_perm.as<uint32_t>(),
                                         c.tani_ws.p, c.cand_idx.as<uint32_t>(), c.cand_score.as<float>(),
                                         c.tau.as<float>(), &dm->blocks_skipped, s));
        } else {
            CK(launch_coarse_fp32_tanimoto(c.xsT.as<float>(), n, np, dp, cap, d_norms, c.tnorm.as<float2>(),
                                           c.cand_idx.as<uint32_t>(), c.cand_score.as<float>(), c.tau.as<float>(), s));
        }
        CK(cudaEventRecord(c.ev[2], s));
        CK(launch_rescore(d_x, n, d, k, cap, cap, c.cand_idx.as<uint32_t>(), c.cand_score.as<float>(),
                          c.tau.as<float>(), d_norms, nullptr, nullptr, nullptr, eps_t, cap < n - 1, 1, nullptr,
                          nullptr, d_idx, d_cos, d_w, c.fb_rows.as<uint32_t>(), c.fb_minsim.as<double>(),
                          &dm->fb_count, dm->max_err_bits, s));
        CK(cudaEventRecord(c.ev[3], s));
        if (cap < n - 1) {
            if (gather_smem(k, d, dp) > 227 * 1024)
                throw Fail{COSTAL_EUNSUPPORTED, "k too large for the GPU regather kernel"};
            CK(launch_gather(d_x, c.xsT.as<float>(), n, np, d, dp, k, d_norms, c.fb_rows.as<uint32_t>(),
                             c.fb_minsim.as<double>(), &dm->fb_count, 0, 1, std::min(n, 4 * c.sm_count), d_idx,
                             d_cos, d_w, s));
        }
    } else {
        CK(ensure(c.cand_idx, (size_t)n * cap * 4));
        CK(ensure(c.cand_score, (size_t)n * cap * 4));
        CK(ensure(c.tau, (size_t)n * 4));
        const double eps = ((double)d + 4.0) * F32_EPS;  // knn.rs:185-187
        if (tc_backend && (fp8 || tc::supported(d, cap))) {
            used_tc = true;
            // Locality order (k-means cells) and per-query-block column lists, nearest blocks first;
            // with a learned threshold, blocks whose bound is below it are skipped. Deep rows (the
            // pruning geometry covers d ≤ 64) keep the input order and visit every column block.
            const bool ordered = prune::supported(d);
            prune::Plan pp{};
            bool learned = false;
            if (ordered) {
                CK(ensure(c.prune_ws, prune::workspace_bytes(n, d)));
                CK(prune::build_order(c.prune_ws.p, c.xsT.as<float>(), n, np, d, s, pp));
            }
            CK(ensure(c.tc_ws, tc::workspace_bytes(n, d, fp8)));
            CK(ensure(c.tc_rows, (size_t)n * 4));
            tc::Plan plan{};
            CK(tc::prepare(c.tc_ws.p, c.xsT.as<float>(), n, np, dp, d, ordered ? pp.perm : nullptr, s, plan, fp8,
                           ordered && !fp8 ? pp.wrows : nullptr));
            if (ordered) {
                // with the early stop, the lists take the per-row bound too (the nearest row of each
                // query block to each column block's centre, from the split operands just made)
                if (o.prune && tc::rowmax_supported(plan)) {
                    CK(ensure(c.rm_ws, tc::rowmax_bytes(pp.ncb, d)));
                    CK(ensure(c.rm_out, (size_t)pp.nqb * pp.ncb * 4));
                    const float* delta = nullptr;
                    CK(tc::launch_rowmax(plan, pp.ccenter_f, pp.ncb, c.rm_ws.p, c.rm_out.as<float>(), &delta,
                                         &dm->timeout_flag, s));
                    pp.rowmax = c.rm_out.as<float>();
                    pp.rm_delta = delta;
                }
                learned = o.learned_prune && c.mlp.ready && c.mlp.d == d && c.mlp.k == k;
                if (learned) {
                    CK(mlp_predict_thresholds(c, pp, s));
                } else {
                    pp.tq = nullptr;
                }
                CK(prune::build_lists(pp, &dm->blocks_skipped, s));
                list_cb = pp.cb;
            }
            if (shard && nrows > 0) {  // the shard's rows: its query blocks in the processing order
                if (ordered)
                    CK(cudaMemcpyAsync(srows, pp.perm + (size_t)qb0 * 128, (size_t)nrows * 4, cudaMemcpyDeviceToDevice,
                                       s));
                else
                    CK(launch_iota(srows, qb0 * 128, nrows, s));
            }
            CK(cudaEventRecord(c.ev[5], s));
            CK(cudaEventRecord(c.ev[6], s));
            if (nrows > 0)
                CK(tc::launch_coarse(plan, cap, ordered ? pp.lists : nullptr,
                                     ordered && o.prune ? pp.list_ub : nullptr, ordered ? pp.counts : nullptr,
                                     ordered ? pp.ncb : 0, ordered ? pp.cb : 0, c.cand_idx.as<uint32_t>(),
                                     c.cand_score.as<float>(),
                                     c.tau.as<float>(), &dm->blocks_stopped, &dm->timeout_flag, c.sm_count, s, qb0,
                                     qb1));
            CK(cudaEventRecord(c.ev[2], s));
            // The split-BF16 certificate with its per-row bound (and, with pruning, the skipped
            // blocks' bound); rows that fail it are listed in tc_rows, re-run over ALL columns by the
            // FP32 coarse kernel and rescored with the FP32 bound, whose failures in turn take the
            // full-row regather.
            if (nrows > 0)
                CK(launch_rescore(d_x, n, d, k, cap, cap, c.cand_idx.as<uint32_t>(), c.cand_score.as<float>(),
                                  c.tau.as<float>(), d_norms, plan.row_eps, learned ? pp.row_ub : nullptr,
                                  &dm->prune_fail_count, 0.0, cap < n - 1, 0, srows, scount, d_idx, d_cos, d_w,
                                  c.tc_rows.as<uint32_t>(), c.fb_minsim.as<double>(), &dm->tc_fail_count,
                                  dm->max_err_bits, s));
            if (coarse_fp32_smem(dp, cap) > 227 * 1024)
                throw Fail{COSTAL_EUNSUPPORTED, "d and k + margin too large for the FP32 re-run of uncertified rows"};
            // How many rows failed decides the re-run's shape (few rows: the columns split across CTAs).
            CK(cudaMemcpyAsync(&c.h_misc->tc_fail_count, &dm->tc_fail_count, sizeof(unsigned), cudaMemcpyDeviceToHost,
                               s));
            CK(cudaStreamSynchronize(s));
            const int nfail = (int)c.h_misc->tc_fail_count;
            if (nfail > 0) {
                const int segs = coarse_fp32_segments(nfail, np, c.sm_count);
                if (segs > 1) {
                    CK(ensure(c.part_idx, (size_t)segs * nfail * cap * 4));
                    CK(ensure(c.part_score, (size_t)segs * nfail * cap * 4));
                    CK(ensure(c.part_tau, (size_t)segs * nfail * 4));
                }
                CK(ensure(c.tfloor, (size_t)n * 4));
                CK(launch_rerun_floor(c.tc_rows.as<uint32_t>(), &dm->tc_fail_count, nfail, cap, c.tau.as<float>(),
                                      c.cand_score.as<float>(), plan.row_eps, eps, c.tfloor.as<float>(), s));
                CK(launch_coarse_fp32_split(c.xsT.as<float>(), n, np, dp, cap, cap, c.tc_rows.as<uint32_t>(),
                                            &dm->tc_fail_count, nfail, segs, c.tfloor.as<float>(),
                                            c.part_idx.as<uint32_t>(),
                                            c.part_score.as<float>(), c.part_tau.as<float>(), c.cand_idx.as<uint32_t>(),
                                            c.cand_score.as<float>(), c.tau.as<float>(), s));
                CK(launch_rescore(d_x, n, d, k, cap, cap, c.cand_idx.as<uint32_t>(), c.cand_score.as<float>(),
                                  c.tau.as<float>(), d_norms, nullptr, nullptr, nullptr, eps, cap < n - 1, 0,
                                  c.tc_rows.as<uint32_t>(), &dm->tc_fail_count, d_idx, d_cos, d_w,
                                  c.fb_rows.as<uint32_t>(), c.fb_minsim.as<double>(), &dm->fb_count, nullptr, s));
            }
            CK(cudaEventRecord(c.ev[3], s));
        } else {
            if (coarse_fp32_smem(dp, cap) > 227 * 1024)
                throw Fail{COSTAL_EUNSUPPORTED, "d and k + margin too large for the FP32 coarse kernel"};
            if (!shard) {
                CK(launch_coarse_fp32(c.xsT.as<float>(), n, np, dp, cap, cap, nullptr, nullptr,
                                      c.cand_idx.as<uint32_t>(), c.cand_score.as<float>(), c.tau.as<float>(), s));
            } else if (nrows > 0) {  // the shard's rows, listed, against all columns
                CK(launch_iota(srows, qb0 * 128, nrows, s));
                CK(launch_coarse_fp32_split(c.xsT.as<float>(), n, np, dp, cap, cap, srows, scount, nrows, 1, nullptr,
                                            nullptr, nullptr, nullptr, c.cand_idx.as<uint32_t>(),
                                            c.cand_score.as<float>(), c.tau.as<float>(), s));
            }
            CK(cudaEventRecord(c.ev[2], s));
            if (nrows > 0)
                CK(launch_rescore(d_x, n, d, k, cap, cap, c.cand_idx.as<uint32_t>(), c.cand_score.as<float>(),
                                  c.tau.as<float>(), d_norms, nullptr, nullptr, nullptr, eps, cap < n - 1, 0, srows,
                                  scount, d_idx, d_cos, d_w, c.fb_rows.as<uint32_t>(), c.fb_minsim.as<double>(),
                                  &dm->fb_count, dm->max_err_bits, s));
            CK(cudaEventRecord(c.ev[3], s));
        }
        if (cap < n - 1) {
            if (gather_smem(k, d, dp) > 227 * 1024)
                throw Fail{COSTAL_EUNSUPPORTED, "k too large for the GPU regather kernel"};
            CK(launch_gather(d_x, c.xsT.as<float>(), n, np, d, dp, k, d_norms, c.fb_rows.as<uint32_t>(),
                             c.fb_minsim.as<double>(), &dm->fb_count, 0, 0, std::min(n, 4 * c.sm_count), d_idx,
                             d_cos, d_w, s));
        }
    }
    CK(cudaEventRecord(c.ev[4], s));
    CK(cudaMemcpyAsync(c.h_misc, dm, sizeof(Misc), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const Misc& hm = *c.h_misc;
    if (hm.bad_row != ~0ull) throw Fail{COSTAL_EINVAL, "row " + std::to_string(hm.bad_row) + " contains NaN or inf"};
    if (hm.timeout_flag == 2) throw Fail{COSTAL_ECUDA, "internal error: a column-block list entry out of range"};
    if (hm.timeout_flag) throw Fail{COSTAL_ETIMEOUT, "a bounded device wait in the tensor-core kernel gave up"};
    if (st) {
        st->fallback_rows = hm.fb_count;
        st->row_block = 128;
        st->col_block = used_tc ? (uint64_t)(list_cb ? list_cb : tc::BLOCK_N) : 128;
        st->blocks_skipped = hm.blocks_skipped;
        st->blocks_stopped = hm.blocks_stopped;
        st->blocks_total = (uint64_t)(qb1 - qb0) * (uint64_t)((n + st->col_block - 1) / st->col_block);
        st->margin = margin;
        st->recomputed_rows = used_tc ? hm.tc_fail_count : 0;
        st->pruned_fallback_rows = hm.prune_fail_count;
        double me;
        std::memcpy(&me, &hm.max_err_bits[0], 8);
        st->max_coarse_err = me;
        std::memcpy(&me, &hm.max_err_bits[1], 8);
        st->max_err_ratio = me;
        st->coarse_kind = used_tc ? (fp8 ? 2 : 1) : 0;
        st->ms_prep = elapsed(c.ev[0], c.ev[1]);
        st->ms_order = elapsed(c.ev[1], c.ev[5]);
        st->ms_coarse = elapsed(c.ev[5], c.ev[2]);
        st->ms_rescore = elapsed(c.ev[2], c.ev[3]);
        st->ms_fallback = elapsed(c.ev[3], c.ev[4]);
        st->ms_total = elapsed(c.ev[0], c.ev[4]);
        st->ms_kernel = used_tc ? elapsed(c.ev[6], c.ev[2]) : st->ms_coarse;
    }
}

costal_knn_opts defaults() {
    costal_knn_opts o{};
    o.margin = UINT32_MAX;
    o.select = COSTAL_SELECT_COSINE;
    o.backend = COSTAL_BACKEND_FP32;
    o.sort_by_norm = 1;
    o.prune = 1;
    return o;
}

template <class F>
int guarded(char* err, size_t errlen, F&& f) {
    Context& c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    int rc = init_locked(c);
    if (rc != COSTAL_OK) {
        put_err(err, errlen, c.init_err);
        return rc;
    }
    try {
        f(c);
    } catch (const Fail& fl) {
        put_err(err, errlen, fl.msg);
        return fl.rc;
    } catch (const std::exception& ex) {
        put_err(err, errlen, ex.what());
        return COSTAL_ECUDA;
    }
    return COSTAL_OK;
}

void check_knn_args(uint64_t n, uint32_t d, uint32_t k) {
    std::string m = knn_arg_error(n, k);
    if (!m.empty()) throw Fail{COSTAL_EINVAL, m};
    if (n > (uint64_t)INT32_MAX) throw Fail{COSTAL_EINVAL, "n=" + std::to_string(n) + " exceeds the int32 index range"};
    if ((uint64_t)n * k > (uint64_t)INT32_MAX)
        throw Fail{COSTAL_EUNSUPPORTED, "n*k exceeds the int32 edge index range of the GPU path"};
    (void)d;
}

// Check an (n, k) neighbour matrix on the device: lib.rs:65-78 reports the first bad value.
void check_neighbours(Context& c, const int32_t* d_idx, const int32_t* h_idx, uint64_t n, uint32_t k, cudaStream_t s) {
    CK(ensure(c.misc, sizeof(Misc)));
    Misc* dm = c.misc.as<Misc>();
    CK(cudaMemsetAsync(&dm->first_bad_idx, 0xff, 8, s));
    CK(launch_check_idx(d_idx, n * k, (int)n, &dm->first_bad_idx, s));
    CK(cudaMemcpyAsync(c.h_misc, dm, sizeof(Misc), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (c.h_misc->first_bad_idx != ~0ull) {
        int32_t bad = h_idx[c.h_misc->first_bad_idx];
        throw Fail{COSTAL_EINVAL, "neighbor index " + std::to_string(bad) + " out of range (n=" + std::to_string(n) + ")"};
    }
}

}  // namespace

extern "C" {

const char* costal_version(void) { return "2.1.0"; }

unsigned long long costal_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int costal_device_ok(char* err, size_t errlen) {
    return guarded(err, errlen, [](Context&) {});
}

int costal_check_f64_conversion(uint64_t* mismatches, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        cudaStream_t s = c.stream;
        CK(ensure(c.misc, sizeof(Misc)));
        Misc* dm = c.misc.as<Misc>();
        CK(cudaMemsetAsync(&dm->conv_mismatches, 0, 8, s));
        CK(launch_check_f64_of(&dm->conv_mismatches, c.sm_count, s));
        CK(cudaMemcpyAsync(c.h_misc, dm, sizeof(Misc), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        *mismatches = c.h_misc->conv_mismatches;
    });
}

int costal_row_l2_norms(const float* x, uint64_t n, uint32_t d, float* out, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        if (n == 0) return;
        cudaStream_t s = c.stream;
        CK(ensure(c.x, n * d * 4ull));
        CK(ensure(c.f32out, n * 4ull));
        CK(cudaMemcpyAsync(c.x.p, x, n * d * 4ull, cudaMemcpyHostToDevice, s));
        CK(launch_row_l2_norms_f32(c.x.as<float>(), (int)n, (int)d, c.f32out.as<float>(), s));
        CK(cudaMemcpyAsync(out, c.f32out.p, n * 4ull, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

int costal_knn_exact(const float* x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts, uint32_t* idx,
                     double* cos, double* norms, costal_knn_stats* stats, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        check_knn_args(n, d, k);
        const costal_knn_opts o = opts ? *opts : defaults();
        cudaStream_t s = c.stream;
        CK(ensure(c.x, n * d * 4ull));
        CK(ensure(c.out_idx, n * k * 4ull));
        CK(ensure(c.out_cos, n * k * 8ull));
        CK(ensure(c.norms, n * 8ull));
        CK(cudaMemcpyAsync(c.x.p, x, n * d * 4ull, cudaMemcpyHostToDevice, s));
        run_knn(c, c.x.as<float>(), (int)n, (int)d, (int)k, o, c.out_idx.as<uint32_t>(), c.out_cos.as<double>(),
                c.norms.as<double>(), nullptr, stats, s);
        CK(cudaMemcpyAsync(idx, c.out_idx.p, n * k * 4ull, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(cos, c.out_cos.p, n * k * 8ull, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(norms, c.norms.p, n * 8ull, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

int costal_knn_exact_device(const float* d_x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts,
                            uint32_t* d_idx, double* d_cos, double* d_norms, costal_knn_stats* stats, void* stream,
                            char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        check_knn_args(n, d, k);
        const costal_knn_opts o = opts ? *opts : defaults();
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.stream;
        run_knn(c, d_x, (int)n, (int)d, (int)k, o, d_idx, d_cos, d_norms, nullptr, stats, s);
    });
}

int costal_knn_bruteforce(const float* x, uint64_t n, uint32_t d, uint32_t k, uint32_t select, uint32_t* idx,
                          double* cos, double* norms, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        check_knn_args(n, d, k);
        cudaStream_t s = c.stream;
        const int dp = coarse_dpad((int)d), np = round_up((int)n, 128);
        CK(ensure(c.x, n * d * 4ull));
        CK(ensure(c.out_idx, n * k * 4ull));
        CK(ensure(c.out_cos, n * k * 8ull));
        CK(ensure(c.norms, n * 8ull));
        CK(ensure(c.xsT, (size_t)dp * np * 4));
        CK(ensure(c.misc, sizeof(Misc)));
        Misc* dm = c.misc.as<Misc>();
        CK(cudaMemsetAsync(&dm->bad_row, 0xff, 8, s));
        CK(cudaMemcpyAsync(c.x.p, x, n * d * 4ull, cudaMemcpyHostToDevice, s));
        CK(launch_prep(c.x.as<float>(), (int)n, (int)d, np, dp, c.norms.as<double>(), c.xsT.as<float>(), &dm->bad_row, s));
        if (gather_smem(k, d, dp) > 227 * 1024) throw Fail{COSTAL_EUNSUPPORTED, "k too large for the GPU scan kernel"};
        CK(launch_gather(c.x.as<float>(), c.xsT.as<float>(), (int)n, np, (int)d, dp, (int)k, c.norms.as<double>(),
                         nullptr, nullptr, nullptr, 1, select == COSTAL_SELECT_TANIMOTO ? 1 : 0,
                         std::min((int)n, 8 * c.sm_count), c.out_idx.as<uint32_t>(), c.out_cos.as<double>(), nullptr, s));
        CK(cudaMemcpyAsync(c.h_misc, dm, sizeof(Misc), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(idx, c.out_idx.p, n * k * 4ull, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(cos, c.out_cos.p, n * k * 8ull, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(norms, c.norms.p, n * 8ull, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (c.h_misc->bad_row != ~0ull)
            throw Fail{COSTAL_EINVAL, "row " + std::to_string(c.h_misc->bad_row) + " contains NaN or inf"};
    });
}

int costal_reweight(uint64_t n, uint32_t k, const int32_t* idx, const double* cos, const double* norms, uint32_t weight,
                    double* out, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        if (weight > COSTAL_WEIGHT_JACCARD) throw Fail{COSTAL_EINVAL, "unknown edge weight"};
        const uint64_t nk = n * k;
        if (nk == 0) return;
        if (nk > (uint64_t)INT32_MAX) throw Fail{COSTAL_EUNSUPPORTED, "n*k exceeds the int32 range of the GPU path"};
        cudaStream_t s = c.stream;
        CK(ensure(c.idx_in, nk * 4));
        CK(ensure(c.cos_in, nk * 8));
        CK(ensure(c.norms_in, n * 8));
        CK(ensure(c.w_in, nk * 8));
        CK(cudaMemcpyAsync(c.idx_in.p, idx, nk * 4, cudaMemcpyHostToDevice, s));
        check_neighbours(c, c.idx_in.as<int32_t>(), idx, n, k, s);
        if (weight == COSTAL_WEIGHT_COSINE) {
            std::memcpy(out, cos, nk * 8);  // weight.rs:51: the rescored cosine itself
            return;
        }
        if (weight == COSTAL_WEIGHT_TANIMOTO) {
            CK(cudaMemcpyAsync(c.cos_in.p, cos, nk * 8, cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(c.norms_in.p, norms, n * 8, cudaMemcpyHostToDevice, s));
            CK(launch_tanimoto_w(c.idx_in.as<uint32_t>(), c.cos_in.as<double>(), c.norms_in.as<double>(), nk, (int)k,
                                 c.w_in.as<double>(), s));
        } else {
            CK(ensure(c.jac, nk * 4));
            CK(launch_jaccard(c.idx_in.as<uint32_t>(), (int)n, (int)k, c.jac.as<uint32_t>(), c.w_in.as<double>(), s));
        }
        CK(cudaMemcpyAsync(out, c.w_in.p, nk * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

namespace {
void run_union(Context& c, const uint32_t* d_idx, const double* d_w, uint64_t n, uint32_t k, int32_t* d_rows,
               int32_t* d_cols, double* d_wout, uint64_t* m, cudaStream_t s) {
    CK(ensure(c.fu_scratch, fuzzy_union_scratch_bytes((int)n, (int)k)));
    CK(ensure(c.misc, sizeof(Misc)));
    Misc* dm = c.misc.as<Misc>();
    CK(launch_fuzzy_union(d_idx, d_w, (int)n, (int)k, c.fu_scratch.p, d_rows, d_cols, d_wout, &dm->m, s));
    CK(cudaMemcpyAsync(&c.h_misc->m, &dm->m, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *m = c.h_misc->m;
}
}  // namespace

int costal_fuzzy_union(uint64_t n, uint32_t k, const int32_t* idx, const double* w, int32_t* rows, int32_t* cols,
                       double* w_out, uint64_t* m, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        *m = 0;
        const uint64_t nk = n * k;
        if (nk == 0) return;
        if (nk > (uint64_t)INT32_MAX) throw Fail{COSTAL_EUNSUPPORTED, "n*k exceeds the int32 range of the GPU path"};
        cudaStream_t s = c.stream;
        CK(ensure(c.idx_in, nk * 4));
        CK(ensure(c.w_in, nk * 8));
        CK(ensure(c.rows, nk * 4));
        CK(ensure(c.cols, nk * 4));
        CK(ensure(c.wout, nk * 8));
        CK(cudaMemcpyAsync(c.idx_in.p, idx, nk * 4, cudaMemcpyHostToDevice, s));
        check_neighbours(c, c.idx_in.as<int32_t>(), idx, n, k, s);
        CK(cudaMemcpyAsync(c.w_in.p, w, nk * 8, cudaMemcpyHostToDevice, s));
        run_union(c, c.idx_in.as<uint32_t>(), c.w_in.as<double>(), n, k, c.rows.as<int32_t>(), c.cols.as<int32_t>(),
                  c.wout.as<double>(), m, s);
        CK(cudaMemcpyAsync(rows, c.rows.p, *m * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(cols, c.cols.p, *m * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(w_out, c.wout.p, *m * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

namespace {
// X (device) -> kNN -> weights -> fuzzy union, all on the device.
void run_build(Context& c, const float* d_x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts& o,
               uint32_t weight, int32_t* d_rows, int32_t* d_cols, double* d_w, uint64_t* m, costal_knn_stats* st,
               cudaStream_t s) {
    if (weight > COSTAL_WEIGHT_JACCARD) throw Fail{COSTAL_EINVAL, "unknown edge weight"};
    const uint64_t nk = n * k;
    CK(ensure(c.out_idx, nk * 4));
    CK(ensure(c.out_cos, nk * 8));
    CK(ensure(c.norms, n * 8));
    CK(ensure(c.out_w, nk * 8));
    double* fused_w = weight == COSTAL_WEIGHT_TANIMOTO ? c.out_w.as<double>() : nullptr;
    run_knn(c, d_x, (int)n, (int)d, (int)k, o, c.out_idx.as<uint32_t>(), c.out_cos.as<double>(), c.norms.as<double>(),
            fused_w, st, s);
    const double* wsrc = c.out_w.as<double>();
    if (weight == COSTAL_WEIGHT_COSINE) {
        wsrc = c.out_cos.as<double>();
    } else if (weight == COSTAL_WEIGHT_JACCARD) {
        CK(ensure(c.jac, nk * 4));
        CK(launch_jaccard(c.out_idx.as<uint32_t>(), (int)n, (int)k, c.jac.as<uint32_t>(), c.out_w.as<double>(), s));
    }
    run_union(c, c.out_idx.as<uint32_t>(), wsrc, n, k, d_rows, d_cols, d_w, m, s);
}
}  // namespace

int costal_build_graph(const float* x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts, uint32_t weight,
                       int32_t* rows, int32_t* cols, double* w, uint64_t* m, uint32_t* idx, double* cos, double* norms,
                       costal_knn_stats* stats, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        check_knn_args(n, d, k);
        const costal_knn_opts o = opts ? *opts : defaults();
        cudaStream_t s = c.stream;
        const uint64_t nk = n * k;
        CK(ensure(c.x, n * d * 4ull));
        CK(ensure(c.rows, nk * 4));
        CK(ensure(c.cols, nk * 4));
        CK(ensure(c.wout, nk * 8));
        CK(cudaMemcpyAsync(c.x.p, x, n * d * 4ull, cudaMemcpyHostToDevice, s));
        run_build(c, c.x.as<float>(), n, d, k, o, weight, c.rows.as<int32_t>(), c.cols.as<int32_t>(),
                  c.wout.as<double>(), m, stats, s);
        CK(cudaMemcpyAsync(rows, c.rows.p, *m * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(cols, c.cols.p, *m * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(w, c.wout.p, *m * 8, cudaMemcpyDeviceToHost, s));
        if (idx) CK(cudaMemcpyAsync(idx, c.out_idx.p, nk * 4, cudaMemcpyDeviceToHost, s));
        if (cos) CK(cudaMemcpyAsync(cos, c.out_cos.p, nk * 8, cudaMemcpyDeviceToHost, s));
        if (norms) CK(cudaMemcpyAsync(norms, c.norms.p, n * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

int costal_build_graph_csr(const float* x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts,
                           uint32_t weight, uint64_t* indptr, uint32_t* nbr, double* w, uint64_t* nnz,
                           costal_knn_stats* stats, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        check_knn_args(n, d, k);
        const uint64_t nk = n * k;
        if (2 * nk > (uint64_t)INT32_MAX) throw Fail{COSTAL_EUNSUPPORTED, "2*n*k exceeds the int32 range of the GPU CSR"};
        const costal_knn_opts o = opts ? *opts : defaults();
        cudaStream_t s = c.stream;
        CK(ensure(c.x, n * d * 4ull));
        CK(ensure(c.rows, nk * 4));
        CK(ensure(c.cols, nk * 4));
        CK(ensure(c.wout, nk * 8));
        CK(cudaMemcpyAsync(c.x.p, x, n * d * 4ull, cudaMemcpyHostToDevice, s));
        uint64_t m = 0;
        run_build(c, c.x.as<float>(), n, d, k, o, weight, c.rows.as<int32_t>(), c.cols.as<int32_t>(),
                  c.wout.as<double>(), &m, stats, s);
        CK(ensure(c.csr_ws, csr_scratch_bytes((int)n, (int)k)));
        CK(ensure(c.csr_indptr, (n + 1) * 8));
        CK(ensure(c.csr_src, 2 * nk * 4));
        CK(ensure(c.csr_nbr, 2 * nk * 4));
        CK(ensure(c.csr_w, 2 * nk * 8));
        Misc* dm = c.misc.as<Misc>();
        CK(launch_csr_from_union(c.rows.as<int32_t>(), c.cols.as<int32_t>(), c.wout.as<double>(), &dm->m, (int)n, (int)k,
                                 c.csr_ws.p, c.csr_indptr.as<uint64_t>(), c.csr_src.as<int32_t>(),
                                 c.csr_nbr.as<int32_t>(), c.csr_w.as<double>(), &dm->nnz, s));
        *nnz = 2 * m;
        CK(cudaMemcpyAsync(indptr, c.csr_indptr.p, (n + 1) * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(nbr, c.csr_nbr.p, *nnz * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(w, c.csr_w.p, *nnz * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

int costal_build_graph_device(const float* d_x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts,
                              uint32_t weight, int32_t* d_rows, int32_t* d_cols, double* d_w, uint64_t* m,
                              costal_knn_stats* stats, void* stream, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        check_knn_args(n, d, k);
        const costal_knn_opts o = opts ? *opts : defaults();
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.stream;
        run_build(c, d_x, n, d, k, o, weight, d_rows, d_cols, d_w, m, stats, s);
    });
}

// ---- row shards (multi-GPU) ------------------------------------------------------------------

uint64_t costal_shard_rows_max(uint64_t n, uint32_t n_shards) {
    if (n_shards == 0) return 0;
    const uint64_t nqb = (n + 127) / 128, most = (nqb + n_shards - 1) / n_shards;
    return std::min<uint64_t>(n, most * 128);
}

int costal_knn_shard_device(const float* d_x, uint64_t n, uint32_t d, uint32_t k, const costal_knn_opts* opts,
                            uint32_t shard, uint32_t n_shards, uint32_t* d_rows, uint64_t* count, uint32_t* d_idx,
                            double* d_cos, double* d_w, double* d_norms, costal_knn_stats* stats, void* stream,
                            char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        check_knn_args(n, d, k);
        if (n_shards == 0 || shard >= n_shards)
            throw Fail{COSTAL_EINVAL, "shard " + std::to_string(shard) + " of " + std::to_string(n_shards)};
        const costal_knn_opts o = opts ? *opts : defaults();
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.stream;
        const uint64_t nk = n * k;
        CK(ensure(c.out_idx, nk * 4));
        CK(ensure(c.out_cos, nk * 8));
        if (d_w) CK(ensure(c.out_w, nk * 8));
        Shard sh;
        sh.index = (int)shard;
        sh.count = (int)n_shards;
        run_knn(c, d_x, (int)n, (int)d, (int)k, o, c.out_idx.as<uint32_t>(), c.out_cos.as<double>(), d_norms,
                d_w ? c.out_w.as<double>() : nullptr, stats, s, &sh);
        *count = (uint64_t)sh.nrows;
        if (sh.nrows > 0) {
            CK(cudaMemcpyAsync(d_rows, c.shard_rows.p, (size_t)sh.nrows * 4, cudaMemcpyDeviceToDevice, s));
            CK(launch_take_rows(c.shard_rows.as<uint32_t>(), sh.nrows, (int)k, c.out_idx.as<uint32_t>(),
                                c.out_cos.as<double>(), d_w ? c.out_w.as<double>() : nullptr, d_idx, d_cos, d_w, s));
        }
        CK(cudaStreamSynchronize(s));
    });
}

int costal_fuzzy_union_device(const int32_t* d_idx, const double* d_w, uint64_t n, uint32_t k, int32_t* d_rows,
                              int32_t* d_cols, double* d_wout, uint64_t* m, void* stream, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        *m = 0;
        const uint64_t nk = n * k;
        if (nk == 0) return;
        if (nk > (uint64_t)INT32_MAX) throw Fail{COSTAL_EUNSUPPORTED, "n*k exceeds the int32 range of the GPU path"};
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.stream;
        CK(ensure(c.misc, sizeof(Misc)));
        Misc* dm = c.misc.as<Misc>();
        CK(cudaMemsetAsync(&dm->first_bad_idx, 0xff, 8, s));
        CK(launch_check_idx(d_idx, nk, (int)n, &dm->first_bad_idx, s));
        CK(cudaMemcpyAsync(c.h_misc, dm, sizeof(Misc), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (c.h_misc->first_bad_idx != ~0ull) {  // lib.rs:65-78: report the first bad value
            int32_t bad = 0;
            CK(cudaMemcpy(&bad, d_idx + c.h_misc->first_bad_idx, 4, cudaMemcpyDeviceToHost));
            throw Fail{COSTAL_EINVAL,
                       "neighbor index " + std::to_string(bad) + " out of range (n=" + std::to_string(n) + ")"};
        }
        run_union(c, reinterpret_cast<const uint32_t*>(d_idx), d_w, n, k, d_rows, d_cols, d_wout, m, s);
    });
}

// ---- the learned block-pruning model ----------------------------------------------------------

int costal_mlp_train(const float* x, uint64_t n, uint32_t d, uint32_t k, const costal_mlp_opts* mo,
                     costal_mlp_stats* stats, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        check_knn_args(n, d, k);
        if (!prune::supported((int)d)) throw Fail{COSTAL_EUNSUPPORTED, "learned pruning supports 1 <= d <= 64"};
        costal_mlp_opts o{};
        o.sample = 200000;
        o.epochs = 30;
        o.batch = 2048;
        o.lr = 2e-3f;
        o.quantile = 0.05f;
        o.margin = UINT32_MAX;
        o.seed = 20241203;
        if (mo) o = *mo;
        cudaStream_t s = c.stream;
        const int N = (int)n, D = (int)d, K = (int)k;
        const int dp = coarse_dpad(D), np = round_up(N, 128);
        const uint64_t margin = o.margin == UINT32_MAX ? (uint64_t)k : (uint64_t)o.margin;
        const int cap = (int)std::min<uint64_t>((uint64_t)k + margin, n - 1);
        if (coarse_slots(cap) == 0 || coarse_fp32_smem(dp, cap) > 227 * 1024)
            throw Fail{COSTAL_EUNSUPPORTED, "k + margin too large for the FP32 label pass"};
        const int m = (int)std::min<uint64_t>(o.sample ? o.sample : n, n);
        const int F = D + MLP_TOPC;
        const size_t P = mlp_param_count(F);
        CK(ensure(c.x, n * d * 4ull));
        CK(ensure(c.norms, n * 8ull));
        CK(ensure(c.xsT, (size_t)dp * np * 4));
        CK(ensure(c.misc, sizeof(Misc)));
        CK(ensure(c.cand_idx, (size_t)n * cap * 4));
        CK(ensure(c.cand_score, (size_t)n * cap * 4));
        CK(ensure(c.tau, n * 4ull));
        CK(ensure(c.out_idx, n * k * 4ull));
        CK(ensure(c.out_cos, n * k * 8ull));
        CK(ensure(c.fb_rows, n * 4ull));
        CK(ensure(c.fb_minsim, n * 8ull));
        CK(ensure(c.mlp_rows, (size_t)std::max(m, std::min(N, MLP_CHUNK)) * 4));
        CK(ensure(c.mlp_y, (size_t)m * 4));
        CK(ensure(c.mlp_feat, (size_t)std::max(m, std::min(N, MLP_CHUNK)) * F * 4));
        CK(ensure(c.mlp_pred, std::max<size_t>(n, m) * 4));
        CK(ensure(c.mlp_params, P * 4));
        CK(ensure(c.mlp_params_bf, P * 4));
        CK(ensure(c.mlp_m1, P * 4));
        CK(ensure(c.mlp_m2, P * 4));
        CK(ensure(c.mlp_grad, P * 4));
        CK(ensure(c.mlp_partial, (size_t)((o.batch + 31) / 32) * P * 4));
        Misc* dm = c.misc.as<Misc>();
        CK(cudaMemsetAsync(dm, 0, sizeof(Misc), s));
        CK(cudaMemsetAsync(&dm->bad_row, 0xff, 8, s));
        CK(cudaMemcpyAsync(c.x.p, x, n * d * 4ull, cudaMemcpyHostToDevice, s));
        CK(cudaEventRecord(c.ev[0], s));
        CK(launch_prep(c.x.as<float>(), N, D, np, dp, c.norms.as<double>(), c.xsT.as<float>(), &dm->bad_row, s));
        // the same cells (and so the same features) as the pruned kNN computes for this data
        CK(ensure(c.prune_ws, prune::workspace_bytes(N, D)));
        prune::Plan pp{};
        CK(prune::build_order(c.prune_ws.p, c.xsT.as<float>(), N, np, D, s, pp));
        // labels: the exact k-th-neighbour cosine of every sampled row, from the plain FP32 path
        uint32_t* rows = c.mlp_rows.as<uint32_t>();
        CK(launch_stride_rows(rows, m, N, s));
        unsigned hm = (unsigned)m;
        CK(cudaMemcpyAsync(&dm->tc_fail_count, &hm, 4, cudaMemcpyHostToDevice, s));
        CK(launch_coarse_fp32(c.xsT.as<float>(), N, np, dp, cap, cap, rows, &dm->tc_fail_count, c.cand_idx.as<uint32_t>(),
                              c.cand_score.as<float>(), c.tau.as<float>(), s));
        const double eps = ((double)d + 4.0) * F32_EPS;
        CK(launch_rescore(c.x.as<float>(), N, D, K, cap, cap, c.cand_idx.as<uint32_t>(), c.cand_score.as<float>(),
                          c.tau.as<float>(), c.norms.as<double>(), nullptr, nullptr, nullptr, eps, cap < N - 1, 0, rows,
                          &dm->tc_fail_count, c.out_idx.as<uint32_t>(), c.out_cos.as<double>(), nullptr,
                          c.fb_rows.as<uint32_t>(), c.fb_minsim.as<double>(), &dm->fb_count, nullptr, s));
        if (cap < N - 1)
            CK(launch_gather(c.x.as<float>(), c.xsT.as<float>(), N, np, D, dp, K, c.norms.as<double>(),
                             c.fb_rows.as<uint32_t>(), c.fb_minsim.as<double>(), &dm->fb_count, 0, 0,
                             std::min(N, 4 * c.sm_count), c.out_idx.as<uint32_t>(), c.out_cos.as<double>(), nullptr, s));
        CK(launch_kth(c.out_cos.as<double>(), rows, m, K, c.mlp_y.as<float>(), s));
        CK(mlp::features(c.xsT.as<float>(), np, D, pp.centroids, pp.K, rows, m, c.mlp_feat.as<float>(), s));
        CK(cudaEventRecord(c.ev[1], s));
        // Adam on the pinball loss, minibatches in sample order
        CK(launch_init_params(c.mlp_params.as<float>(), F, (unsigned long long)o.seed, s));
        CK(cudaMemsetAsync(c.mlp_m1.p, 0, P * 4, s));
        CK(cudaMemsetAsync(c.mlp_m2.p, 0, P * 4, s));
        int t = 0;
        const int B = (int)std::max<uint32_t>(32, o.batch);
        for (uint32_t ep = 0; ep < o.epochs; ++ep) {
            for (int b0 = 0; b0 < m; b0 += B) {
                const int mb = std::min(B, m - b0);
                CK(mlp::gradient(c.mlp_params.as<float>(), F, c.mlp_feat.as<float>() + (size_t)b0 * F,
                                 c.mlp_y.as<float>() + b0, mb, o.quantile, c.mlp_partial.as<float>(),
                                 c.mlp_grad.as<float>(), s));
                CK(mlp::adam(c.mlp_params.as<float>(), c.mlp_grad.as<float>(), c.mlp_m1.as<float>(),
                             c.mlp_m2.as<float>(), P, o.lr, ++t, s));
            }
        }
        CK(mlp::round_bf16(c.mlp_params.as<float>(), c.mlp_params_bf.as<float>(), P, s));
        CK(mlp::forward(c.mlp_params_bf.as<float>(), F, c.mlp_feat.as<float>(), m, c.mlp_pred.as<float>(), s));
        CK(cudaEventRecord(c.ev[2], s));
        std::vector<float> pred(m), y(m);
        CK(cudaMemcpyAsync(pred.data(), c.mlp_pred.p, (size_t)m * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(y.data(), c.mlp_y.p, (size_t)m * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(c.h_misc, dm, sizeof(Misc), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (c.h_misc->bad_row != ~0ull)
            throw Fail{COSTAL_EINVAL, "row " + std::to_string(c.h_misc->bad_row) + " contains NaN or inf"};
        double loss = 0.0, mae = 0.0;
        size_t below = 0;
        for (int i = 0; i < m; ++i) {
            const double r = (double)y[i] - (double)pred[i];
            loss += r >= 0 ? o.quantile * r : (o.quantile - 1.0) * r;
            mae += std::fabs(r);
            below += pred[i] <= y[i];
        }
        c.mlp.ready = true;
        c.mlp.d = D;
        c.mlp.k = K;
        c.mlp.F = F;
        c.mlp.quantile = o.quantile;
        c.mlp.params = c.mlp_params.as<float>();
        c.mlp.params_bf = c.mlp_params_bf.as<float>();
        c.mlp.nparams = P;
        if (stats) {
            stats->samples = (uint64_t)m;
            stats->steps = (uint64_t)t;
            stats->params = (uint64_t)P;
            stats->loss = loss / m;
            stats->mae = mae / m;
            stats->coverage = (double)below / m;
            stats->ms_labels = elapsed(c.ev[0], c.ev[1]);
            stats->ms_train = elapsed(c.ev[1], c.ev[2]);
        }
    });
}

int costal_mlp_get(float* params, uint64_t capacity, uint64_t* count, uint32_t* d, uint32_t* k, float* quantile,
                   char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        if (!c.mlp.ready) throw Fail{COSTAL_EINVAL, "no trained model"};
        *count = c.mlp.nparams;
        *d = (uint32_t)c.mlp.d;
        *k = (uint32_t)c.mlp.k;
        *quantile = c.mlp.quantile;
        if (params && capacity >= c.mlp.nparams) {
            CK(cudaMemcpy(params, c.mlp.params, c.mlp.nparams * 4, cudaMemcpyDeviceToHost));
        }
    });
}

int costal_mlp_set(const float* params, uint64_t count, uint32_t d, uint32_t k, float quantile, char* err,
                   size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        const int F = (int)d + MLP_TOPC;
        const size_t P = mlp_param_count(F);
        if (!prune::supported((int)d) || count != P)
            throw Fail{COSTAL_EINVAL, "parameter block does not match d (expected " + std::to_string(P) + " values)"};
        CK(ensure(c.mlp_params, P * 4));
        CK(ensure(c.mlp_params_bf, P * 4));
        CK(cudaMemcpy(c.mlp_params.p, params, P * 4, cudaMemcpyHostToDevice));
        CK(mlp::round_bf16(c.mlp_params.as<float>(), c.mlp_params_bf.as<float>(), P, c.stream));
        CK(cudaStreamSynchronize(c.stream));
        c.mlp.ready = true;
        c.mlp.d = (int)d;
        c.mlp.k = (int)k;
        c.mlp.F = F;
        c.mlp.quantile = quantile;
        c.mlp.params = c.mlp_params.as<float>();
        c.mlp.params_bf = c.mlp_params_bf.as<float>();
        c.mlp.nparams = P;
    });
}

int costal_mlp_clear(char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) { c.mlp.ready = false; });
}

int costal_mlp_forward(const float* params, uint32_t F, const float* feat, uint64_t m, float* out, char* err,
                       size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        if (F < 1 || F > (uint32_t)MLP_MAXF) throw Fail{COSTAL_EINVAL, "F out of range"};
        const size_t P = mlp_param_count((int)F);
        cudaStream_t s = c.stream;
        CK(ensure(c.mlp_grad, P * 4));
        CK(ensure(c.mlp_feat, m * F * 4));
        CK(ensure(c.mlp_pred, m * 4));
        CK(cudaMemcpyAsync(c.mlp_grad.p, params, P * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(c.mlp_feat.p, feat, m * F * 4, cudaMemcpyHostToDevice, s));
        CK(mlp::forward(c.mlp_grad.as<float>(), (int)F, c.mlp_feat.as<float>(), (int)m, c.mlp_pred.as<float>(), s));
        CK(cudaMemcpyAsync(out, c.mlp_pred.p, m * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

int costal_mlp_gradient(const float* params, uint32_t F, const float* feat, const float* y, uint64_t m,
                        float quantile, float* grad, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        if (F < 1 || F > (uint32_t)MLP_MAXF) throw Fail{COSTAL_EINVAL, "F out of range"};
        const size_t P = mlp_param_count((int)F);
        cudaStream_t s = c.stream;
        CK(ensure(c.mlp_m1, P * 4));
        CK(ensure(c.mlp_grad, P * 4));
        CK(ensure(c.mlp_feat, m * F * 4));
        CK(ensure(c.mlp_y, m * 4));
        CK(ensure(c.mlp_partial, ((m + 31) / 32) * P * 4));
        CK(cudaMemcpyAsync(c.mlp_m1.p, params, P * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(c.mlp_feat.p, feat, m * F * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(c.mlp_y.p, y, m * 4, cudaMemcpyHostToDevice, s));
        CK(mlp::gradient(c.mlp_m1.as<float>(), (int)F, c.mlp_feat.as<float>(), c.mlp_y.as<float>(), (int)m, quantile,
                         c.mlp_partial.as<float>(), c.mlp_grad.as<float>(), s));
        CK(cudaMemcpyAsync(grad, c.mlp_grad.p, P * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

int costal_block_bounds(const float* x, uint64_t n, uint32_t d, uint32_t* perm, double* ccenter, double* cradius,
                        float* rowmax, float* delta, char* err, size_t errlen) {
    return guarded(err, errlen, [&](Context& c) {
        if (n < 2 || n > (uint64_t)INT32_MAX / 2) throw Fail{COSTAL_EINVAL, "n out of range"};
        if (!prune::supported((int)d)) throw Fail{COSTAL_EUNSUPPORTED, "block bounds cover 1 <= d <= 64"};
        cudaStream_t s = c.stream;
        const int N = (int)n, D = (int)d;
        const int dp = coarse_dpad(D), np = round_up(N, 128);
        CK(ensure(c.x, n * d * 4ull));
        CK(ensure(c.norms, n * 8ull));
        CK(ensure(c.xsT, (size_t)dp * np * 4));
        CK(ensure(c.misc, sizeof(Misc)));
        Misc* dm = c.misc.as<Misc>();
        CK(cudaMemsetAsync(dm, 0, sizeof(Misc), s));
        CK(cudaMemsetAsync(&dm->bad_row, 0xff, 8, s));
        CK(cudaMemcpyAsync(c.x.p, x, n * d * 4ull, cudaMemcpyHostToDevice, s));
        CK(launch_prep(c.x.as<float>(), N, D, np, dp, c.norms.as<double>(), c.xsT.as<float>(), &dm->bad_row, s));
        CK(ensure(c.prune_ws, prune::workspace_bytes(N, D)));
        prune::Plan pp{};
        CK(prune::build_order(c.prune_ws.p, c.xsT.as<float>(), N, np, D, s, pp));
        CK(ensure(c.tc_ws, tc::workspace_bytes(N, D, false)));
        tc::Plan plan{};
        CK(tc::prepare(c.tc_ws.p, c.xsT.as<float>(), N, np, dp, D, pp.perm, s, plan, false, pp.wrows));
        CK(ensure(c.rm_ws, tc::rowmax_bytes(pp.ncb, D)));
        CK(ensure(c.rm_out, (size_t)pp.nqb * pp.ncb * 4));
        const float* d_delta = nullptr;
        CK(tc::launch_rowmax(plan, pp.ccenter_f, pp.ncb, c.rm_ws.p, c.rm_out.as<float>(), &d_delta, &dm->timeout_flag,
                             s));
        CK(cudaMemcpyAsync(perm, pp.perm, n * 4ull, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(ccenter, pp.ccenter, (size_t)pp.ncb * D * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(cradius, pp.cradius, (size_t)pp.ncb * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(rowmax, c.rm_out.p, (size_t)pp.nqb * pp.ncb * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(delta, d_delta, 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(c.h_misc, dm, sizeof(Misc), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (c.h_misc->bad_row != ~0ull)
            throw Fail{COSTAL_EINVAL, "row " + std::to_string(c.h_misc->bad_row) + " contains NaN or inf"};
        if (c.h_misc->timeout_flag) throw Fail{COSTAL_ETIMEOUT, "a bounded device wait in the bound kernel gave up"};
    });
}

}  // extern "C"
