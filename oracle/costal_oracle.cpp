// TEST INFRASTRUCTURE ONLY — the CPU oracle for the exact cosine kNN graph.
//
// A C++ restatement of CosTaL 2.1.0's CPU algorithms, used by tests/ as the parity checker, by
// __graft_entry__.smoke() as the checker of one small GPU run, and by bench.py as the timed CPU
// baseline. Nothing in the product library (costal_gb300/) links, loads or calls this file.
//
// Parity status: PINNED. The restatement is checked (tests/test_oracle.py) against every known
// answer the reference's own tests hold for this path — the duplicate tie-break answer
// (crates/costal-core/src/knn.rs:1002-1017), zero rows (:1020-1032), the heap tie-break
// (:1150-1159), the closed-form Tanimoto values (weight.rs:100-109), the Jaccard hand case
// (weight.rs:112-121), the fuzzy-union hand cases (graph.rs:74-95), bitwise equality of the
// blocked path with the brute force (tests/test_knn.py:38-43), and the GOLDEN_PIPELINE digest
// (tests/test_leiden_native.py:123-135) that pins kNN + Tanimoto + fuzzy union + Leiden end to end.
//
// Every function cites the reference file:line it restates. Floating-point expressions keep the
// reference's order of operations; this file is compiled with -ffp-contract=off so that no
// multiply-add is fused (Rust never contracts). Only oracle_tile.cpp (the coarse f32 tile
// product, whose rounding is covered by the coarse-error bound) allows contraction.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" void oracle_tile_nt(const float* a, size_t rows, const float* b, size_t cols, size_t d,
                               float* out, float* scratch_bt);

namespace {

constexpr float F32_EPS = 1.1920928955078125e-07f;  // f32::EPSILON = 2^-23

// knn.rs:290-296 — f64 dot in dimension order (f32×f32 is exact in f64).
inline double dot64(const float* a, const float* b, size_t d) {
    double s = 0.0;
    for (size_t t = 0; t < d; ++t) s += (double)a[t] * (double)b[t];
    return s;
}

// knn.rs:301-312 — cosine for rescoring; 0 for a zero row; -0.0 normalised to +0.0.
inline double cos64(double dot, double ni, double nj) {
    if (ni == 0.0 || nj == 0.0) return 0.0;
    double c = dot / (ni * nj);
    return c == 0.0 ? 0.0 : c;
}

// weight.rs:30-37 — d = a·b·cos; 0 when d == 0, else d / (a² + b² − d).
inline double tani_from_cos(double a, double b, double c) {
    double d = a * b * c;
    if (d == 0.0) return 0.0;
    return d / (a * a + b * b - d);
}

// Rust's f64::total_cmp as an integer key (knn.rs:589-591 sorts with it).
inline int64_t total_key(double v) {
    int64_t b;
    std::memcpy(&b, &v, 8);
    return b ^ (int64_t)(((uint64_t)(b >> 63)) >> 1);
}

struct Cand {
    double score;
    double cos;
    uint32_t j;
};

// knn.rs:589-591 — sort by (score desc, original index asc).
inline void sort_cands(std::vector<Cand>& c) {
    std::sort(c.begin(), c.end(), [](const Cand& a, const Cand& b) {
        int64_t ka = total_key(a.score), kb = total_key(b.score);
        if (ka != kb) return ka > kb;
        return a.j < b.j;
    });
}

// knn.rs:798-801 — heap order: lower score is worse; on equal scores the larger index is worse.
inline bool worse(float sa, uint32_t ia, float sb, uint32_t ib) {
    return sa < sb || (sa == sb && ia > ib);
}

// knn.rs:791-875 — one fixed-capacity min-heap per row of a row block.
struct BlockHeaps {
    size_t cap;
    std::vector<float> scores;
    std::vector<uint32_t> ids;
    std::vector<size_t> lens;
    BlockHeaps(size_t rows, size_t cap_) : cap(cap_), scores(rows * cap_), ids(rows * cap_), lens(rows) {}
    void reset() { std::fill(lens.begin(), lens.end(), 0); }
    float tau(size_t r) const {
        return lens[r] < cap ? -std::numeric_limits<float>::infinity() : scores[r * cap];
    }
    void push(size_t r, float score, uint32_t id) {
        float* s = &scores[r * cap];
        uint32_t* d = &ids[r * cap];
        size_t len = lens[r];
        if (len < cap) {
            size_t pos = len;
            s[pos] = score;
            d[pos] = id;
            while (pos > 0) {
                size_t parent = (pos - 1) / 2;
                if (!worse(s[pos], d[pos], s[parent], d[parent])) break;
                std::swap(s[pos], s[parent]);
                std::swap(d[pos], d[parent]);
                pos = parent;
            }
            lens[r] = len + 1;
            return;
        }
        if (!worse(s[0], d[0], score, id)) return;
        s[0] = score;
        d[0] = id;
        size_t pos = 0;
        for (;;) {
            size_t left = 2 * pos + 1;
            if (left >= cap) break;
            size_t w = left;
            if (left + 1 < cap && worse(s[left + 1], d[left + 1], s[left], d[left])) w = left + 1;
            if (!worse(s[w], d[w], s[pos], d[pos])) break;
            std::swap(s[pos], s[w]);
            std::swap(d[pos], d[w]);
            pos = w;
        }
    }
};

// Selection metrics, knn.rs:136-284.
struct CosineSel {
    static constexpr bool NORMALIZED = true;
    static constexpr bool PRUNES = false;
    float row_state(size_t) const { return 0.0f; }
    float tile_threshold(float, float tau, size_t) const { return tau; }       // :172-174
    float score(float, size_t, float sim) const { return sim; }                // :176-178
    double rescore(double c, double, double) const { return c; }               // :180-182
    double coarse_eps(size_t d) const { return ((double)d + 4.0) * (double)F32_EPS; }  // :185-187
    bool norm_window(float, double*, double*) const { return false; }
};

struct TanimotoSel {
    static constexpr bool NORMALIZED = false;
    static constexpr bool PRUNES = true;
    std::vector<float> norm_sq, block_min, block_max;
    size_t cb;
    // knn.rs:207-227
    TanimotoSel(const std::vector<uint32_t>& perm, const std::vector<double>& norms, size_t cb_) {
        cb = std::max<size_t>(cb_, 1);
        norm_sq.resize(perm.size());
        for (size_t w = 0; w < perm.size(); ++w) {
            double v = norms[perm[w]];
            norm_sq[w] = (float)(v * v);
        }
        for (size_t s = 0; s < norm_sq.size(); s += cb) {
            float lo = std::numeric_limits<float>::infinity(), hi = -lo;
            for (size_t t = s; t < std::min(norm_sq.size(), s + cb); ++t) {
                lo = std::min(lo, norm_sq[t]);
                hi = std::max(hi, norm_sq[t]);
            }
            block_min.push_back(lo);
            block_max.push_back(hi);
        }
    }
    float row_state(size_t row) const { return norm_sq[row]; }
    // knn.rs:239-252
    float tile_threshold(float a, float tau, size_t col_start) const {
        if (tau == -std::numeric_limits<float>::infinity()) return tau;
        float c = tau / (1.0f + tau);
        size_t block = col_start / cb;
        float b = c >= 0.0f ? block_min[block] : block_max[block];
        return c * (a + b);
    }
    // knn.rs:254-261
    float score(float a, size_t col, float dot) const {
        float den = a + norm_sq[col] - dot;
        if (dot == 0.0f || den <= 0.0f) return 0.0f;
        return dot / den;
    }
    double rescore(double c, double ni, double nj) const { return tani_from_cos(ni, nj, c); }
    double coarse_eps(size_t d) const { return 2.0 * ((double)d + 8.0) * (double)F32_EPS; }  // :268-270
    // knn.rs:275-283
    bool norm_window(float tau, double* lo, double* hi) const {
        if (std::isnan(tau) || tau <= 0.0f) return false;
        double t = (double)tau;
        double q = (1.0 + t) / t * (1.0 + 1e-4);
        double disc = std::sqrt(std::max(q * q - 4.0, 0.0));
        *lo = (q - disc) / 2.0;
        *hi = (q + disc) / 2.0;
        return true;
    }
};

struct Scratch {
    std::vector<float> tile, bt;
    BlockHeaps heaps;
    std::vector<Cand> cands;
    Scratch(size_t rb, size_t cb, size_t cap, size_t d)
        : tile(rb * cb), bt(cb * std::max<size_t>(d, 1)), heaps(rb, cap) {}
};

template <class S>
struct Ctx {
    const S& sel;
    const float* x;
    const float* xs;
    const double* norms;
    const uint32_t* perm;
    size_t n, d, k, cap, cb;
    double eps;
    bool prune;

    // knn.rs:758-787 — scan one tile row: a 16-wide "any above the threshold" test, heap pushes on
    // the rare path, self-exclusion by working index.
    void scan_row(float st, const float* row, size_t cols, size_t c0, size_t self_col,
                  BlockHeaps& heaps, size_t r) const {
        const size_t LANES = 16;
        float th = sel.tile_threshold(st, heaps.tau(r), c0);
        size_t base = c0;
        for (size_t off = 0; off < cols; off += LANES) {
            size_t len = std::min(LANES, cols - off);
            bool hit = false;
            for (size_t t = 0; t < len; ++t) hit |= row[off + t] > th;
            if (hit) {
                for (size_t t = 0; t < len; ++t) {
                    float v = row[off + t];
                    size_t col = base + t;
                    if (v > th && col != self_col) {
                        heaps.push(r, sel.score(st, col, v), (uint32_t)col);
                        th = sel.tile_threshold(st, heaps.tau(r), c0);
                    }
                }
            }
            base += len;
        }
    }

    // knn.rs:647-660
    void scan_block(size_t r0, size_t rows, size_t blk, Scratch& scr) const {
        size_t c0 = blk * cb;
        size_t cols = std::min(cb, n - c0);
        oracle_tile_nt(xs + r0 * d, rows, xs + c0 * d, cols, d, scr.tile.data(), scr.bt.data());
        for (size_t r = 0; r < rows; ++r) {
            float st = sel.row_state(r0 + r);
            scan_row(st, &scr.tile[r * cols], cols, c0, r0 + r, scr.heaps, r);
        }
    }

    double norm_at(size_t w) const { return norms[perm[w]]; }

    // knn.rs:669-678
    bool block_window(size_t r0, size_t rows, const BlockHeaps& heaps, double* lo, double* hi) const {
        double l = std::numeric_limits<double>::infinity(), h = -l;
        for (size_t r = 0; r < rows; ++r) {
            double rlo, rhi;
            if (!sel.norm_window(heaps.tau(r), &rlo, &rhi)) return false;
            double a = norm_at(r0 + r);
            l = std::min(l, rlo * a);
            h = std::max(h, rhi * a);
        }
        *lo = l;
        *hi = h;
        return true;
    }

    // knn.rs:603-644 — returns the number of column blocks skipped.
    size_t coarse_block(size_t r0, size_t rows, Scratch& scr) const {
        scr.heaps.reset();
        size_t nblocks = (n + cb - 1) / cb;
        if (!S::PRUNES || !prune) {
            for (size_t blk = 0; blk < nblocks; ++blk) scan_block(r0, rows, blk, scr);
            return 0;
        }
        size_t mid = std::min((r0 + rows / 2) / cb, nblocks - 1);
        scan_block(r0, rows, mid, scr);
        size_t left = mid, right = mid + 1, scanned = 1;
        for (;;) {
            double lo = 0, hi = 0;
            bool win = block_window(r0, rows, scr.heaps, &lo, &hi);
            bool progressed = false;
            if (right < nblocks) {
                if (!win || norm_at(right * cb) <= hi) {
                    scan_block(r0, rows, right, scr);
                    right += 1;
                    scanned += 1;
                    progressed = true;
                } else {
                    right = nblocks;
                }
            }
            if (left > 0) {
                if (!win || norm_at(left * cb - 1) >= lo) {
                    scan_block(r0, rows, left - 1, scr);
                    left -= 1;
                    scanned += 1;
                    progressed = true;
                } else {
                    left = 0;
                }
            }
            if (!progressed) return nblocks - scanned;
        }
    }

    // knn.rs:746-753
    void push_rescored(size_t i, size_t wj, std::vector<Cand>& cands) const {
        uint32_t j = perm[wj];
        double dot = dot64(x + i * d, x + (size_t)j * d, d);
        double c = cos64(dot, norms[i], norms[j]);
        cands.push_back({sel.rescore(c, norms[i], norms[j]), c, j});
    }

    // knn.rs:723-743 — fallback: rescan the whole row, gather f32 score ≥ min_sim, rescore.
    void gather_row(size_t w_row, double min_sim, Scratch& scr) const {
        size_t i = perm[w_row];
        scr.cands.clear();
        const float* a = xs + w_row * d;
        float st = sel.row_state(w_row);
        for (size_t c0 = 0; c0 < n; c0 += cb) {
            size_t cols = std::min(cb, n - c0);
            oracle_tile_nt(a, 1, xs + c0 * d, cols, d, scr.tile.data(), scr.bt.data());
            for (size_t t = 0; t < cols; ++t) {
                size_t wj = c0 + t;
                if (wj != w_row && (double)sel.score(st, wj, scr.tile[t]) >= min_sim)
                    push_rescored(i, wj, scr.cands);
            }
        }
    }

    // knn.rs:688-720 — rescore one row; returns whether the fallback was taken.
    bool finalize_row(size_t w_row, size_t r, Scratch& scr, uint32_t* out_idx, double* out_cos) const {
        size_t i = perm[w_row];
        scr.cands.clear();
        for (size_t t = 0; t < scr.heaps.lens[r]; ++t)
            push_rescored(i, scr.heaps.ids[r * cap + t], scr.cands);
        sort_cands(scr.cands);
        bool fell_back = false;
        if (cap < n - 1) {
            double floor = (double)scr.heaps.tau(r);
            double s_k = scr.cands[k - 1].score;
            if (s_k <= floor + eps) {
                fell_back = true;
                gather_row(w_row, s_k - eps, scr);
                sort_cands(scr.cands);
            }
        }
        for (size_t t = 0; t < k; ++t) {
            out_idx[t] = scr.cands[t].j;
            out_cos[t] = scr.cands[t].cos;
        }
        return fell_back;
    }
};

void row_norms64(const float* x, size_t n, size_t d, double* out) {  // knn.rs:315-323
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) out[i] = std::sqrt(dot64(x + i * d, x + i * d, d));
}

void set_err(char* err, size_t errlen, const char* msg) {
    if (err && errlen) {
        std::snprintf(err, errlen, "%s", msg);
    }
}

// knn.rs:325-342
int validate(const float* x, size_t n, size_t d, size_t k, char* err, size_t errlen) {
    char buf[160];
    if (n > 0xFFFFFFFFull) {
        std::snprintf(buf, sizeof buf, "n=%zu exceeds the u32 index range", n);
        set_err(err, errlen, buf);
        return 2;
    }
    if (k == 0 || k >= n) {
        std::snprintf(buf, sizeof buf, "invalid k=%zu: need 1 <= k <= n-1 (n=%zu)", k, n);
        set_err(err, errlen, buf);
        return 2;
    }
    for (size_t i = 0; i < n; ++i) {
        for (size_t t = 0; t < d; ++t) {
            if (!std::isfinite(x[i * d + t])) {
                std::snprintf(buf, sizeof buf, "row %zu contains NaN or inf", i);
                set_err(err, errlen, buf);
                return 2;
            }
        }
    }
    return 0;
}

struct Stats {
    uint64_t fallback_rows, row_block, col_block, blocks_skipped, blocks_total;
};

// knn.rs:403-512
template <class S, class Make>
void run_blocked(const float* x, size_t n, size_t d, size_t k, size_t margin, size_t row_block,
                 size_t col_block, bool sort_by_norm, bool prune, int threads, Make make,
                 uint32_t* idx, double* cos, double* norms, Stats* st) {
    row_norms64(x, n, d, norms);
    std::vector<uint32_t> perm(n);
    for (size_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
    if (sort_by_norm)  // stable: equal norms keep original-index order (knn.rs:413-418)
        std::stable_sort(perm.begin(), perm.end(),
                         [&](uint32_t a, uint32_t b) { return total_key(norms[a]) < total_key(norms[b]); });
    std::vector<float> xs(n * d, 0.0f);
#pragma omp parallel for schedule(static)
    for (long long w = 0; w < (long long)n; ++w) {  // knn.rs:420-436
        size_t o = perm[w];
        const float* src = x + o * d;
        float* dst = &xs[w * d];
        if (!S::NORMALIZED) {
            std::memcpy(dst, src, d * sizeof(float));
            continue;
        }
        double nrm = norms[o];
        if (nrm > 0.0)
            for (size_t t = 0; t < d; ++t) dst[t] = (float)((double)src[t] / nrm);
    }
    // knn.rs:551-569 with a fixed 1 MiB tile budget in place of the CPU cache probe (block sizes
    // change speed only, never the output).
    size_t budget = (1u << 20) / sizeof(float);
    size_t side = (size_t)1 << ((63 - __builtin_clzll((unsigned long long)budget)) / 2);
    size_t cb = col_block ? col_block : std::min<size_t>(std::max<size_t>(side, 256), 1024);
    cb = std::min<size_t>(std::max<size_t>(cb, 1), n);
    size_t rb = row_block;
    if (!rb) {
        size_t by_cache = budget / cb;
        size_t by_balance = (n + (size_t)threads * 8 - 1) / ((size_t)threads * 8);
        rb = std::min<size_t>(std::max<size_t>(std::min(by_cache, by_balance), 8), 512);
    }
    rb = std::min<size_t>(std::max<size_t>(rb, 1), n);
    S sel = make(perm, std::vector<double>(norms, norms + n), cb);
    size_t cap = std::min(k + margin, n - 1);
    Ctx<S> ctx{sel, x, xs.data(), norms, perm.data(), n, d, k, cap, cb, sel.coarse_eps(d),
               prune && sort_by_norm};
    std::vector<uint32_t> w_idx(n * k);
    std::vector<double> w_cos(n * k);
    size_t nrb = (n + rb - 1) / rb;
    uint64_t skipped = 0, fallbacks = 0;
#pragma omp parallel num_threads(threads) reduction(+ : skipped, fallbacks)
    {
        Scratch scr(rb, cb, cap, d);
#pragma omp for schedule(dynamic, 1)
        for (long long bi = 0; bi < (long long)nrb; ++bi) {
            size_t r0 = (size_t)bi * rb;
            size_t rows = std::min(rb, n - r0);
            skipped += ctx.coarse_block(r0, rows, scr);
            for (size_t r = 0; r < rows; ++r)
                fallbacks += ctx.finalize_row(r0 + r, r, scr, &w_idx[(r0 + r) * k], &w_cos[(r0 + r) * k]);
        }
    }
    // knn.rs:516-543 — working order → original order (out of place here).
    for (size_t w = 0; w < n; ++w) {
        size_t dst = perm[w];
        std::memcpy(idx + dst * k, &w_idx[w * k], k * sizeof(uint32_t));
        std::memcpy(cos + dst * k, &w_cos[w * k], k * sizeof(double));
    }
    st->fallback_rows = fallbacks;
    st->row_block = rb;
    st->col_block = cb;
    st->blocks_skipped = skipped;
    st->blocks_total = ((n + rb - 1) / rb) * ((n + cb - 1) / cb);
}

}  // namespace

extern "C" {

struct oracle_stats {
    uint64_t fallback_rows, row_block, col_block, blocks_skipped, blocks_total;
};

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// knn.rs:365-379 (knn_exact_with_stats). select: 0 cosine, 1 tanimoto. row_block/col_block 0 = derive.
int oracle_knn_exact(const float* x, uint64_t n, uint32_t d, uint32_t k, uint32_t margin, int select,
                     uint32_t row_block, uint32_t col_block, int sort_by_norm, int prune, int n_threads,
                     uint32_t* idx, double* cos, double* norms, oracle_stats* stats, char* err,
                     size_t errlen) {
    int rc = validate(x, n, d, k, err, errlen);
    if (rc) return rc;
    int threads = n_threads > 0 ? n_threads : oracle_max_threads();
    Stats st{};
    if (select == 0) {
        run_blocked<CosineSel>(x, n, d, k, margin, row_block, col_block, sort_by_norm != 0, prune != 0,
                               threads,
                               [](const std::vector<uint32_t>&, const std::vector<double>&, size_t) {
                                   return CosineSel{};
                               },
                               idx, cos, norms, &st);
    } else {
        run_blocked<TanimotoSel>(x, n, d, k, margin, row_block, col_block, sort_by_norm != 0, prune != 0,
                                 threads,
                                 [](const std::vector<uint32_t>& p, const std::vector<double>& nr, size_t cb) {
                                     return TanimotoSel(p, nr, cb);
                                 },
                                 idx, cos, norms, &st);
    }
    if (stats) std::memcpy(stats, &st, sizeof st);
    return 0;
}

// The blocked cosine path restricted to query rows [q0, q1), against all n columns: the same
// per-row work as oracle_knn_exact (tiles, heaps, rescoring, certificate, fallback) for a bounded
// sample of rows. Used to time the CPU baseline on a slice of a large workload. Outputs hold
// (q1 − q0) rows; norms holds all n.
int oracle_knn_rows(const float* x, uint64_t n, uint32_t d, uint32_t k, uint32_t margin, uint64_t q0,
                    uint64_t q1, int n_threads, uint32_t* idx, double* cos, double* norms,
                    uint64_t* fallback_rows, char* err, size_t errlen) {
    int rc = validate(x, n, d, k, err, errlen);
    if (rc) return rc;
    if (q0 > q1 || q1 > n) {
        set_err(err, errlen, "query row range out of bounds");
        return 2;
    }
    int threads = n_threads > 0 ? n_threads : oracle_max_threads();
    row_norms64(x, n, d, norms);
    std::vector<uint32_t> perm(n);
    for (size_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
    std::vector<float> xs(n * (size_t)d, 0.0f);
#pragma omp parallel for schedule(static)
    for (long long w = 0; w < (long long)n; ++w) {
        double nrm = norms[w];
        if (nrm > 0.0)
            for (size_t t = 0; t < d; ++t) xs[w * d + t] = (float)((double)x[w * d + t] / nrm);
    }
    size_t cb = std::min<size_t>(512, n), rb = 64;
    CosineSel sel;
    size_t cap = std::min<size_t>((size_t)k + margin, n - 1);
    Ctx<CosineSel> ctx{sel, x, xs.data(), norms, perm.data(), n, d, k, cap, cb, sel.coarse_eps(d), false};
    size_t rows_total = q1 - q0, nrb = (rows_total + rb - 1) / rb;
    uint64_t fallbacks = 0;
#pragma omp parallel num_threads(threads) reduction(+ : fallbacks)
    {
        Scratch scr(rb, cb, cap, d);
#pragma omp for schedule(dynamic, 1)
        for (long long bi = 0; bi < (long long)nrb; ++bi) {
            size_t r0 = q0 + (size_t)bi * rb;
            size_t rows = std::min(rb, q1 - r0);
            ctx.coarse_block(r0, rows, scr);
            for (size_t r = 0; r < rows; ++r)
                fallbacks += ctx.finalize_row(r0 + r, r, scr, idx + (r0 + r - q0) * k, cos + (r0 + r - q0) * k);
        }
    }
    if (fallback_rows) *fallback_rows = fallbacks;
    return 0;
}

// knn.rs:884-924 — golden brute force: every candidate in f64, full sort.
int oracle_knn_bruteforce(const float* x, uint64_t n, uint32_t d, uint32_t k, int select, int n_threads,
                          uint32_t* idx, double* cos, double* norms, char* err, size_t errlen) {
    int rc = validate(x, n, d, k, err, errlen);
    if (rc) return rc;
    int threads = n_threads > 0 ? n_threads : oracle_max_threads();
    row_norms64(x, n, d, norms);
#pragma omp parallel num_threads(threads)
    {
        std::vector<Cand> all;
        all.reserve(n);
#pragma omp for schedule(dynamic, 16)
        for (long long i = 0; i < (long long)n; ++i) {
            all.clear();
            for (size_t j = 0; j < n; ++j) {
                if (j == (size_t)i) continue;
                double c = cos64(dot64(x + i * d, x + j * d, d), norms[i], norms[j]);
                double s = select == 0 ? c : tani_from_cos(norms[i], norms[j], c);
                all.push_back({s, c, (uint32_t)j});
            }
            sort_cands(all);
            for (size_t t = 0; t < k; ++t) {
                idx[i * k + t] = all[t].j;
                cos[i * k + t] = all[t].cos;
            }
        }
    }
    return 0;
}

// weight.rs:30-37
double oracle_tani_from_cos(double a, double b, double c) { return tani_from_cos(a, b, c); }

// weight.rs:41-92 — weight: 0 tanimoto, 1 cosine, 2 jaccard. idx values must be in [0, n).
int oracle_reweight(uint64_t n, uint32_t k, const uint32_t* idx, const double* cos, const double* norms,
                    int weight, double* out) {
    size_t nk = (size_t)n * k;
    if (weight == 1) {
        std::memcpy(out, cos, nk * sizeof(double));
        return 0;
    }
    if (weight == 0) {
        for (size_t e = 0; e < nk; ++e) out[e] = tani_from_cos(norms[e / k], norms[idx[e]], cos[e]);
        return 0;
    }
    std::vector<uint32_t> sorted(idx, idx + nk);
    for (size_t i = 0; i < n; ++i) std::sort(sorted.begin() + i * k, sorted.begin() + (i + 1) * k);
    for (size_t i = 0; i < n; ++i) {
        const uint32_t* a = &sorted[i * k];
        for (size_t t = 0; t < k; ++t) {
            const uint32_t* b = &sorted[(size_t)idx[i * k + t] * k];
            size_t p = 0, q = 0, c = 0;  // weight.rs:79-93
            while (p < k && q < k) {
                if (a[p] < b[q]) ++p;
                else if (a[p] > b[q]) ++q;
                else { ++c; ++p; ++q; }
            }
            double s = (double)c;
            out[i * k + t] = s / (2.0 * (double)k - s);
        }
    }
    return 0;
}

// graph.rs:24-68 — fuzzy union S + Sᵀ − S∘Sᵀ; upper-triangular, ascending (row, col), exact zeros
// dropped. Outputs hold up to n·k edges; *m receives the edge count.
int oracle_fuzzy_union(uint64_t n, uint32_t k, const uint32_t* idx, const double* w, uint32_t* rows,
                       uint32_t* cols, double* wout, uint64_t* m_out) {
    std::vector<std::pair<uint64_t, double>> e;
    e.reserve((size_t)n * k);
    for (size_t t = 0; t < (size_t)n * k; ++t) {
        uint64_t i = t / k, j = idx[t];
        if (i == j) continue;
        uint64_t lo = std::min(i, j), hi = std::max(i, j);
        e.push_back({(lo << 32) | hi, w[t]});
    }
    std::stable_sort(e.begin(), e.end(),
                     [](const std::pair<uint64_t, double>& a, const std::pair<uint64_t, double>& b) {
                         return a.first < b.first;
                     });
    size_t m = 0, t = 0;
    while (t < e.size()) {
        uint64_t key = e[t].first;
        double a = e[t].second, v;
        if (t + 1 < e.size() && e[t + 1].first == key) {
            double b = e[t + 1].second;
            t += 2;
            v = (a + b) - a * b;
        } else {
            t += 1;
            v = a;
        }
        if (v != 0.0) {
            rows[m] = (uint32_t)(key >> 32);
            cols[m] = (uint32_t)key;
            wout[m] = v;
            ++m;
        }
    }
    *m_out = m;
    return 0;
}

// knn.rs:791-875 — push `count` (score, id) pairs into one heap of capacity `cap` without a
// threshold check, and return the kept ids (the heap_keeps_best_with_index_tiebreak test, :1150-1159).
size_t oracle_heap_keep(const float* scores, const uint32_t* ids, size_t count, size_t cap, uint32_t* out) {
    BlockHeaps h(1, cap);
    for (size_t t = 0; t < count; ++t) h.push(0, scores[t], ids[t]);
    for (size_t t = 0; t < h.lens[0]; ++t) out[t] = h.ids[t];
    return h.lens[0];
}

// lib.rs:34-47 — f32 row norms (the module's smoke function), sequential f32 sum per row.
void oracle_row_l2_norms(const float* x, uint64_t n, uint32_t d, float* out) {
    for (size_t i = 0; i < n; ++i) {
        float s = 0.0f;
        for (size_t t = 0; t < d; ++t) s += x[i * d + t] * x[i * d + t];
        out[i] = std::sqrt(s);
    }
}

}  // extern "C"
