// Host Leiden: the consumer of the device-built kNN graph (`leiden="fast"`).
//
// A C++ restatement of CosTaL 2.1.0's deterministic Leiden (crates/costal-core/src/leiden.rs),
// which the reference runs on the host after building the graph. It is not GPU work: it must give
// the same partition as the reference for the same edge list and seed, so every floating-point
// expression keeps the reference's order of operations (this file is compiled with
// -ffp-contract=off), the random streams are the reference's own xoshiro256** seeded through
// SplitMix64 (leiden.rs:1329-1396), and e^x is the reference's own range-reduced Taylor polynomial
// (leiden.rs:1297-1327). The reference parallelises the refinement and aggregation per cluster and
// per row, which it states never changes the result (leiden.rs:10-18, 630-642); this version runs
// them sequentially and parallelises only independent runs (costal_leiden_many).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "costal_gb300.h"

namespace {

// leiden.rs:28-32. The algorithm reads the graph through the three pointers, which point either into
// the owned vectors (graphs built here) or into a caller's arrays (a CSR built on the GPU).
struct Csr {
    std::vector<size_t> indptr_s{0};
    std::vector<uint32_t> nbr_s;
    std::vector<double> w_s;
    const size_t* indptr = indptr_s.data();
    const uint32_t* nbr = nullptr;
    const double* w = nullptr;
    size_t nodes = 0;
    size_t n() const { return nodes; }
    void bind() {  // after the owned vectors change
        indptr = indptr_s.data();
        nbr = nbr_s.data();
        w = w_s.data();
        nodes = indptr_s.size() - 1;
    }
    Csr() = default;
    Csr(const Csr&) = delete;
    Csr& operator=(const Csr&) = delete;
};
static_assert(sizeof(size_t) == sizeof(uint64_t), "indptr is exchanged as u64");

std::string fmt_f64(double x) {  // Rust's Display for the weights quoted in error messages
    if (std::isnan(x)) return "NaN";
    if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.17g", x);
    return buf;
}

// leiden.rs:52-101 — each undirected edge once; zero weights dropped; rows in edge-list order.
bool csr_from_edges(size_t n, const uint32_t* rows, const uint32_t* cols, const double* w, size_t m,
                    Csr& g, std::string& err) {
    if (n > 0xFFFFFFFFull) {
        err = std::to_string(n) + " nodes exceed the u32 node index";
        return false;
    }
    g.indptr_s.assign(n + 1, 0);
    for (size_t e = 0; e < m; ++e) {
        size_t i = rows[e], j = cols[e];
        double x = w[e];
        if (i >= n || j >= n) {
            err = "edge " + std::to_string(e) + " (" + std::to_string(i) + ", " + std::to_string(j) +
                  ") is out of range (n=" + std::to_string(n) + ")";
            return false;
        }
        if (i == j) {
            err = "edge " + std::to_string(e) + " is a self-loop on node " + std::to_string(i);
            return false;
        }
        if (!(std::isfinite(x) && x >= 0.0)) {
            err = "edge " + std::to_string(e) + " has weight " + fmt_f64(x) +
                  "; weights must be finite and non-negative";
            return false;
        }
        if (x > 0.0) {
            g.indptr_s[i + 1] += 1;
            g.indptr_s[j + 1] += 1;
        }
    }
    for (size_t v = 0; v < n; ++v) g.indptr_s[v + 1] += g.indptr_s[v];
    std::vector<size_t> fill(g.indptr_s.begin(), g.indptr_s.begin() + n);
    g.nbr_s.assign(g.indptr_s[n], 0);
    g.w_s.assign(g.indptr_s[n], 0.0);
    for (size_t e = 0; e < m; ++e) {
        size_t i = rows[e], j = cols[e];
        double x = w[e];
        if (x > 0.0) {
            g.nbr_s[fill[i]] = (uint32_t)j;
            g.w_s[fill[i]] = x;
            fill[i] += 1;
            g.nbr_s[fill[j]] = (uint32_t)i;
            g.w_s[fill[j]] = x;
            fill[j] += 1;
        }
    }
    g.bind();
    return true;
}

// A caller's CSR in the same layout (a graph built on the GPU), checked for what the algorithm
// relies on — indptr from 0 and non-decreasing up to nnz, neighbours in range and not the row
// itself, weights finite and positive — and used in place, without a copy.
bool csr_view(size_t n, const uint64_t* indptr, const uint32_t* nbr, const double* w, Csr& g, std::string& err) {
    if (n > 0xFFFFFFFFull) {
        err = std::to_string(n) + " nodes exceed the u32 node index";
        return false;
    }
    if (indptr[0] != 0) {
        err = "indptr[0] must be 0";
        return false;
    }
    for (size_t v = 0; v < n; ++v) {
        if (indptr[v + 1] < indptr[v]) {
            err = "indptr decreases at row " + std::to_string(v);
            return false;
        }
        for (uint64_t e = indptr[v]; e < indptr[v + 1]; ++e) {
            if (nbr[e] >= n || nbr[e] == v) {
                err = "entry " + std::to_string(e) + " of row " + std::to_string(v) + " has neighbour " +
                      std::to_string(nbr[e]) + " (n=" + std::to_string(n) + ")";
                return false;
            }
            if (!(std::isfinite(w[e]) && w[e] > 0.0)) {
                err = "entry " + std::to_string(e) + " has weight " + fmt_f64(w[e]) + "; CSR weights must be finite and positive";
                return false;
            }
        }
    }
    g.indptr = reinterpret_cast<const size_t*>(indptr);
    g.nbr = nbr;
    g.w = w;
    g.nodes = n;
    return true;
}

// leiden.rs:112-187 — each edge once in either orientation, or a symmetric list; anything else is
// an error.
bool csr_from_coo(size_t n, const uint32_t* rows, const uint32_t* cols, const double* w, size_t m,
                  Csr& g, std::string& err) {
    struct K {
        uint32_t a, b;
        bool up;
        uint32_t e;
        bool operator<(const K& o) const {
            if (a != o.a) return a < o.a;
            if (b != o.b) return b < o.b;
            if (up != o.up) return up < o.up;
            return e < o.e;
        }
    };
    std::vector<K> keyed;
    keyed.reserve(m);
    for (size_t e = 0; e < m; ++e) {
        uint32_t i = rows[e], j = cols[e];
        double x = w[e];
        if ((size_t)i >= n || (size_t)j >= n) {
            err = "edge " + std::to_string(e) + " (" + std::to_string(i) + ", " + std::to_string(j) +
                  ") is out of range (n=" + std::to_string(n) + ")";
            return false;
        }
        if (i == j) {
            err = "edge " + std::to_string(e) + " is a self-loop on node " + std::to_string(i);
            return false;
        }
        if (!(std::isfinite(x) && x >= 0.0)) {
            err = "edge " + std::to_string(e) + " has weight " + fmt_f64(x) +
                  "; weights must be finite and non-negative";
            return false;
        }
        keyed.push_back({std::min(i, j), std::max(i, j), i < j, (uint32_t)e});
    }
    std::sort(keyed.begin(), keyed.end());
    size_t once = 0, both = 0;
    std::vector<uint32_t> lo, hi;
    std::vector<double> ww;
    size_t t = 0;
    while (t < keyed.size()) {
        K cur = keyed[t];
        size_t k = t + 1;
        while (k < keyed.size() && keyed[k].a == cur.a && keyed[k].b == cur.b) ++k;
        if (k - t == 1) {
            once += 1;
        } else if (k - t == 2 && keyed[t + 1].up != cur.up) {
            size_t other = keyed[t + 1].e;
            if (w[cur.e] != w[other]) {
                err = "edges " + std::to_string(cur.e) + " and " + std::to_string(other) + " list the pair (" +
                      std::to_string(cur.a) + ", " + std::to_string(cur.b) +
                      ") in both directions with different weights (" + fmt_f64(w[cur.e]) + " and " +
                      fmt_f64(w[other]) + ")";
                return false;
            }
            both += 1;
        } else {
            std::string list;
            for (size_t q = t; q < k; ++q) list += (q > t ? ", " : "") + std::to_string(keyed[q].e);
            err = "the pair (" + std::to_string(cur.a) + ", " + std::to_string(cur.b) +
                  ") is listed more than once in the same direction (edges " + list +
                  "); combine duplicates before calling";
            return false;
        }
        if (once > 0 && both > 0) {
            err = "some pairs are listed in both directions and others once: give each edge once, or "
                  "every edge in both directions (a symmetric matrix)";
            return false;
        }
        lo.push_back(cur.a);
        hi.push_back(cur.b);
        ww.push_back(w[cur.e]);
        t = k;
    }
    return csr_from_edges(n, lo.data(), hi.data(), ww.data(), lo.size(), g, err);
}

std::vector<double> strengths(const Csr& g) {  // leiden.rs:206-208
    std::vector<double> s(g.n());
    for (size_t v = 0; v < g.n(); ++v) {
        double acc = 0.0;
        for (size_t e = g.indptr[v]; e < g.indptr[v + 1]; ++e) acc += g.w[e];
        s[v] = acc;
    }
    return s;
}

double sum(const std::vector<double>& v) {
    double s = 0.0;
    for (double x : v) s += x;
    return s;
}

// ---------------------------------------------------------------- the reference's own math

constexpr uint64_t GOLDEN = 0x9E3779B97F4A7C15ull;

uint64_t mix(uint64_t z) {  // leiden.rs:1331-1335
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

struct Rng {  // leiden.rs:1338-1396 — xoshiro256** seeded from a list of words
    uint64_t s[4];
    Rng(std::initializer_list<uint64_t> words) {
        uint64_t h = 0x243F6A8885A308D3ull;
        for (uint64_t w : words) h = mix((h + GOLDEN) ^ w);
        for (auto& lane : s) {
            h += GOLDEN;
            lane = mix(h);
        }
        if (!s[0] && !s[1] && !s[2] && !s[3]) s[0] = GOLDEN;
    }
    Rng(const uint64_t* words, size_t nw) {
        uint64_t h = 0x243F6A8885A308D3ull;
        for (size_t i = 0; i < nw; ++i) h = mix((h + GOLDEN) ^ words[i]);
        for (auto& lane : s) {
            h += GOLDEN;
            lane = mix(h);
        }
        if (!s[0] && !s[1] && !s[2] && !s[3]) s[0] = GOLDEN;
    }
    uint64_t next_u64() {
        uint64_t out = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return out;
    }
    uint64_t below(uint64_t n) {  // Lemire's multiply-shift with rejection
        unsigned __int128 m = (unsigned __int128)next_u64() * n;
        if ((uint64_t)m < n) {
            uint64_t threshold = (0 - n) % n;
            while ((uint64_t)m < threshold) m = (unsigned __int128)next_u64() * n;
        }
        return (uint64_t)(m >> 64);
    }
    double unif() { return (double)(next_u64() >> 11) * (1.0 / (double)(1ull << 53)); }
    void shuffle(std::vector<uint32_t>& a) {
        for (size_t i = a.size(); i-- > 1;) {
            size_t j = (size_t)below((uint64_t)i + 1);
            std::swap(a[i], a[j]);
        }
    }
};

struct InvFactorial {  // leiden.rs:1298-1306
    double a[14];
    InvFactorial() {
        a[0] = 1.0;
        for (int k = 1; k < 14; ++k) a[k] = a[k - 1] / (double)k;
    }
};
const InvFactorial INV_FACTORIAL;

double exp_nonpositive(double x) {  // leiden.rs:1313-1327
    if (x < -708.0) return 0.0;
    const double LN2_HI = 6.931471803691238e-1;
    const double LN2_LO = 1.9082149292705877e-10;
    const double LOG2_E = 1.4426950408889634;
    double k = std::round(x * LOG2_E);
    double r = (x - k * LN2_HI) - k * LN2_LO;
    double p = INV_FACTORIAL.a[13];
    for (int c = 12; c >= 0; --c) p = p * r + INV_FACTORIAL.a[c];
    uint64_t bits = ((uint64_t)((int64_t)k + 1023)) << 52;
    double scale;
    std::memcpy(&scale, &bits, 8);
    return p * scale;
}

// ---------------------------------------------------------------- the algorithm

template <class T>
void reset(std::vector<T>& v, size_t n, T x) {
    v.clear();
    v.resize(n, x);
}

struct Groups {  // leiden.rs:598-604
    std::vector<size_t> start, fill;
    std::vector<uint32_t> order;
};

void group_by(const std::vector<uint32_t>& labels, size_t nl, Groups& gr) {  // leiden.rs:1246-1261
    reset(gr.start, nl + 1, (size_t)0);
    for (uint32_t c : labels) gr.start[c + 1] += 1;
    for (size_t c = 0; c < nl; ++c) gr.start[c + 1] += gr.start[c];
    gr.fill.assign(gr.start.begin(), gr.start.begin() + nl);
    reset(gr.order, labels.size(), 0u);
    for (size_t v = 0; v < labels.size(); ++v) gr.order[gr.fill[labels[v]]++] = (uint32_t)v;
}

size_t compact(uint32_t* labels, size_t len, size_t n_ids, std::vector<uint32_t>& map) {  // :1264-1280
    reset(map, n_ids, UINT32_MAX);
    for (size_t i = 0; i < len; ++i) map[labels[i]] = 0;
    uint32_t k = 0;
    for (auto& x : map)
        if (x == 0) x = k++;
    for (size_t i = 0; i < len; ++i) labels[i] = map[labels[i]];
    return k;
}

size_t relabel_by_first_appearance(uint32_t* labels, size_t len, std::vector<uint32_t>& map) {  // :1283-1295
    reset(map, len, UINT32_MAX);
    uint32_t k = 0;
    for (size_t i = 0; i < len; ++i) {
        uint32_t& x = map[labels[i]];
        if (x == UINT32_MAX) x = k++;
        labels[i] = x;
    }
    return k;
}

struct MoveBufs {
    std::vector<double> cw, ewc;
    std::vector<uint32_t> count, unused, order, cand;
    std::vector<char> stable;
};

struct RefineScratch {
    std::vector<double> cw, ext, ewc, gain, w_to, cum;
    std::vector<char> single;
    std::vector<uint32_t> cand, perm, map;
};

struct Level {
    Csr g;
    std::vector<double> nw;
};

struct Workspace {
    std::vector<uint32_t> clu, next_clu, node_of, map;
    MoveBufs moving;
    Groups refine_groups, agg_groups;
    std::vector<uint32_t> pos, local, refined, counts;
    RefineScratch scratch;
    std::vector<double> acc;
    std::vector<uint32_t> touched;
};

// leiden.rs:759-857 — fast local moving. Returns (moved, nc).
std::pair<bool, size_t> move_nodes(const Csr& g, const double* nw, double gamma, std::vector<uint32_t>& clu,
                                   Rng& rng, MoveBufs& b, std::vector<uint32_t>& map) {
    size_t n = g.n();
    if (n <= 1) return {false, n};
    reset(b.cw, n, 0.0);
    reset(b.count, n, 0u);
    for (size_t v = 0; v < n; ++v) {
        b.cw[clu[v]] += nw[v];
        b.count[clu[v]] += 1;
    }
    b.unused.clear();
    for (size_t c = n; c-- > 0;)
        if (b.count[c] == 0) b.unused.push_back((uint32_t)c);
    b.order.resize(n);
    for (size_t v = 0; v < n; ++v) b.order[v] = (uint32_t)v;
    rng.shuffle(b.order);
    reset(b.ewc, n, 0.0);
    b.cand.clear();
    reset(b.stable, n, (char)0);
    size_t n_unstable = n, i = 0;
    bool moved = false;
    for (;;) {
        size_t v = b.order[i];
        size_t cur = clu[v];
        double kv = nw[v];
        b.cw[cur] -= kv;
        b.count[cur] -= 1;
        if (b.count[cur] == 0) {
            b.cw[cur] = 0.0;
            b.unused.push_back((uint32_t)cur);
        }
        b.cand.clear();
        b.cand.push_back(b.unused.back());
        size_t e0 = g.indptr[v], e1 = g.indptr[v + 1];
        for (size_t e = e0; e < e1; ++e) {
            size_t l = clu[g.nbr[e]];
            if (b.ewc[l] == 0.0) b.cand.push_back((uint32_t)l);
            b.ewc[l] += g.w[e];
        }
        size_t best = cur;
        double best_gain = b.ewc[cur] - kv * b.cw[cur] * gamma;
        for (uint32_t lc : b.cand) {
            size_t l = lc;
            double gain = b.ewc[l] - kv * b.cw[l] * gamma;
            if (gain > best_gain) {
                best = l;
                best_gain = gain;
            }
            b.ewc[l] = 0.0;
        }
        b.cw[best] += kv;
        b.count[best] += 1;
        if (!b.unused.empty() && b.unused.back() == (uint32_t)best) b.unused.pop_back();
        b.stable[v] = 1;
        n_unstable -= 1;
        if (best != cur) {
            clu[v] = (uint32_t)best;
            moved = true;
            for (size_t e = e0; e < e1; ++e) {
                size_t u = g.nbr[e];
                if (b.stable[u] && clu[u] != best) {
                    b.stable[u] = 0;
                    n_unstable += 1;
                    size_t p = i + n_unstable;
                    b.order[p < n ? p : p - n] = (uint32_t)u;
                }
            }
        }
        if (n_unstable == 0) break;
        i = i + 1 < n ? i + 1 : 0;
    }
    size_t nc = compact(clu.data(), n, n, map);
    return {moved, nc};
}

// leiden.rs:964-1089 — refine one cluster; `out` holds the sub-cluster of each of its nodes.
uint32_t refine_cluster(const Csr& g, const double* nw, double gamma, double beta, const std::vector<uint32_t>& clu,
                        const std::vector<uint32_t>& pos, uint32_t id, const uint32_t* nodes, size_t m,
                        const uint64_t stream[4], uint32_t* out, RefineScratch& s) {
    for (size_t i = 0; i < m; ++i) out[i] = (uint32_t)i;
    if (m == 1) return 1;
    s.cw.resize(m);
    s.ext.resize(m);
    for (size_t i = 0; i < m; ++i) {
        size_t v = nodes[i];
        s.cw[i] = nw[v];
        double acc = 0.0;
        for (size_t e = g.indptr[v]; e < g.indptr[v + 1]; ++e)
            if (clu[g.nbr[e]] == id) acc += g.w[e];
        s.ext[i] = acc;
    }
    double total = sum(s.cw);
    reset(s.single, m, (char)1);
    reset(s.ewc, m, 0.0);
    s.perm.resize(m);
    for (size_t i = 0; i < m; ++i) s.perm[i] = (uint32_t)i;
    Rng rng(stream, 4);
    rng.shuffle(s.perm);
    bool merged = false;
    for (size_t idx = 0; idx < m; ++idx) {
        size_t i = s.perm[idx];
        if (!s.single[i] || s.ext[i] < s.cw[i] * (total - s.cw[i]) * gamma) continue;
        size_t vi = nodes[i];
        double kv = nw[vi];
        double e_v = s.ext[i];
        s.cw[i] = 0.0;
        s.ext[i] = 0.0;
        s.cand.clear();
        s.cand.push_back((uint32_t)i);
        for (size_t e = g.indptr[vi]; e < g.indptr[vi + 1]; ++e) {
            size_t u = g.nbr[e];
            if (clu[u] != id) continue;
            size_t l = out[pos[u]];
            if (s.ewc[l] == 0.0) s.cand.push_back((uint32_t)l);
            s.ewc[l] += g.w[e];
        }
        s.gain.clear();
        s.w_to.clear();
        double max_gain = -std::numeric_limits<double>::infinity();
        size_t n_ok = 0, last_ok = 0;
        for (size_t j = 0; j < s.cand.size(); ++j) {
            size_t l = s.cand[j];
            double gain = -std::numeric_limits<double>::infinity();
            if (s.ext[l] >= s.cw[l] * (total - s.cw[l]) * gamma) {
                double dd = s.ewc[l] - kv * s.cw[l] * gamma;
                if (dd >= 0.0) {
                    gain = dd;
                    n_ok += 1;
                    last_ok = j;
                }
            }
            max_gain = std::fmax(max_gain, gain);
            s.gain.push_back(gain);
            s.w_to.push_back(s.ewc[l]);
            s.ewc[l] = 0.0;
        }
        size_t pick;
        if (n_ok == 1) {
            pick = last_ok;
        } else {
            s.cum.clear();
            double acc = 0.0;
            for (double gn : s.gain) {
                if (gn > -std::numeric_limits<double>::infinity()) acc += exp_nonpositive((gn - max_gain) / beta);
                s.cum.push_back(acc);
            }
            double r = acc * rng.unif();
            size_t j = (size_t)(std::upper_bound(s.cum.begin(), s.cum.end(), r) - s.cum.begin());
            pick = j < s.cand.size() ? j : last_ok;
        }
        size_t chosen = s.cand[pick];
        s.cw[chosen] += kv;
        s.ext[chosen] += e_v - 2.0 * s.w_to[pick];
        if (chosen != i) {
            out[i] = (uint32_t)chosen;
            s.single[chosen] = 0;
            merged = true;
        }
    }
    return merged ? (uint32_t)compact(out, m, m, s.map) : (uint32_t)m;
}

// leiden.rs:867-941 — refinement of every cluster; the refined partition goes to ws.refined.
size_t refine(const Csr& g, const double* nw, double gamma, double beta, const std::vector<uint32_t>& clu,
              size_t nc, const uint64_t stream[3], Workspace& ws) {
    size_t n = g.n();
    group_by(clu, nc, ws.refine_groups);
    const auto& start = ws.refine_groups.start;
    const auto& order = ws.refine_groups.order;
    reset(ws.pos, n, 0u);
    for (size_t c = 0; c < nc; ++c)
        for (size_t j = start[c]; j < start[c + 1]; ++j) ws.pos[order[j]] = (uint32_t)(j - start[c]);
    reset(ws.local, n, 0u);
    ws.counts.resize(nc);
    for (size_t c = 0; c < nc; ++c) {
        uint64_t st[4] = {stream[0], stream[1], stream[2], (uint64_t)c};
        ws.counts[c] = refine_cluster(g, nw, gamma, beta, clu, ws.pos, (uint32_t)c, &order[start[c]],
                                      start[c + 1] - start[c], st, &ws.local[start[c]], ws.scratch);
    }
    size_t nr = 0;
    for (auto& k : ws.counts) {
        size_t here = k;
        k = (uint32_t)nr;
        nr += here;
    }
    ws.refined.resize(n);
    for (size_t v = 0; v < n; ++v) {
        size_t c = clu[v];
        ws.refined[v] = ws.counts[c] + ws.local[start[c] + ws.pos[v]];
    }
    return nr;
}

// leiden.rs:1095-1243 — aggregate graph of `labels`: summed edge weights between labels, weight
// inside a label dropped, rows in ascending neighbour order.
void aggregate(const Csr& g, const double* nw, const std::vector<uint32_t>& labels, size_t nl, Workspace& ws,
               Level& out) {
    group_by(labels, nl, ws.agg_groups);
    const auto& start = ws.agg_groups.start;
    const auto& order = ws.agg_groups.order;
    out.nw.resize(nl);
    for (size_t r = 0; r < nl; ++r) {
        double s = 0.0;
        for (size_t j = start[r]; j < start[r + 1]; ++j) s += nw[order[j]];
        out.nw[r] = s;
    }
    Csr& csr = out.g;
    csr.indptr_s.assign(1, 0);
    csr.nbr_s.clear();
    csr.w_s.clear();
    reset(ws.acc, nl, 0.0);
    ws.touched.clear();
    for (size_t r = 0; r < nl; ++r) {
        for (size_t j = start[r]; j < start[r + 1]; ++j) {
            size_t v = order[j];
            for (size_t e = g.indptr[v]; e < g.indptr[v + 1]; ++e) {
                uint32_t q = labels[g.nbr[e]];
                if (q != r) {
                    if (ws.acc[q] == 0.0) ws.touched.push_back(q);
                    ws.acc[q] += g.w[e];
                }
            }
        }
        std::sort(ws.touched.begin(), ws.touched.end());
        for (uint32_t q : ws.touched) {
            csr.nbr_s.push_back(q);
            csr.w_s.push_back(ws.acc[q]);
            ws.acc[q] = 0.0;
        }
        ws.touched.clear();
        csr.indptr_s.push_back(csr.nbr_s.size());
    }
    csr.bind();
}

// leiden.rs:648-751 — one iteration on the original graph; returns whether any node moved.
bool one_iteration(const Csr& g0, const double* nw0, double gamma, double beta, uint32_t* clu0,
                   const uint64_t stream[2], Workspace& ws) {
    size_t n0 = g0.n();
    ws.clu.assign(clu0, clu0 + n0);
    Level levels[2];
    int cur_level = -1;  // which of `levels` holds the current aggregate graph, -1 = the original
    bool aggregated = false, moved = false;
    for (uint64_t level = 0;; ++level) {
        const Csr& g = cur_level < 0 ? g0 : levels[cur_level].g;
        const double* nw = cur_level < 0 ? nw0 : levels[cur_level].nw.data();
        Rng rng({stream[0], stream[1], level, 0});
        auto mv = move_nodes(g, nw, gamma, ws.clu, rng, ws.moving, ws.map);
        moved |= mv.first;
        size_t nc = mv.second;
        if (nc == g.n()) break;
        uint64_t stream3[3] = {stream[0], stream[1], level};
        size_t nr = refine(g, nw, gamma, beta, ws.clu, nc, stream3, ws);
        bool refined = nr < g.n();
        const std::vector<uint32_t>& labels = refined ? ws.refined : ws.clu;
        size_t n_labels = refined ? nr : nc;
        int next = cur_level == 0 ? 1 : 0;
        aggregate(g, nw, labels, n_labels, ws, levels[next]);
        if (aggregated) {
            for (auto& x : ws.node_of) x = labels[x];
        } else {
            ws.node_of.assign(labels.begin(), labels.end());
            aggregated = true;
        }
        if (refined) {
            reset(ws.next_clu, nr, 0u);
            for (size_t v = 0; v < ws.refined.size(); ++v) ws.next_clu[ws.refined[v]] = ws.clu[v];
        } else {
            ws.next_clu.resize(nc);
            for (size_t c = 0; c < nc; ++c) ws.next_clu[c] = (uint32_t)c;
        }
        std::swap(ws.clu, ws.next_clu);
        cur_level = next;
    }
    if (aggregated) {
        for (size_t v = 0; v < n0; ++v) clu0[v] = ws.clu[ws.node_of[v]];
    } else {
        std::copy(ws.clu.begin(), ws.clu.end(), clu0);
    }
    return moved;
}

bool check_params(int objective, double resolution, double beta, int32_t n_iterations, std::string& err) {
    (void)objective;
    if (!(std::isfinite(resolution) && resolution >= 0.0)) {  // leiden.rs:486-500
        err = "resolution must be finite and \xE2\x89\xA5 0, got " + fmt_f64(resolution);
        return false;
    }
    if (!(std::isfinite(beta) && beta > 0.0)) {
        err = "beta must be finite and > 0, got " + fmt_f64(beta);
        return false;
    }
    if (n_iterations == 0) {
        err = "n_iterations must be positive, or negative to run until stable";
        return false;
    }
    return true;
}

bool check_labels(const uint32_t* labels, size_t len, size_t n, std::string& err) {  // leiden.rs:476-484
    if (len != n) {
        err = std::to_string(len) + " labels for " + std::to_string(n) + " nodes";
        return false;
    }
    for (size_t i = 0; i < len; ++i)
        if (labels[i] >= n) {
            err = "label " + std::to_string(labels[i]) + " is not below the node count " + std::to_string(n);
            return false;
        }
    return true;
}

constexpr size_t MAX_ITERATIONS = 1000;  // leiden.rs:263

// leiden.rs:514-563 — one run into `clu`; returns false with `err` on bad parameters.
bool run(const Csr& g, const std::vector<double>& nw, int objective, double resolution, double beta,
         int32_t n_iterations, uint64_t seed, const uint32_t* initial, Workspace& ws, uint32_t* clu,
         uint64_t* n_clusters, uint64_t* iterations_out, int* converged_out, std::string& err) {
    if (!check_params(objective, resolution, beta, n_iterations, err)) return false;
    size_t n = g.n();
    if (initial) {
        if (!check_labels(initial, n, n, err)) return false;
        std::copy(initial, initial + n, clu);
    } else {
        for (size_t v = 0; v < n; ++v) clu[v] = (uint32_t)v;
    }
    double total = sum(nw);
    uint64_t iterations = 0;
    bool converged = true;
    if (total > 0.0) {
        double gamma = objective == 0 ? resolution / total : resolution;
        size_t max_it = n_iterations > 0 ? (size_t)n_iterations : MAX_ITERATIONS;
        for (size_t it = 0; it < max_it; ++it) {
            uint64_t stream[2] = {seed, (uint64_t)it};
            bool moved = one_iteration(g, nw.data(), gamma, beta, clu, stream, ws);
            iterations += 1;
            converged = !moved;
            if (n_iterations < 0 && converged) break;
        }
    }
    *n_clusters = relabel_by_first_appearance(clu, n, ws.map);
    *iterations_out = iterations;
    *converged_out = converged ? 1 : 0;
    return true;
}

std::vector<double> node_weights(const Csr& g, int objective) {  // leiden.rs:282-287
    if (objective == 0) return strengths(g);
    return std::vector<double>(g.n(), 1.0);
}

// leiden.rs:452-474
double modularity(const Csr& g, const uint32_t* membership, double resolution) {
    size_t n = g.n();
    std::vector<double> nw = strengths(g);
    double total = sum(nw);
    if (total == 0.0) return 0.0;
    std::vector<double> k_c(n, 0.0);
    double internal = 0.0;
    for (size_t v = 0; v < n; ++v) {
        uint32_t c = membership[v];
        k_c[c] += nw[v];
        for (size_t e = g.indptr[v]; e < g.indptr[v + 1]; ++e)
            if (membership[g.nbr[e]] == c) internal += g.w[e];
    }
    double null = 0.0;
    for (double k : k_c) null += k * k;
    return internal / total - resolution * null / (total * total);
}

// leiden.rs:422-449
double quality(const Csr& g, const uint32_t* membership, int objective, double resolution) {
    if (objective == 0) return modularity(g, membership, resolution);
    size_t n = g.n();
    std::vector<double> size(n, 0.0);
    double internal = 0.0;
    for (size_t v = 0; v < n; ++v) {
        uint32_t c = membership[v];
        size[c] += 1.0;
        for (size_t e = g.indptr[v]; e < g.indptr[v + 1]; ++e)
            if (membership[g.nbr[e]] == c) internal += g.w[e];
    }
    double pairs = 0.0;
    for (double s : size) pairs += s * (s - 1.0);
    return internal - resolution * pairs;
}

void put_err(char* err, size_t errlen, const std::string& msg) {
    if (err && errlen) std::snprintf(err, errlen, "%s", msg.c_str());
}

}  // namespace

extern "C" {

int costal_leiden(uint64_t n, const uint32_t* rows, const uint32_t* cols, const double* weights, uint64_t m,
                  int objective, int from_coo, double resolution, double beta, int32_t n_iterations,
                  uint64_t seed, const uint32_t* initial, uint32_t* membership, uint64_t* n_clusters,
                  uint64_t* iterations, int* converged, double* quality_out, char* err, size_t errlen) {
    std::string e;
    Csr g;
    bool ok = from_coo ? csr_from_coo(n, rows, cols, weights, m, g, e) : csr_from_edges(n, rows, cols, weights, m, g, e);
    if (!ok) {
        put_err(err, errlen, e);
        return COSTAL_EINVAL;
    }
    Workspace ws;
    if (!run(g, node_weights(g, objective), objective, resolution, beta, n_iterations, seed, initial, ws, membership,
             n_clusters, iterations, converged, e)) {
        put_err(err, errlen, e);
        return COSTAL_EINVAL;
    }
    if (quality_out) *quality_out = quality(g, membership, objective, resolution);
    return COSTAL_OK;
}

int costal_leiden_csr(uint64_t n, const uint64_t* indptr, const uint32_t* nbr, const double* weights, int objective,
                      double resolution, double beta, int32_t n_iterations, uint64_t seed, const uint32_t* initial,
                      uint32_t* membership, uint64_t* n_clusters, uint64_t* iterations, int* converged,
                      double* quality_out, char* err, size_t errlen) {
    std::string e;
    Csr g;
    if (!csr_view(n, indptr, nbr, weights, g, e)) {
        put_err(err, errlen, e);
        return COSTAL_EINVAL;
    }
    Workspace ws;
    if (!run(g, node_weights(g, objective), objective, resolution, beta, n_iterations, seed, initial, ws, membership,
             n_clusters, iterations, converged, e)) {
        put_err(err, errlen, e);
        return COSTAL_EINVAL;
    }
    if (quality_out) *quality_out = quality(g, membership, objective, resolution);
    return COSTAL_OK;
}

namespace {
// lib.rs:311-350: every (resolution, seed) run on one graph, resolutions outer; runs in parallel,
// each deterministic.
int many_runs(const Csr& g, uint64_t n, const double* resolutions, uint64_t n_resolutions, const uint64_t* seeds,
              uint64_t n_seeds, double beta, int32_t n_iterations, int n_threads, uint32_t* out, char* err,
              size_t errlen) {
    std::string e;
    size_t runs = (size_t)n_resolutions * n_seeds;
    for (size_t r = 0; r < n_resolutions; ++r)
        if (!check_params(0, resolutions[r], beta, n_iterations, e)) {
            put_err(err, errlen, e);
            return COSTAL_EINVAL;
        }
    if (runs == 0 || n == 0) return COSTAL_OK;
    std::vector<double> nw = strengths(g);
    int threads = n_threads > 0 ? n_threads : 0;
    (void)threads;
#pragma omp parallel num_threads(threads > 0 ? threads : omp_get_max_threads())
    {
        Workspace ws;
#pragma omp for schedule(dynamic, 1)
        for (long long i = 0; i < (long long)runs; ++i) {
            size_t r = (size_t)i / n_seeds, s = (size_t)i % n_seeds;
            uint64_t nc, it;
            int conv;
            std::string local;
            run(g, nw, 0, resolutions[r], beta, n_iterations, seeds[s], nullptr, ws, out + (size_t)i * n, &nc, &it,
                &conv, local);
        }
    }
    return COSTAL_OK;
}
}  // namespace

int costal_leiden_many(uint64_t n, const uint32_t* rows, const uint32_t* cols, const double* weights, uint64_t m,
                       const double* resolutions, uint64_t n_resolutions, const uint64_t* seeds, uint64_t n_seeds,
                       double beta, int32_t n_iterations, int n_threads, uint32_t* out, char* err, size_t errlen) {
    std::string e;
    Csr g;
    if (!csr_from_edges(n, rows, cols, weights, m, g, e)) {
        put_err(err, errlen, e);
        return COSTAL_EINVAL;
    }
    return many_runs(g, n, resolutions, n_resolutions, seeds, n_seeds, beta, n_iterations, n_threads, out, err, errlen);
}

int costal_leiden_many_csr(uint64_t n, const uint64_t* indptr, const uint32_t* nbr, const double* weights,
                           const double* resolutions, uint64_t n_resolutions, const uint64_t* seeds, uint64_t n_seeds,
                           double beta, int32_t n_iterations, int n_threads, uint32_t* out, char* err, size_t errlen) {
    std::string e;
    Csr g;
    if (!csr_view(n, indptr, nbr, weights, g, e)) {
        put_err(err, errlen, e);
        return COSTAL_EINVAL;
    }
    return many_runs(g, n, resolutions, n_resolutions, seeds, n_seeds, beta, n_iterations, n_threads, out, err, errlen);
}

int costal_modularity(uint64_t n, const uint32_t* rows, const uint32_t* cols, const double* weights, uint64_t m,
                      const uint32_t* membership, double resolution, double* q, char* err, size_t errlen) {
    std::string e;
    Csr g;
    if (!csr_from_edges(n, rows, cols, weights, m, g, e) || !check_labels(membership, n, n, e)) {
        put_err(err, errlen, e);
        return COSTAL_EINVAL;
    }
    *q = modularity(g, membership, resolution);
    return COSTAL_OK;
}

}  // extern "C"
