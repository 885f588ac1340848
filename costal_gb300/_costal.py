"""Drop-in replacement of CosTaL 2.1.0's `costal._costal` extension module, on a GB300.

Same functions, signatures, return types and error behaviour as the PyO3 module of
crates/costal-py/src/lib.rs:80-465; the reference's pure-Python package (`costal._api`,
`costal._leiden`) runs unchanged on top of it. Only type
conversion and error mapping live here — as in lib.rs — and every computation is a call into
libcostal_gb300.so: the kNN graph on the GPU, Leiden (the host consumer) in host C++.

Differences from the reference, all documented:
  - `matmul` names a coarse-pass backend of this library: "fp32" (default; "gemm" is accepted as
    its alias), "bf16" (certified tcgen05 tiles: split BF16, or split FP8 e4m3 for d >= 512),
    "bf16x3" (split BF16 at every depth) or "fp8" (split FP8 wherever the query tile is streamed,
    3d > 128). Like the reference's backends they change speed only, never the output.
    "accelerate" is Apple-only and unavailable here, as it is for the reference on Linux.
  - `row_block`, `col_block`, `sort_by_norm` and `n_threads` are accepted and validated but do not
    change the GPU tiling (the reference: they change speed only, knn.rs:39-44). `prune` (speed
    only, as in the reference) switches the exact early stop of the bf16 backend's block lists.
  - The GPU keeps at most 128 candidates a row: k + margin above 128 runs with margin 128 − k, and
    k ≥ 128 with the exact f64 scan of every candidate (the output is the same; the margin in effect
    is reported in the stats).
  - The backend used when a caller passes no `matmul` (as costal.knn and costal.find_communities of the
    reference package never do) is DEFAULT_MATMUL: "fp32" unless the environment variable
    COSTAL_GB300_MATMUL names another backend when this module is imported. Setting it to "bf16" moves
    an unchanged caller onto the certified tensor-core path; the output stays the same bits.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L

__version__ = "2.1.0"

NOT_CONTIGUOUS = "input must be a C-contiguous array; call np.ascontiguousarray first"  # lib.rs:35


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _arr(a, dtype, ndim, name="input"):
    """PyReadonlyArray<T> extraction: exact dtype, C-contiguous (lib.rs:35, 68)."""
    if not isinstance(a, np.ndarray):
        raise TypeError(f"{name} must be a numpy.ndarray of {np.dtype(dtype).name}")
    if a.dtype != np.dtype(dtype):
        raise TypeError(f"{name} must have dtype {np.dtype(dtype).name}, got {a.dtype}")
    if a.ndim != ndim:
        raise TypeError(f"{name} must be {ndim}-dimensional, got {a.ndim}")
    if not a.flags.c_contiguous:
        raise ValueError(NOT_CONTIGUOUS)
    return a


def _call(fn, *args):
    err, size = L.errbuf()
    rc = fn(*args, err, size)
    L.check(rc, err)


def hello() -> str:
    """crates/costal-core/src/lib.rs:23-25."""
    return f"CosTaL core v{core_version()} is alive"


def core_version() -> str:
    return L.lib().costal_version().decode()


def row_l2_norms(x):
    """lib.rs:92-102: (n, d) float32 -> (n,) float32 row norms, on the GPU."""
    x = _arr(x, np.float32, 2, "x")
    n, d = x.shape
    out = np.empty(n, np.float32)
    _call(L.lib().costal_row_l2_norms, _ptr(x), n, d, _ptr(out))
    return out


_SELECT_NAMES = ("cosine", "tanimoto")
_BACKENDS = {"fp32": L.BACKEND_FP32, "gemm": L.BACKEND_FP32, "bf16": L.BACKEND_BF16, "bf16x3": L.BACKEND_BF16X3,
             "fp8": L.BACKEND_FP8}

DEFAULT_MATMUL = os.environ.get("COSTAL_GB300_MATMUL", "fp32")
if DEFAULT_MATMUL not in _BACKENDS:
    raise ImportError(f'COSTAL_GB300_MATMUL="{DEFAULT_MATMUL}" is not a backend of this library ({", ".join(_BACKENDS)})')


def _backend(matmul):
    """The backend name a call runs on: its `matmul`, or DEFAULT_MATMUL when it names none."""
    name = DEFAULT_MATMUL if matmul is None else matmul
    if name == "accelerate":
        raise ValueError("matmul backend accelerate is not available on this platform")  # knn.rs:120-122
    if name not in _BACKENDS:
        raise ValueError(f'unknown matmul backend "{name}"')
    return name


def _parse_select(select):
    if select is None:
        return "cosine"
    if select not in _SELECT_NAMES:
        raise ValueError(f'unknown select "{select}"')  # lib.rs:104-111
    return select


def _opts(select, margin, row_block, col_block, backend, sort_by_norm, prune, learned_prune=False):
    o = L.KnnOpts()
    o.margin = 0xFFFFFFFF if margin is None else int(margin)
    o.select = L.SELECT[select]
    o.backend = backend
    o.row_block = int(row_block or 0)
    o.col_block = int(col_block or 0)
    o.sort_by_norm = int(bool(sort_by_norm))
    o.prune = int(bool(prune))
    o.learned_prune = int(bool(learned_prune))
    return o


def _check_knob(name, v):
    if v is not None and int(v) < 0:
        raise OverflowError(f"can't convert negative int to unsigned ({name})")


def _knn_exact(x, k, *, select=None, margin=None, row_block=None, col_block=None, matmul=None, sort_by_norm=True,
               prune=True, n_threads=None, learned_prune=False):
    """lib.rs:113-167: exact kNN. Returns ((idx int32 (n,k), cos float64 (n,k), norms float64 (n,)), stats).

    GB300 addition: with matmul="bf16" and learned_prune=True, a model trained by _mlp_train on this
    data skips column blocks whose bound is below its prediction (every skip is certified).
    """
    x = _arr(x, np.float32, 2, "x")
    n, d = x.shape
    if n > np.iinfo(np.int32).max:
        raise ValueError(f"n={n} exceeds the int32 index range")
    matmul = _backend(matmul)
    for name, v in (("k", k), ("margin", margin), ("row_block", row_block), ("col_block", col_block),
                    ("n_threads", n_threads)):
        _check_knob(name, v)
    sel = _parse_select(select)
    k = int(k)
    idx = np.empty((n, k), np.uint32)
    cos = np.empty((n, k), np.float64)
    norms = np.empty(n, np.float64)
    st = L.KnnStats()
    o = _opts(sel, margin, row_block, col_block, _BACKENDS[matmul], sort_by_norm, prune, learned_prune)
    _call(L.lib().costal_knn_exact, _ptr(x), n, d, k, C.byref(o), _ptr(idx), _ptr(cos), _ptr(norms), C.byref(st))
    stats = {
        "fallback_rows": int(st.fallback_rows),
        "row_block": int(st.row_block),
        "col_block": int(st.col_block),
        "matmul": matmul,
        "margin": int(st.margin),
        "select": sel,
        "blocks_skipped": int(st.blocks_skipped),
        "blocks_total": int(st.blocks_total),
        # GB300-only counters
        "recomputed_rows": int(st.recomputed_rows),
        "pruned_fallback_rows": int(st.pruned_fallback_rows),
        "max_coarse_err": float(st.max_coarse_err),
        "max_err_ratio": float(st.max_err_ratio),
        "coarse_kind": L.COARSE_KINDS[int(st.coarse_kind)],
        "blocks_stopped": int(st.blocks_stopped),
        "ms_order": float(st.ms_order),
        "ms_coarse": float(st.ms_coarse),
        "ms_total": float(st.ms_total),
    }
    return (idx.view(np.int32), cos, norms), stats


def _knn_bruteforce(x, k, *, select=None, n_threads=None):
    """lib.rs:169-191: every candidate in f64, no blocking (tests and benchmarks only)."""
    x = _arr(x, np.float32, 2, "x")
    n, d = x.shape
    _check_knob("k", k)
    sel = _parse_select(select)
    k = int(k)
    idx = np.empty((n, k), np.uint32)
    cos = np.empty((n, k), np.float64)
    norms = np.empty(n, np.float64)
    _call(L.lib().costal_knn_bruteforce, _ptr(x), n, d, k, L.SELECT[sel], _ptr(idx), _ptr(cos), _ptr(norms))
    return idx.view(np.int32), cos, norms


def _weight_code(weight):
    if weight not in L.WEIGHT:
        raise ValueError(f'unknown edge weight "{weight}"')  # lib.rs:202-203
    return L.WEIGHT[weight]


def _reweight(idx, cos, norms, weight):
    """lib.rs:193-214: edge weights ("tanimoto" / "cosine" / "jaccard") on a kNN."""
    w = _weight_code(weight)
    idx = _arr(idx, np.int32, 2, "idx")
    cos = _arr(cos, np.float64, 2, "cos")
    norms = _arr(norms, np.float64, 1, "norms")
    n, k = idx.shape
    if cos.shape != (n, k) or norms.shape[0] != n:
        raise ValueError("shapes of idx, cos and norms do not match")
    out = np.empty((n, k), np.float64)
    _call(L.lib().costal_reweight, n, k, _ptr(idx), _ptr(cos), _ptr(norms), w, _ptr(out))
    return out


def _fuzzy_union(idx, w):
    """lib.rs:216-239: fuzzy-union symmetrisation -> upper-triangular (rows, cols, weights)."""
    idx = _arr(idx, np.int32, 2, "idx")
    w = _arr(w, np.float64, 2, "w")
    n, k = idx.shape
    if w.shape != (n, k):
        raise ValueError("shapes of idx and w do not match")
    rows = np.empty(n * k, np.int32)
    cols = np.empty(n * k, np.int32)
    wout = np.empty(n * k, np.float64)
    m = C.c_uint64(0)
    _call(L.lib().costal_fuzzy_union, n, k, _ptr(idx), _ptr(w), _ptr(rows), _ptr(cols), _ptr(wout), C.byref(m))
    m = m.value
    return rows[:m].copy(), cols[:m].copy(), wout[:m].copy()


def _build_graph(x, k, *, weight="tanimoto", margin=None, matmul=None, return_knn=False, learned_prune=False):
    """GB300 addition: the fused X -> kNN -> weights -> fuzzy union of _api.py:460-462 on the device.

    Returns (rows int32, cols int32, weights float64), plus (idx, cos, norms) and stats when
    return_knn is true. Bit-identical to calling _knn_exact, _reweight and _fuzzy_union in turn.
    """
    x = _arr(x, np.float32, 2, "x")
    n, d = x.shape
    wc = _weight_code(weight)
    matmul = _backend(matmul)
    k = int(k)
    rows = np.empty(n * k, np.int32)
    cols = np.empty(n * k, np.int32)
    wout = np.empty(n * k, np.float64)
    m = C.c_uint64(0)
    idx = cos = norms = None
    if return_knn:
        idx = np.empty((n, k), np.uint32)
        cos = np.empty((n, k), np.float64)
        norms = np.empty(n, np.float64)
    st = L.KnnStats()
    o = _opts("cosine", margin, None, None, _BACKENDS[matmul], True, True, learned_prune)
    _call(L.lib().costal_build_graph, _ptr(x), n, d, k, C.byref(o), wc, _ptr(rows), _ptr(cols), _ptr(wout),
          C.byref(m), _ptr(idx), _ptr(cos), _ptr(norms), C.byref(st))
    m = m.value
    edges = (rows[:m].copy(), cols[:m].copy(), wout[:m].copy())
    if return_knn:
        return edges, (idx.view(np.int32), cos, norms), st.as_dict()
    return edges


def _build_graph_csr(x, k, *, weight="tanimoto", margin=None, matmul=None, learned_prune=False):
    """GB300 addition: the fused X -> kNN -> weights -> fuzzy union, handed back as the Leiden's CSR
    (leiden.rs:52-101 `Csr::from_edges` of the edge list _build_graph returns), built on the device.

    Returns (indptr uint64[n + 1], nbr uint32[nnz], weights float64[nnz]) for _leiden_csr."""
    x = _arr(x, np.float32, 2, "x")
    n, d = x.shape
    wc = _weight_code(weight)
    matmul = _backend(matmul)
    k = int(k)
    indptr = np.empty(n + 1, np.uint64)
    nbr = np.empty(2 * n * k, np.uint32)
    w = np.empty(2 * n * k, np.float64)
    nnz = C.c_uint64(0)
    st = L.KnnStats()
    o = _opts("cosine", margin, None, None, _BACKENDS[matmul], True, True, learned_prune)
    _call(L.lib().costal_build_graph_csr, _ptr(x), n, d, k, C.byref(o), wc, _ptr(indptr), _ptr(nbr), _ptr(w),
          C.byref(nnz), C.byref(st))
    nnz = nnz.value
    return indptr, nbr[:nnz].copy(), w[:nnz].copy()


def _leiden_csr(n, indptr, nbr, weights, *, resolution, beta=0.01, n_iterations=2, seed=0, n_threads=None):
    """GB300 addition: _leiden on a graph given as the CSR _build_graph_csr returns, used in place.

    Returns (membership int32, n_clusters, iterations, converged), the same as _leiden on the edge
    list the CSR was built from."""
    n = _u64(n, "n")
    indptr = _arr(indptr, np.uint64, 1, "indptr")
    nbr = _arr(nbr, np.uint32, 1, "nbr")
    w = _arr(weights, np.float64, 1, "weights")
    if len(indptr) != n + 1:
        raise ValueError(f"indptr has {len(indptr)} entries for n={n}")
    if int(indptr[-1]) != len(nbr) or len(nbr) != len(w):
        raise ValueError(f"indptr ends at {int(indptr[-1])} but there are {len(nbr)} neighbours and {len(w)} weights")
    memb = np.empty(n, np.uint32)
    ncl, it, conv = C.c_uint64(), C.c_uint64(), C.c_int()
    _call(L.lib().costal_leiden_csr, n, _ptr(indptr), _ptr(nbr), _ptr(w), 0, float(resolution), float(beta),
          int(n_iterations), _u64(seed, "seed"), None, _ptr(memb), C.byref(ncl), C.byref(it), C.byref(conv), None)
    return memb.view(np.int32), int(ncl.value), int(it.value), bool(conv.value)


def _as_u32(a, name):
    """lib.rs:241-249: a non-negative int32 array viewed as u32."""
    a = _arr(a, np.int32, 1, name)
    if a.size and a.min() < 0:
        raise ValueError(f"negative index {int(a[a < 0][0])}")
    return a.view(np.uint32)


def _edges(rows, cols, weights):
    r = _as_u32(rows, "rows")
    c = _as_u32(cols, "cols")
    w = _arr(weights, np.float64, 1, "weights")
    if not (len(r) == len(c) == len(w)):
        raise ValueError(f"edge arrays differ in length: {len(r)} rows, {len(c)} cols, {len(w)} weights")
    return r, c, w


def _u64(v, name):
    v = int(v)
    if v < 0:
        raise OverflowError(f"can't convert negative int to unsigned ({name})")
    return v


def _leiden(n, rows, cols, weights, *, resolution, beta=0.01, n_iterations=2, seed=0, n_threads=None):
    """lib.rs:272-306: Leiden (modularity) on an upper-triangular edge list.

    Returns (membership int32, n_clusters, iterations, converged)."""
    n = _u64(n, "n")
    r, c, w = _edges(rows, cols, weights)
    memb = np.empty(n, np.uint32)
    ncl, it, conv = C.c_uint64(), C.c_uint64(), C.c_int()
    _call(L.lib().costal_leiden, n, _ptr(r), _ptr(c), _ptr(w), len(w), 0, 0, float(resolution), float(beta),
          int(n_iterations), _u64(seed, "seed"), None, _ptr(memb), C.byref(ncl), C.byref(it), C.byref(conv), None)
    return memb.view(np.int32), int(ncl.value), int(it.value), bool(conv.value)


def _leiden_many(n, rows, cols, weights, *, resolutions, seeds, beta=0.01, n_iterations=2, n_threads=None):
    """lib.rs:308-350: Leiden at every (resolution, seed), resolutions outer -> int32 (runs, n)."""
    n = _u64(n, "n")
    r, c, w = _edges(rows, cols, weights)
    res = np.ascontiguousarray([float(v) for v in resolutions], dtype=np.float64)
    sd = np.ascontiguousarray([_u64(v, "seed") for v in seeds], dtype=np.uint64)
    out = np.empty((len(res) * len(sd), n), np.uint32)
    _call(L.lib().costal_leiden_many, n, _ptr(r), _ptr(c), _ptr(w), len(w), _ptr(res), len(res), _ptr(sd), len(sd),
          float(beta), int(n_iterations), int(n_threads or 0), _ptr(out))
    return out.view(np.int32)


def _leiden_many_csr(n, indptr, nbr, weights, *, resolutions, seeds, beta=0.01, n_iterations=2, n_threads=None):
    """GB300 addition: _leiden_many on the CSR _build_graph_csr returns, used in place (the same labels
    as _leiden_many on the edge list the CSR was built from) -> int32 (runs, n)."""
    n = _u64(n, "n")
    indptr = _arr(indptr, np.uint64, 1, "indptr")
    nbr = _arr(nbr, np.uint32, 1, "nbr")
    w = _arr(weights, np.float64, 1, "weights")
    if len(indptr) != n + 1:
        raise ValueError(f"indptr has {len(indptr)} entries for n={n}")
    res = np.ascontiguousarray([float(v) for v in resolutions], dtype=np.float64)
    sd = np.ascontiguousarray([_u64(v, "seed") for v in seeds], dtype=np.uint64)
    out = np.empty((len(res) * len(sd), n), np.uint32)
    _call(L.lib().costal_leiden_many_csr, n, _ptr(indptr), _ptr(nbr), _ptr(w), _ptr(res), len(res), _ptr(sd), len(sd),
          float(beta), int(n_iterations), int(n_threads or 0), _ptr(out))
    return out.view(np.int32)


def _leiden_coo(n, rows, cols, weights, *, objective, resolution, beta, n_iterations, seed, initial=None,
                n_threads=None):
    """lib.rs:352-412: Leiden on an external COO list -> (labels int64, quality, n_clusters, iterations, converged)."""
    if objective not in ("modularity", "cpm"):
        raise ValueError(f"objective must be 'modularity' or 'cpm', got \"{objective}\"")
    n = _u64(n, "n")
    r = _arr(rows, np.uint32, 1, "rows")
    c = _arr(cols, np.uint32, 1, "cols")
    w = _arr(weights, np.float64, 1, "weights")
    if not (len(r) == len(c) == len(w)):
        raise ValueError(f"edge arrays differ in length: {len(r)} rows, {len(c)} cols, {len(w)} weights")
    init = None if initial is None else _arr(initial, np.uint32, 1, "initial")
    memb = np.empty(n, np.uint32)
    ncl, it, conv, q = C.c_uint64(), C.c_uint64(), C.c_int(), C.c_double()
    _call(L.lib().costal_leiden, n, _ptr(r), _ptr(c), _ptr(w), len(w), 0 if objective == "modularity" else 1, 1,
          float(resolution), float(beta), int(n_iterations), _u64(seed, "seed"), _ptr(init), _ptr(memb),
          C.byref(ncl), C.byref(it), C.byref(conv), C.byref(q))
    return memb.astype(np.int64), float(q.value), int(ncl.value), int(it.value), bool(conv.value)


def _modularity(n, rows, cols, weights, membership, resolution):
    """lib.rs:414-428."""
    n = _u64(n, "n")
    r, c, w = _edges(rows, cols, weights)
    m = _as_u32(membership, "membership")
    q = C.c_double()
    _call(L.lib().costal_modularity, n, _ptr(r), _ptr(c), _ptr(w), len(w), _ptr(m), float(resolution), C.byref(q))
    return float(q.value)


def l2_bytes_per_thread():
    """lib.rs:430-434: the reference's CPU cache probe. The GPU kernels do not size tiles from a CPU
    cache, so there is nothing to report (the reference also returns None when unavailable)."""
    return None


def tile_budget_bytes() -> int:
    """lib.rs:436-440: the reference's fallback tile budget (the GPU tiles are fixed at 128 x 128)."""
    return 1 << 20


def default_matmul() -> str:
    """lib.rs:442-446: name of the default coarse-pass backend (DEFAULT_MATMUL)."""
    return DEFAULT_MATMUL


# ---- the learned block-pruning model (GB300 addition; no counterpart in the reference) ----------

def _mlp_train(x, k, *, sample=200_000, epochs=30, batch=2048, lr=2e-3, quantile=0.05, margin=None, seed=20241203):
    """Train the k-th-neighbour-cosine model on x (labels from the plain FP32 path); it stays loaded.

    Returns the training stats (loss, mean absolute error, coverage = share of rows predicted at or
    below their exact k-th cosine, times)."""
    x = _arr(x, np.float32, 2, "x")
    n, d = x.shape
    o = L.MlpOpts()
    o.sample, o.epochs, o.batch = int(sample), int(epochs), int(batch)
    o.margin = 0xFFFFFFFF if margin is None else int(margin)
    o.lr, o.quantile, o.seed = float(lr), float(quantile), int(seed)
    st = L.MlpStats()
    _call(L.lib().costal_mlp_train, _ptr(x), n, d, int(k), C.byref(o), C.byref(st))
    return st.as_dict()


def _mlp_get():
    """The loaded model: (f32 master weights, d, k, quantile)."""
    cnt, d, k, q = C.c_uint64(), C.c_uint32(), C.c_uint32(), C.c_float()
    _call(L.lib().costal_mlp_get, None, 0, C.byref(cnt), C.byref(d), C.byref(k), C.byref(q))
    params = np.empty(cnt.value, np.float32)
    _call(L.lib().costal_mlp_get, _ptr(params), cnt.value, C.byref(cnt), C.byref(d), C.byref(k), C.byref(q))
    return params, int(d.value), int(k.value), float(q.value)


def _mlp_set(params, d, k, quantile=0.05):
    """Load a model (e.g. from a checkpoint, or a constant predictor for an ablation)."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    _call(L.lib().costal_mlp_set, _ptr(params), params.size, int(d), int(k), float(quantile))


def _mlp_clear():
    _call(L.lib().costal_mlp_clear)


def _mlp_forward(params, feat):
    """Test hook: the GPU inference pass (bf16 operands on the tensor cores, FP32 accumulation) for given
    weights and features (m, F)."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    feat = np.ascontiguousarray(feat, dtype=np.float32)
    m, F = feat.shape
    out = np.empty(m, np.float32)
    _call(L.lib().costal_mlp_forward, _ptr(params), F, _ptr(feat), m, _ptr(out))
    return out


def col_block_rows(n):
    """Rows of a column block of the tensor-core path's lists for n rows (prune.h col_block)."""
    return 128 if (n + 127) // 128 <= 8192 else 256


def _block_bounds(x):
    """Test hook: the tensor-core path's per-row block bound data for X (n, d), d <= 64.

    Returns (perm, ccenter, cradius, rowmax, delta): the working order (working -> original row),
    the unit centres (ncb, d) and angular radii (ncb,) of the column blocks (128 working rows while
    ceil(n / 128) <= 8,192, else 256), the largest split-BF16 coarse score of each query block's rows
    (blocks of 128) with each centre (nqb, ncb), and that score's error margin in cosine.
    """
    x = np.ascontiguousarray(x, dtype=np.float32)
    n, d = x.shape
    cb = col_block_rows(n)
    nqb, ncb = (n + 127) // 128, (n + cb - 1) // cb
    perm = np.empty(n, np.uint32)
    ccenter = np.empty((ncb, d), np.float64)
    cradius = np.empty(ncb, np.float64)
    rowmax = np.empty((nqb, ncb), np.float32)
    delta = C.c_float()
    _call(L.lib().costal_block_bounds, _ptr(x), n, d, _ptr(perm), _ptr(ccenter), _ptr(cradius), _ptr(rowmax),
          C.byref(delta))
    return perm, ccenter, cradius, rowmax, float(delta.value)


def _mlp_gradient(params, feat, y, quantile):
    """Test hook: the GPU gradient of the mean pinball loss for given weights, features and labels."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    feat = np.ascontiguousarray(feat, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    m, F = feat.shape
    grad = np.empty(params.size, np.float32)
    _call(L.lib().costal_mlp_gradient, _ptr(params), F, _ptr(feat), _ptr(y), m, float(quantile), _ptr(grad))
    return grad
