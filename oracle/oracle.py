"""TEST INFRASTRUCTURE ONLY — ctypes bindings of the CPU oracle (oracle/_build/libcostal_oracle.so).

Used by tests/, by __graft_entry__.smoke() as the checker, and by bench.py as the timed CPU baseline.
The product (costal_gb300/) never imports this module.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import build_oracle

_lib = None


class OracleStats(C.Structure):
    _fields_ = [(f, C.c_uint64) for f in ("fallback_rows", "row_block", "col_block", "blocks_skipped", "blocks_total")]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle()
        _lib = C.CDLL(str(path))
        P = C.c_void_p
        _lib.oracle_knn_exact.argtypes = [P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_uint32,
                                          C.c_uint32, C.c_int, C.c_int, C.c_int, P, P, P, P, C.c_char_p, C.c_size_t]
        _lib.oracle_knn_rows.argtypes = [P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint64,
                                         C.c_int, P, P, P, P, C.c_char_p, C.c_size_t]
        _lib.oracle_knn_bruteforce.argtypes = [P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int, C.c_int, P, P, P,
                                               C.c_char_p, C.c_size_t]
        _lib.oracle_reweight.argtypes = [C.c_uint64, C.c_uint32, P, P, P, C.c_int, P]
        _lib.oracle_fuzzy_union.argtypes = [C.c_uint64, C.c_uint32, P, P, P, P, P, P]
        _lib.oracle_tani_from_cos.argtypes = [C.c_double, C.c_double, C.c_double]
        _lib.oracle_tani_from_cos.restype = C.c_double
        _lib.oracle_row_l2_norms.argtypes = [P, C.c_uint64, C.c_uint32, P]
        _lib.oracle_max_threads.restype = C.c_int
        _lib.oracle_heap_keep.argtypes = [P, P, C.c_size_t, C.c_size_t, P]
        _lib.oracle_heap_keep.restype = C.c_size_t
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _f32(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    if x.ndim != 2:
        raise ValueError("x must be 2-D")
    return x


def max_threads() -> int:
    return lib().oracle_max_threads()


def knn_exact(x, k, *, margin=None, select="cosine", row_block=0, col_block=0, sort_by_norm=True, prune=True,
              n_threads=0):
    """knn.rs:365 knn_exact_with_stats, restated. Returns ((idx u32, cos f64, norms f64), stats)."""
    x = _f32(x)
    n, d = x.shape
    idx = np.empty((n, k), np.uint32)
    cos = np.empty((n, k), np.float64)
    norms = np.empty(n, np.float64)
    st = OracleStats()
    err = C.create_string_buffer(256)
    rc = lib().oracle_knn_exact(_ptr(x), n, d, k, k if margin is None else margin, 0 if select == "cosine" else 1,
                                row_block, col_block, int(sort_by_norm), int(prune), n_threads, _ptr(idx), _ptr(cos),
                                _ptr(norms), C.byref(st), err, 256)
    if rc:
        raise ValueError(err.value.decode())
    stats = {f: int(getattr(st, f)) for f, _ in OracleStats._fields_}
    return (idx, cos, norms), stats


def knn_rows(x, k, q0, q1, *, margin=None, n_threads=0):
    """The blocked cosine path for query rows [q0, q1) against all rows (the CPU-baseline sample)."""
    x = _f32(x)
    n, d = x.shape
    idx = np.empty((q1 - q0, k), np.uint32)
    cos = np.empty((q1 - q0, k), np.float64)
    norms = np.empty(n, np.float64)
    fb = C.c_uint64(0)
    err = C.create_string_buffer(256)
    rc = lib().oracle_knn_rows(_ptr(x), n, d, k, k if margin is None else margin, q0, q1, n_threads, _ptr(idx),
                               _ptr(cos), _ptr(norms), C.byref(fb), err, 256)
    if rc:
        raise ValueError(err.value.decode())
    return (idx, cos, norms), int(fb.value)


def knn_bruteforce(x, k, *, select="cosine", n_threads=0):
    """knn.rs:884 knn_bruteforce_select, restated."""
    x = _f32(x)
    n, d = x.shape
    idx = np.empty((n, k), np.uint32)
    cos = np.empty((n, k), np.float64)
    norms = np.empty(n, np.float64)
    err = C.create_string_buffer(256)
    rc = lib().oracle_knn_bruteforce(_ptr(x), n, d, k, 0 if select == "cosine" else 1, n_threads, _ptr(idx),
                                     _ptr(cos), _ptr(norms), err, 256)
    if rc:
        raise ValueError(err.value.decode())
    return idx, cos, norms


_WEIGHTS = {"tanimoto": 0, "cosine": 1, "jaccard": 2}


def reweight(idx, cos, norms, weight):
    """weight.rs:41 reweight, restated."""
    idx = np.ascontiguousarray(idx, dtype=np.uint32)
    cos = np.ascontiguousarray(cos, dtype=np.float64)
    norms = np.ascontiguousarray(norms, dtype=np.float64)
    n, k = idx.shape
    out = np.empty((n, k), np.float64)
    lib().oracle_reweight(n, k, _ptr(idx), _ptr(cos), _ptr(norms), _WEIGHTS[weight], _ptr(out))
    return out


def fuzzy_union(idx, w):
    """graph.rs:24 fuzzy_union, restated. Returns (rows u32, cols u32, weights f64)."""
    idx = np.ascontiguousarray(idx, dtype=np.uint32)
    w = np.ascontiguousarray(w, dtype=np.float64)
    n, k = idx.shape
    rows = np.empty(n * k, np.uint32)
    cols = np.empty(n * k, np.uint32)
    wout = np.empty(n * k, np.float64)
    m = C.c_uint64(0)
    lib().oracle_fuzzy_union(n, k, _ptr(idx), _ptr(w), _ptr(rows), _ptr(cols), _ptr(wout), C.byref(m))
    m = m.value
    return rows[:m].copy(), cols[:m].copy(), wout[:m].copy()


def tani_from_cos(a, b, c):
    return lib().oracle_tani_from_cos(a, b, c)


def row_l2_norms(x):
    x = _f32(x)
    out = np.empty(x.shape[0], np.float32)
    lib().oracle_row_l2_norms(_ptr(x), x.shape[0], x.shape[1], _ptr(out))
    return out


def heap_keep(pairs, cap):
    """knn.rs:831-875: push (score, id) pairs into one heap of capacity cap; return the kept ids."""
    scores = np.ascontiguousarray([p[0] for p in pairs], dtype=np.float32)
    ids = np.ascontiguousarray([p[1] for p in pairs], dtype=np.uint32)
    out = np.empty(cap, np.uint32)
    m = lib().oracle_heap_keep(_ptr(scores), _ptr(ids), len(pairs), cap, _ptr(out))
    return sorted(int(v) for v in out[:m])
