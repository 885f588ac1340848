"""ctypes declarations of libcostal_gb300.so (include/costal_gb300.h).

The library is built in-tree by `python -m costal_gb300.build` (or __graft_entry__.build()). There is
no Python or CPU fallback for the kNN path: if the library is missing, importing this module fails,
and if no GB300 is present, every kNN call fails with COSTAL_ECUDA.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libcostal_gb300.so"

COSTAL_OK = 0
COSTAL_EINVAL = 2
COSTAL_ECUDA = 3
COSTAL_ENOMEM = 4
COSTAL_ETIMEOUT = 5
COSTAL_EUNSUPPORTED = 6

BACKEND_FP32 = 0
BACKEND_BF16 = 1
BACKEND_BF16X3 = 2
BACKEND_FP8 = 3
COARSE_KINDS = ("fp32", "bf16", "fp8")
SELECT = {"cosine": 0, "tanimoto": 1}
WEIGHT = {"tanimoto": 0, "cosine": 1, "jaccard": 2}


class KnnOpts(C.Structure):
    _fields_ = [
        ("margin", C.c_uint32),
        ("select", C.c_uint32),
        ("backend", C.c_uint32),
        ("row_block", C.c_uint32),
        ("col_block", C.c_uint32),
        ("sort_by_norm", C.c_int32),
        ("prune", C.c_int32),
        ("learned_prune", C.c_int32),
    ]


class KnnStats(C.Structure):
    _fields_ = [
        ("fallback_rows", C.c_uint64),
        ("row_block", C.c_uint64),
        ("col_block", C.c_uint64),
        ("blocks_skipped", C.c_uint64),
        ("blocks_total", C.c_uint64),
        ("margin", C.c_uint64),
        ("recomputed_rows", C.c_uint64),
        ("pruned_fallback_rows", C.c_uint64),
        ("max_coarse_err", C.c_double),
        ("ms_prep", C.c_double),
        ("ms_coarse", C.c_double),
        ("ms_rescore", C.c_double),
        ("ms_fallback", C.c_double),
        ("ms_total", C.c_double),
        ("ms_order", C.c_double),
        ("ms_kernel", C.c_double),
        ("blocks_stopped", C.c_uint64),
        ("max_err_ratio", C.c_double),
        ("coarse_kind", C.c_uint64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class MlpOpts(C.Structure):
    _fields_ = [
        ("sample", C.c_uint32),
        ("epochs", C.c_uint32),
        ("batch", C.c_uint32),
        ("margin", C.c_uint32),
        ("lr", C.c_float),
        ("quantile", C.c_float),
        ("seed", C.c_uint64),
    ]


class MlpStats(C.Structure):
    _fields_ = [
        ("samples", C.c_uint64),
        ("steps", C.c_uint64),
        ("params", C.c_uint64),
        ("loss", C.c_double),
        ("mae", C.c_double),
        ("coverage", C.c_double),
        ("ms_labels", C.c_double),
        ("ms_train", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


P = C.c_void_p
U64, U32, I32, INT, DBL, SZ, STR = C.c_uint64, C.c_uint32, C.c_int32, C.c_int, C.c_double, C.c_size_t, C.c_char_p

# name -> argtypes (every entry point returns int except costal_version)
SIGNATURES = {
    "costal_device_ok": [STR, SZ],
    "costal_check_f64_conversion": [P, STR, SZ],
    "costal_row_l2_norms": [P, U64, U32, P, STR, SZ],
    "costal_knn_exact": [P, U64, U32, U32, P, P, P, P, P, STR, SZ],
    "costal_knn_exact_device": [P, U64, U32, U32, P, P, P, P, P, P, STR, SZ],
    "costal_knn_bruteforce": [P, U64, U32, U32, U32, P, P, P, STR, SZ],
    "costal_reweight": [U64, U32, P, P, P, U32, P, STR, SZ],
    "costal_fuzzy_union": [U64, U32, P, P, P, P, P, P, STR, SZ],
    "costal_build_graph": [P, U64, U32, U32, P, U32, P, P, P, P, P, P, P, P, STR, SZ],
    "costal_build_graph_csr": [P, U64, U32, U32, P, U32, P, P, P, P, P, STR, SZ],
    "costal_build_graph_device": [P, U64, U32, U32, P, U32, P, P, P, P, P, P, STR, SZ],
    "costal_leiden": [U64, P, P, P, U64, INT, INT, DBL, DBL, I32, U64, P, P, P, P, P, P, STR, SZ],
    "costal_leiden_csr": [U64, P, P, P, INT, DBL, DBL, I32, U64, P, P, P, P, P, P, STR, SZ],
    "costal_leiden_many": [U64, P, P, P, U64, P, U64, P, U64, DBL, I32, INT, P, STR, SZ],
    "costal_leiden_many_csr": [U64, P, P, P, P, U64, P, U64, DBL, I32, INT, P, STR, SZ],
    "costal_modularity": [U64, P, P, P, U64, P, DBL, P, STR, SZ],
    "costal_reweight_jaccard_device_noalloc": [P, U64, U32, P, P, STR, SZ],
    "costal_knn_shard_device": [P, U64, U32, U32, P, U32, U32, P, P, P, P, P, P, P, P, STR, SZ],
    "costal_fuzzy_union_device": [P, P, U64, U32, P, P, P, P, P, STR, SZ],
    "costal_mlp_train": [P, U64, U32, U32, P, P, STR, SZ],
    "costal_mlp_get": [P, U64, P, P, P, P, STR, SZ],
    "costal_mlp_set": [P, U64, U32, U32, C.c_float, STR, SZ],
    "costal_mlp_clear": [STR, SZ],
    "costal_mlp_forward": [P, U32, P, U64, P, STR, SZ],
    "costal_mlp_gradient": [P, U32, P, P, U64, C.c_float, P, STR, SZ],
    "costal_block_bounds": [P, U64, U32, P, P, P, P, P, STR, SZ],
}

_lib = None


def lib() -> C.CDLL:
    """The loaded library; raises ImportError (never falls back) when it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA library first (python -m costal_gb300.build); "
                "there is no CPU fallback for the kNN path"
            )
        lb = C.CDLL(str(LIB_PATH))
        for name, args in SIGNATURES.items():
            fn = getattr(lb, name)
            fn.argtypes = args
            fn.restype = C.c_int
        lb.costal_version.argtypes = []
        lb.costal_version.restype = C.c_char_p
        lb.costal_launch_count.argtypes = []
        lb.costal_launch_count.restype = C.c_ulonglong
        lb.costal_shard_rows_max.argtypes = [U64, U32]
        lb.costal_shard_rows_max.restype = C.c_uint64
        _lib = lb
    return _lib


class CostalError(Exception):
    """A failed C-ABI call that is not a ValueError in the reference (CUDA, memory, timeouts)."""


def check(rc: int, err) -> None:
    if rc == COSTAL_OK:
        return
    msg = err.value.decode(errors="replace")
    if rc == COSTAL_EINVAL:
        raise ValueError(msg)
    if rc == COSTAL_EUNSUPPORTED:
        raise NotImplementedError(msg)
    raise CostalError(f"libcostal_gb300 error {rc}: {msg}")


def errbuf(size: int = 512):
    return C.create_string_buffer(size), size
