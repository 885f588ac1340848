"""The C-ABI library loads and exports every entry point include/*.h declares (no GPU needed)."""

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"^\s*(?:const\s+)?(?:\w+\s+)*\w+\s*\*?\s*(costal_\w+)\s*\(", text, re.M))
    return sorted(names)


def test_header_declares_the_drop_in_surface():
    names = declared_symbols()
    for required in ("costal_knn_exact", "costal_knn_bruteforce", "costal_reweight", "costal_fuzzy_union",
                     "costal_build_graph", "costal_leiden", "costal_leiden_many", "costal_modularity",
                     "costal_row_l2_norms", "costal_version"):
        assert required in names


def test_library_exports_every_declared_symbol(ext):
    from costal_gb300 import _lib

    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # every declared entry point has a ctypes signature in the binding
    bound = set(_lib.SIGNATURES) | {"costal_version", "costal_launch_count", "costal_shard_rows_max"}
    assert set(declared_symbols()) <= bound


def test_version_and_module_surface(ext):
    # lib.rs:448-465: the module's functions, all present
    for name in ("hello", "core_version", "row_l2_norms", "_knn_exact", "_knn_bruteforce", "_reweight",
                 "_fuzzy_union", "_leiden", "_leiden_many", "_modularity", "_leiden_coo", "l2_bytes_per_thread",
                 "tile_budget_bytes", "default_matmul"):
        assert callable(getattr(ext, name))
    assert ext.__version__ == ext.core_version() == "2.1.0"
    assert ext.core_version() in ext.hello()
    assert ext.default_matmul() == "fp32"


def test_argument_errors_are_raised_before_any_device_work(ext):
    x = np.zeros((8, 8), np.float32)[:, ::2]
    with pytest.raises(ValueError, match="C-contiguous"):
        ext.row_l2_norms(x)
    y = np.zeros((5, 3), np.float32)
    with pytest.raises(ValueError, match="unknown select"):
        ext._knn_exact(y, 2, select="jaccard")
    with pytest.raises(ValueError, match="unknown matmul"):
        ext._knn_exact(y, 2, matmul="nope")
    with pytest.raises(ValueError, match="unknown edge weight"):
        ext._reweight(np.zeros((5, 2), np.int32), np.zeros((5, 2)), np.zeros(5), "nope")
    with pytest.raises(ValueError, match="shapes"):
        ext._fuzzy_union(np.zeros((5, 2), np.int32), np.zeros((5, 3)))
    with pytest.raises(ValueError, match="negative index"):
        ext._leiden(3, np.array([-1], np.int32), np.array([1], np.int32), np.ones(1), resolution=1.0)
