import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU; runs the CUDA path through the C ABI")
    config.addinivalue_line("markers", "slow: full-size workloads")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False


@pytest.fixture(scope="session")
def ext():
    """The product module (costal_gb300._costal). Builds libcostal_gb300 if it is missing."""
    from costal_gb300 import build

    build.build_library()
    from costal_gb300 import _costal

    return _costal


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.lib()
    return O


def clustered(n, d, seed, n_centers=8, noise=0.5):
    """Gaussian clusters in the positive orthant (the reference's test_knn.py data shape)."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(0, 4, size=(n_centers, d))
    x = centers[rng.integers(0, n_centers, size=n)] + rng.normal(0, noise, size=(n, d))
    return np.ascontiguousarray(x, dtype=np.float32)


def scaled_clusters(n, d, seed):
    """clustered() rows rescaled per row, so magnitude matters (the reference's tests/test_knn.py:97-102)."""
    x = clustered(n, d, seed)
    x *= np.random.default_rng(seed + 100).uniform(0.5, 3.0, size=(n, 1)).astype(np.float32)
    return np.ascontiguousarray(x)


class Lcg:
    """The reproducible generator of crates/costal-core/src/knn.rs:931-940 (its unit tests' data)."""

    def __init__(self, seed):
        self.s = seed & (2**64 - 1)

    def next_f32(self):
        self.s = (self.s * 6364136223846793005 + 1442695040888963407) & (2**64 - 1)
        return np.float32(np.float32(self.s >> 40) / np.float32(1 << 24))


def lcg_clustered(n, d, seed):
    """knn.rs:943-954: 8 centres in [0,4)^d, rows centre + U[0,1) - 0.55, in f32 arithmetic."""
    g = Lcg(seed)
    centers = [g.next_f32() * np.float32(4.0) for _ in range(8 * d)]
    out = np.empty((n, d), np.float32)
    for i in range(n):
        c = i % 8
        for t in range(d):
            out[i, t] = np.float32(np.float32(centers[c * d + t] + g.next_f32()) - np.float32(0.55))
    return out


def digest(labels) -> str:
    import hashlib

    return hashlib.sha256(np.asarray(labels, dtype="<i8").tobytes()).hexdigest()[:16]


# Fixed partitions published by the reference (tests/test_leiden_native.py:125-126).
GOLDEN_GRAPH = "36b0210aa49dc294"
GOLDEN_PIPELINE = "ab4b3e17a8b1138d"


def planted(n_blocks=12, size=40, p_in=0.15, n_cross=500, seed=0):
    """Upper-triangular planted-partition edge list, weights in (0.5, 1): the generator of the
    reference's tests/test_leiden_native.py:19-39, restated (it defines the GOLDEN_GRAPH input)."""
    rng = np.random.default_rng(seed)
    pairs = {}
    for b in range(n_blocks):
        nodes = np.arange(b * size, (b + 1) * size)
        i, j = np.triu_indices(size, 1)
        keep = rng.random(len(i)) < p_in
        for a, c in zip(nodes[i[keep]], nodes[j[keep]]):
            pairs[(int(a), int(c))] = 0.5 + 0.5 * rng.random()
    n = n_blocks * size
    while n_cross:
        a, c = rng.integers(0, n, 2)
        if a // size != c // size:
            pairs[(int(min(a, c)), int(max(a, c)))] = 0.5 + 0.5 * rng.random()
            n_cross -= 1
    keys = sorted(pairs)
    rows = np.array([k[0] for k in keys], dtype=np.int32)
    cols = np.array([k[1] for k in keys], dtype=np.int32)
    w = np.array([pairs[k] for k in keys])
    return n, rows, cols, w


def csr_from_edges(n, rows, cols, w):
    """leiden.rs:52-101 `Csr::from_edges`, restated: walk the edges in order, append j to row i and i
    to row j (zero weights dropped). Returns (indptr uint64, nbr uint32, weights float64)."""
    rows = np.asarray(rows).astype(np.int64)
    cols = np.asarray(cols).astype(np.int64)
    w = np.asarray(w, dtype=np.float64)
    keep = w > 0
    rows, cols, w = rows[keep], cols[keep], w[keep]
    # entry 2e is edge e seen from its first endpoint, 2e + 1 from its second: a stable sort by row
    # keeps each row's entries in edge order
    src = np.stack([rows, cols], 1).ravel()
    dst = np.stack([cols, rows], 1).ravel()
    ww = np.repeat(w, 2)
    order = np.argsort(src, kind="stable")
    indptr = np.zeros(n + 1, np.uint64)
    np.cumsum(np.bincount(src, minlength=n), out=indptr[1:])
    return indptr, dst[order].astype(np.uint32), ww[order]


def pipeline_input():
    """The GOLDEN_PIPELINE input of the reference's tests/test_leiden_native.py:132-135."""
    rng = np.random.default_rng(7)
    x = np.abs(rng.normal(size=(3000, 16)) + np.repeat(rng.normal(0, 3, size=(6, 16)), 500, axis=0))
    return np.ascontiguousarray(x, dtype=np.float32)
