"""Generate the golden fixtures tests/golden/*.npz from the pinned CPU oracle.

    python tests/golden/make_golden.py

The oracle is pinned against the reference's own known answers and golden digests
(tests/test_oracle.py); these fixtures freeze its outputs on small seeded inputs so that the GPU
tests also have a stored answer to compare with. Inputs: clustered data with mixed-sign values
(arcsinh of a Gaussian mixture, as in the cytometry configs), exact-duplicate prototypes (index
tie-break), and small-integer data with zero rows (massive ties: the regather fallback).
"""

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402


def cases():
    rng = np.random.default_rng(20241203)
    means = rng.normal(0, 2, size=(6, 12))
    lab = rng.integers(0, 6, size=256)
    x = np.arcsinh((means[lab] + rng.normal(0, 0.7, size=(256, 12))) / 5.0).astype(np.float32)
    yield "mixture_256x12_k10", x, 10, 10
    protos = rng.normal(size=(8, 5)).astype(np.float32)
    yield "duplicates_240x5_k10", np.ascontiguousarray(np.tile(protos, (30, 1))), 10, 10
    xi = np.floor(rng.uniform(0, 3, size=(200, 6))).astype(np.float32)
    xi[[0, 77, 199]] = 0.0
    yield "integer_ties_200x6_k12", xi, 12, 12


def main():
    out = Path(__file__).resolve().parent
    for name, x, k, margin in cases():
        (idx, cos, norms), st = O.knn_exact(x, k, margin=margin)
        w = O.reweight(idx, cos, norms, "tanimoto")
        r, c, v = O.fuzzy_union(idx, w)
        np.savez_compressed(out / f"{name}.npz", x=x, k=k, margin=margin, idx=idx, cos=cos, norms=norms, w=w,
                            rows=r, cols=c, ew=v, fallback_rows=st["fallback_rows"])
        print(name, st)


if __name__ == "__main__":
    main()
