"""Why the split-FP8 kind keeps 64 candidates a row: a numpy model of its certificate on the
100,000 x 2,000 scRNA-like stand-in (negative-binomial counts, library-size normalised, log1p).

Each normalised row a is scaled by 2^8 and split into e4m3 pieces hi + lo (round to nearest even,
subnormal quantum 2^-9), the remainder r kept exactly; the bound E_i is the one the kernel uses
(split remainder by Cauchy-Schwarz from the pieces' norms, plus (3d + 16)·2^-21·sum|products| for the
accumulation, plus the normalisation and rescoring terms). A row certifies when its exact k-th cosine
exceeds the cap-th coarse score plus E_i (knn.rs:688-720). With the reference's default margin m = k
(cap 30) the bound is wider than most rows' gap; with 64 candidates every sampled row certifies."""

import numpy as np
import pytest


def e4m3(x):
    a = np.abs(x)
    e = np.floor(np.log2(np.where(a > 0, a, 1.0)))
    q = 2.0 ** (np.maximum(e, -6) - 3)  # below 2^-6 the quantum stays 2^-9 (subnormals)
    return np.sign(x) * np.minimum(np.round(a / q) * q, 448.0)


@pytest.fixture(scope="module")
def model():
    from costal_gb300 import workloads as W

    x = W.scrna_100k().astype(np.float64)
    n, d = x.shape
    nrm = np.linalg.norm(x, axis=1)
    xs = x / np.where(nrm > 0, nrm, 1.0)[:, None]
    u = xs * 256.0
    hi = e4m3(u)
    lo = e4m3(u - hi)
    h, l = hi / 256.0, lo / 256.0
    r = xs - h - l
    nh, nl, nr, nhl = (np.linalg.norm(v, axis=1) for v in (h, l, r, h + l))
    split = nl * nl.max() + nhl * nr.max() + nr * nhl.max() + nr * nr.max()
    acc = (3 * d + 16) * 2.0 ** -21 * (nh * nh.max() + nh * nl.max() + nl * nh.max())
    E = split + acc + 2.0001 * 2.0 ** -24 + (d + 8) * 2.0 ** -52
    return xs, h.astype(np.float32), l.astype(np.float32), E


def test_split_fp8_certifies_with_64_candidates(model):
    xs, h, l, E = model
    k = 15
    rows = np.sort(np.random.default_rng(0).choice(len(xs), 300, replace=False))
    ex = xs[rows] @ xs.T
    co = (h[rows] @ h.T + h[rows] @ l.T + l[rows] @ h.T).astype(np.float64)
    ex[np.arange(len(rows)), rows] = -np.inf
    co[np.arange(len(rows)), rows] = -np.inf
    ok = np.isfinite(ex)
    diff = np.subtract(ex, co, where=ok, out=np.zeros_like(ex))
    assert (np.abs(diff) <= E[rows][:, None]).all(), "the bound must hold in the model"
    sk = -np.sort(-ex, axis=1)[:, k - 1]
    cs = -np.sort(-co, axis=1)
    rate = {cap: float(np.mean(sk > cs[:, cap - 1] + E[rows])) for cap in (30, 45, 64, 115)}
    print("certified share by candidates a row:", rate, "E median", float(np.median(E)))
    assert rate[30] < 0.6 and rate[64] >= 0.99
