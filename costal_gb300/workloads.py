"""Seeded synthetic inputs with the shapes and value distributions of the five benchmark workloads.

They stand in for the reference's real cytometry / scRNA-seq datasets (Levine_32, Mosmann_rare,
2,000-gene scRNA sets), which are not available offline. All are float32, C-contiguous, and
deterministic for a seed (numpy's PCG64 `default_rng`).

    name               n          d      k   margin  description
    mixture_20k        20,000     32     10  10      20-cluster Gaussian mixture, arcsinh(x/5)
    rare_400k          400,000    15     10  8       12 clusters + one 400-cell cluster 3σ off its neighbour
    dense_dup_160k     160,000    32     30  30      24 clusters + 10% uniform noise + 1% exact duplicates
    scrna_100k         100,000    2000   15  15      negative-binomial counts, library-size norm, log1p
    zipf_2m            2,000,000  40     10  10      50 clusters with Zipf(1.2) sizes, arcsinh(x/5)
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Workload:
    name: str
    n: int
    d: int
    k: int
    margin: int
    seed: int


WORKLOADS = {
    "mixture_20k": Workload("mixture_20k", 20_000, 32, 10, 10, 0),
    "rare_400k": Workload("rare_400k", 400_000, 15, 10, 8, 1),
    "dense_dup_160k": Workload("dense_dup_160k", 160_000, 32, 30, 30, 2),
    "scrna_100k": Workload("scrna_100k", 100_000, 2000, 15, 15, 3),
    "zipf_2m": Workload("zipf_2m", 2_000_000, 40, 10, 10, 4),
}


def _mixture(rng, sizes, d, mean_sd=2.0, std_lo=0.3, std_hi=1.0):
    """Gaussian mixture: means N(0, mean_sd²), per-cluster diagonal std U(std_lo, std_hi)."""
    k = len(sizes)
    means = rng.normal(0.0, mean_sd, size=(k, d))
    stds = rng.uniform(std_lo, std_hi, size=(k, d))
    out = np.empty((int(np.sum(sizes)), d), np.float32)
    pos = 0
    for c, m in enumerate(sizes):
        out[pos:pos + m] = means[c] + stds[c] * rng.standard_normal((m, d), dtype=np.float32)
        pos += m
    return out, means, stds


def _shuffle(rng, x, labels=None):
    """Rows in a seeded random order; with `labels` (one per row), also those labels in that order."""
    perm = rng.permutation(len(x))
    if labels is None:
        return np.ascontiguousarray(x[perm])
    return np.ascontiguousarray(x[perm]), labels[perm]


def mixture_20k(n=20_000, d=32, seed=0):
    rng = np.random.default_rng(seed)
    sizes = rng.multinomial(n, np.full(20, 1 / 20))
    x, _, _ = _mixture(rng, sizes, d)
    return _shuffle(rng, np.arcsinh(x / 5.0).astype(np.float32))


def rare_400k(n=400_000, d=15, seed=1):
    rng = np.random.default_rng(seed)
    rare = max(1, round(n * 0.001))
    sizes = rng.multinomial(n - rare, np.full(12, 1 / 12))
    x, means, stds = _mixture(rng, sizes, d)
    # the rare population: centred 3σ (three of cluster c's standard deviations, along a random
    # direction) from the centre of cluster c, which is then its nearest neighbouring cluster
    c = int(rng.integers(12))
    direction = rng.normal(size=d)
    direction /= np.linalg.norm(direction)
    centre = means[c] + 3.0 * stds[c] * direction
    if int(np.argmin(np.linalg.norm(means - centre, axis=1))) != c:
        raise ValueError("seed places the rare population nearer another cluster than the one it is offset from")
    r = centre + 0.5 * stds[c] * rng.standard_normal((rare, d))
    x = np.vstack([x, r.astype(np.float32)])
    return _shuffle(rng, np.arcsinh(x / 5.0).astype(np.float32))


def dense_dup_160k(n=160_000, d=32, seed=2):
    rng = np.random.default_rng(seed)
    n_noise = n // 10
    n_dup = n // 100
    n_mix = n - n_noise - n_dup
    sizes = rng.multinomial(n_mix, np.full(24, 1 / 24))
    x, _, _ = _mixture(rng, sizes, d)
    lo, hi = x.min(axis=0), x.max(axis=0)
    noise = rng.uniform(lo, hi, size=(n_noise, d)).astype(np.float32)
    base = np.vstack([x, noise])
    dup = base[rng.integers(0, len(base), size=n_dup)]
    x = np.vstack([base, dup])
    return _shuffle(rng, np.arcsinh(x / 5.0).astype(np.float32))


def scrna_100k(n=100_000, d=2000, seed=3, chunk=10_000):
    """Negative-binomial counts (15 cluster log-normal mean profiles, dispersion 0.5), library-size
    normalised to 1e4, log1p, dense float32."""
    rng = np.random.default_rng(seed)
    profiles = np.exp(rng.normal(-3.0, 1.6, size=(15, d)))  # ~90% zeros at these means
    labels = rng.integers(0, 15, size=n)
    r = 1.0 / 0.5  # dispersion 0.5 -> NB shape r = 2
    out = np.empty((n, d), np.float32)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        mu = profiles[labels[a:b]] * rng.lognormal(0.0, 0.3, size=(b - a, 1))
        p = r / (r + mu)
        counts = rng.negative_binomial(r, p).astype(np.float64)
        lib = counts.sum(axis=1, keepdims=True)
        lib[lib == 0] = 1.0
        out[a:b] = np.log1p(counts / lib * 1e4)
    return out


def zipf_2m(n=2_000_000, d=40, seed=4, return_labels=False):
    """With return_labels, also each row's mixture component (0 = the largest of the 50)."""
    rng = np.random.default_rng(seed)
    w = 1.0 / np.arange(1, 51) ** 1.2
    sizes = rng.multinomial(n, w / w.sum())
    x, _, _ = _mixture(rng, sizes, d)
    x, labels = _shuffle(rng, np.arcsinh(x / 5.0).astype(np.float32), np.repeat(np.arange(50), sizes))
    return (x, labels) if return_labels else x


GENERATORS = {
    "mixture_20k": mixture_20k,
    "rare_400k": rare_400k,
    "dense_dup_160k": dense_dup_160k,
    "scrna_100k": scrna_100k,
    "zipf_2m": zipf_2m,
}


def make(name: str, n: int | None = None) -> tuple[np.ndarray, Workload]:
    """The workload's matrix (optionally a smaller n with the same generator) and its parameters."""
    wl = WORKLOADS[name]
    gen = GENERATORS[name]
    x = gen(seed=wl.seed) if n is None else gen(n=n, seed=wl.seed)
    return x, wl
