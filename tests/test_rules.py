"""The arithmetic rules the GPU rescoring relies on, restated and checked on random cases (CPU).

k_rescore drops, before the f64 rescoring, every candidate whose coarse score is below c_k − 2E, where
c_k is the k-th largest coarse score of the row's candidates and E bounds |coarse − exact|: such a
candidate scores below the exact k-th score s_k, so it can neither be in the top k nor change s_k (the
certificate's other input). The f32 → f64 widening of the f64 dot products is done with integer
operations; its restatement must give the conversion's bits for every class of f32.
"""

import numpy as np
import pytest


def top_k(scores, ids, k):
    order = np.lexsort((ids, -scores))  # (score desc, index asc)
    return ids[order[:k]], scores[order[:k]]


@pytest.mark.parametrize("seed", range(20))
def test_skipping_below_kth_minus_two_bounds_keeps_the_top_k_and_s_k(seed):
    rng = np.random.default_rng(seed)
    for _ in range(200):
        cap = int(rng.integers(2, 129))
        k = int(rng.integers(1, cap + 1))
        e = float(rng.choice([1e-6, 1e-4, 1e-2]))
        exact = rng.choice([rng.uniform(-1, 1, cap), np.round(rng.uniform(-1, 1, cap), 2)])  # with ties
        coarse = exact + rng.uniform(-e, e, cap)  # |coarse − exact| ≤ E
        ids = rng.permutation(10 * cap)[:cap]
        c_k = np.sort(coarse)[::-1][k - 1]
        keep = ~(coarse < c_k - 2 * e)
        want_ids, want_s = top_k(exact, ids, k)
        got_ids, got_s = top_k(exact[keep], ids[keep], k)
        np.testing.assert_array_equal(got_ids, want_ids)
        np.testing.assert_array_equal(got_s, want_s)


def f64_of(u32):
    """The integer widening of f32 bit patterns (finite) to f64 bit patterns."""
    u = np.asarray(u32, dtype=np.uint64)
    v = u & 0x7FFFFFFF
    sgn = (u & 0x80000000) << 32
    normal = (((v >> 3) + 0x38000000) << 32) | ((v << 29) & 0xFFFFFFFF)
    # subnormal: leading bit p, value 2^(p−149)·(1.f)
    p = np.zeros_like(v)
    nz = v > 0
    p[nz] = np.floor(np.log2(v[nz].astype(np.float64))).astype(np.uint64)
    sub = ((p + 874) << 52) | ((v << (52 - p)) & 0x000FFFFFFFFFFFFF)
    out = np.where(v >= 0x00800000, normal, np.where(v == 0, 0, sub))
    return out | sgn


def test_integer_widening_restated_on_every_class():
    rng = np.random.default_rng(3)
    pats = np.concatenate([
        rng.integers(0, 1 << 32, 2_000_000, dtype=np.uint64),           # any pattern
        np.arange(0, 1 << 23, 97, dtype=np.uint64),                      # subnormals
        np.arange(0, 1 << 23, 97, dtype=np.uint64) | 0x80000000,         # negative subnormals
        np.array([0, 0x80000000, 1, 0x80000001, 0x007FFFFF, 0x00800000, 0x7F7FFFFF, 0xFF7FFFFF], np.uint64),
    ]).astype(np.uint32)
    pats = pats[(pats & 0x7F800000) != 0x7F800000]  # finite only
    want = pats.view(np.float32).astype(np.float64).view(np.uint64)
    np.testing.assert_array_equal(f64_of(pats), want)


@pytest.mark.parametrize("d", [1, 5, 16, 40, 64, 300])
def test_coarse_tanimoto_stays_within_its_bound(d):
    # The GPU's coarse Tanimoto score: T = dot / (A + B − dot), dot = a·b·ĉ with ĉ the f32 dot of the
    # f32-normalised rows and a, A the f32 norm and squared norm; within 2(d+12)·2⁻²³ of the exact T.
    rng = np.random.default_rng(d)
    n = 400
    x = rng.normal(size=(n, d)) * rng.uniform(0.01, 100.0, size=(n, 1))
    x[rng.random(x.shape) < 0.3] = 0.0
    x = x.astype(np.float32)
    x64 = x.astype(np.float64)
    nrm = np.sqrt((x64 * x64).sum(1))
    xs = np.where(nrm[:, None] > 0, x64 * (1.0 / np.where(nrm > 0, nrm, 1.0))[:, None], 0.0).astype(np.float32)
    i = rng.integers(0, n, 20000)
    j = rng.integers(0, n, 20000)
    dot64 = (x64[i] * x64[j]).sum(1)
    with np.errstate(invalid="ignore", divide="ignore"):
        cos = np.where((nrm[i] > 0) & (nrm[j] > 0), dot64 / (nrm[i] * nrm[j]), 0.0)
        d_ex = nrm[i] * nrm[j] * cos
        t_ex = np.where(d_ex == 0, 0.0, d_ex / (nrm[i] ** 2 + nrm[j] ** 2 - d_ex))
    c32 = np.zeros(len(i), np.float32)
    for t in range(d):  # one rounding per step, like the GPU's FMA chain within the (d+4)·2⁻²³ bound
        c32 = (c32 + xs[i, t] * xs[j, t]).astype(np.float32)
    a = nrm.astype(np.float32)
    sq = (nrm * nrm).astype(np.float32)
    dn = (a[i] * a[j]).astype(np.float32) * c32
    den = (sq[i] + sq[j]).astype(np.float32) - dn
    with np.errstate(invalid="ignore", divide="ignore"):
        t32 = np.where((dn == 0) | (den <= 0), np.float32(0), dn / den).astype(np.float64)
    bound = 2.0 * (d + 12) * 2.0 ** -23
    assert np.abs(t32 - t_ex).max() <= bound


def bf16_rne(v32):
    """f32 → bf16 (round to nearest even), returned as f32 values."""
    u = np.asarray(v32, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def to_f32_toward_zero(x64):
    f = x64.astype(np.float32)
    away = np.abs(f.astype(np.float64)) > np.abs(x64)
    f[away] = np.nextafter(f[away], np.float32(0))
    return f


@pytest.mark.parametrize("d", [3, 15, 40, 64, 200])
def test_split_bf16_coarse_score_within_its_row_bound(d):
    # The split A = [hi | lo | hi], B = [hi | hi | lo] and the per-row bound E_i of k_row_eps, against an
    # accumulation model worse than the hardware's: products of each 16-wide step summed exactly, then
    # truncated to f32, and the f32 accumulator truncated after every step.
    rng = np.random.default_rng(100 + d)
    n = 300
    x = rng.normal(size=(n, d)) + rng.normal(0, 3, size=(1, d))
    x64 = x / np.linalg.norm(x, axis=1, keepdims=True)
    a = x64.astype(np.float32)
    hi = bf16_rne(a)
    lo = bf16_rne((a - hi).astype(np.float32))
    rem = ((a - hi).astype(np.float32) - lo).astype(np.float64)
    h64, l64 = hi.astype(np.float64), lo.astype(np.float64)
    nh, nl, nr = (np.linalg.norm(v, axis=1) for v in (h64, l64, rem))
    npn = np.linalg.norm(h64 + l64, axis=1)
    Mh, Ml, Mr, Mp = nh.max(), nl.max(), nr.max(), npn.max()
    K = 3 * d
    split = nl * Ml + npn * Mr + nr * Mp + nr * Mr
    acc = (K + 16) * 2.0 ** -21 * (nh * Mh + nl * Mh + nh * Ml)
    E = split + acc + 2.0001 * 2.0 ** -24 + (d + 8) * 2.0 ** -52
    A = np.concatenate([h64, l64, h64], 1)
    B = np.concatenate([h64, h64, l64], 1)
    i = rng.integers(0, n, 3000)
    j = rng.integers(0, n, 3000)
    accum = np.zeros(len(i), np.float32)
    for k0 in range(0, K, 16):
        step = (A[i, k0:k0 + 16] * B[j, k0:k0 + 16]).sum(1)  # exact enough in f64 for bf16 products
        accum = to_f32_toward_zero(accum.astype(np.float64) + to_f32_toward_zero(step).astype(np.float64))
    exact = (x64[i] * x64[j]).sum(1)
    assert (np.abs(accum.astype(np.float64) - exact) <= E[i]).all()
