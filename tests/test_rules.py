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
