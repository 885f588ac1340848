"""The CPU oracle against the reference's own known answers and golden digests (no GPU needed).

Each test names the reference test it restates. Together they pin the oracle: it is the
checker of every GPU parity test, so it must first reproduce what the reference itself asserts.
"""

import numpy as np
import pytest

from conftest import GOLDEN_PIPELINE, Lcg, clustered, csr_from_edges, digest, lcg_clustered, pipeline_input


def same(a, b):
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)


def test_matches_bruteforce_exactly(oracle):
    # knn.rs:960-967
    x = lcg_clustered(1500, 32, 1)
    (idx, cos, norms), st = oracle.knn_exact(x, 10)
    same((idx, cos, norms), oracle.knn_bruteforce(x, 10))


@pytest.mark.parametrize("rb,cb", [(1, 1), (8, 64), (33, 129), (512, 4096)])
@pytest.mark.parametrize("sort", [False, True])
def test_independent_of_blocks_and_layout(oracle, rb, cb, sort):
    # knn.rs:969-999
    x = lcg_clustered(900, 17, 2)
    want = oracle.knn_bruteforce(x, 7)
    for threads in (1, 4):
        got, _ = oracle.knn_exact(x, 7, row_block=rb, col_block=cb, sort_by_norm=sort, n_threads=threads)
        same(got, want)


def test_exact_duplicates_break_ties_by_original_index(oracle):
    # knn.rs:1001-1017: 10 prototypes × 30 copies; row 0's neighbours are 10, 20, …, 100
    d, k = 5, 10
    g = Lcg(3)
    protos = np.array([np.float32(g.next_f32() - np.float32(0.3)) for _ in range(10 * d)], np.float32).reshape(10, d)
    x = np.ascontiguousarray(protos[np.arange(300) % 10])
    (idx, cos, norms), _ = oracle.knn_exact(x, k)
    same((idx, cos, norms), oracle.knn_bruteforce(x, k))
    assert list(idx[0]) == [10, 20, 30, 40, 50, 60, 70, 80, 90, 100]


def test_zero_rows_and_integer_ties(oracle):
    # knn.rs:1019-1032
    n, d, k = 400, 6, 12
    g = Lcg(4)
    x = np.array([np.floor(g.next_f32() * np.float32(3.0)) for _ in range(n * d)], np.float32).reshape(n, d)
    x[[0, 57, 399]] = 0.0
    want = oracle.knn_bruteforce(x, k)
    same(oracle.knn_exact(x, k)[0], want)
    assert (want[1][0] == 0.0).all()


@pytest.mark.parametrize("k", [1, 23, 24])
def test_k_close_to_n(oracle, k):
    # knn.rs:1034-1044
    x = lcg_clustered(25, 4, 5)
    same(oracle.knn_exact(x, k)[0], oracle.knn_bruteforce(x, k))


def test_rejects_bad_input(oracle):
    # knn.rs:1046-1067
    x = np.ones((4, 3), np.float32)
    with pytest.raises(ValueError, match="invalid k=4"):
        oracle.knn_exact(x, 4)
    with pytest.raises(ValueError, match="invalid k=0"):
        oracle.knn_exact(x, 0)
    y = x.copy()
    y.reshape(-1)[7] = np.nan
    with pytest.raises(ValueError, match="row 2 contains NaN"):
        oracle.knn_exact(y, 1)


def test_heap_keeps_best_with_index_tiebreak(oracle):
    # knn.rs:1149-1159
    pairs = [(0.5, 7), (0.9, 3), (0.5, 2), (0.7, 9), (0.5, 1), (0.95, 0)]
    assert oracle.heap_keep(pairs, 3) == [0, 3, 9]


def test_tanimoto_selection_matches_bruteforce(oracle):
    # knn.rs:1076-1101: rows rescaled so that magnitude matters
    n, d, k = 1200, 16, 10
    x = lcg_clustered(n, d, 6)
    x *= (np.float32(1.0) + ((np.arange(n) % 7).astype(np.float32) * np.float32(0.4)))[:, None]
    want = oracle.knn_bruteforce(x, k, select="tanimoto")
    assert not np.array_equal(want[0], oracle.knn_bruteforce(x, k)[0])
    for rb, cb in [(1, 7), (16, 128), (300, 2000)]:
        for sort in (False, True):
            same(oracle.knn_exact(x, k, select="tanimoto", row_block=rb, col_block=cb, sort_by_norm=sort)[0], want)


def test_tanimoto_norm_window_prunes_and_stays_exact(oracle):
    # knn.rs:1118-1138
    n, d, k = 3000, 8, 10
    x = lcg_clustered(n, d, 9)
    x *= (np.float32(1.0) + (np.arange(n) % 50).astype(np.float32))[:, None]
    want = oracle.knn_bruteforce(x, k, select="tanimoto")
    got, st = oracle.knn_exact(x, k, select="tanimoto", row_block=32, col_block=64)
    same(got, want)
    assert st["blocks_skipped"] * 4 > st["blocks_total"]
    assert oracle.knn_exact(x, k)[1]["blocks_skipped"] == 0


def test_tanimoto_closed_forms(oracle):
    # weight.rs:99-109
    t = oracle.tani_from_cos
    assert t(1.0, 2.0, 1.0) == 2.0 / 3.0
    assert abs(t(3.0, 3.0, 0.6) - 0.6 / (2.0 - 0.6)) < 1e-15
    assert t(0.0, 2.0, 0.9) == 0.0
    assert abs(t(1.0, 1.0, -1.0) + 1.0 / 3.0) < 1e-15


def test_jaccard_hand_case(oracle):
    # weight.rs:111-121
    idx = np.array([1, 2, 0, 2, 0, 1, 0, 1], np.uint32).reshape(4, 2)
    w = oracle.reweight(idx, np.zeros((4, 2)), np.ones(4), "jaccard").ravel()
    assert w[0] == 1.0 / 3.0 and w[6] == 1.0 / 3.0 and w[4] == 1.0 / 3.0


def test_fuzzy_union_hand_cases(oracle):
    # graph.rs:74-95
    idx = np.array([1, 2, 0, 2, 1, 0], np.uint32).reshape(3, 2)
    w = np.array([0.5, 0.3, 0.4, 0.2, 0.0, 0.6]).reshape(3, 2)
    r, c, v = oracle.fuzzy_union(idx, w)
    assert list(r) == [0, 0, 1] and list(c) == [1, 2, 2]
    assert list(v) == [(0.5 + 0.4) - 0.5 * 0.4, (0.3 + 0.6) - 0.3 * 0.6, 0.2]
    r, c, v = oracle.fuzzy_union(np.array([[1], [2], [0]], np.uint32), np.array([[0.0], [0.7], [0.0]]))
    assert (list(r), list(c), list(v)) == ([1], [2], [0.7])


# ---- the reference's Python tests (tests/test_knn.py), restated against the oracle -------------

@pytest.mark.parametrize("seed", [0, 1])
def test_blocked_equals_bruteforce_bitwise(oracle, seed):
    # test_knn.py:36-43
    x = clustered(3000, 32, seed)
    got, st = oracle.knn_exact(x, 10)
    same(got, oracle.knn_bruteforce(x, 10))
    assert st["fallback_rows"] == 0


def test_independent_numpy_f64_oracle(oracle):
    # test_knn.py:46-61
    x = clustered(1500, 20, 2)
    (idx, cos, _), _ = oracle.knn_exact(x, 12)
    x64 = x.astype(np.float64)
    xn = x64 / np.linalg.norm(x64, axis=1, keepdims=True)
    sim = xn @ xn.T
    np.fill_diagonal(sim, -np.inf)
    order = np.argsort(-sim, axis=1, kind="stable")[:, :13]
    want = np.take_along_axis(sim, order, axis=1)
    np.testing.assert_allclose(cos, want[:, :12], rtol=0, atol=1e-12)
    clear = (want[:, 11] - want[:, 12]) > 1e-9
    assert clear.mean() > 0.99
    for i in np.flatnonzero(clear):
        assert set(idx[i]) == set(order[i, :12])


def test_tie_heavy_integer_data_takes_the_fallback(oracle):
    # test_knn.py:87-94
    rng = np.random.default_rng(5)
    x = np.floor(rng.uniform(0, 3, size=(500, 6))).astype(np.float32)
    x[[0, 99, 499]] = 0.0
    got, st = oracle.knn_exact(x, 12)
    same(got, oracle.knn_bruteforce(x, 12))
    assert st["fallback_rows"] > 0


def original_tani_from_cos(a, b, c):
    d = a * b * c
    return 0 if d == 0 else d / (a * a + b * b - d)


def test_tanimoto_weights_match_the_1_0_formula(oracle):
    # test_knn.py:195-206: bit-identical to CosTaL 1.0's order of operations
    (idx, cos, norms), _ = oracle.knn_exact(clustered(600, 12, 8), 10)
    w = oracle.reweight(idx, cos, norms, "tanimoto")
    want = np.array([[original_tani_from_cos(norms[i], norms[j], c) for j, c in zip(idx[i], cos[i])]
                     for i in range(len(idx))])
    np.testing.assert_array_equal(w, want)


def test_jaccard_matches_the_1_0_formula(oracle):
    # test_knn.py:208-211
    (idx, cos, norms), _ = oracle.knn_exact(clustered(400, 8, 9), 10)
    k = idx.shape[1]
    want = np.array([[len(set(idx[i]) & set(idx[j])) for j in idx[i]] for i in range(len(idx))], float)
    want = want / (2 * k - want)
    np.testing.assert_array_equal(oracle.reweight(idx, cos, norms, "jaccard"), want)


def test_fuzzy_union_matches_scipy(oracle):
    # test_knn.py:217-237: S + Sᵀ − S∘Sᵀ, setdiag(0), triu, eliminate_zeros
    sp = pytest.importorskip("scipy.sparse")
    (idx, cos, norms), _ = oracle.knn_exact(clustered(1000, 16, 10), 10)
    w = oracle.reweight(idx, cos, norms, "tanimoto")
    n, k = idx.shape
    csr = sp.csr_matrix((w.ravel(), (np.repeat(np.arange(n), k), idx.ravel().astype(np.int64))), shape=(n, n))
    csr = csr + csr.transpose() - csr.multiply(csr.transpose())
    csr.setdiag(0)
    csr = sp.triu(csr).tocsr()
    csr.eliminate_zeros()
    src, dst = csr.nonzero()
    got = oracle.fuzzy_union(idx, w)
    np.testing.assert_array_equal(got[0], src)
    np.testing.assert_array_equal(got[1], dst)
    np.testing.assert_array_equal(got[2], csr.data)


def test_golden_pipeline_digest(oracle, ext):
    # test_leiden_native.py:129-135: kNN + Tanimoto + fuzzy union (oracle) → host Leiden → digest
    x = pipeline_input()
    (idx, cos, norms), _ = oracle.knn_exact(x, 10)
    w = oracle.reweight(idx, cos, norms, "tanimoto")
    r, c, v = oracle.fuzzy_union(idx, w)
    m = ext._leiden(len(x), r.view(np.int32), c.view(np.int32), v, resolution=0.8, n_iterations=2, seed=3)[0]
    assert digest(m.astype(np.int64)) == GOLDEN_PIPELINE


def test_golden_pipeline_on_the_csr_layout(oracle, ext):
    # The Leiden's CSR of the union's edge list (leiden.rs:52-101): every row comes out ascending,
    # the property the GPU's sorted buckets reproduce, and the host Leiden run on that CSR in place
    # gives the golden labels.
    x = pipeline_input()
    (idx, cos, norms), _ = oracle.knn_exact(x, 10)
    w = oracle.reweight(idx, cos, norms, "tanimoto")
    r, c, v = oracle.fuzzy_union(idx, w)
    indptr, nbr, cw = csr_from_edges(len(x), r, c, v)
    for i in range(len(x)):
        assert (np.diff(nbr[indptr[i]:indptr[i + 1]].astype(np.int64)) > 0).all()
    m = ext._leiden_csr(len(x), indptr, nbr, cw, resolution=0.8, n_iterations=2, seed=3)[0]
    assert digest(m.astype(np.int64)) == GOLDEN_PIPELINE


def test_golden_fixtures_reproduce(oracle):
    # tests/golden/*.npz were made by tests/golden/make_golden.py from the (pinned) oracle
    from pathlib import Path

    gold = Path(__file__).parent / "golden"
    files = sorted(p for p in gold.glob("*.npz") if not p.name.startswith("dropin"))  # (dropin_*: the replay record)
    assert files, "golden fixtures missing"
    for f in files:
        z = np.load(f)
        x, k = z["x"], int(z["k"])
        (idx, cos, norms), st = oracle.knn_exact(x, k, margin=int(z["margin"]))
        np.testing.assert_array_equal(idx, z["idx"])
        np.testing.assert_array_equal(cos, z["cos"])
        np.testing.assert_array_equal(norms, z["norms"])
        w = oracle.reweight(idx, cos, norms, "tanimoto")
        np.testing.assert_array_equal(w, z["w"])
        r, c, v = oracle.fuzzy_union(idx, w)
        np.testing.assert_array_equal(r, z["rows"])
        np.testing.assert_array_equal(c, z["cols"])
        np.testing.assert_array_equal(v, z["ew"])
