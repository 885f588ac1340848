"""GPU parity: the CUDA path (through the C ABI, via costal_gb300._costal) against the CPU oracle.

Integer and index outputs must be bit-identical, and so must the f64 cosines, norms and weights
(the reference's order of operations is restated on the device). Restates the reference's
tests/test_knn.py and knn.rs unit tests, plus full-size checks on the benchmark workloads through
row samples (the oracle answers a sample of query rows against all n columns).
"""

import numpy as np
import pytest

from conftest import GOLDEN_PIPELINE, Lcg, clustered, csr_from_edges, digest, lcg_clustered, pipeline_input

pytestmark = pytest.mark.gpu


def same(a, b):
    for u, v in zip(a, b):
        np.testing.assert_array_equal(np.asarray(u), np.asarray(v))


def as_oracle(res):
    idx, cos, norms = res
    return idx.view(np.uint32), cos, norms


@pytest.mark.parametrize("seed", [0, 1])
def test_exact_matches_bruteforce_bitwise(ext, oracle, seed):
    # test_knn.py:36-43
    x = clustered(3000, 32, seed)
    got, stats = ext._knn_exact(x, 10)
    same(as_oracle(got), oracle.knn_bruteforce(x, 10))
    same(as_oracle(ext._knn_bruteforce(x, 10)), oracle.knn_bruteforce(x, 10))
    assert stats["fallback_rows"] == 0


def test_matches_independent_numpy_oracle(ext):
    # test_knn.py:46-61
    x = clustered(1500, 20, 2)
    idx, cos, _ = ext._knn_exact(x, 12)[0]
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


def test_output_independent_of_knobs_and_backend(ext, oracle):
    # test_knn.py:64-75: blocks, backend, layout and threads never change the output
    x = clustered(1200, 17, 3)
    want = oracle.knn_bruteforce(x, 7)
    for backend in ("gemm", ext.default_matmul(), "bf16"):
        for rb, cb in [(1, 7), (16, 128), (200, 5000)]:
            for sort in (False, True):
                got, _ = ext._knn_exact(x, 7, row_block=rb, col_block=cb, matmul=backend, sort_by_norm=sort,
                                        n_threads=3)
                same(as_oracle(got), want)


def test_ties_break_by_original_index(ext, oracle):
    # test_knn.py:78-84
    rng = np.random.default_rng(4)
    protos = rng.normal(size=(10, 5)).astype(np.float32)
    x = np.ascontiguousarray(np.tile(protos, (30, 1)))
    idx, cos, norms = ext._knn_exact(x, 10)[0]
    same(as_oracle((idx, cos, norms)), oracle.knn_bruteforce(x, 10))
    np.testing.assert_array_equal(idx[0], np.arange(10, 101, 10))


def test_tie_heavy_integer_data_stays_exact(ext, oracle):
    # test_knn.py:87-94: massive exact ties must take the regather fallback
    rng = np.random.default_rng(5)
    x = np.floor(rng.uniform(0, 3, size=(500, 6))).astype(np.float32)
    x[[0, 99, 499]] = 0.0
    got, stats = ext._knn_exact(x, 12)
    same(as_oracle(got), oracle.knn_bruteforce(x, 12))
    assert stats["fallback_rows"] > 0


def test_integer_f64_conversion_matches_the_instruction(ext):
    """The f64 dot products widen f32 with integer operations; every finite f32 must come out the same."""
    import ctypes as C

    from costal_gb300 import _lib

    bad = C.c_uint64(99)
    err, size = _lib.errbuf()
    _lib.check(_lib.lib().costal_check_f64_conversion(C.addressof(bad), err, size), err)
    assert bad.value == 0


@pytest.mark.parametrize("matmul", ["gemm", "bf16"])
def test_subnormal_and_signed_zero_entries(ext, oracle, matmul):
    """Subnormal, ±0 and tiny entries go through the same f64 rescoring bit for bit."""
    rng = np.random.default_rng(21)
    x = clustered(900, 24, 4)
    x[rng.random(x.shape) < 0.15] = np.float32(-0.0)
    x[rng.random(x.shape) < 0.05] = 0.0
    sub = (rng.integers(1, 1 << 23, size=x.shape).astype(np.uint32)).view(np.float32)  # subnormal magnitudes
    sign = np.where(rng.random(x.shape) < 0.5, np.float32(-1), np.float32(1))
    m = rng.random(x.shape) < 0.1
    x[m] = (sub * sign)[m]
    x[7] = (sub[7] * sign[7])  # a row of subnormals only
    x = np.ascontiguousarray(x, dtype=np.float32)
    got, _ = ext._knn_exact(x, 9, matmul=matmul)
    same(as_oracle(got), oracle.knn_bruteforce(x, 9))


def test_lcg_known_answers(ext, oracle):
    # knn.rs:1001-1044 on the reference's own generator
    g = Lcg(3)
    protos = np.array([np.float32(g.next_f32() - np.float32(0.3)) for _ in range(50)], np.float32).reshape(10, 5)
    x = np.ascontiguousarray(protos[np.arange(300) % 10])
    idx = ext._knn_exact(x, 10)[0][0]
    assert list(idx[0]) == [10, 20, 30, 40, 50, 60, 70, 80, 90, 100]
    g = Lcg(4)
    x = np.array([np.floor(g.next_f32() * np.float32(3.0)) for _ in range(2400)], np.float32).reshape(400, 6)
    x[[0, 57, 399]] = 0.0
    got = ext._knn_exact(x, 12)[0]
    same(as_oracle(got), oracle.knn_bruteforce(x, 12))
    assert (got[1][0] == 0.0).all()
    x = lcg_clustered(25, 4, 5)
    for k in (1, 23, 24):
        same(as_oracle(ext._knn_exact(x, k)[0]), oracle.knn_bruteforce(x, k))


@pytest.mark.parametrize("n,d,k,margin", [(1001, 1, 5, None), (777, 5, 1, 0), (1500, 15, 10, 8), (1300, 17, 7, None),
                                          (900, 33, 30, None), (640, 64, 12, 3), (2000, 40, 10, 118), (129, 3, 20, 0),
                                          (700, 65, 10, None), (600, 300, 15, None), (500, 2000, 15, 15),
                                          (300, 130, 40, 60)])
def test_shapes_and_margins(ext, oracle, n, d, k, margin):
    rng = np.random.default_rng(n * 31 + d)
    means = rng.normal(0, 2, size=(7, d))
    x = np.arcsinh((means[rng.integers(0, 7, n)] + rng.normal(0, 0.6, size=(n, d))) / 5.0).astype(np.float32)
    got, st = ext._knn_exact(x, k, margin=margin)
    want, ost = oracle.knn_exact(x, k, margin=margin)
    same(as_oracle(got), want)
    same(as_oracle(got), oracle.knn_bruteforce(x, k))


@pytest.mark.parametrize("n,d,k,margin", [(900, 1, 6, None), (800, 8, 10, None), (1100, 16, 12, 4), (700, 24, 10, None),
                                          (1000, 31, 20, 30), (1200, 32, 10, None), (900, 33, 15, None),
                                          (1300, 39, 10, 10), (1500, 40, 10, None), (600, 40, 30, 30)])
def test_compact_operands_on_the_tensor_cores(ext, oracle, n, d, k, margin):
    """Around the compact operand range (22 ≤ d ≤ 32: 2d-wide [hi | lo] column rows, two MMA chains)
    and the 3d-wide resident form on either side of it."""
    rng = np.random.default_rng(3 * n + d)
    means = rng.normal(0, 2, size=(9, d))
    x = np.arcsinh((means[rng.integers(0, 9, n)] + rng.normal(0, 0.6, size=(n, d))) / 5.0).astype(np.float32)
    got, st = ext._knn_exact(x, k, margin=margin, matmul="bf16")
    same(as_oracle(got), oracle.knn_bruteforce(x, k))


@pytest.mark.parametrize("n,d,k,margin", [(700, 43, 10, None), (600, 300, 15, None), (500, 2000, 15, 15),
                                          (400, 130, 20, 40), (650, 41, 10, None), (640, 42, 12, 12)])
def test_deep_rows_on_the_tensor_cores(ext, oracle, n, d, k, margin):
    """Rows with 3d > 128 run the tensor-core K loop (with the locality order, block lists and early
    stop up to d = 64, in row order above); d = 41, 42 the resident 3d-wide form at its upper end: same
    exact output."""
    rng = np.random.default_rng(n + d)
    means = rng.normal(0, 2, size=(9, d))
    x = np.arcsinh((means[rng.integers(0, 9, n)] + rng.normal(0, 0.6, size=(n, d))) / 5.0).astype(np.float32)
    got, st = ext._knn_exact(x, k, margin=margin, matmul="bf16")
    same(as_oracle(got), oracle.knn_bruteforce(x, k))


def test_tanimoto_selection_matches_bruteforce(ext, oracle):
    # test_knn.py:118-126
    x = clustered(1500, 12, 14)
    x *= np.random.default_rng(114).uniform(0.5, 3.0, size=(1500, 1)).astype(np.float32)
    x = np.ascontiguousarray(x)
    got, stats = ext._knn_exact(x, 10, select="tanimoto")
    assert stats["select"] == "tanimoto"
    same(as_oracle(got), oracle.knn_bruteforce(x, 10, select="tanimoto"))
    same(as_oracle(ext._knn_bruteforce(x, 10, select="tanimoto")), oracle.knn_bruteforce(x, 10, select="tanimoto"))
    assert not np.array_equal(got[0], ext._knn_exact(x, 10)[0][0])


@pytest.mark.parametrize("n,d,k,margin", [(2000, 16, 10, None), (1200, 40, 15, 5), (900, 65, 8, None),
                                          (600, 300, 12, 12), (700, 7, 30, 0)])
def test_tanimoto_selection_shapes(ext, oracle, n, d, k, margin):
    # knn.rs:197-284 on the GPU: the FP32 pass with the coarse Tanimoto score (both the resident and
    # the chunked kernel), rescoring by T and its certificate; rows of very different norms
    rng = np.random.default_rng(n + 7 * d)
    means = rng.normal(0, 2, size=(6, d))
    x = (means[rng.integers(0, 6, n)] + rng.normal(0, 0.7, size=(n, d))) * rng.uniform(0.2, 5.0, size=(n, 1))
    x = np.ascontiguousarray(np.abs(x), dtype=np.float32)
    got, st = ext._knn_exact(x, k, select="tanimoto", margin=margin)
    same(as_oracle(got), oracle.knn_bruteforce(x, k, select="tanimoto"))


def test_tanimoto_selection_ties_take_the_regather(ext, oracle):
    # integer rows repeat exactly: equal Tanimoto scores everywhere, certificate failures, and the
    # regather filtered by the coarse Tanimoto score
    rng = np.random.default_rng(15)
    x = np.floor(rng.uniform(0, 3, size=(600, 5))).astype(np.float32)
    x[[3, 300]] = 0.0
    got, st = ext._knn_exact(x, 12, select="tanimoto")
    same(as_oracle(got), oracle.knn_bruteforce(x, 12, select="tanimoto"))
    assert st["fallback_rows"] > 0


@pytest.mark.parametrize("weight", ["tanimoto", "cosine", "jaccard"])
def test_reweight_bitwise(ext, oracle, weight):
    x = clustered(2000, 12, 8)
    idx, cos, norms = ext._knn_exact(x, 10)[0]
    np.testing.assert_array_equal(ext._reweight(idx, cos, norms, weight),
                                  oracle.reweight(idx.view(np.uint32), cos, norms, weight))


def test_reweight_rejects_out_of_range(ext):
    idx = np.array([[1, 2], [0, 5], [0, 1]], np.int32)
    with pytest.raises(ValueError, match="neighbor index 5 out of range"):
        ext._reweight(idx, np.zeros((3, 2)), np.ones(3), "tanimoto")


def test_fuzzy_union_bitwise(ext, oracle):
    x = clustered(3000, 16, 10)
    idx, cos, norms = ext._knn_exact(x, 10)[0]
    w = ext._reweight(idx, cos, norms, "tanimoto")
    got = ext._fuzzy_union(idx, w)
    want = oracle.fuzzy_union(idx.view(np.uint32), w)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b.astype(a.dtype) if a.dtype != np.float64 else b)


def test_fuzzy_union_edge_cases(ext, oracle):
    # self-loops, exact zeros, one-sided and two-sided pairs, a hub with a large in-degree
    rng = np.random.default_rng(0)
    n, k = 5000, 6
    idx = rng.integers(0, n, size=(n, k)).astype(np.int32)
    idx[:, 0] = np.arange(n)          # self-loops are dropped
    idx[::3, 1] = 7                   # node 7: in-degree > 1600 (the large-bucket sort path)
    for i in range(n):                # de-duplicate within rows (kNN rows hold distinct neighbours)
        row = list(dict.fromkeys(idx[i].tolist()))
        while len(row) < k:
            c = int(rng.integers(0, n))
            if c not in row:
                row.append(c)
        idx[i] = row
    w = rng.uniform(-0.3, 1.0, size=(n, k))
    w[rng.random((n, k)) < 0.05] = 0.0
    got = ext._fuzzy_union(idx, w)
    want = oracle.fuzzy_union(idx.view(np.uint32), w)
    np.testing.assert_array_equal(got[0], want[0].astype(np.int32))
    np.testing.assert_array_equal(got[1], want[1].astype(np.int32))
    np.testing.assert_array_equal(got[2], want[2])


@pytest.mark.parametrize("weight", ["tanimoto", "cosine", "jaccard"])
def test_fused_build_graph_equals_separate_calls(ext, weight):
    x = clustered(2500, 20, 11)
    (rows, cols, w), knn, st = ext._build_graph(x, 10, weight=weight, return_knn=True)
    idx, cos, norms = ext._knn_exact(x, 10)[0]
    same(knn, (idx, cos, norms))
    want = ext._fuzzy_union(idx, ext._reweight(idx, cos, norms, weight))
    same((rows, cols, w), want)


def test_golden_pipeline_digest_on_gpu(ext):
    # test_leiden_native.py:129-135 with the graph built on the GPU and Leiden on the host
    x = pipeline_input()
    (idx, cos, norms), _ = ext._knn_exact(x, 10, select="cosine")
    w = ext._reweight(idx, cos, norms, "tanimoto")
    rows, cols, ew = ext._fuzzy_union(idx, w)
    m = ext._leiden(len(x), rows, cols, ew, resolution=0.8, n_iterations=2, seed=3)[0]
    assert digest(m.astype(np.int64)) == GOLDEN_PIPELINE
    rows2, cols2, ew2 = ext._build_graph(x, 10)
    m2 = ext._leiden(len(x), rows2, cols2, ew2, resolution=0.8, n_iterations=2, seed=3)[0]
    assert digest(m2.astype(np.int64)) == GOLDEN_PIPELINE


def test_graph_csr_built_on_the_device(ext):
    # The Leiden's CSR (leiden.rs:52-101 of the union's edge list) built on the GPU: the same arrays
    # as the host construction, and the golden labels from the host Leiden run on it in place.
    x = pipeline_input()
    indptr, nbr, w = ext._build_graph_csr(x, 10)
    rows, cols, ew = ext._build_graph(x, 10)
    want = csr_from_edges(len(x), rows, cols, ew)
    for got, exp in zip((indptr, nbr, w), want):
        np.testing.assert_array_equal(got, exp)
    m = ext._leiden_csr(len(x), indptr, nbr, w, resolution=0.8, n_iterations=2, seed=3)[0]
    assert digest(m.astype(np.int64)) == GOLDEN_PIPELINE
    # hubs: two centres, each the nearest neighbour of the ~6,000 rows around it (rows of the CSR
    # longer than one warp's bucket sort and than one shared-memory run of the large-bucket sort)
    rng = np.random.default_rng(8)
    d = 64
    u = rng.normal(size=(12000, d))
    side = np.arange(12000) % 2
    u[np.arange(12000), side] = 0.0  # spokes orthogonal to their centre e_0 or e_1
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    pts = np.eye(d)[side] + 0.3 * u
    x = np.ascontiguousarray(np.vstack([np.eye(d)[:2], pts]), dtype=np.float32)
    for matmul in ("gemm", "bf16"):
        indptr, nbr, w = ext._build_graph_csr(x, 15, matmul=matmul)
        rows, cols, ew = ext._build_graph(x, 15, matmul=matmul)
        want = csr_from_edges(len(x), rows, cols, ew)
        assert np.diff(want[0].astype(np.int64)).max() > 4096
        for got, exp in zip((indptr, nbr, w), want):
            np.testing.assert_array_equal(got, exp)


def test_golden_fixtures(ext):
    from pathlib import Path

    for f in sorted(p for p in (Path(__file__).parent / "golden").glob("*.npz") if not p.name.startswith("dropin")):
        z = np.load(f)
        (idx, cos, norms), st = ext._knn_exact(z["x"], int(z["k"]), margin=int(z["margin"]))
        np.testing.assert_array_equal(idx, z["idx"].view(np.int32))
        np.testing.assert_array_equal(cos, z["cos"])
        np.testing.assert_array_equal(norms, z["norms"])
        w = ext._reweight(idx, cos, norms, "tanimoto")
        np.testing.assert_array_equal(w, z["w"])
        r, c, v = ext._fuzzy_union(idx, w)
        np.testing.assert_array_equal(r, z["rows"].view(np.int32))
        np.testing.assert_array_equal(c, z["cols"].view(np.int32))
        np.testing.assert_array_equal(v, z["ew"])


def test_input_validation(ext):
    # test_knn.py:151-171 (through the module surface)
    x = clustered(50, 4, 7)
    with pytest.raises(ValueError, match="invalid k=50"):
        ext._knn_exact(x, 50)
    with pytest.raises(ValueError, match="invalid k=0"):
        ext._knn_exact(x, 0)
    bad = x.copy()
    bad[3, 1] = np.nan
    with pytest.raises(ValueError, match="row 3 contains NaN"):
        ext._knn_exact(bad, 5)
    bad[3, 1] = np.inf
    with pytest.raises(ValueError, match="NaN or inf"):
        ext._knn_bruteforce(bad, 5)
    # the context stays usable after an input error
    same(as_oracle(ext._knn_exact(x, 5)[0]), as_oracle(ext._knn_bruteforce(x, 5)))


def test_row_l2_norms(ext):
    # test_smoke.py:18-26
    rng = np.random.default_rng(0)
    x = rng.standard_normal((257, 33), dtype=np.float32)
    got = ext.row_l2_norms(x)
    assert got.dtype == np.float32 and got.shape == (257,)
    np.testing.assert_allclose(got, np.linalg.norm(x, axis=1), rtol=1e-5, atol=1e-5)


# ---- the benchmark workloads -------------------------------------------------------------------

def test_mixture_20k_full_parity_and_labels(ext, oracle):
    """Config 1 (20,000 × 32, k = 10): the whole kNN, weights, graph and Leiden labels."""
    from costal_gb300 import workloads as W

    x, wl = W.make("mixture_20k")
    (idx, cos, norms), st = ext._knn_exact(x, wl.k)
    want, _ = oracle.knn_exact(x, wl.k)
    same(as_oracle((idx, cos, norms)), want)
    rows, cols, w = ext._build_graph(x, wl.k)
    ow = oracle.reweight(want[0], want[1], want[2], "tanimoto")
    orows, ocols, oew = oracle.fuzzy_union(want[0], ow)
    np.testing.assert_array_equal(rows, orows.view(np.int32))
    np.testing.assert_array_equal(cols, ocols.view(np.int32))
    np.testing.assert_array_equal(w, oew)
    m = ext._leiden(len(x), rows, cols, w, resolution=0.8, n_iterations=2, seed=0)[0]
    mo = ext._leiden(len(x), orows.view(np.int32), ocols.view(np.int32), oew, resolution=0.8, n_iterations=2, seed=0)[0]
    np.testing.assert_array_equal(m, mo)


def check_invariants(idx, cos):
    """Every row: no self, distinct neighbours, sorted by (cos desc, index asc)."""
    n = len(idx)
    assert not (idx == np.arange(n)[:, None]).any()
    d = np.diff(cos, axis=1)
    assert (d <= 0).all()
    assert (np.diff(idx, axis=1)[d == 0] > 0).all()
    assert (np.diff(np.sort(idx, axis=1), axis=1) > 0).all()


_FULL_ORACLE = {}


def full_oracle(oracle, name):
    """The oracle's whole answer for a workload (kNN, Tanimoto weights, fuzzy-union edges), computed once."""
    if name not in _FULL_ORACLE:
        from costal_gb300 import workloads as W

        x, wl = W.make(name)
        (oidx, ocos, onorms), _ = oracle.knn_exact(x, wl.k, margin=wl.margin)
        ow = oracle.reweight(oidx, ocos, onorms, "tanimoto")
        _FULL_ORACLE[name] = (x, wl, (oidx, ocos, onorms), oracle.fuzzy_union(oidx, ow))
    return _FULL_ORACLE[name]


@pytest.mark.timeout(1800)
@pytest.mark.parametrize("name", ["rare_400k", "dense_dup_160k"])
@pytest.mark.parametrize("backend", ["fp32", "bf16"])
def test_full_size_whole_output_parity(ext, oracle, name, backend):
    """Configs 2 and 3 at full size (400,000 x 15 with its 400-cell rare population, k = 10, m = 8;
    160,000 x 32 with 1% exact duplicates, k = 30, m = 30): every row's neighbours, cosines and norms,
    every Tanimoto weight and every fuzzy-union edge equal the oracle's, bit for bit."""
    x, wl, want, wedges = full_oracle(oracle, name)
    (idx, cos, norms), st = ext._knn_exact(x, wl.k, margin=wl.margin, matmul=backend)
    same(as_oracle((idx, cos, norms)), want)
    check_invariants(idx, cos)
    rows, cols, w = ext._build_graph(x, wl.k, margin=wl.margin, matmul=backend)
    np.testing.assert_array_equal(rows.view(np.uint32), wedges[0])
    np.testing.assert_array_equal(cols.view(np.uint32), wedges[1])
    np.testing.assert_array_equal(w, wedges[2])
    print(f"{name} {backend}: {len(x)} rows, {len(w)} edges identical; recomputed {st['recomputed_rows']}, "
          f"regathered {st['fallback_rows']}, max err / bound {st['max_err_ratio']:.3g}")


@pytest.mark.timeout(1800)
@pytest.mark.parametrize("name,rows", [("zipf_2m", 20_000), ("scrna_100k", 2_000)])
@pytest.mark.parametrize("backend", ["fp32", "bf16"])
def test_full_size_row_sample_parity(ext, oracle, name, rows, backend):
    """Configs 5 and 4 at full size: the GPU answer for a contiguous block of query rows (the rows are
    in seeded random order, so the block is a random sample; at 2,000,000 x 40 it holds rows of every
    one of the 50 Zipf components, the smallest included) equals the oracle's answer for those rows
    against all n columns, bit for bit; every row satisfies the output invariants; on the tensor-core
    path every row equals the plain FP32 path's."""
    from costal_gb300 import workloads as W

    wl = W.WORKLOADS[name]
    if name == "zipf_2m":
        x, labels = W.zipf_2m(seed=wl.seed, return_labels=True)
    else:
        x, labels = W.make(name)[0], None
    n = len(x)
    (idx, cos, norms), st = ext._knn_exact(x, wl.k, margin=wl.margin, matmul=backend)
    q0 = int(np.random.default_rng(wl.seed).integers(0, n - rows))
    if labels is not None:
        per = np.bincount(labels[q0:q0 + rows], minlength=50)
        assert per.min() >= 20, f"component sizes in the sample: {per}"
    (oidx, ocos, onorms), _ = oracle.knn_rows(x, wl.k, q0, q0 + rows, margin=wl.margin)
    np.testing.assert_array_equal(norms, onorms)
    np.testing.assert_array_equal(idx[q0:q0 + rows].view(np.uint32), oidx)
    np.testing.assert_array_equal(cos[q0:q0 + rows], ocos)
    check_invariants(idx, cos)
    if backend == "bf16":
        # every row, including those the tensor-core certificate sent to the FP32 re-run (merged over
        # column segments) or a learned skip sent back: the same answer as the plain FP32 path
        (fidx, fcos, _), _ = ext._knn_exact(x, wl.k, margin=wl.margin, matmul="fp32")
        np.testing.assert_array_equal(idx, fidx)
        np.testing.assert_array_equal(cos, fcos)
    print(f"{name} {backend}: {rows} of {n} rows against the oracle; max err / bound {st['max_err_ratio']:.3g}")


def adversarial_rows(kind, n, d, seed):
    """Inputs built against the split-BF16 accumulation bound.

    cancel: every row is one fixed magnitude profile with random signs, the profile's entries spread
            over 2^-14 .. 1, so each pair's products all have the same magnitudes (sum |products| is
            the whole squared norm) and cancel to cosines near 0, with a few near-copies for ties;
    spread: entries of random sign with exponents spread over 2^-24 .. 2^0 independently per entry;
    near:   tight clusters (cosines within 1e-6 of 1) whose rows differ in the last bits of their
            bf16 lo parts.
    """
    rng = np.random.default_rng(seed)
    if kind == "cancel":
        prof = np.exp2(-rng.uniform(0, 14, size=d))
        x = prof * rng.choice([-1.0, 1.0], size=(n, d))
        x[: n // 10] = x[n // 10: 2 * (n // 10)] * (1 + 1e-7 * rng.standard_normal((n // 10, 1)))
    elif kind == "spread":
        x = np.exp2(-rng.uniform(0, 24, size=(n, d))) * rng.choice([-1.0, 1.0], size=(n, d))
    else:
        base = rng.standard_normal((8, d))
        x = base[rng.integers(0, 8, n)] * (1 + 1e-6 * rng.standard_normal((n, d)))
    return np.ascontiguousarray(x, dtype=np.float32)


@pytest.mark.parametrize("d", [1, 8, 40, 41, 130, 2000])
@pytest.mark.parametrize("kind", ["cancel", "spread", "near"])
def test_certificate_bound_holds_on_adversarial_rows(ext, oracle, kind, d):
    """knn.rs:688-720: the certificate is sound only if |coarse - exact| never exceeds the bound it
    uses. On rows built to stress the split-BF16 tensor-core accumulation (large sum |products| with
    full cancellation, exponents spread across K, near-identical rows), the largest ratio of the two
    over every rescored candidate, as the device measured it, stays below 1 on both backends, and the
    answer equals the oracle's brute force."""
    n = 2000 if d < 2000 else 1200
    x = adversarial_rows(kind, n, d, 100 + d)
    want = oracle.knn_bruteforce(x, 10)
    for backend in ("bf16", "fp32", "fp8"):
        (idx, cos, norms), st = ext._knn_exact(x, 10, margin=54, matmul=backend)
        same(as_oracle((idx, cos, norms)), want)
        print(f"{kind} d={d} {backend}: max |coarse - exact| {st['max_coarse_err']:.3g}, "
              f"max ratio to the bound {st['max_err_ratio']:.3g}, recomputed {st['recomputed_rows']}")
        assert st["max_err_ratio"] < 1.0, st


@pytest.mark.parametrize("n,d,k,margin", [(5000, 16, 100, None), (3000, 60, 40, 40), (1500, 8, 150, None),
                                          (1200, 24, 300, 5)])
@pytest.mark.parametrize("backend", ["fp32", "bf16"])
def test_large_k_and_margin(ext, oracle, n, d, k, margin, backend):
    """knn.rs:449 accepts any 1 <= k <= n-1 with cap = min(k + m, n - 1): beyond the candidates the
    GPU coarse pass holds, the margin in effect shrinks (the output is the same) and for k >= 128 every
    candidate is scanned in f64; the answer equals the oracle's brute force bit for bit."""
    x = clustered(n, d, 40 + d)
    (idx, cos, norms), st = ext._knn_exact(x, k, margin=margin, matmul=backend)
    same(as_oracle((idx, cos, norms)), oracle.knn_bruteforce(x, k))
    assert st["margin"] <= (k if margin is None else margin)


@pytest.mark.parametrize("n,d,k,spread,signed", [(20_000, 12, 10, 8.0, False), (6000, 40, 15, 3.0, False),
                                                 (5000, 16, 10, 4.0, True), (3000, 64, 30, 6.0, False)])
def test_tanimoto_norm_window(ext, oracle, n, d, k, spread, signed):
    """knn.rs:595-644 on the GPU: with pruning on, each query block walks outward through the norm
    order and stops a side at the first tile outside every row's norm window. The answer equals the
    oracle's (and the pass without the window); on positive rows of widely spread norms tiles are
    skipped, and none with prune=False. Signed rows can have thresholds <= 0, where no window exists."""
    rng = np.random.default_rng(n + d)
    means = rng.normal(0, 2, size=(10, d))
    x = means[rng.integers(0, 10, n)] + rng.normal(0, 0.6, size=(n, d))
    if not signed:
        x = np.abs(x)
    x = x * np.exp(rng.uniform(0, np.log(spread), size=(n, 1)))
    x[:3] = 0.0  # zero rows: Tanimoto 0 with every row
    x = np.ascontiguousarray(x, dtype=np.float32)
    want = oracle.knn_bruteforce(x, k, select="tanimoto")
    got, st = ext._knn_exact(x, k, select="tanimoto")
    same(as_oracle(got), want)
    got0, st0 = ext._knn_exact(x, k, select="tanimoto", prune=False)
    same(as_oracle(got0), want)
    assert st0["blocks_skipped"] == 0
    print(f"n={n} d={d} spread={spread} signed={signed}: window skipped {st['blocks_skipped']} of "
          f"{st['blocks_total']} tiles, regathered {st['fallback_rows']}")
    if not signed and spread >= 6.0:
        assert st["blocks_skipped"] > 0.2 * st["blocks_total"], st


@pytest.mark.parametrize("d", [130, 512, 2000])
def test_split_fp8_kind(ext, oracle, d):
    """The split-FP8 kind (e4m3 pieces of the rows scaled by 2^8, kind::f8f6f4 MMAs, 64 candidates a
    row): on deep scRNA-like rows the answer equals the oracle's and the plain FP32 path's bit for
    bit, every rescored candidate's error stays inside its row's bound, and the default tensor-core
    backend picks this kind from d = 512 on."""
    from costal_gb300 import workloads as W

    x = W.scrna_100k(n=6000, d=d)
    want, _ = oracle.knn_exact(x, 15)
    (idx, cos, norms), st = ext._knn_exact(x, 15, matmul="fp8")
    same(as_oracle((idx, cos, norms)), want)
    assert st["coarse_kind"] == "fp8" and st["max_err_ratio"] < 1.0, st
    _, st_auto = ext._knn_exact(x, 15, matmul="bf16")
    assert st_auto["coarse_kind"] == ("fp8" if d >= 512 else "bf16")
    (i3, c3, _), st3 = ext._knn_exact(x, 15, matmul="bf16x3")
    same(as_oracle((i3, c3, norms)), want)
    assert st3["coarse_kind"] == "bf16"
    print(f"d={d}: fp8 recomputed {st['recomputed_rows']} of {len(x)} rows, max err / bound "
          f"{st['max_err_ratio']:.3g}, max err {st['max_coarse_err']:.3g}")


@pytest.mark.timeout(1800)
def test_early_stop_beyond_8192_column_blocks(ext):
    """2,200,000 rows of the Zipf generator: 8,594 column blocks of 256, past the 8,192 keys one list
    sort of 16 keys a thread holds; the lists are sorted with 32 keys a thread (up to 16,384 blocks),
    so the exact early stop still leaves blocks out, and every row equals the plain FP32 path's."""
    from costal_gb300 import workloads as W

    x = W.zipf_2m(n=2_200_000)
    (idx, cos, norms), st = ext._knn_exact(x, 10, matmul="bf16")
    assert st["blocks_stopped"] > 0.5 * st["blocks_total"], st
    (fidx, fcos, fnorms), _ = ext._knn_exact(x, 10, matmul="fp32")
    np.testing.assert_array_equal(idx, fidx)
    np.testing.assert_array_equal(cos, fcos)
    print(f"n=2,200,000: stopped {st['blocks_stopped']} of {st['blocks_total']} tiles")


def test_leiden_ensemble_on_the_device_graph(ext, oracle):
    """_leiden_many (lib.rs:311-350, the ensemble of find_communities_multiscale, _multiscale.py:170-175)
    fed the GPU-built graph, as an edge list and as the device-built CSR used in place: the labels of
    every (resolution, seed) run equal the ensemble's on the oracle's graph of the same input."""
    from costal_gb300 import workloads as W

    x, wl = W.make("mixture_20k")
    res, seeds = [0.2, 0.8, 1.6, 3.2], [0, 1, 2]
    (oidx, ocos, onorms), _ = oracle.knn_exact(x, wl.k)
    orows, ocols, ow = oracle.fuzzy_union(oidx, oracle.reweight(oidx, ocos, onorms, "tanimoto"))
    want = ext._leiden_many(len(x), orows.view(np.int32), ocols.view(np.int32), ow, resolutions=res, seeds=seeds)
    for matmul in ("fp32", "bf16"):
        rows, cols, w = ext._build_graph(x, wl.k, matmul=matmul)
        np.testing.assert_array_equal(ext._leiden_many(len(x), rows, cols, w, resolutions=res, seeds=seeds), want)
        indptr, nbr, cw = ext._build_graph_csr(x, wl.k, matmul=matmul)
        np.testing.assert_array_equal(ext._leiden_many_csr(len(x), indptr, nbr, cw, resolutions=res, seeds=seeds), want)
