"""The host Leiden (leiden="fast", the consumer of the device graph): host C++ in libcostal_gb300,
no GPU needed. Restates the reference's tests/test_leiden_native.py and leiden.rs unit tests."""

import numpy as np
import pytest

from conftest import GOLDEN_GRAPH, csr_from_edges, digest, planted


def test_golden_graph_digest(ext):
    # test_leiden_native.py:129-131: the same bits as the reference on every platform
    n, rows, cols, w = planted(n_blocks=20, size=50, p_in=0.1, n_cross=2000, seed=11)
    m = ext._leiden(n, rows, cols, w, resolution=1.3, seed=12345)[0]
    assert digest(m) == GOLDEN_GRAPH


def test_recovers_planted_blocks_and_is_thread_independent(ext):
    # test_leiden_native.py:46-53
    n, rows, cols, w = planted(p_in=0.3)
    m, k, iterations, _ = ext._leiden(n, rows, cols, w, resolution=1.0, seed=0)
    assert k == 12 and iterations == 2
    assert all(len(np.unique(m[b * 40:(b + 1) * 40])) == 1 for b in range(12))
    for threads in (1, 2, 4):
        assert np.array_equal(ext._leiden(n, rows, cols, w, resolution=1.0, seed=5, n_threads=threads)[0],
                              ext._leiden(n, rows, cols, w, resolution=1.0, seed=5)[0])


def test_many_matches_single_runs(ext):
    # test_leiden_native.py:84-89
    n, rows, cols, w = planted(seed=4)
    many = ext._leiden_many(n, rows, cols, w, resolutions=[0.5, 1.0, 2.0], seeds=[0, 7])
    assert many.shape == (6, n)
    for i, (res, seed) in enumerate([(r, s) for r in (0.5, 1.0, 2.0) for s in (0, 7)]):
        assert np.array_equal(many[i], ext._leiden(n, rows, cols, w, resolution=res, seed=seed)[0])


def test_until_stable_and_bad_arguments(ext):
    # test_leiden_native.py:92-101
    n, rows, cols, w = planted(seed=6)
    m, _, iterations, converged = ext._leiden(n, rows, cols, w, resolution=1.0, n_iterations=-1, seed=0)
    assert converged and iterations >= 1
    with pytest.raises(ValueError, match="n_iterations"):
        ext._leiden(n, rows, cols, w, resolution=1.0, n_iterations=0)
    with pytest.raises(ValueError, match="resolution"):
        ext._leiden(n, rows, cols, w, resolution=-1.0)
    with pytest.raises(ValueError, match="out of range"):
        ext._leiden(n - 1, rows, cols, w, resolution=1.0)


def test_modularity_of_a_known_partition(ext):
    # leiden.rs:452-474 on a two-triangle graph: Q = 1/2 − 1/2 · γ · ... computed by hand
    rows = np.array([0, 0, 1, 3, 3, 4, 2], np.int32)
    cols = np.array([1, 2, 2, 4, 5, 5, 3], np.int32)
    w = np.ones(7)
    m = np.array([0, 0, 0, 1, 1, 1], np.int32)
    # 2m = 14; internal (both directions) = 12; strengths: 2,2,3,3,2,2 -> K_c = 7, 7
    q = ext._modularity(6, rows, cols, w, m, 1.0)
    assert q == pytest.approx(12 / 14 - (49 + 49) / 196, abs=1e-15)


def test_coo_forms_and_errors(ext):
    # leiden.rs:1569-1600: each edge once in either orientation, or a symmetric list; errors otherwise
    u = lambda a: np.array(a, np.uint32)  # noqa: E731
    f = lambda a: np.array(a, np.float64)  # noqa: E731
    base = dict(objective="modularity", resolution=1.0, beta=0.01, n_iterations=2, seed=1)
    once = ext._leiden_coo(4, u([0, 2, 1]), u([1, 1, 3]), f([0.5, 1.0, 0.25]), **base)
    both = ext._leiden_coo(4, u([0, 1, 2, 1, 1, 3]), u([1, 0, 1, 2, 3, 1]), f([0.5, 0.5, 1.0, 1.0, 0.25, 0.25]), **base)
    upper = ext._leiden_coo(4, u([0, 1, 1]), u([1, 2, 3]), f([0.5, 1.0, 0.25]), **base)
    assert np.array_equal(once[0], upper[0]) and np.array_equal(both[0], upper[0])
    assert once[1] == upper[1] == both[1]
    err = lambda r, c, w: ext._leiden_coo(3, u(r), u(c), f(w), **base)  # noqa: E731
    for (r, c, w), msg in [
        (([0, 0], [1, 1], [1.0, 1.0]), "same direction"),
        (([0, 1], [1, 0], [1.0, 2.0]), "different weights"),
        (([0, 1, 1], [1, 0, 2], [1.0, 1.0, 1.0]), "others once"),
        (([0], [0], [1.0]), "self-loop"),
        (([0], [3], [1.0]), "out of range"),
        (([0], [1], [np.nan]), "weight"),
        (([0], [1], [-1.0]), "weight"),
    ]:
        with pytest.raises(ValueError, match=msg):
            err(r, c, w)


def test_cpm_quality_matches_its_definition(ext):
    # leiden.rs:1602-1620: Σ_c [2 w_c − γ n_c (n_c − 1)]
    edges = [(0, 1, 0.3), (0, 2, 0.9), (1, 2, 0.4), (2, 3, 0.2), (3, 4, 0.7), (3, 5, 0.6), (4, 5, 0.8)]
    r = np.array([e[0] for e in edges], np.uint32)
    c = np.array([e[1] for e in edges], np.uint32)
    w = np.array([e[2] for e in edges])
    init = np.array([0, 0, 0, 1, 1, 1], np.uint32)
    labels, q, *_ = ext._leiden_coo(6, r, c, w, objective="cpm", resolution=0.1, beta=0.01, n_iterations=1, seed=0,
                                    initial=init)
    sizes = np.bincount(labels)
    internal = sum(x for a, b, x in edges if labels[a] == labels[b])
    assert q == pytest.approx(2 * internal - 0.1 * float((sizes * (sizes - 1)).sum()), abs=1e-12)


def test_csr_entry_matches_the_edge_list_and_checks_its_input(ext):
    # the same Leiden on the graph given as its CSR (the GPU-built layout), used in place
    n, rows, cols, w = planted(n_blocks=20, size=50, p_in=0.1, n_cross=2000, seed=11)
    indptr, nbr, cw = csr_from_edges(n, rows, cols, w)
    m = ext._leiden_csr(n, indptr, nbr, cw, resolution=1.3, seed=12345)[0]
    assert digest(m) == GOLDEN_GRAPH
    for seed in (0, 7):
        a = ext._leiden(n, rows, cols, w, resolution=0.9, seed=seed)
        b = ext._leiden_csr(n, indptr, nbr, cw, resolution=0.9, seed=seed)
        assert np.array_equal(a[0], b[0]) and a[1:] == b[1:]
    bad = indptr.copy()
    bad[0] = 1
    with pytest.raises(ValueError, match="indptr"):
        ext._leiden_csr(n, bad, nbr, cw, resolution=1.0)
    bad = indptr.copy()
    bad[5], bad[6] = bad[6], bad[5]
    with pytest.raises(ValueError, match="decreases"):
        ext._leiden_csr(n, bad, nbr, cw, resolution=1.0)
    for v in (np.uint32(n), np.uint32(0)):  # out of range; a self-loop on row 0
        nb = nbr.copy()
        nb[0] = v
        with pytest.raises(ValueError, match="neighbour"):
            ext._leiden_csr(n, indptr, nb, cw, resolution=1.0)
    ww = cw.copy()
    ww[3] = 0.0
    with pytest.raises(ValueError, match="positive"):
        ext._leiden_csr(n, indptr, nbr, ww, resolution=1.0)
    with pytest.raises(ValueError, match="entries"):
        ext._leiden_csr(n + 1, indptr, nbr, cw, resolution=1.0)


def test_many_on_a_csr_matches_the_edge_list(ext):
    """The ensemble of lib.rs:311-350 on a graph given as the Leiden's CSR (leiden.rs:52-101 of the
    edge list, as the GPU builds it), used in place: the same labels as on the edge list."""
    n, rows, cols, w = planted(seed=4)
    many = ext._leiden_many(n, rows, cols, w, resolutions=[0.5, 1.0, 2.0], seeds=[0, 7])
    indptr, nbr, cw = csr_from_edges(n, rows, cols, w)
    got = ext._leiden_many_csr(n, indptr, nbr, cw, resolutions=[0.5, 1.0, 2.0], seeds=[0, 7])
    np.testing.assert_array_equal(got, many)
