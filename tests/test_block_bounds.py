"""The per-row block bound of the tensor-core path, checked against f64 arithmetic on the same rows.

For a query block Q (128 working rows) and a column block B (128 working rows, unit centre c_B,
angular radius r_B), the device computes M = max over q in Q of the split-BF16 coarse score q.c_B
and its margin delta; the column lists then use cos(max(0, acos(M + delta) - r_B)) as an upper
bound of every cosine between a row of Q and a row of B (the early stop relies on it). Two checks:
|M - exact M| <= delta, and the bound above every exact block maximum. Shapes cover the three
operand layouts (3d-wide resident, compact, K loop), a ragged last query block and more than one
tile of centres.
"""

import numpy as np
import pytest

from conftest import clustered, scaled_clusters

pytestmark = pytest.mark.gpu


def _exact_block_max(w, nqb, ncb, cb):
    """max over (q in Q, x in B) of the exact cosine, from f64 unit rows in working order."""
    n = len(w)
    out = np.full((nqb, ncb), -np.inf)
    cstarts = np.arange(0, n, cb)
    for q0 in range(0, n, 1024):
        s = w[q0:q0 + 1024] @ w.T
        colmax = np.maximum.reduceat(s, cstarts, axis=1)  # rows x ncb
        qs = np.arange(0, len(s), 128)
        out[q0 // 128:q0 // 128 + len(qs)] = np.maximum.reduceat(colmax, qs, axis=0)
    return out


@pytest.mark.parametrize(
    "n,d,gen",
    [
        (3000, 8, clustered),          # 3d-wide, resident; ragged last query block (56 rows)
        (5000, 30, scaled_clusters),   # compact operands
        (4100, 40, clustered),         # 3d-wide, two K blocks
        (3000, 50, clustered),         # K-loop shape (3d > 128), streamed operands in the coarse pass
        (2600, 64, scaled_clusters),
        (16400, 16, clustered),        # 129 column blocks: a second tile of centres with one centre
    ],
)
def test_row_bound_holds(n, d, gen):
    from costal_gb300 import _costal as ext

    x = gen(n, d, 7)
    perm, cc, cr, rm, delta = ext._block_bounds(x)
    cb = ext.col_block_rows(n)
    assert cb == 128
    nqb, ncb = (n + 127) // 128, (n + cb - 1) // cb
    assert rm.shape == (nqb, ncb) and cc.shape == (ncb, d)
    assert sorted(perm.tolist()) == list(range(n))
    assert 0 < delta < 2e-4
    x64 = x.astype(np.float64)
    w = (x64 / np.linalg.norm(x64, axis=1, keepdims=True))[perm]
    # the coarse scores against the exact ones
    g = w @ cc.T
    m_exact = np.maximum.reduceat(g, np.arange(0, n, 128), axis=0)
    err = np.abs(rm.astype(np.float64) - m_exact)
    assert err.max() <= delta, (err.max(), delta)
    # the bound over every exact block maximum
    ub = np.cos(np.maximum(0.0, np.arccos(np.minimum(1.0, rm.astype(np.float64) + delta)) - cr[None, :]))
    exact = _exact_block_max(w, nqb, ncb, cb)
    assert (exact <= ub + 1e-12).all(), float((exact - ub).max())
