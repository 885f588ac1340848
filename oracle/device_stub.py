"""TEST INFRASTRUCTURE ONLY — the library's device entry points answered by the CPU oracle.

`DeviceStub` stands in for the loaded libcostal_gb300 object behind costal_gb300._lib.lib() on a
machine without a GPU. The entry points that run on the GPU in the product (`costal_knn_exact`,
`costal_knn_bruteforce`, `costal_reweight`, `costal_fuzzy_union`, `costal_row_l2_norms`) are
answered by the oracle's restatement of the reference (knn.rs, weight.rs, graph.rs), with the same
pointer arguments, status codes and messages as the C ABI (include/costal_gb300.h); every other entry
point (the host Leiden, versions) is the real library's. With it installed, the whole Python layer of
costal_gb300._costal runs unchanged on the CPU, which is how tests/golden/make_dropin.py records what
the reference's own Python package asks of `costal._costal`. It is never used by the product, and the
replay of that record on a GB300 goes through the real library.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import oracle as O

OK, EINVAL = 0, 2
_SELECT = {0: "cosine", 1: "tanimoto"}
_WEIGHT = {0: "tanimoto", 1: "cosine", 2: "jaccard"}


def _view(ptr, ctype, shape):
    """A numpy view of `shape` elements of `ctype` at the address held by a c_void_p (or int)."""
    addr = ptr.value if isinstance(ptr, C.c_void_p) else int(ptr)
    count = int(np.prod(shape)) if len(shape) else 1
    if count == 0:
        return np.empty(shape, np.dtype(ctype))
    return np.ctypeslib.as_array((ctype * count).from_address(addr)).reshape(shape)


def _obj(ref):
    """The ctypes object behind C.byref(obj)."""
    return getattr(ref, "_obj", ref)


def _fail(err, errlen, msg, rc=EINVAL):
    err.value = msg.encode()[: max(0, int(errlen) - 1)]
    return rc


class DeviceStub:
    """Device entry points on the oracle; everything else forwarded to the real library."""

    def __init__(self, real):
        self._real = real

    def __getattr__(self, name):
        return getattr(self._real, name)

    def costal_row_l2_norms(self, x, n, d, out, err, errlen):
        xs = _view(x, C.c_float, (n, d))
        _view(out, C.c_float, (n,))[:] = O.row_l2_norms(xs)
        return OK

    def costal_knn_exact(self, x, n, d, k, opts, idx, cos, norms, stats, err, errlen):
        o = _obj(opts)
        margin = None if o.margin == 0xFFFFFFFF else int(o.margin)
        try:
            (i, c, nm), st = O.knn_exact(_view(x, C.c_float, (n, d)), k, margin=margin, select=_SELECT[o.select])
        except ValueError as e:
            return _fail(err, errlen, str(e))
        _view(idx, C.c_uint32, (n, k))[:] = i
        _view(cos, C.c_double, (n, k))[:] = c
        _view(norms, C.c_double, (n,))[:] = nm
        s = _obj(stats)
        s.fallback_rows = st["fallback_rows"]
        s.row_block, s.col_block = st["row_block"], st["col_block"]
        s.blocks_skipped, s.blocks_total = st["blocks_skipped"], st["blocks_total"]
        s.margin = k if margin is None else margin
        return OK

    def costal_knn_bruteforce(self, x, n, d, k, select, idx, cos, norms, err, errlen):
        try:
            i, c, nm = O.knn_bruteforce(_view(x, C.c_float, (n, d)), k, select=_SELECT[select])
        except ValueError as e:
            return _fail(err, errlen, str(e))
        _view(idx, C.c_uint32, (n, k))[:] = i
        _view(cos, C.c_double, (n, k))[:] = c
        _view(norms, C.c_double, (n,))[:] = nm
        return OK

    @staticmethod
    def _check_idx(ix, n, err, errlen):
        """lib.rs:66-75: every neighbour index must lie in [0, n)."""
        bad = ix[(ix < 0) | (ix >= n)]
        if bad.size:
            return _fail(err, errlen, f"neighbor index {int(bad[0])} out of range (n={n})")
        return OK

    def costal_reweight(self, n, k, idx, cos, norms, weight, out, err, errlen):
        ix = _view(idx, C.c_int32, (n, k))
        if self._check_idx(ix, n, err, errlen):
            return EINVAL
        w = O.reweight(ix.view(np.uint32), _view(cos, C.c_double, (n, k)), _view(norms, C.c_double, (n,)),
                       _WEIGHT[weight])
        _view(out, C.c_double, (n, k))[:] = w
        return OK

    def costal_fuzzy_union(self, n, k, idx, w, rows, cols, wout, m, err, errlen):
        ix = _view(idx, C.c_int32, (n, k))
        if self._check_idx(ix, n, err, errlen):
            return EINVAL
        r, c, ww = O.fuzzy_union(ix.view(np.uint32), _view(w, C.c_double, (n, k)))
        e = len(ww)
        _view(rows, C.c_uint32, (e,))[:] = r
        _view(cols, C.c_uint32, (e,))[:] = c
        _view(wout, C.c_double, (e,))[:] = ww
        _obj(m).value = e
        return OK


def install():
    """Put the stub behind costal_gb300._lib.lib(); returns a function that takes it out again."""
    from costal_gb300 import _lib as L

    real = L.lib()
    L._lib = DeviceStub(real)

    def remove():
        L._lib = real

    return remove
