"""The no-allocation Jaccard entry point, through the C ABI, against costal_reweight.

costal_reweight_jaccard_device_noalloc serves callers that hand the library device buffers but may not
let it allocate device memory (its scratch is a fixed array inside the library). This file is named
so that pytest collects it last: if it fails, a run that stops at the first failure has already run
every other test. It also passes alone in a fresh process.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ENTRIES = 4 << 20  # the fixed scratch holds this many neighbour entries


def call_noalloc(lib, d_idx, n, k, d_out, stream):
    err = C.create_string_buffer(512)
    rc = lib.costal_reweight_jaccard_device_noalloc(C.c_void_p(d_idx.data_ptr()), n, k,
                                                    C.c_void_p(d_out.data_ptr()), C.c_void_p(stream), err, 512)
    return rc, err.value.decode()


def knn_graph(ext, n, d, seed):
    rng = np.random.default_rng(seed)
    centers = rng.uniform(0, 4, size=(8, d))
    x = np.ascontiguousarray(centers[rng.integers(0, 8, n)] + rng.normal(0, 0.5, size=(n, d)), dtype=np.float32)
    return ext._knn_exact(x, 10)[0]


def test_noalloc_jaccard_matches_reweight_twice_in_a_row(ext):
    torch = pytest.importorskip("torch")
    from costal_gb300 import _lib as L

    lib = L.lib()
    stream = torch.cuda.current_stream().cuda_stream
    # two different inputs in a row: the second call must not see the first one's scratch contents
    for n, d, seed in ((5000, 12, 1), (3000, 20, 2)):
        idx, cos, norms = knn_graph(ext, n, d, seed)
        k = idx.shape[1]
        want = ext._reweight(idx, cos, norms, "jaccard")
        d_idx = torch.from_numpy(idx).cuda()
        d_out = torch.full((n, k), float("nan"), dtype=torch.float64, device="cuda")
        rc, msg = call_noalloc(lib, d_idx, n, k, d_out, stream)
        assert rc == 0, msg
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d_out.cpu().numpy(), want)


def test_noalloc_allocates_nothing_and_holds_its_stated_maximum(ext, oracle):
    """At n*k exactly the scratch's capacity the result equals the oracle's Jaccard (weight.rs:64-92),
    and the device's free memory does not move across calls: the library allocates nothing."""
    torch = pytest.importorskip("torch")
    from costal_gb300 import _lib as L

    lib = L.lib()
    stream = torch.cuda.current_stream().cuda_stream
    n, k = MAX_ENTRIES // 16, 16
    rng = np.random.default_rng(5)
    idx = rng.integers(0, n, size=(n, k), dtype=np.int32)
    want = oracle.reweight(idx.view(np.uint32), np.zeros((n, k)), np.ones(n), "jaccard")
    d_idx = torch.from_numpy(idx).cuda()
    d_out = torch.full((n, k), float("nan"), dtype=torch.float64, device="cuda")
    rc, msg = call_noalloc(lib, d_idx, n, k, d_out, stream)  # warm-up: the module is loaded by now
    assert rc == 0, msg
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        d_out.fill_(float("nan"))
        rc, msg = call_noalloc(lib, d_idx, n, k, d_out, stream)
        assert rc == 0, msg
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d_out.cpu().numpy(), want)
    assert torch.cuda.mem_get_info()[0] == free_before
    # one entry more than the scratch holds is refused before any device work
    rc, msg = call_noalloc(lib, d_idx, MAX_ENTRIES + 1, 1, d_out, stream)
    assert rc == L.COSTAL_EINVAL and "exceeds the fixed scratch" in msg
    # a product that would wrap around 64 bits is refused too, not taken for an empty input
    rc, msg = call_noalloc(lib, d_idx, 1 << 62, 4, d_out, stream)
    assert rc == L.COSTAL_EINVAL and "exceeds the fixed scratch" in msg


def test_noalloc_rejects_what_it_cannot_hold(ext):
    torch = pytest.importorskip("torch")
    from costal_gb300 import _lib as L

    lib = L.lib()
    stream = torch.cuda.current_stream().cuda_stream
    # beyond the fixed scratch: a clear error, before any device work (the buffers are never read)
    dummy = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc, msg = call_noalloc(lib, dummy, MAX_ENTRIES // 10 + 1, 10, dummy, stream)
    assert rc == L.COSTAL_EINVAL and "exceeds the fixed scratch" in msg
    # an index outside [0, n) is reported like costal_reweight reports it
    idx = np.array([[1, 2], [0, 5], [0, 1]], np.int32)
    d_idx = torch.from_numpy(idx).cuda()
    d_out = torch.empty((3, 2), dtype=torch.float64, device="cuda")
    rc, msg = call_noalloc(lib, d_idx, 3, 2, d_out, stream)
    assert rc == L.COSTAL_EINVAL and "neighbor index 5 out of range" in msg
