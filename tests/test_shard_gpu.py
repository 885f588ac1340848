"""Row shards on the GPU, through the C ABI (costal_knn_shard_device, costal_fuzzy_union_device).

One GPU computes every shard of a split in turn (no shard waits on another); the shards' rows must
partition the rows, each shard's neighbours must equal the same rows of the whole-input answer bit
for bit (on the plain FP32 path the shards are the input-order blocks; on the tensor-core path,
blocks of the locality order), and the fuzzy union of the assembled kNN must equal the one-call graph.
"""

import numpy as np
import pytest

from conftest import clustered

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("backend", ["fp32", "bf16"])
@pytest.mark.parametrize("n,world", [(30_000, 1), (30_000, 3), (30_000, 8), (300, 4)])
def test_shards_assemble_to_the_whole_graph(ext, backend, n, world):
    import torch

    from costal_gb300 import shard as S

    k, margin = 10, 10
    x = clustered(n, 24, 11)
    (widx, wcos, wnorms), _ = ext._knn_exact(x, k, margin=margin, matmul=backend)
    erows, ecols, ew = ext._build_graph(x, k, margin=margin, matmul=backend)
    xd = torch.from_numpy(x).cuda()
    idx = np.full((n, k), -1, np.int32)
    cos = np.zeros((n, k))
    w = np.zeros((n, k))
    seen = np.zeros(n, np.int64)
    for s in range(world):
        part = S.shard_device(xd, k, s, world, margin=margin, matmul=backend)
        rows = part["rows"].cpu().numpy()
        assert len(rows) <= S.rows_max(n, world)
        if backend == "fp32":
            r0, r1 = S.shard_rows(n, s, world)
            np.testing.assert_array_equal(rows, np.arange(r0, r1))
        seen[rows] += 1
        idx[rows] = part["idx"].cpu().numpy()
        cos[rows] = part["cos"].cpu().numpy()
        w[rows] = part["w"].cpu().numpy()
        np.testing.assert_array_equal(part["norms"].cpu().numpy(), wnorms)
    assert (seen == 1).all()
    np.testing.assert_array_equal(idx, widx)
    np.testing.assert_array_equal(cos, wcos)
    np.testing.assert_array_equal(w, ext._reweight(widx, wcos, wnorms, "tanimoto"))
    r, c, v = S.union_device(torch.from_numpy(idx).cuda(), torch.from_numpy(w).cuda())
    np.testing.assert_array_equal(r.cpu().numpy(), erows)
    np.testing.assert_array_equal(c.cpu().numpy(), ecols)
    np.testing.assert_array_equal(v.cpu().numpy(), ew)


def test_device_union_rejects_bad_indices(ext):
    import torch

    from costal_gb300 import shard as S

    idx = torch.tensor([[1, 2], [0, 7], [0, 1]], dtype=torch.int32, device="cuda")
    w = torch.ones((3, 2), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError, match="neighbor index 7 out of range"):
        S.union_device(idx, w)


@pytest.mark.parametrize("backend", ["fp32", "bf16"])
def test_sharded_build_through_nccl_on_one_rank(ext, backend):
    """The multi-GPU step as bench.py and a user run it (shard, NCCL all-gather, device union) in a
    one-rank process group: the same edges and kNN as the one-call graph."""
    import socket

    import torch
    import torch.distributed as dist

    from costal_gb300 import shard as S

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        x = clustered(20_000, 24, 5)
        (r, c, w), (idx, cos, norms), _ = S.build_graph_sharded(torch.from_numpy(x).cuda(), 10, matmul=backend)
        er, ec, ew = ext._build_graph(x, 10, matmul=backend)
        np.testing.assert_array_equal(r.cpu().numpy(), er)
        np.testing.assert_array_equal(c.cpu().numpy(), ec)
        np.testing.assert_array_equal(w.cpu().numpy(), ew)
        (widx, wcos, wnorms), _ = ext._knn_exact(x, 10, matmul=backend)
        np.testing.assert_array_equal(idx.cpu().numpy(), widx)
        np.testing.assert_array_equal(cos.cpu().numpy(), wcos)
    finally:
        dist.destroy_process_group()
