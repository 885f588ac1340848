"""Row shards across ranks (knn.rs:403-512's unit of work, a block of query rows against all columns),
tested on CPU ranks over gloo: each rank computes its shard of the rows with the oracle, the ranks
all-gather them through costal_gb300.shard.gather_rows, and every rank's whole graph (kNN, Tanimoto
weights, fuzzy-union edges) equals the single-process oracle's bit for bit."""

import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, n, d, k, margin, out):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import torch
    import torch.distributed as dist

    from conftest import clustered
    from costal_gb300 import shard as S
    from oracle import oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        x = clustered(n, d, 3)

        def compute(xt, k, shard, n_shards, margin=None, matmul=None):
            r0, r1 = S.shard_rows(len(xt), shard, n_shards)
            (idx, cos, norms), _ = O.knn_rows(xt.numpy(), k, r0, r1, margin=margin, n_threads=2)
            return {"rows": torch.arange(r0, r1, dtype=torch.int32), "idx": torch.from_numpy(idx.view(np.int32)),
                    "cos": torch.from_numpy(cos), "norms": torch.from_numpy(norms)}

        def weights(idx, cos, norms):
            return torch.from_numpy(O.reweight(idx.numpy().view(np.uint32), cos.numpy(), norms.numpy(), "tanimoto"))

        def union(idx, w):
            r, c, v = O.fuzzy_union(idx.numpy().view(np.uint32), w.numpy())
            return torch.from_numpy(r.view(np.int32)), torch.from_numpy(c.view(np.int32)), torch.from_numpy(v)

        (r, c, w), (idx, cos, norms), _ = S.build_graph_sharded(torch.from_numpy(x), k, margin=margin, compute=compute,
                                                               weights=weights, union=union)
        np.savez(out / f"rank{rank}.npz", rows=r.numpy(), cols=c.numpy(), w=w.numpy(), idx=idx.numpy(),
                 cos=cos.numpy(), norms=norms.numpy())
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_graph_equals_the_single_process_oracle(oracle, tmp_path, world):
    import torch.multiprocessing as mp

    from conftest import clustered

    n, d, k, margin = 2100, 12, 10, 10
    mp.start_processes(_rank_main, args=(world, _free_port(), n, d, k, margin, tmp_path), nprocs=world, join=True,
                       start_method="spawn")
    x = clustered(n, d, 3)
    (idx, cos, norms), _ = oracle.knn_exact(x, k, margin=margin)
    w = oracle.reweight(idx, cos, norms, "tanimoto")
    rows, cols, ew = oracle.fuzzy_union(idx, w)
    for rank in range(world):
        z = np.load(tmp_path / f"rank{rank}.npz")
        np.testing.assert_array_equal(z["idx"].view(np.uint32), idx)
        np.testing.assert_array_equal(z["cos"], cos)
        np.testing.assert_array_equal(z["norms"], norms)
        np.testing.assert_array_equal(z["rows"].view(np.uint32), rows)
        np.testing.assert_array_equal(z["cols"].view(np.uint32), cols)
        np.testing.assert_array_equal(z["w"], ew)


def test_shards_partition_the_rows():
    from costal_gb300 import shard as S

    for n in (1, 127, 128, 129, 1000, 2_000_000):
        for world in (1, 2, 3, 8, 64):
            spans = [S.shard_rows(n, s, world) for s in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert all(e - s <= S.rows_max(n, world) for s, e in spans)
            assert all(s % S.ROW_BLOCK == 0 for s, _ in spans)
