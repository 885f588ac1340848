"""bench.py's host logic on the CPU: the multi-rank side (gloo, two ranks: every rank reports the slowest
rank's time, and the job's throughput counts the cells of every replica) and the DRAM-traffic estimate
from the committed ncu captures. No GPU needed."""

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        ws, r, local = bench.dist_env()
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank)  # rank 1 is the slower one
        Path(outdir, f"rank{rank}").write_text(f"{ws} {r} {local} {slowest!r}")
    finally:
        dist.destroy_process_group()


def test_two_ranks_report_the_slowest_time(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    mp.spawn(_worker, args=(_free_port(), str(tmp_path)), nprocs=2, join=True)
    for rank in (0, 1):
        ws, r, local, slowest = Path(tmp_path, f"rank{rank}").read_text().split()
        assert (int(ws), int(r), int(local)) == (2, rank, rank)
        assert float(slowest) == 15.0
    del torch


def test_single_process_and_job_throughput():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(12.5) == 12.5  # no process group: the value itself
    # two replicas of 1,000 cells, the slower one in 15 ms: 2 · 1000 / 0.015 cells/s
    assert bench.job_cells_per_s(1000, 2, 15.0) == pytest.approx(2 * 1000 / 0.015)
    assert bench.job_cells_per_s(2_000_000, 1, 250.0) == pytest.approx(8_000_000.0)


def test_traffic_estimate_from_the_committed_captures():
    import json

    sys.path.insert(0, str(ROOT))
    import bench

    table = json.loads((ROOT / "profiles" / "dram_traffic.json").read_text())
    pairs = 1e9
    # resident tensor-core form (3d <= 128): bytes per computed pair
    assert bench.traffic_per_launch("bf16", pairs, 40) == pytest.approx(table["bf16"]["bytes_per_pair"] * pairs)
    # K loop (3d > 128): bytes per pair per padded K
    kp = (3 * 2000 + 63) // 64 * 64
    assert bench.traffic_per_launch("bf16", pairs, 2000) == pytest.approx(
        table["bf16_kloop"]["bytes_per_pair_per_k"] * kp * pairs)
    assert bench.traffic_per_launch("fp32", pairs, 40) == pytest.approx(table["fp32"]["bytes_per_pair"] * pairs)
    assert bench.traffic_per_launch("no-such-backend", pairs, 40) is None
