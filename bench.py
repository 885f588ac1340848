"""Benchmark: exact kNN-graph cells/s on one GB300 (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--backend bf16|fp32]
    python bench.py --impl reference ...      # the CPU implementation of the path on the host cores

Default workload: 2,000,000 × 40 f32, 50 clusters with Zipf(1.2) sizes, arcsinh(x/5), k = 10, m = 10
(the learned-prune configuration), certified split-BF16 tensor-core coarse pass with learned block
pruning, against the plain FP32 GPU path on the same input.

A step is one pass of the hot path over one batch: X (n × d f32) -> norms, normalised tiles, top-(k+m)
selection, f64 rescoring + certificate (+ recomputation / regather), Tanimoto weights, fuzzy-union
edge list. With the learned backend the step also includes the k-means locality order, the model's
inference and the block lists; the model itself is trained once before timing (reported as `train`).

  value  — n / step time with X already resident in HBM (CUDA events on the launching stream, L2
           flushed between steps by writing a 512 MB buffer outside the timed events);
  e2e    — the same through the host C-ABI call costal_build_graph: pinned host X in, pinned host
           edge list out, copies inside the timed region (wall clock around the synchronous call);
  plain_fp32 — the plain FP32 GPU path on the same input (device-resident, same timing);
  without_learned — the certified BF16 path with the exact early stop but no learned threshold;
  roofline — the dominant kernel (the coarse tile + selection kernel): algorithmic FLOP/s (2·d per
           visited pair: pairs of the tiles neither skipped by the learned threshold nor left out by
           the exact early stop) over its CUDA-event duration;
  cpu_baseline — the oracle (C++ restatement of the reference's CPU path) on a bounded sample of
           query rows, all host threads.

Multi-GPU (torchrun, N > 1): the rows are split across the ranks (costal_gb300.shard): every rank
holds all of X, computes its shard of the query rows against every column, the ranks all-gather the
shards' neighbours, cosines and weights over NCCL, and every rank builds the fuzzy union; the total
work is fixed at n ("strong" scaling) and value = n / the slowest rank's step time.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "exact kNN-graph cells/s, certified BF16+learned prune vs plain FP32, one GB300"
L2_FLUSH_BYTES = 512 << 20


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [s.strip() for s in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for name, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def traffic_per_launch(backend, pairs, d):
    """DRAM bytes (read + write) per launch of the dominant kernel: bytes per computed pair from the
    committed ncu capture summaries (profiles/dram_traffic.json), times this launch's computed pairs;
    for the tensor-core K loop (3d > 128) per pair and per padded K. None without a capture."""
    p = ROOT / "profiles" / "dram_traffic.json"
    if not p.exists():
        return None
    table = json.loads(p.read_text())
    if backend == "bf16" and 3 * d > 128:
        rec = table.get("bf16_kloop")
        return rec["bytes_per_pair_per_k"] * ((3 * d + 63) // 64 * 64) * pairs if rec else None
    rec = table.get(backend)
    return rec["bytes_per_pair"] * pairs if rec else None


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, device="cpu"):
    """The largest x over all ranks of the initialised process group (a job's time is its slowest
    rank's); x itself without one. Every rank must call it."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_cells_per_s(n, ws, ms):
    """Whole-job throughput: ws graphs of n cells each built in (at most) ms; the sharded benchmark
    builds one graph of n cells across all ranks (ws = 1)."""
    return ws * n / (ms / 1e3)


def cpu_baseline(x, wl, target_s=15.0, threads=0):
    """The oracle's blocked CPU path on a bounded sample of query rows against all n columns, sized
    to about `target_s` seconds of CPU work. Returns (cells/s, cores, sample description)."""
    from oracle import oracle as O

    n = len(x)
    cores = threads or O.max_threads()
    probe = max(64, min(n, 256))
    t = time.perf_counter()
    O.knn_rows(x, wl.k, 0, probe, margin=wl.margin, n_threads=cores)
    dt = time.perf_counter() - t
    rows = probe
    for _ in range(3):  # grow the sample until it takes at least half the target time (or covers n)
        rows = max(64, int(min(n, max(probe, rows * target_s / max(dt, 1e-6)))))
        q0 = (n - rows) // 2
        t = time.perf_counter()
        O.knn_rows(x, wl.k, q0, q0 + rows, margin=wl.margin, n_threads=cores)
        dt = time.perf_counter() - t
        if dt >= 0.5 * target_s or rows >= n:
            break
    return rows / dt, cores, f"{rows} query rows x all {n} columns (kNN incl. f64 rescoring), {dt:.1f} s"


def cpu_crosscheck(x, wl, sampled, args):
    """The CPU port on one thread (a sample of rows), and in full on 200,000- and 400,000-row draws of
    the same generator, extrapolated by n^2 to the workload's n: a check of the sampled all-core
    figure."""
    from costal_gb300 import workloads as W
    from oracle import oracle as O

    v1, _, s1 = cpu_baseline(x, wl, target_s=args.cpu_seconds, threads=1)
    full = {}
    for m in (200_000, 400_000):
        xm = W.make(wl.name, n=m)[0]
        t = time.perf_counter()
        O.knn_exact(xm, wl.k, margin=wl.margin)
        full[m] = time.perf_counter() - t
    est = {m: full[m] * (wl.n / m) ** 2 for m in full}
    return {"one_core_value": v1, "one_core_sample": s1,
            "full_runs_s": {str(m): full[m] for m in full},
            "extrapolated_s_at_n": {str(m): est[m] for m in est},
            "extrapolated_cells_per_s": {str(m): wl.n / est[m] for m in est},
            "sampled_cells_per_s": sampled}


def _hubs(spokes, d=64, seed=8):
    """Two centres, each the nearest neighbour of half the spokes (long rows in the Leiden CSR)."""
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(spokes, d))
    side = np.arange(spokes) % 2
    u[np.arange(spokes), side] = 0.0
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    return np.ascontiguousarray(np.vstack([np.eye(d)[:2], np.eye(d)[side] + 0.3 * u]), dtype=np.float32)


def _profile_case(name):
    from costal_gb300 import _costal as ext
    from costal_gb300 import workloads as W

    if name in ("coarse_fp32_kc", "split_wide", "coarse_tc_fp8"):
        x = W.scrna_100k(n=20_000)
        matmul = {"coarse_fp32_kc": "fp32", "split_wide": "bf16x3", "coarse_tc_fp8": "fp8"}[name]
        return [lambda: ext._knn_exact(x, 15, matmul=matmul)[1]]
    if name == "gather":  # integer rows: ties everywhere, every row regathered
        x = np.floor(np.random.default_rng(5).uniform(0, 3, size=(50_000, 6))).astype(np.float32)
        return [lambda: ext._knn_exact(x, 12)[1]]
    if name == "merge_parts":  # 300 near-identical rows fail the split-BF16 certificate
        x = W.mixture_20k(n=200_000, d=16)
        rng = np.random.default_rng(9)
        base = rng.uniform(0, 1, size=(1, 16))
        x[:300] = (base * (1 + 1e-6 * rng.standard_normal((300, 16)))).astype(np.float32)
        return [lambda: ext._knn_exact(np.ascontiguousarray(x), 10, matmul="bf16")[1]]
    if name == "tanimoto_window":
        x, wl = W.make("rare_400k", n=200_000)
        return [lambda: ext._knn_exact(x, wl.k, margin=wl.margin, select="tanimoto")[1]]
    if name == "jaccard":
        x = W.mixture_20k(n=400_000)
        idx, cos, norms = ext._knn_exact(x, 10)[0]
        return [lambda: {"shape": ext._reweight(idx, cos, norms, "jaccard").shape}]
    if name == "csr":
        x = _hubs(12_000)
        return [lambda: {"nnz": len(ext._build_graph_csr(x, 15)[1])}]
    raise ValueError(name)


PROFILE_CASES = {
    "coarse_fp32_kc": "k_coarse_fp32_kc: the FP32 pass for deep rows (20,000 x 2,000 scRNA-like)",
    "split_wide": "k_split_wide: the split-BF16 operands of deep rows (20,000 x 2,000)",
    "coarse_tc_fp8": "k_coarse_tc<.., FP8>: the split-FP8 tensor-core pass (20,000 x 2,000)",
    "gather": "k_gather: the full-row regather (50,000 x 6 integer rows)",
    "merge_parts": "k_merge_parts: column-segment lists of re-run rows merged (200,000 x 16, 300 near-copies)",
    "tanimoto_window": "k_coarse_tani_window: Tanimoto selection with the norm window (200,000 x 15)",
    "jaccard": "k_sort_rows + k_jaccard: Jaccard weights (400,000 x 10 neighbours)",
    "csr": "k_sort_big + k_csr_emit: the Leiden CSR with two hub rows of ~6,000 entries",
}


def run_profile_case(name):
    calls = _profile_case(name)
    for _ in range(2):
        out = calls[0]()
    keep = ("coarse_kind", "recomputed_rows", "fallback_rows", "blocks_skipped", "blocks_total", "ms_kernel")
    print(json.dumps({"profile_case": name, "what": PROFILE_CASES[name],
                      "result": {k_: v for k_, v in out.items() if k_ in keep or k_ in ("shape", "nnz")}}))


def run_reference(args, wl, x):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O

    cores = O.max_threads()
    vals = []
    sample = None
    for step in range(args.warmup + args.steps):
        v, cores, sample = cpu_baseline(x, wl, target_s=args.ref_seconds, threads=cores)
        if step >= args.warmup:
            vals.append(v)
    v = float(np.median(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wl.n / v * 1e3, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f32 coarse + f64 rescoring", "data": "synthetic (seeded, shapes of the workload)",
        "config": {"workload": wl.name, "n": wl.n, "d": wl.d, "k": wl.k, "margin": wl.margin,
                   "l2": "inputs resident in host memory (CPU run)"},
        "cpu_baseline": {"value": v, "unit": "cells/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="zipf_2m")
    ap.add_argument("--n", type=int, default=None, help="a smaller n from the same generator (profiling)")
    ap.add_argument("--backend", default="bf16", choices=["fp32", "bf16", "bf16x3", "fp8"],
                    help="bf16: tensor cores (split BF16; split FP8 for d >= 512); bf16x3 / fp8: that kind only")
    ap.add_argument("--no-learned", action="store_true", help="bf16 backend without the learned pruning")
    ap.add_argument("--train-sample", type=int, default=200_000)
    ap.add_argument("--train-epochs", type=int, default=60)
    ap.add_argument("--train-quantile", type=float, default=0.01, help="pinball-loss quantile of the model")
    ap.add_argument("--mlp-save", default=None, help="write the trained model here (.npz)")
    ap.add_argument("--mlp-load", default=None,
                    help="load a model saved with --mlp-save instead of training (e.g. to profile the steps alone)")
    ap.add_argument("--plain-steps", type=int, default=2, help="timed steps of the plain FP32 leg (0: skip)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--cpu-crosscheck", action="store_true",
                    help="also time the CPU port on one thread and in full at n = 200,000 and 400,000 (n^2 check)")
    ap.add_argument("--sharded", action="store_true",
                    help="time the multi-GPU (row-shard) step even on one GPU (a one-rank process group)")
    ap.add_argument("--profile-case", choices=sorted(PROFILE_CASES),
                    help="run one small case that launches the named kernel twice (for ncu captures) and exit")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.profile_case:
        return run_profile_case(args.profile_case)

    from costal_gb300 import workloads as W

    x, wl = W.make(args.workload, n=args.n)
    if args.n is not None:
        import dataclasses

        wl = dataclasses.replace(wl, n=len(x))
    if args.impl == "reference":
        return run_reference(args, wl, x)

    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    import torch.distributed as dist

    if ws > 1:
        dist.init_process_group("nccl")
    elif args.sharded:  # the sharded step on one rank (a one-process NCCL group)
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29531")
        dist.init_process_group("nccl", rank=0, world_size=1)
    from costal_gb300 import _lib as L

    lib = L.lib()
    n, d, k = wl.n, wl.d, wl.k
    learned = args.backend != "fp32" and not args.no_learned and wl.d <= 64
    err, errlen = L.errbuf()

    def make_opts(backend, learned_prune):
        o = L.KnnOpts()
        o.margin = wl.margin
        o.select = 0
        o.backend = {"fp32": L.BACKEND_FP32, "bf16": L.BACKEND_BF16, "bf16x3": L.BACKEND_BF16X3,
                     "fp8": L.BACKEND_FP8}[backend]
        o.sort_by_norm = 1
        o.prune = 1
        o.learned_prune = 1 if learned_prune else 0
        return o

    opts = make_opts(args.backend, learned)
    weight = L.WEIGHT["tanimoto"]
    stream = torch.cuda.current_stream()

    # ---- the model (trained once on this input, labels from the plain FP32 path; untimed)
    train = None
    if learned and args.mlp_load:
        from costal_gb300 import _costal as ext

        z = np.load(args.mlp_load)
        ext._mlp_set(z["params"], int(z["d"]), int(z["k"]), float(z["quantile"]))
        train = {"loaded": args.mlp_load}
    elif learned:
        mo = L.MlpOpts()
        mo.sample, mo.epochs, mo.batch = min(args.train_sample, n), args.train_epochs, 2048
        mo.margin, mo.lr, mo.quantile, mo.seed = wl.margin, 2e-3, args.train_quantile, 20241203
        ms_ = L.MlpStats()
        t = time.perf_counter()
        L.check(lib.costal_mlp_train(x.ctypes.data_as(C.c_void_p), n, d, k, C.byref(mo), C.byref(ms_), err, errlen),
                err)
        train = {kk: v for kk, v in ms_.as_dict().items()}
        train["wall_s"] = time.perf_counter() - t
        if args.mlp_save:
            from costal_gb300 import _costal as ext

            params, md, mk, mq = ext._mlp_get()
            np.savez(args.mlp_save, params=params, d=md, k=mk, quantile=mq)

    dx = torch.from_numpy(x).cuda()
    d_rows = torch.empty(n * k, dtype=torch.int32, device="cuda")
    d_cols = torch.empty(n * k, dtype=torch.int32, device="cuda")
    d_w = torch.empty(n * k, dtype=torch.float64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    m = C.c_uint64()
    st = L.KnnStats()

    sharded = ws > 1 or args.sharded
    shard_stats = {}

    def step_sharded(o, xd):
        from costal_gb300 import shard as S

        (r, c, w), _, stt = S.build_graph_sharded(
            xd, k, margin=wl.margin, matmul=args.backend if o.backend != L.BACKEND_FP32 else "fp32",
            learned_prune=bool(o.learned_prune))
        shard_stats.update(stt)
        m.value = r.shape[0]
        return r, c, w

    def step_device(o, xin=None):
        xin = dx if xin is None else xin
        if sharded:
            r, c, w = step_sharded(o, xin)
            d_rows[: r.shape[0]].copy_(r)
            d_cols[: c.shape[0]].copy_(c)
            d_w[: w.shape[0]].copy_(w)
            return
        rc = lib.costal_build_graph_device(C.c_void_p(xin.data_ptr()), n, d, k, C.byref(o), weight,
                                           C.c_void_p(d_rows.data_ptr()), C.c_void_p(d_cols.data_ptr()),
                                           C.c_void_p(d_w.data_ptr()), C.byref(m), C.byref(st),
                                           C.c_void_p(stream.cuda_stream), err, errlen)
        L.check(rc, err)

    def timed_device(o, warmup, steps, clocks=None, xin=None):
        for _ in range(warmup):
            flush.zero_()
            step_device(o, xin)
        torch.cuda.synchronize()
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()
        times, stats = [], []
        l0 = lib.costal_launch_count()
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step_device(o, xin)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            stats.append(dict(shard_stats) if sharded else st.as_dict())
        launches = lib.costal_launch_count() - l0
        torch.cuda.synchronize()
        ms = max_over_ranks(float(np.mean(times)), "cuda")
        if ws > 1:
            dist.barrier()
        return ms, stats, launches, int(m.value)

    # ---- device-resident value
    with ClockSampler(local) as clocks:
        ms, stats, launches, edges = timed_device(opts, args.warmup, args.steps)

    # ---- end to end through the host C ABI (pinned host buffers, copies inside the timed region)
    hx = torch.from_numpy(x).pin_memory()
    h_rows = torch.empty(n * k, dtype=torch.int32, pin_memory=True)
    h_cols = torch.empty(n * k, dtype=torch.int32, pin_memory=True)
    h_w = torch.empty(n * k, dtype=torch.float64, pin_memory=True)
    m2 = C.c_uint64()
    st_host = L.KnnStats()  # the kNN stage's device time inside the host call

    def step_host():
        if sharded:  # X from pinned host memory to this rank's GPU, the sharded step, the edges back
            xd = hx.to("cuda", non_blocking=True)
            r, c, w = step_sharded(opts, xd)
            e = r.shape[0]
            h_rows[:e].copy_(r)
            h_cols[:e].copy_(c)
            h_w[:e].copy_(w)
            m2.value = e
            return
        rc = lib.costal_build_graph(C.c_void_p(hx.data_ptr()), n, d, k, C.byref(opts), weight,
                                    C.c_void_p(h_rows.data_ptr()), C.c_void_p(h_cols.data_ptr()),
                                    C.c_void_p(h_w.data_ptr()), C.byref(m2), None, None, None, C.byref(st_host), err,
                                    errlen)
        L.check(rc, err)

    for _ in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize()
        step_host()
    e2e_t, e2e_knn = [], []
    with ClockSampler(local) as e2e_clocks:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            step_host()
            e2e_t.append(time.perf_counter() - t)
            if not sharded:
                e2e_knn.append(st_host.ms_total)
    e2e_s = max_over_ranks(float(np.mean(e2e_t)), "cuda")
    # parity guard: the timed host result equals the device-resident one
    assert int(m2.value) == edges
    host_edges = (h_rows[:edges].numpy().copy(), h_cols[:edges].numpy().copy(), h_w[:edges].numpy().copy())

    # ---- the plain FP32 GPU path on the same input (the comparison the metric names)
    plain = None
    if args.backend != "fp32" and args.plain_steps > 0:
        pms, pstats, _, pedges = timed_device(make_opts("fp32", False), 1, args.plain_steps)
        same = pedges == edges and all(
            np.array_equal(a, b.cpu().numpy()[:edges]) for a, b in zip(host_edges, (d_rows, d_cols, d_w)))
        plain = {"ms_per_step": pms, "value": job_cells_per_s(n, 1, pms), "unit": "cells/s", "steps": args.plain_steps,
                 "warmup": 1, "ms_kernel": float(np.mean([s_["ms_kernel"] for s_ in pstats])),
                 "speedup": pms / ms, "identical_edges": bool(same)}

    # ---- the same certified path without the learned threshold (exact early stop only)
    stop_only = None
    if learned:
        sms, sstats, _, sedges = timed_device(make_opts("bf16", False), 1, args.steps)
        stop_only = {"ms_per_step": sms, "value": job_cells_per_s(n, 1, sms), "unit": "cells/s", "steps": args.steps,
                     "warmup": 1, "ms_kernel": float(np.mean([s_["ms_kernel"] for s_ in sstats])),
                     "blocks_stopped": sstats[-1]["blocks_stopped"], "same_edge_count": sedges == edges}
        if plain is not None:
            stop_only["speedup_vs_plain"] = plain["ms_per_step"] / sms

    # ---- the model trained on this draw, reused unchanged on another draw of the same generator
    reuse = None
    if learned and args.workload == "zipf_2m" and args.n is None:
        x2 = W.zipf_2m(seed=wl.seed + 1)
        dx2 = torch.from_numpy(x2).cuda()
        rms, rstats, _, redges = timed_device(opts, 1, 2, xin=dx2)
        r_edges = (d_rows[:redges].clone(), d_cols[:redges].clone(), d_w[:redges].clone())
        sms2, sstats2, _, sedges2 = timed_device(make_opts("bf16", False), 1, 2, xin=dx2)
        same2 = redges == sedges2 and all(torch.equal(a, b[:redges]) for a, b in zip(r_edges, (d_rows, d_cols, d_w)))
        reuse = {"input": f"zipf_2m seed {wl.seed + 1} (another draw; the model trained on seed {wl.seed})",
                 "ms_per_step": rms, "value": job_cells_per_s(n, 1, rms), "stop_only_ms_per_step": sms2,
                 "blocks_skipped": rstats[-1]["blocks_skipped"], "blocks_stopped": rstats[-1]["blocks_stopped"],
                 "pruned_fallback_rows": rstats[-1]["pruned_fallback_rows"],
                 "identical_edges_vs_stop_only": bool(same2)}
        del dx2

    if rank == 0:
        pk, pk_kind = peaks()
        s0 = stats[-1]
        kms = float(np.mean([s_["ms_kernel"] for s_ in stats]))
        total_blocks = s0["blocks_total"]
        tensor = args.backend != "fp32"
        skipped = s0["blocks_skipped"] + s0["blocks_stopped"] if tensor else 0
        visited = 1.0 - skipped / total_blocks if total_blocks else 1.0
        pairs = float(n) * float(n) * visited  # dense pairs of the visited (query block, column block) tiles
        flops = 2.0 * d * pairs
        kind = s0.get("coarse_kind", 1 if tensor else 0)
        if tensor and kind == 2:
            # split FP8: e4m3 MMAs, K = 3d padded to 128; the dense FP8 rate is twice the BF16 one
            kpad = (3 * d + 127) // 128 * 128
            tiles = (total_blocks - skipped)
            executed = 2.0 * kpad * tiles * 128 * 256
            bound, peak, unit = "tensor", 2.0 * pk.get("bf16_tflops_sustained", pk["bf16_tflops"]), "TFLOP/s"
            kernel = "k_coarse_tc (split-FP8 e4m3 tcgen05 tiles + top-(k+m) selection)"
            peak_kind = f"fp8 dense = 2 x bf16 dense sustained ({pk_kind}; no fp8 figure is measured)"
        elif tensor:
            kpad = (3 * d + 63) // 64 * 64
            tiles = (total_blocks - skipped)
            executed = 2.0 * kpad * tiles * 128 * 256
            bound, peak, unit = "tensor", pk.get("bf16_tflops_sustained", pk["bf16_tflops"]), "TFLOP/s"
            kernel = "k_coarse_tc (split-BF16 tcgen05 tiles + top-(k+m) selection)"
            peak_kind = f"bf16 dense sustained, {pk_kind}"
        else:
            executed = flops
            # FP32 FFMA peak of the GB300 (152 SMs x 128 lanes x 2 FLOP x max SM clock); MEASURED_PEAKS
            # has no CUDA-core figure, so it is derived from the measured max clock.
            bound, unit = "fp32-fma", "TFLOP/s"
            peak = 152 * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
            kernel = "k_coarse_fp32 (FP32 tiles + top-(k+m) selection)"
            peak_kind = "derived FP32-FFMA peak at max SM clock"
        achieved = flops / (kms * 1e-3) / 1e12
        traffic = traffic_per_launch("bf16" if kind else "fp32", pairs, d) if kind != 2 else None
        line = {
            "metric": METRIC,
            "value": job_cells_per_s(n, 1, ms),
            "unit": "cells/s",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms,
            "higher_is_better": True,
            "scaling": "strong",
            "vs_baseline": None,
            "dtype": ({0: "f32 tiles", 1: "split-bf16 tcgen05 tiles (fp32 accumulate)",
                       2: "split-fp8 e4m3 tcgen05 tiles (fp32 accumulate)"}[kind] + " + f64 rescoring"),
            "data": "synthetic (seeded generator with the workload's shapes and distributions)",
            "config": {"workload": wl.name, "n": n, "d": d, "k": k, "margin": wl.margin, "backend": args.backend,
                       "learned_prune": learned, "weight": "tanimoto",
                       "l2": "flushed between steps (512 MB write outside the timed events)"},
            "e2e": {"value": job_cells_per_s(n, 1, e2e_s * 1e3), "unit": "cells/s", "ms_per_step": e2e_s * 1e3,
                    "ms_steps": [round(t_ * 1e3, 2) for t_ in e2e_t],
                    "ms_knn_device": float(np.mean(e2e_knn)) if e2e_knn else None, "clocks": e2e_clocks.summary(),
                    "h2d_bytes_per_step": n * d * 4 * ws,
                    "d2h_bytes_per_step": edges * 16},
            "gpu_launches": int(launches),
            "gpu_launches_per_step": launches / args.steps,
            "roofline": {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit, "frac": achieved / peak,
                         "traffic": traffic, "kernel": kernel, "peak_kind": peak_kind,
                         "ms_per_launch": kms, "pairs_per_launch": pairs,
                         "executed_tflops": executed / (kms * 1e-3) / 1e12,
                         "executed_frac": executed / (kms * 1e-3) / 1e12 / peak},
            "pair_dots_per_s": float(n) * (n - 1) / (ms * 1e-3),
            "edges": edges,
            "plain_fp32": plain,
            "without_learned": stop_only,
            "reused_model": reuse,
            "train": train,
            "stats": {kk: s0[kk] for kk in ("fallback_rows", "recomputed_rows", "pruned_fallback_rows",
                                             "blocks_skipped", "blocks_stopped", "blocks_total", "max_coarse_err", "ms_prep",
                                             "ms_order", "ms_coarse", "ms_kernel", "ms_rescore", "ms_fallback",
                                             "ms_total")},
            "clocks": clocks.summary(),
        }
        if train is not None and "ms_train" in train:
            line["value_incl_training"] = job_cells_per_s(n, 1, ms + train["ms_labels"] + train["ms_train"])
        if not args.no_cpu:
            v, cores, sample = cpu_baseline(x, wl, target_s=args.cpu_seconds)
            line["cpu_baseline"] = {"value": v, "unit": "cells/s", "cores": cores, "kind": "port", "sample": sample}
            if args.cpu_crosscheck:
                line["cpu_baseline"]["crosscheck"] = cpu_crosscheck(x, wl, v, args)
        print(json.dumps(line), flush=True)
    if dist.is_initialized():
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
