"""Benchmark: exact kNN-graph cells/s on one GB300 (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--backend fp32|bf16]
    python bench.py --impl reference ...      # the CPU implementation of the path on the host cores

A step is one pass of the hot path over one batch: X (n × d f32) -> norms, normalised tiles, top-(k+m)
selection, f64 rescoring + certificate (+ regather), Tanimoto weights, fuzzy-union edge list.

  value  — n / step time with X already resident in HBM (CUDA events on the launching stream, L2
           flushed between steps by writing a 512 MB buffer outside the timed events);
  e2e    — the same through the host C-ABI call costal_build_graph: pinned host X in, pinned host
           edge list out, copies inside the timed region (wall clock around the synchronous call);
  roofline — the dominant kernel (the coarse tile + selection kernel), achieved algorithmic FLOP/s
           (2·n·(n−1)·d per launch, dense-equivalent) over its CUDA-event duration;
  cpu_baseline — the oracle (C++ restatement of the reference's CPU path) on a bounded sample of
           query rows, all host threads.

Multi-GPU (torchrun): every rank runs an independent replica of the workload on its own GPU
(no collective on the data path); value = total cells of all ranks / max step time.
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


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


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
    rows = int(min(n, max(probe, probe * target_s / max(dt, 1e-6))))
    rows = max(64, rows)
    q0 = (n - rows) // 2
    t = time.perf_counter()
    O.knn_rows(x, wl.k, q0, q0 + rows, margin=wl.margin, n_threads=cores)
    dt = time.perf_counter() - t
    return rows / dt, cores, f"{rows} query rows x all {n} columns (kNN incl. f64 rescoring), {dt:.1f} s"


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
        "warmup": args.warmup, "ms_per_step": wl.n / v * 1e3, "higher_is_better": True, "scaling": "weak",
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
    ap.add_argument("--workload", default="rare_400k")
    ap.add_argument("--n", type=int, default=None, help="a smaller n from the same generator (profiling)")
    ap.add_argument("--backend", default="fp32", choices=["fp32", "bf16"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

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
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from costal_gb300 import _lib as L

    lib = L.lib()
    n, d, k = wl.n, wl.d, wl.k
    opts = L.KnnOpts()
    opts.margin = wl.margin
    opts.select = 0
    opts.backend = L.BACKEND_BF16 if args.backend == "bf16" else L.BACKEND_FP32
    opts.sort_by_norm = 1
    opts.prune = 1
    weight = L.WEIGHT["tanimoto"]
    stream = torch.cuda.current_stream()
    dx = torch.from_numpy(x).cuda()
    d_rows = torch.empty(n * k, dtype=torch.int32, device="cuda")
    d_cols = torch.empty(n * k, dtype=torch.int32, device="cuda")
    d_w = torch.empty(n * k, dtype=torch.float64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    m = C.c_uint64()
    st = L.KnnStats()
    err, errlen = L.errbuf()

    def step_device():
        rc = lib.costal_build_graph_device(C.c_void_p(dx.data_ptr()), n, d, k, C.byref(opts), weight,
                                           C.c_void_p(d_rows.data_ptr()), C.c_void_p(d_cols.data_ptr()),
                                           C.c_void_p(d_w.data_ptr()), C.byref(m), C.byref(st),
                                           C.c_void_p(stream.cuda_stream), err, errlen)
        L.check(rc, err)

    # ---- device-resident value
    for _ in range(args.warmup):
        flush.zero_()
        step_device()
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    times, coarse_ms, stats = [], [], []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step_device()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            coarse_ms.append(st.ms_coarse)
            stats.append(st.as_dict())
    torch.cuda.synchronize()
    ms = float(np.mean(times))
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    edges = int(m.value)

    # ---- end to end through the host C ABI (pinned host buffers, copies inside the timed region)
    hx = torch.from_numpy(x).pin_memory()
    h_rows = torch.empty(n * k, dtype=torch.int32, pin_memory=True)
    h_cols = torch.empty(n * k, dtype=torch.int32, pin_memory=True)
    h_w = torch.empty(n * k, dtype=torch.float64, pin_memory=True)
    m2 = C.c_uint64()

    def step_host():
        rc = lib.costal_build_graph(C.c_void_p(hx.data_ptr()), n, d, k, C.byref(opts), weight,
                                    C.c_void_p(h_rows.data_ptr()), C.c_void_p(h_cols.data_ptr()),
                                    C.c_void_p(h_w.data_ptr()), C.byref(m2), None, None, None, None, err, errlen)
        L.check(rc, err)

    for _ in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize()
        step_host()
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        step_host()
        e2e_t.append(time.perf_counter() - t)
    e2e_s = float(np.mean(e2e_t))
    if ws > 1:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    # parity guard: the timed host result equals the device-resident one
    assert int(m2.value) == edges

    if rank == 0:
        pk, pk_kind = peaks()
        cm = float(np.mean(coarse_ms))
        flops = 2.0 * n * (n - 1) * d
        s0 = stats[-1]
        if args.backend == "bf16":
            bound, peak, unit = "tensor", pk["bf16_tflops"], "TFLOP/s"
        else:
            # FP32 FFMA peak of the GB300 (152 SMs x 128 lanes x 2 FLOP x max SM clock); MEASURED_PEAKS
            # has no CUDA-core figure, so it is derived from the measured max clock.
            bound, unit = "fp32-fma", "TFLOP/s"
            peak = 152 * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
        achieved = flops / (cm * 1e-3) / 1e12
        line = {
            "metric": METRIC,
            "value": ws * n / (ms * 1e-3),
            "unit": "cells/s",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 tiles + f64 rescoring" if args.backend == "fp32" else "split-bf16 tcgen05 tiles + f64 rescoring",
            "data": "synthetic (seeded generator with the workload's shapes and distributions)",
            "config": {"workload": wl.name, "n": n, "d": d, "k": k, "margin": wl.margin, "backend": args.backend,
                       "weight": "tanimoto", "l2": "flushed between steps (512 MB write outside the timed events)"},
            "e2e": {"value": ws * n / e2e_s, "unit": "cells/s", "h2d_bytes_per_step": n * d * 4,
                    "d2h_bytes_per_step": edges * 16},
            "gpu_launches": None,
            "roofline": {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit, "frac": achieved / peak,
                         "traffic": None, "kernel": "coarse tile + top-(k+m) selection",
                         "peak_kind": ("derived FP32-FFMA peak at max SM clock" if args.backend == "fp32"
                                       else f"bf16 dense, {pk_kind}")},
            "pair_dots_per_s": ws * n * (n - 1) / (ms * 1e-3),
            "edges": edges,
            "stats": {kk: s0[kk] for kk in ("fallback_rows", "recomputed_rows", "max_coarse_err", "ms_prep",
                                             "ms_coarse", "ms_rescore", "ms_fallback", "ms_total")},
            "clocks": clocks.summary(),
        }
        if not args.no_cpu:
            v, cores, sample = cpu_baseline(x, wl, target_s=args.cpu_seconds)
            line["cpu_baseline"] = {"value": v, "unit": "cells/s", "cores": cores, "kind": "port", "sample": sample}
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
