"""The exact kNN graph split by query rows across the ranks of a torch.distributed group.

The reference's unit of parallel work is a block of query rows against all columns
(crates/costal-core/src/knn.rs:403-512, `run_blocked` over row blocks). Here each rank (one GPU) keeps
all of X and computes one shard of the query rows against every column (costal_knn_shard_device:
query blocks of 128 rows in the order the coarse pass processes them, shard s of S taking the
contiguous blocks [s*B/S, (s+1)*B/S)); the ranks then all-gather their rows' neighbours, cosines and
Tanimoto weights, and every rank builds the fuzzy union (costal_fuzzy_union_device) of the whole
graph. No tile of another rank's memory is ever read: every remote byte arrives through the
collective into local buffers. The output is the same bits as the one-GPU path.

`compute`, `weights` and `union` can be swapped for stand-ins, which is how the exchange itself is
tested on CPU ranks over gloo (the oracle computing each rank's rows).
"""

from __future__ import annotations

import ctypes as C

from . import _lib as L
from ._costal import _BACKENDS, _backend, _call, _opts

ROW_BLOCK = 128  # rows per query block, the unit shards are made of


def shard_rows(n: int, shard: int, n_shards: int) -> tuple[int, int]:
    """The [start, end) positions, in the processing order, of shard `shard` of `n_shards`."""
    nqb = (n + ROW_BLOCK - 1) // ROW_BLOCK
    qb0, qb1 = nqb * shard // n_shards, nqb * (shard + 1) // n_shards
    return min(n, qb0 * ROW_BLOCK), min(n, qb1 * ROW_BLOCK)


def rows_max(n: int, n_shards: int) -> int:
    """The most rows one of `n_shards` shards holds (costal_shard_rows_max)."""
    return int(L.lib().costal_shard_rows_max(int(n), int(n_shards)))


def _tptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def shard_device(x, k, shard, n_shards, *, margin=None, matmul=None, weights=True, learned_prune=False):
    """The kNN of one shard of the rows of x (a float32 CUDA tensor (n, d)) on x's device.

    Returns a dict of tensors on that device: rows (int32 original ids), idx (int32) and cos
    (float64) of shape (rows, k), w (the Tanimoto weights, when `weights`), norms (float64, all n
    rows), and the call's stats."""
    import torch

    if not (x.is_cuda and x.dtype == torch.float32 and x.dim() == 2 and x.is_contiguous()):
        raise TypeError("x must be a C-contiguous float32 CUDA tensor of shape (n, d)")
    n, d = x.shape
    k = int(k)
    cap = rows_max(n, n_shards)
    dev = x.device
    rows = torch.empty(max(cap, 1), dtype=torch.int32, device=dev)
    idx = torch.empty((max(cap, 1), k), dtype=torch.int32, device=dev)
    cos = torch.empty((max(cap, 1), k), dtype=torch.float64, device=dev)
    w = torch.empty((max(cap, 1), k), dtype=torch.float64, device=dev) if weights else None
    norms = torch.empty(n, dtype=torch.float64, device=dev)
    count = C.c_uint64(0)
    st = L.KnnStats()
    o = _opts("cosine", margin, None, None, _BACKENDS[_backend(matmul)], True, True, learned_prune)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _call(L.lib().costal_knn_shard_device, _tptr(x), n, d, k, C.byref(o), int(shard), int(n_shards), _tptr(rows),
          C.byref(count), _tptr(idx), _tptr(cos), _tptr(w), _tptr(norms), C.byref(st), C.c_void_p(stream))
    m = count.value
    out = {"rows": rows[:m], "idx": idx[:m], "cos": cos[:m], "norms": norms, "stats": st.as_dict()}
    if weights:
        out["w"] = w[:m]
    return out


def union_device(idx, w):
    """lib.rs:219-239 `_fuzzy_union` on CUDA tensors: idx int32 (n, k), w float64 (n, k) ->
    (rows int32, cols int32, weights float64) on the same device."""
    import torch

    n, k = idx.shape
    rows = torch.empty(max(n * k, 1), dtype=torch.int32, device=idx.device)
    cols = torch.empty_like(rows)
    wout = torch.empty(max(n * k, 1), dtype=torch.float64, device=idx.device)
    m = C.c_uint64(0)
    stream = torch.cuda.current_stream(idx.device).cuda_stream
    _call(L.lib().costal_fuzzy_union_device, _tptr(idx.contiguous()), _tptr(w.contiguous()), n, k, _tptr(rows),
          _tptr(cols), _tptr(wout), C.byref(m), C.c_void_p(stream))
    m = m.value
    return rows[:m], cols[:m], wout[:m]


def gather_rows(part, n, group=None):
    """All-gather every rank's rows: part holds `rows` (int32, m) and per-row tensors (m, k) under
    `idx`, `cos` and optionally `w`. Returns the whole (n, k) tensors, each row placed at its id.
    Checks that the shards cover every row exactly once."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rows = part["rows"]
    dev = rows.device
    cnt = torch.tensor([rows.shape[0]], dtype=torch.int64, device=dev)
    counts = [torch.zeros_like(cnt) for _ in range(world)]
    dist.all_gather(counts, cnt, group=group)
    counts = [int(c.item()) for c in counts]
    if sum(counts) != n:
        raise RuntimeError(f"the shards hold {sum(counts)} rows, not n={n}")
    cap = max(max(counts), 1)

    def padded(t):
        out = torch.zeros((cap,) + tuple(t.shape[1:]), dtype=t.dtype, device=dev)
        out[: t.shape[0]] = t
        return out

    keys = [key for key in ("idx", "cos", "w") if key in part]
    got_rows = [torch.empty(cap, dtype=rows.dtype, device=dev) for _ in range(world)]
    dist.all_gather(got_rows, padded(rows), group=group)
    all_rows = torch.cat([r[:c] for r, c in zip(got_rows, counts)]).long()
    seen = torch.zeros(n, dtype=torch.int32, device=dev)
    seen.index_add_(0, all_rows, torch.ones_like(all_rows, dtype=torch.int32))
    if not bool((seen == 1).all()):
        raise RuntimeError("the shards do not cover every row exactly once")
    full = {}
    for key in keys:
        t = part[key]
        got = [torch.empty((cap,) + tuple(t.shape[1:]), dtype=t.dtype, device=dev) for _ in range(world)]
        dist.all_gather(got, padded(t), group=group)
        whole = torch.empty((n,) + tuple(t.shape[1:]), dtype=t.dtype, device=dev)
        whole[all_rows] = torch.cat([g[:c] for g, c in zip(got, counts)])
        full[key] = whole
    return full


def build_graph_sharded(x, k, *, margin=None, matmul=None, learned_prune=False, group=None, compute=None,
                        weights=None, union=None):
    """The exact kNN graph of x, this rank computing its shard of the rows.

    x: this rank's copy of the whole input (a CUDA tensor for the GPU path). Returns
    ((rows, cols, w) edges, (idx, cos, norms), stats) on every rank, the same bits as the one-GPU
    path. `compute(x, k, shard, n_shards, margin=, matmul=)` returns the shard's dict (default:
    shard_device); `weights(idx, cos, norms)` makes the Tanimoto weights when compute gives none;
    `union(idx, w)` builds the edges (default: union_device)."""
    import torch.distributed as dist

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    if compute is None:
        part = shard_device(x, k, rank, world, margin=margin, matmul=matmul, learned_prune=learned_prune)
    else:
        part = compute(x, k, rank, world, margin=margin, matmul=matmul)
    full = gather_rows(part, x.shape[0], group)
    if "w" not in full:
        full["w"] = weights(full["idx"], full["cos"], part["norms"])
    edges = (union or union_device)(full["idx"], full["w"])
    return edges, (full["idx"], full["cos"], part["norms"]), part.get("stats", {})
