"""Multi-GPU layout of the visibility-edge path: replicas with a sharded work
list, no data-path collective.

Visibility shards by pair rows (or, for a batch, by parts): every rank traces
its own rows against replicated BVHs; the only exchange is gathering the edge
lists when one process needs them all. Scoring shards by parts the same way.
With one GPU per process this is what `torchrun --nproc-per-node N bench.py`
runs: N independent replicas, a barrier around the timed region and the max
time over ranks.
"""
from __future__ import annotations

import numpy as np


def row_weights(n: int) -> np.ndarray:
    """Pairs per row i of the upper triangle (i < j < n)."""
    return np.arange(n - 1, -1, -1, dtype=np.int64)


def shard_rows(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous rows [r0, r1) of an n-vertex pair triangle for `rank`, with
    about equal pair counts per rank."""
    w = np.cumsum(row_weights(n))
    total = int(w[-1]) if n else 0
    lo = total * rank // world
    hi = total * (rank + 1) // world
    r0 = int(np.searchsorted(w, lo, side="right")) if rank else 0
    r1 = int(np.searchsorted(w, hi, side="right")) if rank < world - 1 else n
    return min(r0, n), min(max(r1, r0), n)


def shard_parts(costs, rank: int, world: int) -> list[int]:
    """Greedy longest-first assignment of parts (by cost, e.g. pair count) to
    ranks; returns this rank's part indices in ascending order."""
    order = np.argsort(-np.asarray(costs, dtype=np.float64), kind="stable")
    load = np.zeros(world)
    owner = np.empty(len(order), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return sorted(int(i) for i in np.nonzero(owner == rank)[0])


def gather_edges(edges: np.ndarray):
    """All ranks' edge lists, concatenated in rank order (torch.distributed)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size()
    t = torch.from_numpy(np.ascontiguousarray(edges.astype(np.int64)).reshape(-1, 2))
    n = torch.tensor([t.shape[0]], dtype=torch.int64)
    counts = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(counts, n)
    m = int(max(c.item() for c in counts))
    pad = torch.zeros((m, 2), dtype=torch.int64)
    pad[: t.shape[0]] = t
    bufs = [torch.zeros((m, 2), dtype=torch.int64) for _ in range(world)]
    dist.all_gather(bufs, pad)
    return np.concatenate([b[: int(c.item())].numpy() for b, c in zip(bufs, counts)]).astype(np.uint32)


def max_over_ranks(x: float) -> float:
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
