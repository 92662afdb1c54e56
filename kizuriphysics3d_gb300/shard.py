"""Independent worlds across GPUs: one context per rank holding a contiguous range of worlds.

Worlds never interact (each is its own PhysicsWorld in the reference; here a world id keys the
broad phase, so a merged context steps them side by side), so splitting a batch of worlds across
ranks needs no exchange on the step path: each rank steps its own range and only the metrics are
gathered.  The ranges are contiguous in world order and balanced by summed body count, the
linear-partition rule (smallest possible largest share).  A single world never splits: its giant
island is one Gauss-Seidel chain with a barrier per dependency level.
"""
from __future__ import annotations

from typing import Callable, List, Sequence, Tuple

import numpy as np


def partition_worlds(sizes: Sequence[int], nranks: int) -> List[Tuple[int, int]]:
    """Contiguous [start, end) world ranges, one per rank, whose largest summed size is as small as
    possible (binary search on that bound; ties go to the earliest split).  Ranks past the number
    of worlds get empty ranges."""
    sizes = [int(s) for s in sizes]
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    if any(s < 0 for s in sizes):
        raise ValueError("world sizes must be >= 0")

    def cuts(bound: int):
        out, start, acc = [], 0, 0
        for i, s in enumerate(sizes):
            if acc + s > bound and i > start:
                out.append((start, i))
                start, acc = i, 0
            acc += s
        out.append((start, len(sizes)))
        return out

    if not sizes:
        return [(0, 0)] * nranks
    lo, hi = max(sizes), sum(sizes)
    while lo < hi:
        mid = (lo + hi) // 2
        if len(cuts(mid)) <= nranks:
            hi = mid
        else:
            lo = mid + 1
    ranges = cuts(lo)
    while len(ranges) < nranks:  # fewer pieces than ranks: empty ranges at the end
        ranges.append((len(sizes), len(sizes)))
    return ranges


def shard_scene(worlds, start: int, end: int):
    """The merged scene (and world ids, renumbered from 0) of worlds[start:end] for one rank."""
    from .scenes import merge_worlds
    if end <= start:
        return None, np.zeros(0, np.uint32)
    return merge_worlds(list(worlds[start:end]))


def gather_metrics(pg, body_steps: float, elapsed_ms: float) -> Tuple[float, float]:
    """Whole-job body-steps and the slowest rank's time (the only exchange: after the timed steps)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([body_steps, elapsed_ms], dtype=torch.float64)
    if pg is not None and dist.is_initialized():
        dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(pg) == "nccl" else torch.device("cpu")
        s = t[:1].to(dev)
        m = t[1:].to(dev)
        dist.all_reduce(s, op=dist.ReduceOp.SUM, group=pg)
        dist.all_reduce(m, op=dist.ReduceOp.MAX, group=pg)
        return float(s.item()), float(m.item())
    return float(t[0]), float(t[1])


def run_shard(worlds, rank: int, nranks: int, step: Callable, steps: int, pg=None):
    """Partition, step this rank's range with `step(scene, world_ids, steps) -> elapsed_ms`, gather.
    Returns (my range, whole-job body-steps, slowest rank's ms)."""
    sizes = [len(w.bodies) for w in worlds]
    ranges = partition_worlds(sizes, nranks)
    start, end = ranges[rank]
    scene, ids = shard_scene(worlds, start, end)
    n_dyn = scene.num_dynamic if scene is not None else 0
    ms = step(scene, ids, steps) if scene is not None else 0.0
    total, slowest = gather_metrics(pg, float(n_dyn * steps), ms)
    return (start, end), total, slowest
