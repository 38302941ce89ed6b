"""Placement of independent scenes on the GPUs of one node (one process per GPU).

A single scene does not shard (its neighbour search would need halo exchange
every pass), so one-scene runs on N GPUs are replicas.  Batched and served
scenes are independent units: they are dealt to ranks by particle count, with
no collective in the step; the only communication is the host-side reduction
of counts and times for reporting.
"""
from __future__ import annotations

import heapq


def partition_scenes(counts, world_size: int) -> list[list[int]]:
    """Longest-processing-time-first bin packing of scenes (by particle count)
    onto `world_size` ranks.  Deterministic: ties go to the lower scene index
    and the lower rank.  Returns, per rank, its scene indices in ascending
    order."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(counts)), key=lambda i: (-int(counts[i]), i))
    heap = [(0, r) for r in range(world_size)]
    out: list[list[int]] = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + int(counts[i]), r))
    return [sorted(p) for p in out]


def rank_scenes(counts, world_size: int, rank: int) -> list[int]:
    """The scenes of `rank` under partition_scenes."""
    if not 0 <= rank < world_size:
        raise ValueError("rank out of range")
    return partition_scenes(counts, world_size)[rank]


def job_throughput(units: float, seconds: float, dist=None) -> tuple[float, float]:
    """Whole-job totals across ranks: the sum of the units all ranks processed
    and the slowest rank's time (torch.distributed all-reduce when `dist` is
    an initialised torch.distributed module, else this rank's own)."""
    if dist is None:
        return float(units), float(seconds)
    import torch

    u = torch.tensor([float(units)], dtype=torch.float64)
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(u.item()), float(t.item())
