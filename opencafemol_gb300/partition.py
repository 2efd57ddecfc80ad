"""Whole systems across GPUs: the host-side partition of an ensemble.

Independent trajectories shard without any exchange: every system runs on
exactly one device, in that device's own batch, and nothing crosses devices
while they run.  The partition is a longest-processing-time-first greedy
assignment (sort by estimated cost, give each system to the device with the
least work so far; ties go to the lower rank), which is deterministic, so
every rank computes the same assignment from the same list without talking
to the others.  Results come back to one rank in the ensemble's own order
through ``torch.distributed`` object gathers (gloo on the host, NCCL on
GPUs) after the runs; this is reporting, not part of the time step.

The reference has no counterpart: it runs one system per process.
"""
from __future__ import annotations

import heapq
from dataclasses import dataclass

import numpy as np


def system_cost(n_beads: int) -> float:
    """Estimated device time of one system per step: the batched kernel's
    time grows with the bead count, with a floor for the per-step barriers
    of small systems (measured: about 4 us per step at 50 beads, 13 us at
    400, 33 us at 800 on one SM)."""
    return max(float(n_beads), 150.0)


def assign(costs, n_ranks: int) -> list[list[int]]:
    """Indices of the systems each rank runs (largest first per rank)."""
    if n_ranks < 1:
        raise ValueError("need at least one rank")
    costs = np.asarray(costs, dtype=float)
    order = sorted(range(len(costs)), key=lambda k: (-costs[k], k))
    heap = [(0.0, r) for r in range(n_ranks)]
    heapq.heapify(heap)
    parts: list[list[int]] = [[] for _ in range(n_ranks)]
    for k in order:
        load, r = heapq.heappop(heap)
        parts[r].append(k)
        heapq.heappush(heap, (load + float(costs[k]), r))
    return parts


def balance(costs, parts) -> float:
    """Largest rank load over the mean load (1.0 = perfect)."""
    costs = np.asarray(costs, dtype=float)
    loads = np.array([costs[p].sum() if len(p) else 0.0 for p in parts])
    return float(loads.max() / max(loads.mean(), 1e-300))


@dataclass
class Shard:
    rank: int
    world: int
    indices: list[int]  # positions in the ensemble of this rank's systems


def shard(sizes, rank: int, world: int) -> Shard:
    """This rank's share of an ensemble given its systems' bead counts."""
    parts = assign([system_cost(int(n)) for n in sizes], world)
    return Shard(rank, world, parts[rank])


def gather_in_order(local: dict, total: int, world: int, dst: int = 0):
    """Collect {ensemble index: result} from every rank; rank ``dst`` gets
    the list of all ``total`` results in ensemble order, the others None."""
    if world == 1:
        return [local[k] for k in range(total)]
    import torch.distributed as dist
    rank = dist.get_rank()
    bucket = [None] * world if rank == dst else None
    dist.gather_object(local, bucket, dst=dst)
    if rank != dst:
        return None
    merged = {}
    for part in bucket:
        overlap = merged.keys() & part.keys()
        if overlap:
            raise RuntimeError(f"systems {sorted(overlap)[:5]} came back from two ranks")
        merged.update(part)
    missing = [k for k in range(total) if k not in merged]
    if missing:
        raise RuntimeError(f"systems {missing[:5]} came back from no rank")
    return [merged[k] for k in range(total)]
