"""Sharding independent solves across ranks (one process per GPU).

Batched and served SDPs are independent units, so N GPUs split the
instances by a cost model and solve them with no exchange on the data path.
The only collectives are on the host side: the max-over-ranks timing and,
when a caller wants every result on rank 0, one gather of the per-rank
results.  Everything here runs with any ``torch.distributed`` backend (gloo
on CPU, NCCL on GPUs).
"""

from __future__ import annotations

import heapq
from typing import Callable, List, Sequence

__all__ = ["solve_cost", "shard_by_cost", "max_over_ranks", "gather_to_root", "solve_sharded"]


def solve_cost(model) -> float:
    """Relative cost of one interior-point iteration: sum n^3 over the PSD
    blocks plus m^3 / 3 for the Schur Cholesky plus the sparse assembly."""
    c = sum(float(n) ** 3 for n in model.sides) + float(model.m) ** 3 / 3.0
    for A in model.A:
        c += float(A.nnz) ** 2 / max(1, model.m)
    return c


def shard_by_cost(costs: Sequence[float], world: int) -> List[List[int]]:
    """Longest-processing-time assignment: instances in decreasing cost, each
    to the rank with the least assigned cost (ties to the lower rank).  Every
    index appears in exactly one shard; each shard is in increasing order."""
    if world <= 0:
        raise ValueError("world must be positive")
    heap = [(0.0, r) for r in range(world)]
    shards: List[List[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in shards]


def max_over_ranks(value: float) -> float:
    """The maximum of `value` over all ranks (the value itself without a
    process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_to_root(local: list, shard: Sequence[int], total: int):
    """Reassemble per-rank results in global order on rank 0 (None elsewhere)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        out = [None] * total
        for i, r in zip(shard, local):
            out[i] = r
        return out
    parts = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
    dist.gather_object((list(shard), local), parts, dst=0)
    if dist.get_rank() != 0:
        return None
    out = [None] * total
    for idx, res in parts:
        for i, r in zip(idx, res):
            out[i] = r
    return out


def solve_sharded(models: Sequence, solve: Callable[[list], list], rank: int, world: int):
    """Solve this rank's shard of `models` with `solve` (a list of models to a
    list of results) and gather every result on rank 0 in input order."""
    shards = shard_by_cost([solve_cost(m) for m in models], world)
    mine = shards[rank]
    local = solve([models[i] for i in mine]) if mine else []
    if len(local) != len(mine):
        raise RuntimeError("solve returned a different number of results than it was given")
    return gather_to_root(local, mine, len(models))
