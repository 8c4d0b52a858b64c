"""Multi-GPU runs as replicas: one process per GPU (torchrun), each with its
own plans and states, and no collective on the data path.

A single solve does not shard cheaply (every pass needs whole pencils, so a
decomposition would need an all-to-all transpose per pass, which the
reference does not have either).  Work lists of independent solves -- an
ensemble, a request stream -- split by instance: ``shard`` assigns each rank a
set of solves with about equal cost, the ranks run them alone, and the host
combines timings and counts with ``reduce_max`` / ``reduce_sum``.
"""
from __future__ import annotations

from typing import List, Sequence

import torch


def shard(costs: Sequence[float], rank: int, world: int) -> List[int]:
    """Indices of the items rank ``rank`` of ``world`` runs: longest item
    first to the least loaded rank (ties: lower rank), deterministic on every
    rank.  Returned in increasing index order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} out of range for world {world}")
    load = [0.0] * world
    mine: List[int] = []
    for i in sorted(range(len(costs)), key=lambda k: (-float(costs[k]), k)):
        r = min(range(world), key=lambda q: (load[q], q))
        load[r] += float(costs[i])
        if r == rank:
            mine.append(i)
    return sorted(mine)


def _reduce(x: float, op) -> float:
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def reduce_max(x: float) -> float:
    """Maximum over ranks (a run's time is its slowest rank's)."""
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.MAX)


def reduce_sum(x: float) -> float:
    """Sum over ranks (solves, cell updates)."""
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.SUM)
