"""Multi-GPU execution of the integration path: independent replicas, no data-path collective.

Loop integrals are independent, so N GPUs run N independent batches (one process per GPU,
torchrun environment); the only collectives are host-side bookkeeping: a barrier before the
timed region and the maximum of the ranks' elapsed times after it.  `partition_by_cost` splits
one list of integrals over ranks by quadrature points (cost model = product of the orders) for
callers that shard a fixed workload instead of replicating it.
"""
from __future__ import annotations

import os
from typing import Sequence


def dist_env():
    """(rank, world size, local rank) from the torchrun environment (1 process: 0, 1, 0)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(x: float, device=None) -> float:
    """Maximum of `x` over the ranks of the default process group (x itself without one)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: int, steps: int, world: int, max_elapsed_s: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return units_per_rank * steps * world / max_elapsed_s


def partition_by_cost(costs: Sequence[float], world: int):
    """Contiguous ranges [lo, hi) of `costs`, one per rank, with nearly equal total cost
    (greedy prefix split at multiples of total/world).  Every index lands in exactly one range."""
    n = len(costs)
    total = float(sum(costs))
    bounds = [0]
    acc = 0.0
    r = 1
    for i, c in enumerate(costs):
        acc += c
        while r < world and acc >= total * r / world and len(bounds) <= r:
            bounds.append(i + 1)
            r += 1
    while len(bounds) < world:
        bounds.append(n)
    bounds.append(n)
    return [(bounds[k], bounds[k + 1]) for k in range(world)]
