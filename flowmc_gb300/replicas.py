"""Independent sampler replicas, one process per GPU.

Chains are independent, so N ranks run N replicas of the whole schedule with
distinct seeds and no collective on the data path ("replicas only"). The
job's timing is the slowest rank's (maximum over ranks) and its throughput
the sum of the ranks' work over that time.
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def replica_seed(base_seed: int, rank: int) -> int:
    """Seed of replica `rank`: distinct per rank, rank 0 keeps the base seed."""
    return int(base_seed) + 1000003 * int(rank)


def world_size() -> int:
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of `value` over all ranks (the value itself on one rank)."""
    if world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, seconds: float, world: int | None = None) -> float:
    """Whole-job units/s: every rank processed `units_per_rank` in `seconds` (the slowest rank's time)."""
    return units_per_rank * (world_size() if world is None else world) / seconds
