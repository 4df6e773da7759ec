"""Replica-parallel runs: one independent VMC replica per GPU.

Each rank runs its own replica of the workload with its own seed: a replica's chains never
interact with another's, and no collective touches the data path. Ranks only meet at the
timing barriers, and the reported time is the slowest rank's (weak scaling).
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def world() -> int:
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def rank() -> int:
    return dist.get_rank() if dist.is_available() and dist.is_initialized() else 0


def replica_seed(base: int, rank_: int) -> int:
    """Seed of a replica: every rank samples its own chains."""
    return int(base) + int(rank_)


def barrier() -> None:
    if world() > 1:
        dist.barrier()


def max_over_ranks(x: float, device: torch.device | str = "cpu") -> float:
    """The maximum of a per-rank value (the slowest rank's elapsed time)."""
    if world() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, elapsed_max: float) -> float:
    """Whole-job throughput under weak scaling: every rank processed units_per_rank units."""
    return world() * float(units_per_rank) / float(elapsed_max)
