"""Replicas across GPUs: the SpMM path does not shard, so N GPUs run N independent replicas.

Each rank packs its own weights (distinct seeds), runs the same number of steps, and the job's
time is the slowest rank's.  There is no collective on the data path: the only cross-rank
traffic is one barrier before the timed region and one MAX reduction of the measured time.
"""
from __future__ import annotations


def shard_seed(rank: int, replica: int) -> int:
    """Seed of replica `replica` on rank `rank`: distinct for every (rank, replica) below 1000 replicas."""
    if replica < 0 or replica >= 1000 or rank < 0:
        raise ValueError(f"replica {replica} / rank {rank} out of range")
    return 1000 * (rank + 1) + replica


def max_over_ranks(ms: float, device=None) -> float:
    """Slowest rank's time (ms).  One process (no process group) returns `ms` itself."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank_step: float, steps: int, world: int, ms: float) -> float:
    """Units of all ranks per second: every rank processed `units_per_rank_step` per step (weak scaling)."""
    if ms <= 0 or steps <= 0 or world <= 0:
        raise ValueError("steps, world and the measured time must be positive")
    return units_per_rank_step * steps * world / (ms / 1e3)
