"""Host logic of multi-GPU runs: one process per GPU, independent replicas (no collective on the
data path), timings reduced to the slowest rank.

The reference runs on one device. Here N ranks each run the whole workload on their own GPU and
the job's throughput is N x steps / (slowest rank's time) ("weak" scaling). For the naive path a
target-range split (`target_range`, the `nb_naive_accel_range` hook) shards one system across
ranks; its per-step exchange (an all-gather of positions) is not needed by any configuration
measured here.
"""

from __future__ import annotations

import os


def dist_env():
    """(world size, rank, local rank) from the torch.distributed launcher's environment."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def target_range(n: int, rank: int, world_size: int):
    """Contiguous [begin, end) of n targets for `rank`; sizes differ by at most one."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError(f"rank {rank} outside world of {world_size}")
    q, r = divmod(n, world_size)
    begin = rank * q + min(rank, r)
    return begin, begin + q + (1 if rank < r else 0)


def max_over_ranks(value: float, device=None) -> float:
    """Largest value over all ranks (the value itself without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, seconds_per_rank: float, world_size: int,
                   device=None) -> float:
    """Units all ranks processed divided by the slowest rank's time."""
    slowest = max_over_ranks(seconds_per_rank, device)
    return world_size * units_per_rank / slowest
