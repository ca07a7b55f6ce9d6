"""Replica aggregation for N GPUs of one node.

The CASPT2 path does not shard on this target: each rank runs complete, independent solves
on its own GPU (weak scaling, no collective on the data path). The only cross-rank step is
the timing of a benchmark: every rank times its own steps, the slowest rank's time bounds
the job, and the whole-job throughput counts every rank's solves.
"""
from __future__ import annotations

from typing import Sequence, Tuple


def max_over_ranks(values: Sequence[float]) -> Tuple[float, ...]:
    """Element-wise maximum of per-rank values over the default process group (identity on
    a single process)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return tuple(float(v) for v in values)
    import torch
    t = torch.tensor(list(values), dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return tuple(float(x) for x in t)


def replica_throughput(seconds: Sequence[float], steps: int, world: int) -> Tuple[float, ...]:
    """Whole-job solves/s for each timed leg: world * steps / (slowest rank's seconds)."""
    worst = max_over_ranks(seconds)
    return tuple(world * steps / s if s > 0 else float("inf") for s in worst)


def barrier() -> None:
    """Process-group barrier (no-op on a single process)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()
