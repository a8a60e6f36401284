"""Multi-rank bookkeeping of the benchmark: one process per GPU, each running
an independent replica of the whole mesh (the timestep is not sharded across
GPUs in this build).  The helpers work with any torch.distributed backend
(NCCL on GPUs, gloo on CPU for the tests)."""
from __future__ import annotations

import os


def rank_env() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment (1, 0, 0 when absent)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(value: float, device="cpu") -> float:
    """The largest value over all ranks (the slowest replica's time); the value
    itself when no process group is initialised."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, units_per_rank: int, steps: int, total_ms: float) -> float:
    """Units processed by all ranks per second, timed by the slowest rank (weak
    scaling: every rank holds the same work)."""
    return world * units_per_rank * steps / (total_ms * 1e-3)
