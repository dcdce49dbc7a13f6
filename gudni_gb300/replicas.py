"""Multi-GPU form of the raster path: replicas.

Frames (and the scenes of a batch) are independent, so N ranks, one per GPU, each
render their own frames with no data-path collective (weak scaling).  The only
communication is the timing: the job takes as long as its slowest rank, and its
throughput is the units every rank processed over that time.  Ranks are started by
torch.distributed.run (RANK / LOCAL_RANK / WORLD_SIZE / MASTER_ADDR / MASTER_PORT).
"""
from __future__ import annotations

import os
from typing import Tuple


def ranks() -> Tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(world: int, backend: str) -> None:
    """Join the process group when there is more than one rank."""
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend)


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value: float, world: int, device="cpu") -> float:
    """The largest `value` over all ranks (the job's time is its slowest rank's)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job throughput: every rank's units over the slowest rank's time."""
    return world * units_per_rank / seconds
