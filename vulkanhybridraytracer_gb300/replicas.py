"""Replicas: one process per GPU, no data-path collective.

The hybrid pass exchanges nothing between GPUs: every pixel and ray is
independent and the BVH is read-only, so each rank renders its own frames
from its own copy of the scene.  The only cross-rank traffic is the timing of
a weak-scaling run: a barrier before the timed region, each rank's device
time, the maximum over ranks, and whole-job throughput = the units of all
ranks / that maximum.  Ranks are launched by torchrun (RANK, LOCAL_RANK,
WORLD_SIZE, MASTER_ADDR/PORT in the environment).
"""
from __future__ import annotations

import os


def env():
    """(world_size, rank, local_rank) from the launcher's environment (1, 0, 0 without one)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str | None = None) -> bool:
    """Joins the process group when there is more than one rank; True if it did."""
    ws, _, _ = env()
    if ws <= 1:
        return False
    import torch
    import torch.distributed as dist

    if not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))
    return True


def barrier():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(seconds: float, device=None) -> float:
    """The slowest rank's time (the value itself on a single rank)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(seconds)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def throughput(units_per_rank: float, seconds_max: float, world_size: int) -> float:
    """Whole-job rate: the units every rank processed / the slowest rank's time."""
    return units_per_rank * world_size / seconds_max


def finalize():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
