"""Replica harness of the benchmark: one process per GPU, each training its
own replica (the step has no cross-GPU exchange), started by torchrun.  The
ranks meet at a barrier around the timed region; the job's time is the
slowest rank's, and the job's throughput counts every rank's steps."""
from __future__ import annotations

import os


def dist_env():
    """(world size, rank, local rank) from torchrun's environment."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init(ws: int):
    """Join the process group (gloo: only host-side scalars cross ranks)."""
    if ws > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("gloo")


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws: int, x: float) -> float:
    """The largest x over the ranks (every rank gets it)."""
    if ws == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(ws: int, steps_per_rank: int, slowest_s: float) -> float:
    """Whole-job throughput: all ranks' steps over the slowest rank's time."""
    return ws * steps_per_rank / slowest_s


def finish(ws: int):
    if ws > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()
