"""Host-side logic of replica runs: one process per GPU, independent solves.

SLQ probes are independent until the final mean, so N GPUs run N independent
solve streams; the only cross-rank traffic is timing bookkeeping (a barrier
before and after the timed region and the maximum of the per-rank times), and
no collective touches the data path.  These helpers work with the nccl
backend (GPU ranks) and the gloo backend (CPU ranks, used by the tests).
"""

from __future__ import annotations

import os

import torch


def world() -> tuple[int, int, int]:
    """(rank, world_size, local_rank) from the torchrun environment (defaults: single process)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _device():
    import torch.distributed as dist

    return torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")


def barrier(world_size: int) -> None:
    if world_size > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world_size: int) -> float:
    """Largest value of x over all ranks (the slowest rank's time)."""
    if world_size == 1:
        return float(x)
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, world_size: int) -> float:
    if world_size == 1:
        return float(x)
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def aggregate_throughput(units_this_rank: float, seconds_this_rank: float, world_size: int) -> float:
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    total = sum_over_ranks(units_this_rank, world_size)
    slowest = max_over_ranks(seconds_this_rank, world_size)
    return total / slowest
