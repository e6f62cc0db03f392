"""Multi-GPU form of the path: independent replicas.

Rays, pixels and scenes are independent and the path has no exchange step,
so N GPUs run N full replicas of the workload (one process per GPU, launched
by torchrun). The only cross-rank traffic is host bookkeeping: a barrier
around the timed region and the maximum of the per-rank times, from which
the whole-job throughput is (units per rank * ranks) / max time.
"""
from __future__ import annotations

import os


def init(backend: str | None = None):
    """Returns (world, rank, local_rank); initialises torch.distributed for N > 1."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))
    return world, rank, local


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, world: int, max_seconds: float) -> float:
    """Whole-job units per second of `world` replicas timed by the slowest."""
    return units_per_rank * world / max_seconds
