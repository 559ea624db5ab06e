"""Independent replicas across GPUs (one process per GPU, launched by
torchrun): the soups of one rank never interact with those of another, so the
only cross-rank steps are a barrier around the timed region and the
reduction of the results (work summed over ranks, time maximised over ranks).

    rank, world, local = replicas.env()
    group = replicas.init()                  # None when world == 1
    replicas.barrier(group)
    ... timed work ...
    replicas.barrier(group)
    units, seconds = replicas.reduce(units, seconds, group)
"""
from __future__ import annotations

import os
from datetime import timedelta
from typing import Optional, Tuple


def env() -> Tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: Optional[str] = None, timeout_s: float = 300.0):
    """Joins the default process group when WORLD_SIZE > 1 (NCCL when CUDA is
    available, else gloo); returns it, or None for a single process."""
    rank, world, _ = env()
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29517")
        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend, rank=rank, world_size=world,
                                timeout=timedelta(seconds=timeout_s))
    return dist.group.WORLD


def barrier(group) -> None:
    if group is None:
        return
    import torch.distributed as dist
    dist.barrier(group=group)


def reduce(units: float, seconds: float, group) -> Tuple[float, float]:
    """(units summed over ranks, seconds maximised over ranks)."""
    if group is None:
        return float(units), float(seconds)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    s = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(s, op=dist.ReduceOp.MAX, group=group)
    return float(u.item()), float(s.item())


def replica_seed(seed: int, rank: int) -> int:
    """Rank 0 runs the configured seed; rank r > 0 an independent soup of the
    same configuration with seed + r."""
    return seed + rank
