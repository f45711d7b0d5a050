"""Multi-GPU use of the engine: replicas only.

A single A* instance does not shard (the reference has no multi-GPU path and
a hash-distributed search would need an all-to-all of successors every
round).  Streams of independent instances shard across GPUs with no data-path
collective: rank r of N takes instances r, r+N, r+2N, ...  The only
collective is the timing reduction (max over ranks) and a barrier around the
timed region.
"""
from __future__ import annotations

import os
from typing import Sequence, TypeVar

T = TypeVar("T")


def dist_env() -> tuple[int, int, int]:
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def shard(items: Sequence[T], rank: int, world: int) -> list[T]:
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return list(items[rank::world])


def max_over_ranks(value: float) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier() -> None:
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()
