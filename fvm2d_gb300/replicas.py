"""Replicas across GPUs: the hot path does not shard (one mesh's iteration
has no exchange step), so N GPUs run N independent batches of meshes.
Only timing scalars cross ranks (barrier, max of elapsed time, sum of work);
no collective touches the solver data."""
from __future__ import annotations

import os

import torch
import torch.distributed as dist


def world() -> tuple[int, int, int]:
    """(rank, local_rank, world_size) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def init(backend: str | None = None) -> bool:
    """Join the process group when launched with more than one rank."""
    rank, local, size = world()
    if size <= 1 or dist.is_initialized():
        return dist.is_initialized()
    if backend is None:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend=backend, rank=rank, world_size=size)
    return True


def _dev():
    if dist.is_initialized() and dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def barrier() -> None:
    if dist.is_initialized():
        dist.barrier()


def max_over_ranks(x: float) -> float:
    if not dist.is_initialized():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_dev())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float) -> float:
    if not dist.is_initialized():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_dev())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def shard(items, rank: int, size: int):
    """Round-robin share of a list of independent work items."""
    return [it for i, it in enumerate(items) if i % size == rank]


def seed_for(rank: int, k: int) -> int:
    """Distinct grid seeds per rank and replica."""
    return 1000 * rank + k + 2


def finish() -> None:
    if dist.is_initialized():
        dist.destroy_process_group()
