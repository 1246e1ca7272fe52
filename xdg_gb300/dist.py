"""Multi-GPU helpers: the ray queries shard by index range with no data-path
collective (every rank holds the whole geometry and traces its own rays).
The only communication is timing: a barrier around the timed region and a
max-reduction of the elapsed time."""
from __future__ import annotations

import os


def env_rank():
    """(rank, world_size, local_rank) from the torchrun environment."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def shard_range(n: int, rank: int, world: int):
    """Contiguous [lo, hi) slice of n items for this rank (sizes differ by <= 1)."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def rank_seed(seed: int, rank: int) -> int:
    """Independent per-rank stream of synthetic inputs (weak scaling)."""
    return (seed * 1000003 + 7919 * rank) & 0x7FFFFFFF


def max_over_ranks(value: float, world: int) -> float:
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, world: int) -> float:
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
