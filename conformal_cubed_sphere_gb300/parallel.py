"""Ensemble sharding across ranks (one process per GPU).

Members are independent, so an ensemble shards by member with no collective on
the data path: rank r of W advances members r, r + W, r + 2W, ...  The only
collectives are outside the data path: a barrier around the timed region and a
max-reduction of the per-rank time (the slowest rank bounds the job).
"""
from __future__ import annotations

import os


def dist_env() -> tuple[int, int, int]:
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard_members(n_members: int, rank: int, world: int) -> list[int]:
    """Member indices owned by `rank` (round robin, every member exactly once)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    return list(range(rank, n_members, world))


def slowest_rank_seconds(seconds: float, group=None) -> float:
    """Max over ranks of a per-rank duration (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(seconds)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
