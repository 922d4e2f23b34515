"""Process-group helpers for multi-GPU runs.

Galaxies are independent, so a multi-GPU run gives every rank its own galaxies and
exchanges nothing on the data path; ranks only agree on timings (max over ranks) and
totals (sum over ranks).  One process per GPU, launched by torchrun.
"""

from __future__ import annotations

import os

import torch


def world_info():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _reduce(value: float, op) -> float:
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = torch.device("cuda", torch.cuda.current_device()) \
        if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(value: float) -> float:
    import torch.distributed as dist

    return _reduce(value, dist.ReduceOp.MAX)


def sum_over_ranks(value: float) -> float:
    import torch.distributed as dist

    return _reduce(value, dist.ReduceOp.SUM)


def rank_seed(base: int, rank: int) -> int:
    """Seed of the galaxy rendered by ``rank`` (independent galaxies per rank)."""
    return int(base) + 7919 * int(rank)
