"""Multi-GPU form of the path: independent replicas, no collective on the data path.

The reference shards one BFS over a 2D R x C process grid and reduces
frontier slices between ranks (cpu_2d/globalbfs.hh:772-967); at one GPU per
process the single-root search does not shard, and the batched and serving
forms shard by roots: every rank holds the whole graph and runs its own share
of the roots.  The only inter-rank traffic is host-side bookkeeping: the
timing barrier, the max of the ranks' times and the sum of their throughput.
"""
from __future__ import annotations

import os
from typing import Sequence

import numpy as np


def world() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard_roots(roots: Sequence[int], per_rank: int, rank: int, world_size: int) -> np.ndarray:
    """This rank's roots: the rank-th block of per_rank roots out of the
    world_size * per_rank roots drawn for the whole job (blocks are disjoint,
    so the ranks search different roots)."""
    roots = np.asarray(roots, np.int64)
    if per_rank < 1 or world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("bad shard request")
    if len(roots) < per_rank * world_size:
        raise ValueError(f"{len(roots)} roots for {world_size} ranks x {per_rank}")
    return roots[rank * per_rank:(rank + 1) * per_rank].copy()


def _device(dist):
    import torch
    return torch.device("cuda") if dist.get_backend() == "nccl" else torch.device("cpu")


def barrier(dist) -> None:
    """Barrier over the ranks (no-op for a single process), then a device sync."""
    import torch
    if dist is not None:
        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def reduce_max(x: float, dist) -> float:
    """Max of x over the ranks (the job's time is its slowest rank's)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(x: float, dist) -> float:
    """Sum of x over the ranks (whole-job throughput)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
