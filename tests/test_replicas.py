"""Multi-GPU host logic on CPU: two gloo ranks shard the roots, time with a
barrier and take the max of their times and the sum of their throughput (the
path itself has no collective)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from gpugraph500_gb300 import replicas  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, roots, per_rank, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = replicas.shard_roots(roots, per_rank, rank, world)
        t = torch.from_numpy(mine)
        got = [torch.empty_like(t) for _ in range(world)]
        dist.all_gather(got, t)
        replicas.barrier(dist)
        mx = replicas.reduce_max(float(rank + 1), dist)
        sm = replicas.reduce_sum(float(10 * (rank + 1)), dist)
        out[rank] = (torch.cat(got).tolist(), mx, sm)
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_and_reduce():
    world, per_rank = 2, 5
    roots = np.arange(100, 100 + world * per_rank + 3, dtype=np.int64)
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, _free_port(), roots, per_rank, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        gathered, mx, sm = res[rank]
        # disjoint blocks that together are the first world * per_rank roots
        assert gathered == roots[: world * per_rank].tolist()
        assert mx == 2.0 and sm == 30.0


def test_shard_roots_single_and_errors():
    roots = np.arange(8)
    assert replicas.shard_roots(roots, 8, 0, 1).tolist() == list(range(8))
    assert replicas.shard_roots(roots, 4, 1, 2).tolist() == [4, 5, 6, 7]
    with pytest.raises(ValueError):
        replicas.shard_roots(roots, 5, 0, 2)  # too few roots for the job
    with pytest.raises(ValueError):
        replicas.shard_roots(roots, 4, 2, 2)  # rank out of range
    assert replicas.reduce_max(3.5, None) == 3.5 and replicas.reduce_sum(2.0, None) == 2.0
