"""Multi-rank host logic on CPU: two gloo ranks agree on max time and total work."""

import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from rubix_gb300 import dist as rd

    t = rd.max_over_ranks(10.0 + rank)
    n = rd.sum_over_ranks(1000 * (rank + 1))
    out.put((rank, t, n, rd.world_info(), rd.rank_seed(5, rank)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, n, info, seed in res:
        assert t == 11.0 and n == 3000.0
        assert info == (2, rank, rank)
    assert res[0][4] != res[1][4]
