"""Replica partitioning across ranks (world_size 2, gloo on CPU): disjoint, complete shares and
the max/sum reductions of the timing path."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, n_items, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch
    import torch.distributed as dist
    from gwgb300 import dist as gd

    d = gd.init("gloo")
    b, e = gd.partition(n_items, world, rank)
    share = torch.zeros(n_items, dtype=torch.int64)
    share[b:e] = 1
    dist.all_reduce(share)
    t_max = gd.max_over_ranks(d, float(rank + 1) * 1.5)
    total = gd.sum_over_ranks(d, float(e - b))
    gd.barrier(d)
    q.put((rank, share.tolist(), t_max, total))
    dist.destroy_process_group()


@pytest.mark.parametrize("n_items", [1, 7, 256])
def test_two_rank_partition_gloo(n_items):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n_items, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, share, t_max, total in res:
        assert share == [1] * n_items      # every item on exactly one rank
        assert t_max == 3.0 and total == n_items


def test_partition_bounds():
    from gwgb300.dist import partition

    for n in (0, 1, 5, 1024):
        for w in (1, 2, 3, 8):
            spans = [partition(n, w, r) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(w - 1))
            assert max(e - b for b, e in spans) - min(e - b for b, e in spans) <= 1
