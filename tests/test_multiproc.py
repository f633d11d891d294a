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


def _spec_worker(rank, world, port, ncru, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch
    import torch.distributed as dist
    from gwgb300 import dist as gd
    from gwgb300.engine import Ensemble

    d = gd.init("gloo")
    out = {}
    for prec in ("fp32", "fp64"):
        b, e, cl, tile = Ensemble.partition_spec(ncru, world, rank, prec)
        t = torch.tensor([b, e, cl, tile], dtype=torch.int64)
        got = [torch.zeros(4, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(got, t)
        out[prec] = [g.tolist() for g in got]
    gd.barrier(d)
    q.put((rank, out))
    dist.destroy_process_group()


def test_two_rank_ensemble_partition_spec_gloo(enginelib):
    """Two ranks take contiguous, complete shares of a heterogeneous ensemble, and both shares get
    the launch shape of one context holding every cell (so the split reproduces it bit for bit);
    the cell_base of a share is its first global cell."""
    from gwgb300.engine import Ensemble

    ncru = [2000, 12500, 500, 7000, 64, 3000, 9000]
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_spec_worker, args=(r, world, port, ncru, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for prec in ("fp32", "fp64"):
        whole = Ensemble.partition_spec(ncru, 1, 0, prec)
        assert whole[:2] == (0, len(ncru))
        for rank, out in res:
            specs = out[prec]
            assert specs[0][0] == 0 and specs[-1][1] == len(ncru) and specs[0][1] == specs[1][0]
            assert all(s[2:] == list(whole[2:]) for s in specs)
