"""Multi-process path of bench.py: replicas only (the calling path has no data
exchange).  Each rank times its own replica; the reported step time is the
maximum over ranks.  Exercised with the gloo backend on CPU, world size 2."""
import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = torch.tensor([10.0 + 5.0 * rank], dtype=torch.float64)   # per-rank step time
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    sites = torch.tensor([1000], dtype=torch.int64)
    dist.all_reduce(sites, op=dist.ReduceOp.SUM)
    q.put((rank, float(t.item()), int(sites.item())))
    dist.destroy_process_group()


def test_replica_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 15.0, 2000), (1, 15.0, 2000)]
