"""Multi-process path of bench.py: replicas only (the calling path has no data
exchange).  Each rank runs its own replica; the reported step time is the
maximum over ranks and the rate is every rank's sites over that time
(bench.replica_max, bench.replica_rate).  Exercised with the gloo backend on
CPU, world size 2: each rank also loads the native library and builds the
prior and rank tables through the C ABI (gsnp_prior_table, gsnp_rank_table,
host code), and the ranks check that their replicas' tables agree."""
import hashlib
import os
import sys

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from gsnp_gb300 import api, native

    r, w, _ = bench.dist_info()
    lib = native()
    p = api.params_from_flags(["-L", "100", "-t", "-u"], api.PRECISION_FP32_FIXUP)
    prior = np.empty(128, dtype=np.float64)
    rank_tab = np.empty(64 * 64 * 2048, dtype=np.float64)
    rc = lib.gsnp_prior_table(p, prior.ctypes.data) | lib.gsnp_rank_table(rank_tab.ctypes.data)
    digest = hashlib.sha256(prior.tobytes() + rank_tab.tobytes()).digest()
    # every replica's tables equal: the byte-wise max and min of the digests agree
    d = torch.tensor(list(digest), dtype=torch.int64)
    hi, lo = d.clone(), d.clone()
    dist.all_reduce(hi, op=dist.ReduceOp.MAX)
    dist.all_reduce(lo, op=dist.ReduceOp.MIN)
    step = bench.replica_max(dist, 10.0 + 5.0 * rank, device="cpu")
    rate = bench.replica_rate(w, 1000, step)
    q.put((r, w, rc, bool(torch.equal(hi, lo)), step, rate))
    dist.destroy_process_group()


def test_replicas_reduce_and_agree():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 2, 0, True, 15.0, 2000 / 15.0), (1, 2, 0, True, 15.0, 2000 / 15.0)]


def test_replica_helpers_without_a_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.replica_max(None, 12.5) == 12.5
    assert bench.replica_rate(1, 5.0e7, 0.018) == 5.0e7 / 0.018
