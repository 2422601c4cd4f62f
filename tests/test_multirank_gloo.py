"""The multi-rank path on CPU: two gloo ranks split the seeds of a trace-log
task, gather once, and produce the single-process seed average bit for bit.
The oracle stands in for each rank's GPU."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from msmodel_gb300.sharding import run_tracelog_sharded
    from oracle import Oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    o = Oracle()
    ks = np.array([0.7 - 0.05j, 1.6 - 0.2j, 2.8 - 0.05j])

    def compute(seed):
        v, _ = o.tracelog_batch(3, 40, o.fill_medium(3, 40, seed), ks, nthreads=1)
        return v

    def gather(obj):
        out = [None] * world
        dist.all_gather_object(out, obj)
        return out

    res = run_tracelog_sharded(3, 40, ks, nseed=5, rank=rank, world=world, compute=compute, gather=gather)
    q.put((rank, res))
    dist.destroy_process_group()


def test_two_rank_seed_split_matches_single_process():
    import multiprocessing as mp
    from msmodel_gb300.sharding import rank_seeds, seed_average
    from oracle import Oracle
    assert rank_seeds(5, 0, 2) == [1, 3, 5] and rank_seeds(5, 1, 2) == [2, 4]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    o = Oracle()
    ks = np.array([0.7 - 0.05j, 1.6 - 0.2j, 2.8 - 0.05j])
    want = seed_average([o.tracelog_batch(3, 40, o.fill_medium(3, 40, s), ks, nthreads=1)[0] for s in range(1, 6)])
    assert np.array_equal(got[0], want) and np.array_equal(got[1], want)
