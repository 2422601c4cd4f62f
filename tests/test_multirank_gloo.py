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


SIZES = [30, 46, 24, 38]
DOM = (0.5, 3.0, -1.0, 0.0)


def _aberth_compute(rs):
    """The resonance search of realisations rs (n = SIZES[r-1], seed r) by the
    oracle, 8 Halton targets sorted by -Im, standing in for a rank's GPU."""
    from oracle import Oracle
    from msmodel_gb300 import halton_points
    o = Oracle()
    z0 = halton_points(DOM, 8)
    z0 = z0[np.argsort(-z0.imag, kind="stable")]
    return {r: o.solve_aberth(3, SIZES[r - 1], o.fill_medium(3, SIZES[r - 1], r), DOM, z0)[0] for r in rs}


def _aberth_worker(rank, world, port, q):
    import torch.distributed as dist
    from msmodel_gb300.sharding import run_aberth_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)

    def gather(obj):
        out = [None] * world
        dist.all_gather_object(out, obj)
        return out

    roots, hist = run_aberth_sharded(SIZES, rank, world, compute=_aberth_compute, gather=gather, dom=DOM, nbin=10)
    q.put((rank, roots, hist))
    dist.destroy_process_group()


def test_two_rank_resonance_search_gathers_roots_and_histogram():
    """Realisations dealt by n^3 cost, root lists of uneven length joined and
    the ranks' Im k histograms added: the single-process result exactly."""
    import multiprocessing as mp
    from msmodel_gb300.sharding import deal_by_cost
    assert deal_by_cost([n ** 3 for n in SIZES], 2) == [[1], [0, 2, 3]]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_aberth_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = {rank: (roots, hist) for rank, roots, hist in (q.get(timeout=300) for _ in procs)}
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = _aberth_compute(range(1, len(SIZES) + 1))
    allr = np.concatenate(list(want.values()))
    want_hist, _ = np.histogram(allr.imag, bins=10, range=(DOM[2], DOM[3]))
    for rank in (0, 1):
        roots, hist = got[rank]
        assert sorted(roots) == [1, 2, 3, 4]
        for r in roots:
            assert np.array_equal(roots[r], want[r])
        assert np.array_equal(hist, want_hist) and hist.sum() == allr.size


def _cut_worker(rank, world, port, q):
    import torch.distributed as dist
    from msmodel_gb300.sharding import run_cut_sharded
    from oracle import Oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    o = Oracle()
    pos = o.fill_medium(3, 48, 1)
    ks = 0.5 + 2.5 * np.arange(11) / 10 - 0.05j

    def compute(block):
        return o.tracelog_batch(3, 48, pos, block, nthreads=1)[0]

    def gather(obj):
        out = [None] * world
        dist.all_gather_object(out, obj)
        return out

    q.put((rank, run_cut_sharded(ks, rank, world, compute, gather)))
    dist.destroy_process_group()


def test_two_rank_cut_split_matches_single_process():
    """Strong scaling of one realisation's cut: 11 points split in blocks of 6
    and 5 over two ranks, one gather, the single-process cut bit for bit."""
    import multiprocessing as mp
    from msmodel_gb300.sharding import split_points
    from oracle import Oracle
    assert list(split_points(11, 0, 2)) == list(range(6)) and list(split_points(11, 1, 2)) == list(range(6, 11))
    assert sum(len(split_points(4096, r, 8)) for r in range(8)) == 4096
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_cut_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    o = Oracle()
    ks = 0.5 + 2.5 * np.arange(11) / 10 - 0.05j
    want = o.tracelog_batch(3, 48, o.fill_medium(3, 48, 1), ks, nthreads=1)[0]
    assert np.array_equal(got[0], want) and np.array_equal(got[1], want)
