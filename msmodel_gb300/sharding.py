"""Multi-GPU sharding of the trace-log task: one process per GPU.

The (seed, k) points of run_tracelog_omp (reference src/core/ms_core.c:96-141)
are independent, so ranks split the seeds (rank r takes seeds r+1, r+1+W,
...), evaluate them on their own GPU with no data-path collective, and only
the final per-seed results are gathered once so that every rank can form the
reference's running average in seed order (ms_core.c:127) -- bit-identical to
the single-process result.
"""
import numpy as np


def rank_seeds(nseed, rank, world):
    """Seeds 1..nseed dealt round-robin: rank r gets r+1, r+1+world, ..."""
    return list(range(rank + 1, nseed + 1, world))


def seed_average(per_seed):
    """Running average over seeds in seed order, the reference's recurrence
    data = ((s-1) data + v_s) / s (ms_core.c:127)."""
    data = np.zeros_like(per_seed[0])
    for s, v in enumerate(per_seed, start=1):
        data = ((s - 1) * data + v) / s
    return data


def run_tracelog_sharded(d, n, ks, nseed, rank, world, compute=None, gather=None, model="maximum", params=(),
                         shape="ball", ratio=1.0, precision="fp64"):
    """ln det/n averaged over seeds 1..nseed, the seeds split over `world` ranks.

    compute(seed) -> complex array over ks; defaults to this rank's GPU.
    gather(obj) -> list of every rank's obj (e.g. torch.distributed.all_gather_object).
    """
    ks = np.atleast_1d(np.asarray(ks, dtype=np.complex128))
    if compute is None:
        from . import api

        def compute(seed):
            med = api.Medium(d, n, model=model, params=params, shape=shape, ratio=ratio, seed=seed)
            v, st = api.tracelog_batch([med], ks, precision=precision)
            if np.any(st != 0):
                raise api.MsgpuError(f"status {st[st != 0][:4]} for seed {seed}")
            return v
    mine = {s: compute(s) for s in rank_seeds(nseed, rank, world)}
    parts = gather(mine) if gather is not None else [mine]
    allv = {}
    for p in parts:
        allv.update(p)
    assert sorted(allv) == list(range(1, nseed + 1)), "missing seeds after gather"
    return seed_average([allv[s] for s in range(1, nseed + 1)])
