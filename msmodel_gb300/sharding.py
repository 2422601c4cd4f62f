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


def split_points(npoint, rank, world):
    """Point indices of this rank when the points of one realisation are split
    over `world` ranks: contiguous blocks, the first npoint % world ranks one
    point longer (strong scaling of a complex cut or map)."""
    base, extra = divmod(npoint, world)
    start = rank * base + min(rank, extra)
    return np.arange(start, start + base + (1 if rank < extra else 0))


def run_cut_sharded(ks, rank, world, compute, gather=None):
    """ln det/n of one realisation at every k of a cut or map, the points split
    over `world` ranks (split_points); each rank evaluates its block on its GPU
    with no data-path collective, and one gather returns every rank the whole
    result in point order.

    compute(ks block) -> complex array over the block.
    gather(obj) -> list of every rank's obj (e.g. torch.distributed.all_gather_object)."""
    ks = np.atleast_1d(np.asarray(ks, dtype=np.complex128))
    idx = split_points(len(ks), rank, world)
    mine = (int(idx[0]) if len(idx) else 0, np.asarray(compute(ks[idx]) if len(idx) else np.zeros(0, complex)))
    parts = gather(mine) if gather is not None else [mine]
    out = np.empty(len(ks), dtype=np.complex128)
    seen = 0
    for start, vals in sorted(parts, key=lambda p: p[0]):
        out[start:start + len(vals)] = vals
        seen += len(vals)
    assert seen == len(ks), "missing points after gather"
    return out


def deal_by_cost(costs, world):
    """Indices dealt to `world` ranks, largest cost first, each to the rank with
    the least work so far (ties to the lowest rank): the uneven realisation
    sizes of the batched resonance search balance without any exchange."""
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def run_aberth_sharded(sizes, rank, world, compute=None, gather=None, dom=(0.5, 3.0, -1.0, 0.0), ntarget=32,
                       nbin=40, precision="mixed"):
    """The batched resonance search over realisations r = 1..len(sizes) (n_r =
    sizes[r-1], positions from fill_medium(seed=r)), split over `world` ranks by
    n^3 cost.  Each rank searches its own realisations on its GPU; one gather
    then joins the variable-length root lists and adds the ranks' histograms
    of Im k (nbin bins on [dom[2], dom[3]]).

    compute(list of realisation indices r) -> {r: roots}; defaults to this
    rank's GPU (find_eigenstates, method "determinant").
    gather(obj) -> list of every rank's obj (e.g. torch.distributed.all_gather_object).
    Returns ({r: roots} for every realisation, histogram counts)."""
    mine = deal_by_cost([float(n) ** 3 for n in sizes], world)[rank]
    reals = [i + 1 for i in mine]
    if compute is None:
        from . import api

        def compute(rs):
            if not rs:
                return {}
            media = [api.Medium(3, sizes[r - 1], seed=r) for r in rs]
            roots, _ = api.find_eigenstates(media, list(dom), ntarget, precision=precision)
            return dict(zip(rs, roots))
    roots = compute(reals)
    allr = np.concatenate([np.asarray(v) for v in roots.values()]) if roots else np.zeros(0, complex)
    hist, _ = np.histogram(allr.imag, bins=nbin, range=(dom[2], dom[3]))
    parts = gather((roots, hist)) if gather is not None else [(roots, hist)]
    every, total = {}, np.zeros(nbin, dtype=np.int64)
    for r_part, h_part in parts:
        every.update(r_part)
        total += h_part
    assert sorted(every) == list(range(1, len(sizes) + 1)), "missing realisations after gather"
    return every, total
