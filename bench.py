"""Benchmark: ln det M(k) evaluations per second on one GB300.

Workload (the configuration the headline metric is quoted on): d = 3, N = 1024
scatterers uniform in a ball at density 1 (seed 1, the reference's generator),
model "maximum", ln det M(k)/N on the complex cut of 4096 equispaced k on
Re k in [0.5, 3] at Im k = -0.05 (the central samples of a reference kcut with
sample = 4096).  One step = the hot path over the whole cut.

  value  : evals/s with positions and k already resident in HBM (msgpu_job_run)
  e2e    : evals/s through the C-ABI call a user makes with host buffers
           (msgpu_tracelog_batch: H2D of inputs, the kernels, D2H of results)
  roofline: the engine's binding unit (the FP64 pipe, peak = a DFMA probe run
           here) with achieved = 8/3 N^3 flops per ln det / step time, and
           the DRAM traffic of one ncu capture scaled to the launch
  cpu_baseline: the reference algorithm on all host cores, bounded sample
  clocks: nvidia-smi samples during the timed region
  gpu_launches: this library's kernel launches in the timed region
  mixed / aberth: the mixed-precision engine on the same cut, and the
           resonance search (mixed over 256 realisations, FP64 over the first
           32, the reference algorithm on the first 16, root lists compared)
  configs: compact legs of the other configurations -- C1 (d=3 N=64 map),
           C3 (d=2 N=2048 map, its 16x16 subgrid) and C5 (wavefunction
           N=4096, 256 k; FP64 on every 16th k) -- each with both engines,
           its accuracy against FP64 and the oracle, and a CPU baseline

Other configurations print one line each with --workload map64 | map2d |
aberth | wave; --workload eigvals times the eigenvalues of M(k) behind the
mu-plane histograms (batches at n = 128, 256, 512) against LAPACK zgeev.

Multi-GPU (torchrun): weak scaling by default -- each rank evaluates the full
cut for its own realisation (seed = rank + 1); --scaling strong splits the
4096 points of one realisation's cut over the ranks in contiguous blocks.  No
collective on the data path either way.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
  python bench.py --impl reference ...   (the reference algorithm on the host cores)
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

D, N, NK = 3, 1024, 4096
KMIN, KMAX = 0.5 - 0.05j, 3.0 - 0.05j
METRIC = "ln det M(k) evals/s at N=1024 d=3 (complex cut, 4096 k)"
UNIT = "evals/s"


def workload_ks():
    from msmodel_gb300 import kcut_args
    return kcut_args(NK, KMIN, KMAX)[4::3][:NK].copy()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, lr


TRAFFIC_FILE = os.path.join("profiles", "dram_traffic.json")


def recorded_traffic(precision, points):
    """DRAM bytes of one engine launch over `points` cut points at N=1024: the
    per-ln-det bytes of an ncu capture (dram__bytes_read + write of one
    304-point launch, recorded in the data file TRAFFIC_FILE with its command)
    times the points.  Not measured by this run: ncu cannot run inside it."""
    try:
        with open(os.path.join(ROOT, TRAFFIC_FILE)) as f:
            rec = json.load(f)["kcut_d3_n1024"][precision]
    except (OSError, KeyError, ValueError):
        return None, "no recorded capture"
    per_eval = (rec["dram_read"] + rec["dram_write"]) / rec["points"]
    return per_eval * points, (f"recorded ncu capture ({TRAFFIC_FILE}: {rec['kernel']}, one {rec['points']}-point "
                               f"launch), per-ln-det bytes x {points} points")


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        self.f.flush()
        rows = []
        with open(self.f.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    try:
                        rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
                    except ValueError:
                        pass
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def oracle_cut(o):
    """The 4096 cut points and the N=1024 seed-1 positions from the oracle
    alone (the reference arm and the CPU baselines load no library of this
    package): central samples of the reference kcut, get_arg_ccut order."""
    ks = o.kcut_args(NK, KMIN, KMAX)[4::3][:NK].copy()
    return ks, o.fill_medium(D, N, 1)


def strided_indices(nk, step, per_step, stride=128):
    """`per_step` indices of cut points for step `step`, strided across the
    whole cut: offsets step, step + stride, ... (mod stride), so that successive
    steps walk every residue class and the sample spans Re k in [0.5, 3]."""
    out = []
    r = step
    while len(out) < per_step:
        out.extend(range(r % stride, nk, stride)[: per_step - len(out)])
        r += 1
    return np.asarray(out)


def strided_sample(ks, step, per_step, stride=128):
    return ks[strided_indices(len(ks), step, per_step, stride)]


_ORACLE_SAMPLE = {}


def cpu_baseline(seconds=15.0):
    """The reference algorithm (oracle port: reference assembly + OpenBLAS
    zgetrf, one LAPACK thread per OpenMP thread, as run_tracelog_omp) on all
    host cores, on a bounded sample of the same cut strided across all 4096 k."""
    from oracle import Oracle
    o = Oracle()
    threads = os.cpu_count() or 1
    ks, pos = oracle_cut(o)
    per_chunk = 2 * threads
    done, t0, i = 0, time.perf_counter(), 0
    idx, vals = [], []
    while True:
        ix = strided_indices(len(ks), i, per_chunk)
        vals.append(o.tracelog_batch(D, N, pos, ks[ix], nthreads=threads)[0])
        idx.append(ix)
        done += len(ix)
        i += 1
        el = time.perf_counter() - t0
        if el >= seconds and i >= 2:
            break
    # the oracle's values, for the GPU engines' error on these points (taken out of the line)
    _ORACLE_SAMPLE["idx"], _ORACLE_SAMPLE["values"] = np.concatenate(idx), np.concatenate(vals)
    return {"value": done / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{done} of the 4096 cut points taken every 128th across the cut (offsets 0..{i - 1}), "
                      f"N=1024 d=3 seed 1, {threads} OpenMP threads x 1 OpenBLAS thread "
                      f"({' '.join(o.lapack_config().split()[0:2])})", "seconds": el}


def measure_mixed(ms, torch, med, ks, out64, args, stream, flush, ws, barrier):
    """The mixed-precision engine on the same workload in the same process:
    throughput (resident and end to end), its ratio to the FP64 engine, and
    the ln det error of every point against the FP64 results."""
    job = ms.Job("tracelog", [med], ks, precision="mixed")
    for _ in range(args.warmup):
        job.run(stream.cuda_stream)
    barrier()
    l0 = ms.launch_count()
    times = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        job.run(stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    barrier()
    launches = ms.launch_count() - l0
    tot = sum(times)
    if ws > 1:
        t = torch.tensor([tot], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        tot = float(t.item())
    value = args.steps * len(ks) * ws / tot
    outm, st = job.results()
    assert np.all(st == 0), "non-zero status in the mixed results"
    lnd64, lndm = out64 * med.n, outm * med.n
    relerr = np.abs(lndm.real - lnd64.real) / np.abs(lnd64.real)
    t0 = time.perf_counter()
    o2, _ = ms.tracelog_batch([ms.Medium(D, med.n, pos=ms.fill_medium(D, med.n, med.seed), seed=med.seed)], ks,
                              precision="mixed")
    e_el = time.perf_counter() - t0
    n = med.n
    # bf16 tensor work actually executed: 40 real n x n x 32 slice products per
    # 32-column panel step (4 real products x 10 slice pairs), i.e. 80/3 n^3 flops
    tensor_flops = 80.0 / 3.0 * n ** 3 * len(ks) / (tot / args.steps)
    return {"_out": outm, "value": value, "unit": UNIT, "ms_per_step": 1e3 * tot / args.steps,
            "gpu_launches": launches, "ratio_vs_fp64": None,
            "e2e": {"value": len(ks) * ws / e_el, "unit": UNIT, "steps": 1},
            "lndet_rel_err_vs_fp64": {"max": float(relerr.max()), "median": float(np.median(relerr)),
                                      "points": int(relerr.size)},
            "im_branch_max_dist": float(np.max(np.abs(((lndm.imag - lnd64.imag) + np.pi) % (2 * np.pi) - np.pi))),
            "roofline": {"bound": "tensor", "achieved": tensor_flops / 1e12,
                         "traffic": recorded_traffic("mixed", len(ks))[0] if n == N else None,
                         "peak": read_peaks().get("bf16_tflops_sustained", 1728.6), "unit": "TFLOP/s",
                         "frac": tensor_flops / 1e12 / read_peaks().get("bf16_tflops_sustained", 1728.6),
                         "counted": "bf16 tensor flops executed (80/3 n^3 per ln det)",
                         "algorithmic_tflops": 8.0 / 3.0 * n ** 3 * len(ks) / (tot / args.steps) / 1e12}}


ABERTH_DOM = [0.5, 3.0, -1.0, 0.0]


def match_count(got, want, tol):
    """Roots of `want` that have a distinct root of `got` within tol*|k|."""
    got = list(np.asarray(got))
    n = 0
    for w in np.asarray(want):
        if not got:
            break
        dist = np.abs(np.asarray(got) - w)
        j = int(np.argmin(dist))
        if dist[j] <= tol * max(abs(w), 1.0):
            got.pop(j)
            n += 1
    return n


def aberth_media(ms, count):
    """Realisations r = 1..count of the batched resonance search: d=3, N_r drawn
    from [100, 600] by the reference generator (init_random(0), in order),
    positions from fill_medium(seed=r)."""
    sizes = ms.realisation_sizes(count, seed=0)
    return [ms.Medium(D, n, seed=r + 1) for r, n in enumerate(sizes)]


def measure_aberth(ms, torch, count, fp64_count, cpu_sample):
    """Resonance search (Aberth-Ehrlich on dlogf, 32 Halton seeds, nexpsup 4,
    maxit 30, toler 1e-10): roots/s of the mixed search (mixed dlogf far from
    the roots, FP64 near them, FP64 update) over `count` realisations and of
    the FP64 search over the first `fp64_count`, the agreement of their root
    lists there, the reference algorithm on the first `cpu_sample` on all host
    cores with both GPU searches checked against its root lists, and the
    40-bin histogram of Im k over every mixed root."""
    media = aberth_media(ms, count)
    z0 = ms.halton_points(ABERTH_DOM, 32)
    res, roots = {}, {}
    nf = min(count, fp64_count)
    for prec, meds in (("fp64", media[:nf]), ("mixed", media)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rs, ne = ms.solve_aberth_batch(meds, ABERTH_DOM, z0, 4, 30, 1e-10, precision=prec)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        nr = sum(len(r) for r in rs)
        roots[prec] = rs
        res[prec] = {"roots_per_s": nr / el, "roots": nr, "realisations": len(meds), "dlogf_evals": ne,
                     "dlogf_per_s": ne / el, "seconds": el}
    found = sum(match_count(roots["mixed"][i], roots["fp64"][i], 1e-8) for i in range(nf))
    res["mixed_matches_fp64"] = {"matched": found, "fp64_roots": res["fp64"]["roots"],
                                 "mixed_roots": sum(len(r) for r in roots["mixed"][:nf]), "realisations": nf}
    allim = np.concatenate([r.imag for r in roots["mixed"]]) if res["mixed"]["roots"] else np.zeros(0)
    hist, _ = np.histogram(allim, bins=40, range=(-1.0, 0.0))
    res["imag_histogram"] = {"range": [-1.0, 0.0], "bins": 40, "counts": hist.tolist()}
    if cpu_sample:
        import concurrent.futures as cf
        from oracle import Oracle
        o = Oracle()
        sample = media[:min(cpu_sample, nf)]
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
            outs = list(ex.map(lambda m: o.solve_aberth(D, m.n, m.pos, ABERTH_DOM, z0)[0], sample))
        el = time.perf_counter() - t0
        nr = sum(len(r) for r in outs)
        res["cpu_baseline"] = {"roots_per_s": nr / el, "roots": nr, "realisations": len(sample),
                               "cores": os.cpu_count(), "kind": "port", "seconds": el}
        # the GPU searches against the oracle's root lists on the same realisations
        for prec in ("fp64", "mixed"):
            got = roots[prec][:len(sample)]
            res[prec + "_matches_oracle"] = {
                "matched": sum(match_count(got[i], outs[i], 1e-8) for i in range(len(sample))),
                "oracle_roots": nr, "gpu_roots": sum(len(r) for r in got), "realisations": len(sample)}
    res["config"] = {"realisations": count, "natom": "100..600 (reference generator, seed 0)", "seeds": 32,
                     "domain": ABERTH_DOM, "nexpsup": 4, "maxit": 30, "toler": 1e-10}
    return res


# ------------------------------------------------------------------ other configurations
# Measurement lines for the other configurations of the hot path (one JSON
# line each, `--workload`); the default line above is the headline.

def _wall(torch, fn):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return r, time.perf_counter() - t0


def _resident(ms, torch, kind, media, ks, precision, steps, warmup, item_med=None):
    """evals/s of a resident job (inputs in HBM), CUDA events on torch's stream."""
    job = ms.Job(kind, media, ks, item_med=item_med, precision=precision)
    st = torch.cuda.current_stream()
    for _ in range(warmup):
        job.run(st.cuda_stream)
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        job.run(st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1) * 1e-3
    out, status = job.results()
    return len(ks) * steps / tot, out, status


def workload_map64(ms, torch, args):
    """Complex map of ln det M(k)/N, d=3 N=64 seed 1, 64x64 k on [0.5,3] x [-0.5,0]."""
    med = ms.Medium(3, 64, seed=1)
    ks = ms.kplane_args(64, 64, 0.5, 3.0, -0.5, 0.0)
    v64, o64, s64 = _resident(ms, torch, "tracelog", [med], ks, "fp64", args.steps, args.warmup)
    vmx, omx, smx = _resident(ms, torch, "tracelog", [med], ks, "mixed", args.steps, args.warmup)
    (_, _), e2e = _wall(torch, lambda: ms.tracelog_batch([med], ks, precision="fp64"))
    err = np.abs((omx - o64).real) / np.abs(o64.real)
    line = {"workload": "kplane d=3 N=64 64x64 Re[0.5,3] Im[-0.5,0]", "unit": "evals/s",
            "fp64": v64, "mixed": vmx, "e2e_fp64": len(ks) / e2e,
            "mixed_lndet_rel_err": {"max": float(err.max()), "median": float(np.median(err))},
            "status_nonzero": int(np.count_nonzero(s64) + np.count_nonzero(smx))}
    if not args.no_cpu:
        from oracle import Oracle
        o = Oracle()
        _, el = _wall(torch, lambda: o.tracelog_batch(3, 64, med.pos, ks, nthreads=os.cpu_count()))
        ref = o.tracelog_batch(3, 64, med.pos, ks, nthreads=os.cpu_count())
        line["cpu_baseline"] = {"value": len(ks) / el, "cores": os.cpu_count(), "kind": "port",
                                "sample": "the whole 4096-point map"}
        line["fp64_vs_oracle_max_rel"] = float(np.max(np.abs((o64 - ref[0]).real) / np.abs(ref[0].real)))
    return line


def workload_map2d(ms, torch, args):
    """Complex map d=2 N=2048 seed 1, 256x256 k on [0.5,4] x [-0.3,0]: the mixed
    engine on the whole map, the FP64 engine on every 16th row and column, and
    the mixed ln det error against FP64 on that subgrid."""
    med = ms.Medium(2, 2048, seed=1)
    ks = ms.kplane_args(256, 256, 0.5, 4.0, -0.3, 0.0)
    sub = ks.reshape(256, 256)[::16, ::16].reshape(-1).copy()
    frac = args.sample if args.sample else 1.0
    kmix = ks[:int(len(ks) * frac)]
    vmx, omx, smx = _resident(ms, torch, "tracelog", [med], kmix, "mixed", 1, 1)
    v64, o64, s64 = _resident(ms, torch, "tracelog", [med], sub, "fp64", 1, 1)
    osub, _ = ms.tracelog_batch([med], sub, precision="mixed")
    lnd64, lndm = o64 * 2048, osub * 2048
    err = np.abs(lndm.real - lnd64.real) / np.abs(lnd64.real)
    stats = ms.engine_stats() if os.environ.get("MSGPU_STATS") else None
    cpu = None
    if not args.no_cpu:
        from oracle import Oracle
        o = Oracle()
        th = os.cpu_count() or 1
        sample = sub[:2 * th]
        t0 = time.perf_counter()
        o.tracelog_batch(2, 2048, med.pos, sample, nthreads=th)
        el = time.perf_counter() - t0
        cpu = {"value": len(sample) / el, "unit": "evals/s", "cores": th, "kind": "port",
               "sample": f"{len(sample)} points of the 16x16 subgrid, {th} OpenMP threads x 1 OpenBLAS thread"}
    return {**({"phase_cycles_last_mixed_job": stats} if stats else {}), **({"cpu_baseline": cpu} if cpu else {}),
            "workload": f"kplane d=2 N=2048 256x256 Re[0.5,4] Im[-0.3,0] (mixed on {len(kmix)} points)",
            "unit": "evals/s", "mixed": vmx, "fp64": v64, "ratio": vmx / v64,
            "mixed_lndet_rel_err_subgrid": {"max": float(err.max()), "median": float(np.median(err)),
                                            "points": int(err.size)},
            "im_branch_max_dist": float(np.max(np.abs(((lndm.imag - lnd64.imag) + np.pi) % (2 * np.pi) - np.pi))),
            "status_nonzero": {"mixed": int(np.count_nonzero(smx)), "fp64": int(np.count_nonzero(s64))}}


def workload_aberth(ms, torch, args):
    """Batched resonance search over realisations 1..count (N from [100,600]):
    roots/s of the mixed (FP64-finished) search on all of them, the FP64 search
    on the first `fp64_count`, the root-set agreement there, and the histogram
    of Im k of every root (40 bins on [-1, 0])."""
    count = args.count or 4096
    media = aberth_media(ms, count)
    z0 = ms.halton_points(ABERTH_DOM, 32)
    (rm, nem), elm = _wall(torch, lambda: ms.find_eigenstates(media, ABERTH_DOM, 32, 30, 1e-10, "mixed"))
    nf = min(count, args.fp64_count)
    (r64, ne64), el64 = _wall(torch, lambda: ms.find_eigenstates(media[:nf], ABERTH_DOM, 32, 30, 1e-10, "fp64"))
    nrm, nr64 = sum(len(r) for r in rm), sum(len(r) for r in r64)
    matched = sum(match_count(rm[i], r64[i], 1e-8) for i in range(nf))
    extra = sum(len(rm[i]) for i in range(nf)) - matched
    hist, edges = np.histogram(np.concatenate([r.imag for r in rm]) if nrm else np.zeros(0), bins=40,
                               range=(-1.0, 0.0))
    line = {"workload": f"aberth d=3 N in [100,600] {count} realisations, 32 Halton seeds",
            "unit": "roots/s", "mixed": nrm / elm, "mixed_roots": nrm, "mixed_dlogf_evals": nem,
            "mixed_seconds": elm, "fp64": nr64 / el64, "fp64_realisations": nf, "fp64_roots": nr64,
            "fp64_seconds": el64, "match_on_fp64_subset": {"matched": matched, "fp64_roots": nr64,
                                                           "mixed_only": extra},
            "imag_histogram": {"edges": [float(edges[0]), float(edges[-1])], "counts": hist.tolist()}}
    if not args.no_cpu:
        import concurrent.futures as cf
        from oracle import Oracle
        o = Oracle()
        ns = min(count, os.cpu_count() or 1)
        z0s = z0[np.argsort(-z0.imag, kind="stable")]
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
            outs = list(ex.map(lambda m: o.solve_aberth(3, m.n, m.pos, ABERTH_DOM, z0s)[0], media[:ns]))
        el = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": sum(len(r) for r in outs) / el, "cores": os.cpu_count(), "kind": "port",
                                "sample": f"realisations 1..{ns}, one per thread"}
    return line


def workload_wave(ms, torch, args):
    """Wavefunction d=3 N=4096 seed 1, plane wave along +x at nk real k in
    [0.5,3], psi on 512x512 pixels of the z=0 plane over [-R,R]^2: solves and
    grid per second, mixed (refined) and FP64, with the solve residual."""
    n, nk, npx = 4096, args.nk_wave, 512
    med = ms.Medium(3, n, seed=1)
    rad = (n / (4.0 / 3.0 * np.pi)) ** (1.0 / 3.0)
    dom = [-rad, rad, -rad, rad]
    ks = 0.5 + 2.5 * np.arange(nk) / max(nk - 1, 1) + 0j
    res = {}
    for prec in args.legs.split(","):
        (f, d, _, a), el = _wall(torch, lambda: ms.wave_function_batch([med], ks, npx, npx, dom, prec,
                                                                       want_psi=False))
        res[prec] = (f, a[0], el)
    line = {"workload": f"wavefunction d=3 N=4096 {nk} real k in [0.5,3], {npx}x{npx} grid z=0", "unit": "k/s"}
    for prec, (_, _, el) in res.items():
        line[prec] = nk / el
        line[prec + "_seconds"] = el
    if "mixed" in res:
        line["pair_evals_per_s_mixed"] = nk * npx * npx * n / res["mixed"][2]
    if len(res) < 2:
        return line
    f_m, a_m, el_m = res["mixed"]
    f_d, a_d, el_d = res["fp64"]
    line["fun_max_abs_diff_vs_fp64"] = float(np.max(np.abs(f_m - f_d)))
    line["fun_max_abs"] = float(np.max(np.abs(f_d)))
    line["amp_max_rel_diff_vs_fp64"] = float(np.max(np.abs(a_m - a_d)) / np.max(np.abs(a_d)))
    # residual of the solves against M(k) assembled in FP64 by this library
    # (the drop-in build_ms_matrix, pinned element-wise to the reference)
    worst = {"mixed": 0.0, "fp64": 0.0}
    for j in sorted({0, nk // 2, nk - 1}):
        m = ms.build_ms_matrix(med, ks[j])
        phi = np.exp(1j * ks[j] * med.pos[0::3])
        for prec, a in (("mixed", a_m), ("fp64", a_d)):
            r = np.max(np.abs(phi - m @ a[j]))
            worst[prec] = max(worst[prec], float(r / np.max(np.abs(phi))))
            # normwise backward error |phi - M a| / (|M| |a| + |phi|), infinity norms
            bw = r / (np.max(np.sum(np.abs(m), axis=1)) * np.max(np.abs(a[j])) + np.max(np.abs(phi)))
            worst[prec + "_backward"] = max(worst.get(prec + "_backward", 0.0), float(bw))
    line["residual_max"] = worst
    if not args.no_cpu:
        from oracle import Oracle
        o = Oracle()
        # the reference's per-k cost: the N=4096 solve (with a 2x2 grid), then the grid alone (192x192,
        # from those amplitudes) timed per pixel
        t0 = time.perf_counter()
        amp, _ = o.wavefunction(3, n, med.pos, ks[nk // 2], 2, 2, dom, nthreads=os.cpu_count())
        t_solve = time.perf_counter() - t0
        t0 = time.perf_counter()
        o.psi_grid(3, n, med.pos, ks[nk // 2], 192, 192, dom, amp, nthreads=os.cpu_count())
        t_px = (time.perf_counter() - t0) / (192 * 192)
        per_k = t_solve + t_px * npx * npx
        line["cpu_baseline"] = {"value": 1.0 / per_k, "unit": "k/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"one k: N=4096 zgesv {t_solve:.2f} s + {t_px * 1e6:.2f} us per pixel "
                                          f"(192x192 grid), scaled to {npx}x{npx} pixels"}
    return line


def config_legs(ms, torch, no_cpu):
    """Compact measurements of the other configurations, carried by the
    default line: C1 (the whole 64x64 map, both engines), C3 (the 16x16
    subgrid of the 256x256 map, both engines) and C5 (mixed on all 256 k, FP64
    on every 16th k).  Each reports throughput, its accuracy against FP64 and
    the oracle, and its CPU baseline on a bounded sample."""
    from oracle import Oracle
    o = None if no_cpu else Oracle()
    th = os.cpu_count() or 1
    legs = {}
    # C1: d=3 N=64 seed 1, 64x64 kplane on [0.5,3] x [-0.5,0]
    med = ms.Medium(3, 64, seed=1)
    ks = ms.kplane_args(64, 64, 0.5, 3.0, -0.5, 0.0)
    v64, o64, s64 = _resident(ms, torch, "tracelog", [med], ks, "fp64", 3, 3)
    vmx, omx, smx = _resident(ms, torch, "tracelog", [med], ks, "mixed", 3, 3)
    err = np.abs((omx - o64).real) / np.abs(o64.real)
    c1 = {"workload": "kplane d=3 N=64 64x64 Re[0.5,3] Im[-0.5,0]", "unit": "evals/s", "fp64": v64,
          "mixed": vmx, "mixed_lndet_rel_err_vs_fp64": {"max": float(err.max()), "median": float(np.median(err))},
          "status_nonzero": int(np.count_nonzero(s64) + np.count_nonzero(smx))}
    if o is not None:
        t0 = time.perf_counter()
        ref, _ = o.tracelog_batch(3, 64, med.pos, ks, nthreads=th)
        el = time.perf_counter() - t0
        c1["cpu_baseline"] = {"value": len(ks) / el, "unit": "evals/s", "cores": th, "kind": "port",
                              "sample": "the whole 4096-point map"}
        c1["lndet_rel_err_vs_oracle"] = {
            "fp64": float(np.max(np.abs((o64 - ref).real) / np.abs(ref.real))),
            "mixed": float(np.max(np.abs((omx - ref).real) / np.abs(ref.real)))}
    legs["C1"] = c1
    # C3: d=2 N=2048 seed 1, the 16x16 subgrid (every 16th row and column) of the 256x256 map
    med = ms.Medium(2, 2048, seed=1)
    ks = ms.kplane_args(256, 256, 0.5, 4.0, -0.3, 0.0).reshape(256, 256)[::16, ::16].reshape(-1).copy()
    vmx, omx, smx = _resident(ms, torch, "tracelog", [med], ks, "mixed", 1, 1)
    v64, o64, s64 = _resident(ms, torch, "tracelog", [med], ks, "fp64", 1, 1)
    err = np.abs((omx - o64).real * 2048) / np.abs(o64.real * 2048)
    c3 = {"workload": "kplane d=2 N=2048 256x256 Re[0.5,4] Im[-0.3,0]: its 16x16 subgrid", "unit": "evals/s",
          "fp64": v64, "mixed": vmx, "ratio": vmx / v64,
          "mixed_lndet_rel_err_vs_fp64": {"max": float(err.max()), "median": float(np.median(err)),
                                          "points": int(err.size)},
          "im_branch_max_dist": float(np.max(np.abs(((omx.imag - o64.imag) * 2048 + np.pi) % (2 * np.pi) - np.pi))),
          "status_nonzero": {"mixed": int(np.count_nonzero(smx)), "fp64": int(np.count_nonzero(s64))}}
    if o is not None:
        idx = np.arange(0, len(ks), len(ks) // (2 * th))[:2 * th]
        t0 = time.perf_counter()
        ref, _ = o.tracelog_batch(2, 2048, med.pos, ks[idx], nthreads=th)
        el = time.perf_counter() - t0
        c3["cpu_baseline"] = {"value": len(idx) / el, "unit": "evals/s", "cores": th, "kind": "port",
                              "sample": f"{len(idx)} points spread over the subgrid, {th} OpenMP threads x 1 "
                                        "OpenBLAS thread"}
        c3["lndet_rel_err_vs_oracle"] = {
            "fp64": float(np.max(np.abs((o64[idx] - ref).real) / np.abs(ref.real))),
            "mixed": float(np.max(np.abs((omx[idx] - ref).real) / np.abs(ref.real))), "points": int(len(idx))}
    legs["C3"] = c3
    # C5: d=3 N=4096 seed 1, plane wave along +x, 256 real k in [0.5,3], psi on 512x512 pixels at z=0
    n, nk, npx = 4096, 256, 512
    med = ms.Medium(3, n, seed=1)
    rad = (n / (4.0 / 3.0 * np.pi)) ** (1.0 / 3.0)
    dom = [-rad, rad, -rad, rad]
    ks = 0.5 + 2.5 * np.arange(nk) / (nk - 1) + 0j
    sub = np.arange(0, nk, 16)
    (f_m, _, _, a_m), el_m = _wall(torch, lambda: ms.wave_function_batch([med], ks, npx, npx, dom, "mixed",
                                                                         want_psi=False))
    (f_d, _, _, a_d), el_d = _wall(torch, lambda: ms.wave_function_batch([med], ks[sub], npx, npx, dom, "fp64",
                                                                         want_psi=False))
    c5 = {"workload": "wavefunction d=3 N=4096 256 real k in [0.5,3], 512x512 grid z=0", "unit": "k/s",
          "mixed": nk / el_m, "mixed_seconds": el_m, "fp64": len(sub) / el_d, "fp64_seconds": el_d,
          "fp64_sample": f"every 16th k ({len(sub)} of {nk}): {len(sub)} N=4096 solves on as many CTAs, "
                         "so this rate is the latency of one FP64 solve, not the engine's throughput",
          "fun_max_abs_diff_vs_fp64": float(np.max(np.abs(f_m[sub] - f_d))),
          "fun_max_abs": float(np.max(np.abs(f_d))),
          "amp_max_rel_diff_vs_fp64": float(np.max(np.abs(a_m[0][sub] - a_d[0])) / np.max(np.abs(a_d[0])))}
    worst = {"mixed": 0.0, "fp64": 0.0}
    for j in (0, len(sub) - 1):
        k = ks[sub[j]]
        m = ms.build_ms_matrix(med, k)
        phi = np.exp(1j * k * med.pos[0::3])
        for prec, a in (("mixed", a_m[0][sub[j]]), ("fp64", a_d[0][j])):
            worst[prec] = max(worst[prec], float(np.max(np.abs(phi - m @ a)) / np.max(np.abs(phi))))
    c5["solve_residual_max"] = worst
    if o is not None:
        # the solve (with a 2x2 grid), then the grid alone from its amplitudes, timed per pixel
        t0 = time.perf_counter()
        amp, _ = o.wavefunction(3, n, med.pos, ks[nk // 2], 2, 2, dom, nthreads=th)
        t_solve = time.perf_counter() - t0
        t0 = time.perf_counter()
        o.psi_grid(3, n, med.pos, ks[nk // 2], 96, 96, dom, amp, nthreads=th)
        t_px = (time.perf_counter() - t0) / (96 * 96)
        c5["cpu_baseline"] = {"value": 1.0 / (t_solve + t_px * npx * npx), "unit": "k/s", "cores": th,
                              "kind": "port", "sample": f"one k: N=4096 zgesv {t_solve:.2f} s + "
                                                        f"{t_px * 1e6:.2f} us per pixel (96x96 grid), scaled to "
                                                        f"{npx}x{npx} pixels"}
    legs["C5"] = c5
    return legs


_ZGEEV_TIMER = r"""
import json, os, sys, time
import numpy as np
sys.path.insert(0, os.getcwd())
from oracle import Oracle
o = Oracle()
out = {}
for n, reps in ((128, 4), (256, 4), (512, 2)):
    mats = [o.ms_matrix(3, n, o.fill_medium(3, n, s + 1), 1.3 + 0j) for s in range(reps)]
    t0 = time.perf_counter()
    for m in mats:
        np.linalg.eigvals(m)
    out[n] = (time.perf_counter() - t0) / reps
print(json.dumps(out))
"""


def workload_eigvals(ms, torch, args):
    """Eigenvalues of M(k) (eigvals, zgeev) for the mu-plane histograms: batches
    of `count` d=3 realisations at n = 128, 256, 512 (k = 1.3) through the
    public call (positions in, eigenvalues out), checked against LAPACK zgeev
    (numpy) on the first two matrices of each batch; the CPU baseline is that
    zgeev, one matrix per core (OPENBLAS_NUM_THREADS=1), as the reference's
    OpenMP loop over realisations runs it."""
    from oracle import Oracle
    count = args.count or 304
    res = {}
    for n in (128, 256, 512):
        media = [ms.Medium(3, n, seed=s) for s in range(1, 9)]
        im = (np.arange(count) % len(media)).astype(np.int32)
        ks = np.full(count, 1.3 + 0.0j)
        ms.eigvals_batch(media[:1], ks[:1], np.zeros(1, dtype=np.int32))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mus, st = ms.eigvals_batch(media, ks, im)
        dt = time.perf_counter() - t0
        err = 0.0
        for j in range(2):
            want = list(np.linalg.eigvals(Oracle().ms_matrix(3, n, media[j].pos, 1.3 + 0j)))
            scale = max(abs(w) for w in want)
            for m in mus[j]:
                i = int(np.argmin([abs(m - w) for w in want]))
                err = max(err, abs(m - want[i]) / scale)
                want.pop(i)
        res[n] = {"matrices_per_s": count / dt, "seconds": dt, "nonconverged": int(np.count_nonzero(st)),
                  "max_rel_err_vs_zgeev": err}
    cpu = None
    if not args.no_cpu:
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
        r = subprocess.run([sys.executable, "-c", _ZGEEV_TIMER], capture_output=True, text=True, env=env, check=True)
        per = {int(k): v for k, v in json.loads(r.stdout.strip().splitlines()[-1]).items()}
        th = os.cpu_count() or 1
        cpu = {"value": {str(n): th / per[n] for n in per}, "unit": "matrices/s", "cores": th, "kind": "port",
               "sample": "LAPACK zgeev (numpy's OpenBLAS, 1 thread) on the oracle's M(k): 4 matrices at n=128 and "
                         "256, 2 at n=512, seconds per matrix times the cores (one matrix per core)",
               "seconds_per_matrix_1core": {str(n): per[n] for n in per}}
    return {**({"cpu_baseline": cpu} if cpu else {}),
            "workload": f"eigvals d=3 k=1.3, batches of {count} realisations at n=128,256,512", "unit": "matrices/s",
            "gpu": {str(n): res[n] for n in res}, "gpu_launches_per_batch": 1,
            "data": "synthetic (seeded scatterers drawn by the reference's generator)"}


WORKLOADS = {"map64": workload_map64, "map2d": workload_map2d, "aberth": workload_aberth, "wave": workload_wave,
             "eigvals": workload_eigvals}


def run_workload(args):
    import torch
    import msmodel_gb300 as ms
    torch.cuda.set_device(0)
    ms.init(0)
    l0 = ms.launch_count()
    with Clocks(0) as clk:
        line = WORKLOADS[args.workload](ms, torch, args)
    line["gpu_launches"] = ms.launch_count() - l0
    line["clocks"] = clk.summary()
    line["data"] = "synthetic (seeded scatterers drawn by the reference's generator)"
    print(json.dumps(line))
    return 0


def run_reference(args):
    """The reference's CPU path on the host cores: the oracle port (reference
    assembly restated + LAPACK zgetrf, OpenMP over points with one LAPACK
    thread each, as run_tracelog_omp).  Positions and k come from the oracle;
    nothing of this package is loaded.  Each step is a bounded sample of the
    cut: 2 points per host thread, strided across all 4096 k."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import Oracle
    o = Oracle()
    threads = os.cpu_count() or 1
    ks, pos = oracle_cut(o)
    per_step = threads * 2
    for w in range(args.warmup):
        o.tracelog_batch(D, N, pos, strided_sample(ks, 127 - w, threads), nthreads=threads)
    t0 = time.perf_counter()
    done = 0
    for s in range(args.steps):
        o.tracelog_batch(D, N, pos, strided_sample(ks, s, per_step), nthreads=threads)
        done += per_step
    el = time.perf_counter() - t0
    v = done / el
    sample = (f"{per_step} cut points per step taken every 128th across the 4096-point cut (step s: offsets "
              f"s, s+1, ...), {threads} OpenMP threads x 1 OpenBLAS thread, reference assembly restated + "
              "LAPACK zgetrf")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64)",
            "data": "synthetic (seeded scatterers, reference generator)",
            "config": {"workload": "kcut d=3 N=1024 4096k Im=-0.05", "d": D, "natom": N, "nk": NK,
                       "model": "maximum", "shape": "ball", "sample_per_step": per_step,
                       "sample": "strided across the whole cut (every 128th point)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--nk", type=int, default=NK, help="cut points per step (default: the full 4096)")
    ap.add_argument("--natom", type=int, default=N, help="scatterers (default 1024; smaller only for profiling)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision leg of an fp64 run")
    ap.add_argument("--aberth", type=int, default=256, help="realisations of the resonance-search leg (0: skip)")
    ap.add_argument("--aberth-fp64", type=int, default=32,
                    help="realisations of the resonance-search leg also searched in FP64")
    ap.add_argument("--scaling", default="weak", choices=["weak", "strong"],
                    help="weak: each GPU the whole cut of its own realisation; strong: one realisation's cut "
                         "split over the GPUs")
    ap.add_argument("--no-legs", dest="legs_default", action="store_false",
                    help="skip the compact C1/C3/C5 legs of the default line")
    ap.add_argument("--workload", default="cut", choices=["cut"] + sorted(WORKLOADS),
                    help="cut: the headline line; others: one measurement line of that configuration")
    ap.add_argument("--count", type=int, default=0, help="aberth workload: realisations (default 4096); eigvals: matrices per batch (default 304)")
    ap.add_argument("--fp64-count", type=int, default=64, help="aberth workload: realisations searched in FP64")
    ap.add_argument("--nk-wave", type=int, default=256, help="wave workload: wave numbers")
    ap.add_argument("--legs", default="mixed,fp64", help="wave workload: precisions to run")
    ap.add_argument("--sample", type=float, default=0.0, help="map2d workload: fraction of the map (default all)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "cut":
        return run_workload(args)

    import torch
    import msmodel_gb300 as ms
    ws, rank, lr = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(lr)
    ms.init(lr)
    natom = args.natom
    ks = workload_ks()[:args.nk]
    nk_total = len(ks)
    if args.scaling == "strong":
        # one realisation (seed 1), its cut split over the ranks in contiguous blocks
        from msmodel_gb300.sharding import split_points
        seed = 1
        ks = ks[split_points(nk_total, rank, ws)].copy()
    else:
        seed = rank + 1  # weak: each rank its own realisation, the whole cut
    med = ms.Medium(D, natom, seed=seed)
    job = ms.Job("tracelog", [med], ks, precision=args.precision)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        job.run(stream.cuda_stream)
    barrier()
    l0 = ms.launch_count()
    times = []
    with Clocks(lr) as clk:
        for _ in range(args.steps):
            flush.zero_()  # L2 flush between steps (outside the event bracket)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            job.run(stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
    barrier()
    launches = ms.launch_count() - l0
    phase_cycles = ms.engine_stats() if os.environ.get("MSGPU_STATS") and args.precision == "mixed" else None
    clocks = clk.summary()
    tot = sum(times)
    if ws > 1:
        t = torch.tensor([tot], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        tot = float(t.item())
    units = args.steps * (nk_total if args.scaling == "strong" else len(ks) * ws)
    value = units / tot
    out, st = job.results()
    assert np.all(st == 0), "non-zero status in the benchmark results"

    # dominant kernel: the persistent engine is the only launch of a step
    flops_per_launch = job.flops
    achieved = flops_per_launch / (tot / args.steps) / 1e12
    peaks = read_peaks()
    if args.precision == "fp64":
        peak = ms.probe_fp64_tflops()
        # the FP64 tensor path (warp-level m8n8k4 MMA) measured beside it: the engine
        # runs on whichever is faster, DFMA on GB300
        peak_mma = ms.probe_fp64_mma_tflops()
        roof = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": "measured DFMA probe on this GPU (MEASURED_PEAKS.json has no FP64 entry)",
                "fp64_mma_probe_tflops": peak_mma,
                "algorithmic": "8/3 N^3 real flops per ln det (complex LU), N=1024: 2.863e9",
                "traffic": None}
    else:
        peak = peaks.get("bf16_tflops_sustained", 1728.6)
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained",
                "algorithmic": "8/3 N^3 real flops per ln det", "traffic": None}
    if natom == N:
        roof["traffic"], roof["traffic_source"] = recorded_traffic(args.precision, len(ks))

    e2e = None
    if not args.no_e2e:
        nsteps = min(args.steps, 2)
        t0 = time.perf_counter()
        for _ in range(nsteps):
            pos = ms.fill_medium(D, natom, seed)
            m2 = ms.Medium(D, natom, pos=pos, seed=seed)
            o2, s2 = ms.tracelog_batch([m2], ks, precision=args.precision)
        e_el = time.perf_counter() - t0
        h2d = pos.nbytes + ks.nbytes + 4 * len(ks) * 2 + 40
        d2h = 16 * len(ks) + 4 * len(ks)
        e2e = {"value": nsteps * len(ks) * ws / e_el, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "steps": nsteps,
               "api": "msgpu_tracelog_batch (host buffers; includes medium fill, upload, kernels, download)"}
        assert np.max(np.abs(o2 - out)) == 0.0 or np.max(np.abs(o2 - out) / np.abs(out)) < 1e-12

    mixed = None
    if args.precision == "fp64" and not args.no_mixed:
        mixed = measure_mixed(ms, torch, med, ks, out, args, stream, flush, ws, barrier)
        if os.environ.get("MSGPU_STATS"):
            mixed["phase_cycles"] = ms.engine_stats()

    aberth = None
    if rank == 0 and args.aberth > 0 and args.precision == "fp64":
        aberth = measure_aberth(ms, torch, args.aberth, args.aberth_fp64,
                                0 if args.no_cpu else min(args.aberth, os.cpu_count() or 1))

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline()

    legs = None
    if rank == 0 and args.legs_default and args.precision == "fp64":
        legs = config_legs(ms, torch, args.no_cpu)

    if mixed:
        mixed["ratio_vs_fp64"] = mixed["value"] / value
    outm = mixed.pop("_out") if mixed else None
    if cpu and _ORACLE_SAMPLE and natom == N and len(out) == NK:
        # the engines against the oracle on the cut points its CPU leg evaluated
        ix, ref = _ORACLE_SAMPLE["idx"], _ORACLE_SAMPLE["values"]
        rel = lambda v: np.abs((v[ix] - ref).real) / np.abs(ref.real)
        cmp = {args.precision: out, **({"mixed": outm} if outm is not None else {})}
        cpu["lndet_rel_err_vs_oracle"] = {"points": int(ix.size),
                                          **{f"{k}_max": float(rel(v).max()) for k, v in cmp.items()},
                                          **{f"{k}_median": float(np.median(rel(v))) for k, v in cmp.items()}}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
                "scaling": args.scaling, "vs_baseline": None, "dtype": "c128 (f64)" if args.precision == "fp64" else
                "c128 in / bf16-split tensor LU",
                "data": "synthetic (seeded scatterers drawn by the reference's generator; no dataset)",
                "config": {"workload": f"kcut d=3 N={natom} {len(ks)}k Im=-0.05", "d": D, "natom": natom, "nk": len(ks),
                           "model": "maximum", "shape": "ball", "precision": args.precision,
                           "parallelism": (f"replicas x{ws} (one realisation per GPU)" if args.scaling == "weak"
                                           else f"points split x{ws} (one realisation, {nk_total} k over the GPUs)"),
                           "l2": "flushed between steps (256 MB write); per-CTA working set 5 GB > L2"},
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "gpu_launches": launches,
                **({"mixed": mixed} if mixed else {}),
                **({"aberth": aberth} if aberth else {}),
                **({"configs": legs} if legs else {}),
                **({"phase_cycles": phase_cycles} if phase_cycles else {}),
                "precision": args.precision}
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
