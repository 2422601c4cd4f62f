"""The symbol-compatible drop-ins called from C exactly as the reference's
callers call them (double _Complex by value, Medium* layout)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from helpers import branch_distance, rel

pytestmark = pytest.mark.gpu


def test_dropin_program(ms, oracle, tmp_path):
    from msmodel_gb300 import build
    lib = build.build()
    exe = tmp_path / "dropin_check"
    r = subprocess.run(["gcc", "-O1", "-std=gnu11", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "dropin_check.c"), "-o", str(exe), lib,
                        "-Wl,-rpath," + os.path.dirname(lib), "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    n = 80
    out = subprocess.run([str(exe), str(n)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    vals = {}
    cut = {}
    rfun = {}
    for line in out.stdout.splitlines():
        f = line.split()
        if f[0] == "cut":
            cut[int(f[1])] = complex(float(f[2]), float(f[3]))
        elif f[0] == "rfun":
            rfun[int(f[1])] = float(f[2])
        elif f[0] == "sigma":
            vals["sigma"] = float(f[1])
        elif f[0] in ("chist0", "chist1"):
            vals.setdefault(f[0], []).append(complex(float(f[2]), float(f[3])))
        elif f[0] == "ihist":
            vals.setdefault("ihist", []).append(complex(float(f[2]), float(f[3])))
        elif f[0] == "ihist_info":
            vals["ihist_info"] = [float(x) for x in f[1:]]
        elif f[0] == "pos0":
            vals["pos0"] = [float(x) for x in f[1:]]
        elif f[0] == "chist_realtime":
            vals[f"chist_realtime{f[1]}"] = float(f[2])
        elif f[0].startswith("["):
            continue
        else:
            vals[f[0]] = complex(float(f[1]), float(f[2]))
    k = 1.3 - 0.07j
    pos = oracle.fill_medium(3, n, 1)
    m = oracle.ms_matrix(3, n, pos, k)
    assert rel(vals["M01"], m[0, 1]) < 1e-15
    t = oracle.tracelog_lu(m)
    assert rel(vals["tracelog"].real, t.real) < 1e-11
    assert branch_distance(vals["tracelog"].imag, t.imag, n) < 1e-9
    assert rel(vals["dlogf"], oracle.dk_log_det(3, n, pos, k)) < 1e-10
    assert rel(vals["sigma"], oracle.total_cross_section(3, n, pos, 1.3)) < 1e-10
    ks = oracle.kcut_args(4, 0.5 - 0.05j, 3.0 - 0.05j)
    acc = np.zeros(ks.size, dtype=complex)
    for s in (1, 2):
        v, _ = oracle.tracelog_batch(3, n, oracle.fill_medium(3, n, s), ks)
        acc = ((s - 1) * acc + v) / s
    got = np.array([cut[l] for l in range(ks.size)])
    assert np.max(rel(got.real, acc.real)) < 1e-11
    # run_random_function_omp: bins sorted over seeds 1..3, k on the reference's log grid
    import math
    for i in range(4):
        kb = 0.5 * math.exp(i * math.log(2.5 / 0.5) / 3)
        want = sorted(oracle.total_cross_section(3, n, oracle.fill_medium(3, n, s), kb) for s in (1, 2, 3))
        got = [rfun[3 * i + g] for g in range(3)]
        assert np.max(rel(np.array(got), np.array(want))) < 1e-10
    # run_chistogram_omp: the eigenvalues of seeds 1 and 2, in seed order, handed to fill_chist;
    # M(k) and the normalized N(k) = i - G(k)/I(k,0)
    kc = 1.1 + 0j
    iz = oracle.free_green_imag(3, kc, 0.0)
    for mt in (0, 1):
        mus = vals[f"chist{mt}"]
        assert len(mus) == 2 * n and vals[f"chist_realtime{mt}"] > 0
        for s in (1, 2):
            mm = oracle.ms_matrix(3, n, oracle.fill_medium(3, n, s), kc)
            if mt == 1:
                mm = (mm - np.diag(np.diag(mm))) / iz + 1j * np.eye(n)
            want = list(np.linalg.eigvals(mm))
            scale = max(abs(w) for w in want)
            for m in mus[(s - 1) * n:s * n]:
                j = int(np.argmin([abs(m - w) for w in want]))
                assert abs(m - want[j]) < 1e-10 * scale
                want.pop(j)
    # run_imag_mu_histogram_omp: seeds 1 and 2 of M(1.1) in seed order, the range from seed 1,
    # avgx = Re I(k, 0), the variances, one normalisation, med left holding seed 1
    mus = vals["ihist"]
    assert len(mus) == 2 * n
    want_all, trg = [], []
    for s in (1, 2):
        mm = oracle.ms_matrix(3, n, oracle.fill_medium(3, n, s), kc)
        want = list(np.linalg.eigvals(mm))
        scale = max(abs(w) for w in want)
        got = mus[(s - 1) * n:s * n]
        for m in got:
            j = int(np.argmin([abs(m - w) for w in want]))
            assert abs(m - want[j]) < 1e-10 * scale
            want.pop(j)
        want_all.append(got)
        iu = np.triu_indices(n, 1)
        trg.append(2.0 * np.sum(np.abs(mm[iu]) ** 2) / n)
    xmin, xmax, avgx, vt, ve, nnorm, rt = vals["ihist_info"]
    y1 = np.array(want_all[0]).imag
    assert xmin == np.min(y1[y1 > 0]) / 2 and xmax == 2 * np.max(y1)
    assert rel(avgx, iz.real) < 1e-13
    y = np.concatenate([np.array(g).imag for g in want_all])
    assert rel(vt, np.mean((y - avgx) ** 2)) < 1e-12
    assert rel(ve, 0.25 * np.mean(trg)) < 1e-12
    assert nnorm == 1 and rt > 0
    assert vals["pos0"] == list(oracle.fill_medium(3, n, 1)[:3])


def test_dropin_eigenstates_and_wave(ms, oracle, ref_runs, tmp_path):
    """find_eigenstates_serial_1/2/3 and compute_eigenstates called from C as
    run_eigenstate_list_serial calls them, against the reference's own runs;
    run_wave_function_omp against the oracle's seed average."""
    from msmodel_gb300 import build
    from helpers import cplx, match_root_sets
    lib = build.build()
    exe = tmp_path / "dropin_roots_check"
    r = subprocess.run(["gcc", "-O1", "-std=gnu11", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "dropin_roots_check.c"), "-o", str(exe), lib,
                        "-Wl,-rpath," + os.path.dirname(lib), "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def zs(z):
        return " ".join(f"{float(v.real)!r} {float(v.imag)!r}" for v in z)

    ab = [c for c in ref_runs["cases"] if c["kind"] == "aberth"][0]
    mu = {c["method"]: c for c in ref_runs["cases"] if c["kind"] == "roots_muller"}
    ii = [c for c in ref_runs["cases"] if c["kind"] == "inverse_iteration"]
    z0 = ms.halton_points(ab["dom"], ab["nseed"])
    lines = [f"roots 0 {ab['d']} {ab['n']} {ab['seed']} {ab['maxit']} {ab['toler']!r} {len(z0)} "
             + " ".join(repr(v) for v in ab["dom"]) + " " + zs(z0)]
    for m, name in ((1, "mineigval"), (2, "invtraceinv")):
        c = mu[name]
        z = cplx(c["z0"])
        lines.append(f"roots {m} {c['d']} {c['n']} {c['seed']} {c['maxit']} {c['toler']!r} {len(z)} "
                     + " ".join(repr(v) for v in c["dom"]) + " " + zs(z))
    lines.append(f"eig 3 100 1 {len(ii)} " + zs([complex(*c["k"]) for c in ii]))
    d, n, k, nx, ny, dom = 2, 60, 2.0 + 0.0j, 12, 10, [-6.0, 6.0, -5.0, 5.0]
    lines.append(f"wave {d} {n} 1 3 {k.real!r} {k.imag!r} {nx} {ny} " + " ".join(repr(v) for v in dom))
    kc, nbin, xmin, xmax = 1.5 - 0.01j, 17, -8.0, 8.0
    lines.append(f"cut 3 60 2 3 {kc.real!r} {kc.imag!r} {nbin} {xmin!r} {xmax!r}")
    dcs = [c for c in ref_runs["cases"] if c["kind"] == "diff_cross_section"]
    for c in dcs:
        lines.append(f"dcs {c['d']} {c['n']} {c['iseed']} {c['nseed']} {c['k']!r} {c['nbin']} {c['thmin']!r} "
                     f"{c['thmax']!r} {c['nq']} {c['nc']}")
    out = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    roots = {0: [], 1: [], 2: []}
    nroot, states, vecs, wave = {}, {}, {}, {}
    checked = None
    for line in out.stdout.splitlines():
        f = line.split()
        if not f:
            continue
        if f[0] == "nroot":
            nroot[int(f[1])] = (int(f[2]), float(f[3]))
        elif f[0] == "root":
            roots[int(f[1])].append(complex(float(f[3]), float(f[4])))
        elif f[0] == "state":
            states[int(f[1])] = (complex(float(f[2]), float(f[3])), complex(float(f[4]), float(f[5])))
        elif f[0] == "vec":
            vecs.setdefault(int(f[1]), []).append(complex(float(f[3]), float(f[4])))
        elif f[0] == "wave":
            wave[int(f[1])] = (float(f[2]), float(f[3]))
        elif f[0] == "wave_pos0":
            wave["pos0"] = [float(f[1]), float(f[2])]
        elif f[0] == "checked":
            checked = int(f[1])
        elif f[0] == "cut":
            wave[("cut", int(f[1]), int(f[2]))] = complex(float(f[3]), float(f[4]))
        elif f[0] == "cut_med_kept":
            wave["cut_med_kept"] = int(f[1])
        elif f[0].startswith("dcs_"):
            wave.setdefault((f[0], int(f[1])), {})[int(f[2])] = float(f[3])
    # determinant method: the reference's root set; Muller methods: the same list in the same order
    want = cplx(ab["roots"])
    assert nroot[0][0] == len(want) and nroot[0][1] > 0
    assert not match_root_sets(np.array(roots[0]), want, 1e-8)
    for m, name in ((1, "mineigval"), (2, "invtraceinv")):
        want = cplx(mu[name]["roots"])
        got = np.array(roots[m])
        assert len(got) == len(want), (name, got, want)
        assert np.max(np.abs(got - want) / np.abs(want)) < 1e-8
    # compute_eigenstates: every root's state through the reference's list functions
    assert checked == len(ii)
    for i, c in enumerate(ii):
        kr, lam = states[i]
        assert kr == complex(*c["k"])
        if c["conv"]:
            assert abs(lam - complex(*c["lam"])) < 1e-9
            assert np.max(np.abs(np.array(vecs[i]) - cplx(c["vec"]))) < 1e-8
        else:
            assert abs(lam - complex(*c["lam"])) < 1e-6 * abs(complex(*c["lam"]))
    # run_wave_function_omp: the average over seeds 1..3, med left holding seed 3
    f_acc = np.zeros(nx * ny)
    d_acc = np.zeros(nx * ny)
    for s in (1, 2, 3):
        _, p = oracle.wavefunction(d, n, oracle.fill_medium(d, n, s), k, nx, ny, dom)
        f_acc += p.real
        d_acc += np.abs(p) ** 2
    fun = np.array([wave[l][0] for l in range(nx * ny)])
    den = np.array([wave[l][1] for l in range(nx * ny)])
    assert np.max(np.abs(fun - f_acc / 3)) < 1e-10 * np.max(np.abs(f_acc))
    assert np.max(np.abs(den - d_acc / 3)) < 1e-9 * np.max(d_acc)
    assert wave["pos0"] == list(oracle.fill_medium(d, n, 3)[:2])
    # run_wave_function_cut_omp: psi of seeds 2..4 on the cut, handed bin-major to store_data_wfcut;
    # the caller's medium untouched
    for s in range(3):
        pos = oracle.fill_medium(3, 60, 2 + s)
        want = oracle.wavefunction(3, 60, pos, kc, nbin, 2, [xmin, xmax, -1.0, 0.0])[1][:nbin]
        got = np.array([wave[("cut", s, i)] for i in range(nbin)])
        assert np.max(np.abs(got - want)) < 1e-10 * np.max(np.abs(want))
    assert wave["cut_med_kept"] == 1
    # run_differential_cross_section_omp: the reference's quantiles, mean and curves
    for c in dcs:
        scale = np.max(np.array(c["samples"]))
        for key, want in (("dcs_data", c["data"]), ("dcs_mean", c["mean"]), ("dcs_curve", c["curve"])):
            w = np.array(want).reshape(-1)
            got = wave[(key, c["d"])]
            g = np.array([got[l] for l in range(w.size)])
            assert np.max(np.abs(g - w)) < 1e-10 * scale, (key, c["d"])
