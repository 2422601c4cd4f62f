"""Generate the golden fixtures under tests/golden/ (run in a container that
has the reference tree; the fixtures are committed so that nothing at test
time reads the reference).

1. ``reference_tests.json`` -- the known-answer values held by the reference's
   own tests, read as text:
   * src/test/test_ms_matrix.c: test_tracelog, test_dk_log_det_ms,
     test_total_cross_section (Mathematica values, d=2 N=50/20 hardsphere 0.4,
     seed 1);
   * src/test/test_green_bessel_data.h: GREEN_DATA, DK_GREEN_DATA,
     GREEN_IMAG_DATA, BESSEL_K_DATA, HYP0F1_SERIES_DATA (rows
     [order, Re z, Im z, Re f, Im f], r = 1).
2. ``reference_runs.json`` -- outputs of the reference itself, compiled from
   its sources into oracle/_ref, on the hot-path configurations at sizes that
   finish in seconds (seeded scatterers, ln det / N, dlogf, roots, psi).

Usage:  [MSMODEL_REF=<reference tree>] python tests/golden/make_golden.py [--chistogram-only]
"""
import ast
import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# the reference tree: $MSMODEL_REF, default /root/reference
REF = os.environ.get("MSMODEL_REF", "/root/reference")
sys.path.insert(0, ROOT)


def _c(z):
    z = complex(z)
    return [z.real, z.imag]


def _cl(zs):
    return [_c(z) for z in zs]


def _array_text(src, name):
    m = re.search(r"\b" + re.escape(name) + r"\s*\[\]\s*=\s*\{(.*?)\};", src, re.S)
    return m.group(1)


def _c_complex_list(src, name):
    items = [s.strip() for s in _array_text(src, name).split(",") if s.strip()]
    return [complex(ast.literal_eval(s.replace("*I", "j"))) for s in items]


def _rows5(src, name):
    m = re.search(r"\b" + re.escape(name) + r"\s*\[\]\[5\]\s*=\s*\{(.*?)\};", src, re.S)
    nums = re.findall(r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?", m.group(1))
    vals = [float(x) for x in nums]
    assert len(vals) % 5 == 0, name
    return [vals[i:i + 5] for i in range(0, len(vals), 5)]


def reference_tests():
    t = open(os.path.join(REF, "src/test/test_ms_matrix.c")).read()
    body = lambda fn: t[t.index("void " + fn + "()"):]
    tr = body("test_tracelog")
    dk = body("test_dk_log_det_ms")
    cs = body("test_total_cross_section")
    out = {
        "source": "src/test/test_ms_matrix.c, src/test/test_green_bessel_data.h (values computed by the "
                  "reference author in Wolfram Mathematica)",
        "medium": {"d": 2, "model": "hardsphere", "params": [0.4], "shape": "ball", "ratio": 1.0, "seed": 1},
        "tracelog": {"n": 50, "ks": _cl(_c_complex_list(tr, "ks")),
                     "expected": _cl(_c_complex_list(tr, "logdet_expc")),
                     "cite": "src/test/test_ms_matrix.c:52-57 (only Re is compared, :69)"},
        "dk_log_det": {"n": 50, "ks": _cl(_c_complex_list(dk, "ks")),
                       "expected": _cl(_c_complex_list(dk, "res_expc")),
                       "cite": "src/test/test_ms_matrix.c:99-103"},
        "total_cross_section": {"n": 20, "ks": [z.real for z in _c_complex_list(cs, "ks")],
                                "expected": [z.real for z in _c_complex_list(cs, "cs_expc")],
                                "cite": "src/test/test_ms_matrix.c:187-188"},
    }
    g = open(os.path.join(REF, "src/test/test_green_bessel_data.h")).read()
    for name in ("GREEN_DATA", "DK_GREEN_DATA", "GREEN_IMAG_DATA", "BESSEL_K_DATA", "HYP0F1_SERIES_DATA"):
        out[name] = _rows5(g, name)
    return out


def _pos_digest(pos):
    return hashlib.sha256(np.ascontiguousarray(pos, dtype="<f8").tobytes()).hexdigest()


def reference_runs():
    from oracle import Oracle, Reference
    r = Reference()
    o = Oracle()
    runs = {"lapack": o.lapack_config(), "cases": []}

    def add(kind, **kw):
        kw["kind"] = kind
        runs["cases"].append(kw)

    # seeded media of every configuration (digest + head), drawn by the reference's fill_medium
    for d, n, seed in [(3, 64, 1), (3, 1024, 1), (2, 2048, 1), (3, 4096, 1), (2, 50, 1), (3, 100, 7), (3, 600, 4096)]:
        pos = r.fill_medium(d, n, seed)
        add("medium", d=d, n=n, seed=seed, sha256=_pos_digest(pos), head=pos[:6].tolist())
    # N for the batched realisations: N_r = 100 + floor(501 u), u from init_random(seed 0) in order
    st = np.zeros(4, dtype=np.uint64)
    o.L.orc_rng_init(st, 0)
    add("realisation_sizes", seed=0, sizes=[100 + int(501 * o.L.orc_rng_double(st)) for _ in range(64)])

    # ln det / N: d=3 N=64 kplane subsample, d=3 N=1024 kcut subsample, d=2 N=2048 kplane subsample
    ks = o.kplane_args(64, 64, 0.5, 3.0, -0.5, 0.0)
    sel = list(range(0, 4096, 97))
    add("tracelog", d=3, n=64, seed=1, model="maximum", idx=sel, ks=_cl(ks[sel]),
        out=_cl(r.tracelog(3, 64, 1, ks[sel])))
    kc = 0.5 + 2.5 * np.arange(4096) / 4095 - 0.05j
    sel = [0, 1365, 2730, 4095]
    add("tracelog", d=3, n=1024, seed=1, model="maximum", idx=sel, ks=_cl(kc[sel]),
        out=_cl(r.tracelog(3, 1024, 1, kc[sel])))
    kp = o.kplane_args(256, 256, 0.5, 4.0, -0.3, 0.0)
    sel = [0, 32768 + 128, 65535]
    add("tracelog", d=2, n=2048, seed=1, model="maximum", idx=sel, ks=_cl(kp[sel]),
        out=_cl(r.tracelog(2, 2048, 1, kp[sel])))
    # small cases with other models and shapes
    for model, params in (("hardsphere", (0.4,)), ("softsphere", (0.1,)), ("resonant", (10.0, -0.1))):
        for d in (2, 3):
            kk = [1.0 - 0.3j, 4.0 - 0.05j, 7.5 - 1.0j]
            add("tracelog", d=d, n=40, seed=3, model=model, params=list(params), ks=_cl(kk),
                out=_cl(r.tracelog(d, 40, 3, kk, model, params)))
    # dlogf = tr(M^-1 dM/dk)
    kk = [0.7 - 0.2j, 1.9 - 0.05j, 2.8 - 0.6j]
    add("dlogf", d=3, n=200, seed=5, model="maximum", ks=_cl(kk), out=_cl(r.dlogf(3, 200, 5, kk)))
    kk = [1.0 - 0.1j, 3.3 - 0.02j]
    add("dlogf", d=2, n=300, seed=2, model="maximum", ks=_cl(kk), out=_cl(r.dlogf(2, 300, 2, kk)))
    # Aberth resonance search on dlogf (find_eigenstates_serial_1), 32 Halton seeds
    dom = [0.5, 3.0, -1.0, 0.0]
    for n, seed in ((100, 1), (140, 2)):
        z0 = o.halton_points(dom, 32)
        roots = r.solve_aberth(3, n, seed, dom, z0, nexpsup=4, maxit=30, toler=1e-10)
        add("aberth", d=3, n=n, seed=seed, dom=dom, nseed=32, nexpsup=4, maxit=30, toler=1e-10, roots=_cl(roots))
    # wavefunction: a = M^-1 phi, psi on a small grid of the z=0 plane
    n = 256
    rad = (n / (4.0 / 3.0 * np.pi)) ** (1.0 / 3.0)
    dom = [-rad, rad, -rad, rad]
    amp, psi = r.wavefunction(3, n, 1, 1.5 + 0j, 16, 16, dom)
    add("wavefunction", d=3, n=n, seed=1, k=[1.5, 0.0], nx=16, ny=16, dom=dom, amp=_cl(amp), psi=_cl(psi))
    # total cross section (zgesv path)
    for k in (0.5, 2.0):
        add("total_cross_section", d=3, n=120, seed=9, k=k, out=r.total_cross_section(3, 120, 9, k))
    # traceinv, inverse iteration (compute_eigenstates) and the Muller root methods
    kk = [1.1 - 0.1j, 2.3 - 0.02j, 0.7 - 0.4j]
    add("traceinv", d=3, n=80, seed=2, ks=_cl(kk), out=_cl(r.traceinv(3, 80, 2, kk)))
    ab = [c for c in runs["cases"] if c["kind"] == "aberth" and c["n"] == 100][0]
    for k in [complex(*ab["roots"][0]), complex(*ab["roots"][3]), 1.7 - 0.2j]:
        lam, vec, conv = r.inverse_iteration(3, 100, 1, k)
        add("inverse_iteration", d=3, n=100, seed=1, k=[k.real, k.imag], lam=[lam.real, lam.imag],
            vec=_cl(vec), conv=int(conv))
    dom = [0.5, 3.0, -1.0, 0.0]
    z0 = o.halton_points(dom, 12)
    z0 = z0[np.argsort(-z0.imag, kind="stable")]
    for method in ("invtraceinv", "mineigval"):
        roots = r.roots_muller(method, 3, 100, 1, dom, z0, maxit=30, toler=1e-10)
        add("roots_muller", method=method, d=3, n=100, seed=1, dom=dom, z0=_cl(z0), maxit=30, toler=1e-10,
            roots=_cl(roots))
    # eigenvalues of M(k) (eigvals, zgeev): the input of the mu-plane histograms
    for d, n, seed, k in ((3, 60, 1, 1.2 - 0.05j), (2, 50, 2, 0.8 + 0.0j)):
        add("eigvals", d=d, n=n, seed=seed, k=[k.real, k.imag], mu=_cl(r.eigvals(d, n, seed, k)))
    runs["cases"].extend(chistogram_cases(r))
    runs["cases"].extend(logcut_cases(r))
    runs["cases"].extend(wfcut_cases(r))
    runs["cases"].extend(dcs_cases(r))
    runs["cases"].extend(section_cases(r))
    # random functions (run_random_function_omp): cross section and DOS, seeds 1..nseed, sorted bins
    for kind, d, n in (("crsec", 3, 60), ("dos", 3, 60), ("dos", 2, 80)):
        data = r.random_function(kind, d, n, 5, 4, 0.4, 3.5)
        add("random_function", type=kind, d=d, n=n, nseed=5, nbin=4, xmin=0.4, xmax=3.5, data=data.tolist())
    return runs


def chistogram_cases(r):
    """mu-plane histograms (run_chistogram_omp, ms_core.c:173-232): the
    eigenvalues of M(k) (or of the normalized N(k), build_normalized_matrix) of
    seeds 1..nseed binned by the reference's fill_chist; the [muplane] section
    its save_chistogram writes for each; the eigenvalues of N(k) of one
    realisation; the Im mu histogram task (run_imag_mu_histogram_omp) with its
    [imag_mu] section; and a [wavefunction] section (save_wfun)."""
    out = []
    for mtype, d, n, nseed, k, xbin, ybin, mbin, color in (
            ("msmatrix", 3, 60, 3, 1.3, 16, 12, 10, "magma seq 3"),
            ("msmatrix", 2, 50, 2, 2.0, 12, 9, 8, "viridis div 2.5 rev"),
            ("normalized", 3, 50, 2, 1.1, 10, 8, 6, "magma seq 3")):
        eig = r.eigvals_normalized if mtype == "normalized" else r.eigvals
        mus = [eig(d, n, s, k) for s in range(1, nseed + 1)]
        data, mdata, info = r.chistogram(np.concatenate(mus), xbin, ybin, mbin)
        title = f"{mtype} d={d}"
        text = r.save_chistogram(np.concatenate(mus), mtype == "normalized", complex(k), nseed, xbin, ybin, mbin,
                                 title, color, 2.5)
        out.append({"kind": "chistogram", "mtype": mtype, "d": d, "n": n, "nseed": nseed, "k": [k, 0.0],
                    "xbin": xbin, "ybin": ybin, "mbin": mbin, "mu": [_cl(m) for m in mus],
                    "data": data.ravel().tolist(), "mdata": [float(v) for v in mdata], "info": info,
                    "muplane": {"title": title, "color": color, "realtime": 2.5, "text": text}})
    d, n, seed, k = 3, 60, 1, complex(1.2, -0.05)
    out.append({"kind": "eigvals", "mtype": "normalized", "d": d, "n": n, "seed": seed, "k": [k.real, k.imag],
                "mu": _cl(r.eigvals_normalized(d, n, seed, k))})
    # the Im mu histogram task on one thread, its [imag_mu] section, the reference's
    # eigenvalues per seed and Tr[G^+ G]/N of each M(k) (the oracle's matrix)
    from oracle import Oracle
    o = Oracle()
    d, n, k, nseed, nbin = 3, 40, 1.3, 3, 8
    text, data, info = r.imag_mu(d, n, k, nseed, nbin, "imu", 0.75)
    trg = []
    for s in range(1, nseed + 1):
        m = o.ms_matrix(d, n, o.fill_medium(d, n, s), complex(k))
        trg.append(float(2.0 * np.sum(np.abs(m[np.triu_indices(n, 1)]) ** 2) / n))
    out.append({"kind": "imag_mu", "d": d, "n": n, "k": k, "nseed": nseed, "nbin": nbin, "title": "imu",
                "realtime": 0.75, "text": text, "data": data.tolist(), "info": info,
                "mu": [_cl(r.eigvals(d, n, s, complex(k))) for s in range(1, nseed + 1)], "trg2_of_m": trg})
    # the [wavefunction] section save_wfun writes for seeded values
    rng = np.random.default_rng(5)
    nx, ny, dom, k = 4, 3, [-2.5, 2.5, -1.25, 1.25], complex(1.1, -0.02)
    fun, den = rng.standard_normal(nx * ny) * 10, rng.random(nx * ny)
    out.append({"kind": "wavefunction_file", "nx": nx, "ny": ny, "dom": dom, "k": [k.real, k.imag], "nseed": 3,
                "iseed": 1, "realtime": 4.5, "color1": "magma seq 3", "color2": "viridis div 2 rev",
                "function": fun.tolist(), "density": den.tolist(),
                "text": r.save_wfun(nx, ny, dom, k, 3, 1, 4.5, "magma seq 3", "viridis div 2 rev", fun, den)})
    return out


def logcut_cases(r):
    """The log cut (init_logcut's mesh, log_cut_util.c:93-96) that run_tracelog_omp
    evaluates for a [logkcut] task (ms_core.c:734-740): the reference's mesh, its
    ln det/N there and the [logkcut] section save_logcut writes for them."""
    d, n, seed, ns, rek, imkmin, imkmax = 3, 64, 1, 24, 2.5, -1e-6, -0.4
    k, _ = r.logcut(ns, rek, imkmin, imkmax)
    vals = r.tracelog(d, n, seed, k)
    _, text = r.logcut(ns, rek, imkmin, imkmax, vals, 1, "log cut", 1.5)
    return [{"kind": "logcut", "d": d, "n": n, "seed": seed, "ns": ns, "rek": rek, "imkmin": imkmin,
             "imkmax": imkmax, "k": _cl(k), "values": _cl(vals), "title": "log cut", "realtime": 1.5,
             "text": text}]


def wfcut_cases(r):
    """The wavefunction cut's statistics (store_data_wfcut, wave_function_cut_util.c:92-114,
    called by run_wave_function_cut_omp, ms_core.c:701): mean and quartiles per bin of
    seeded psi samples, including one seed, two seeds and tied samples."""
    rng = np.random.default_rng(11)
    out = []
    for ns, nb in ((1, 3), (2, 4), (9, 5), (40, 6)):
        psi = rng.standard_normal((ns, nb)) + 1j * rng.standard_normal((ns, nb))
        if ns >= 9:
            psi[3, :] = psi[1, :]  # ties
        re, im, den = r.wfcut_stats(psi)
        out.append({"kind": "wfcut_stats", "nseed": ns, "nbin": nb, "psi": [_cl(row) for row in psi],
                    "repsi": re.tolist(), "impsi": im.tolist(), "density": den.tolist()})
    # the [wavefunction_cut] section save_wfcut writes for the last statistics
    k = complex(1.5, -0.01)
    text = r.save_wfcut(nb, -8.0, 8.0, k, ns, 2, 3.25, re, im, den)
    out.append({"kind": "wavefunction_cut_file", "nbin": nb, "xmin": -8.0, "xmax": 8.0, "k": [k.real, k.imag],
                "nseed": ns, "iseed": 2, "realtime": 3.25, "repsi": re.tolist(), "impsi": im.tolist(),
                "density": den.tolist(), "text": text})
    return out


def dcs_cases(r):
    """The differential cross section (run_differential_cross_section_omp,
    ms_core.c:526-594) with the reference's own steps on one thread: the samples
    per seed and angle, the quantiles, mean and curves, and the
    [diff_cross_section] section save_diff_cross_section writes."""
    out = []
    for d, n, k, nseed, iseed, nbin, thmin, thmax, nq, nc in ((3, 50, 1.2, 5, 1, 7, 1.0, 180.0, 5, 2),
                                                             (2, 40, 2.0, 4, 3, 6, 0.5, 170.0, 3, 1)):
        title = f"dcs d={d}"
        smp, data, mean, curve, text = r.diff_cross_section(d, n, k, nseed, iseed, nbin, thmin, thmax, nq, nc,
                                                            title, 1.5)
        out.append({"kind": "diff_cross_section", "d": d, "n": n, "k": k, "nseed": nseed, "iseed": iseed,
                    "nbin": nbin, "thmin": thmin, "thmax": thmax, "nq": nq, "nc": nc, "title": title,
                    "realtime": 1.5, "samples": smp.tolist(), "data": data.tolist(), "mean": mean.tolist(),
                    "curve": curve.tolist(), "text": text})
    return out


def section_cases(r):
    """The [medium], [kcut], [kplane], [random_function] and [eigenstate_list]
    sections the reference's own writers append for seeded values, including
    signed zeros and NaNs, infinities and extreme exponents."""
    rng = np.random.default_rng(21)
    odd = [complex(-0.0, 0.0), complex(np.copysign(np.nan, -1.0), np.nan), complex(np.inf, -np.inf),
           complex(1e-300, -2.5e300), complex(np.nan, np.copysign(np.nan, -1.0))]

    def cvals(m):
        v = list(rng.standard_normal(m) * 10.0 ** rng.integers(-8, 9, m) + 1j * rng.standard_normal(m))
        return v[:max(0, m - len(odd))] + odd[:m]

    def cl(z):
        """IEEE bit patterns (JSON keeps neither a NaN's sign nor -0 reliably): re, im, ..."""
        return np.ascontiguousarray(np.asarray(z, dtype=np.complex128)).view(np.uint64).tolist()

    out = {"kind": "dat_sections"}
    out["medium"] = [{"d": d, "n": n, "model": mo, "params": list(pa), "shape": sh, "ratio": ra,
                      "text": r.save_medium(d, n, mo, pa, sh, ra)}
                     for d, n, mo, pa, sh, ra in ((3, 1024, "maximum", (), "ball", 1.0),
                                                   (2, 50, "resonant", (1.5, 0.25), "cube", 2.5))]
    kc = cvals(15)
    out["kcut"] = {"ns": 3, "zmin": [0.5, -0.05], "zmax": [3.0, -0.05], "nseed": 2, "title": "Trace-log",
                   "realtime": 1.25, "data": cl(kc),
                   "text": r.save_kcut(3, complex(0.5, -0.05), complex(3.0, -0.05), 2, "Trace-log", 1.25, kc)}
    kp = cvals(6)
    out["kplane"] = {"nx": 3, "ny": 2, "xrange": [0.5, 3.0], "yrange": [-0.5, 0.0], "nseed": 3, "title": "Map",
                     "realtime": 12.5, "color": "viridis div 2.5 rev", "data": cl(kp),
                     "text": r.save_kplane(3, 2, 0.5, 3.0, -0.5, 0.0, 3, "Map", 12.5, "viridis div 2.5 rev", kp)}
    rf = rng.standard_normal(6) * 1e3
    rf[1] = np.copysign(np.nan, -1.0)
    rf[4] = -0.0
    out["random_function"] = {"kind": "dos", "nseed": 2, "nbin": 3, "xmin": 0.4, "xmax": 3.5, "title": "DOS",
                              "realtime": 2.0, "data": rf.view(np.uint64).tolist(),
                              "text": r.save_rfun("dos", 2, 3, 0.4, 3.5, "DOS", 2.0, rf)}
    kr, mu = cvals(2), [complex(1e-12, 2e-13), complex(0.0, -3e-11)]
    ev = [cvals(4), cvals(4)]
    out["eigenstate_list"] = {"d": 3, "n": 4, "seed": 7, "method": "mineigval", "ntarget": 32,
                              "dom": [0.5, 3.0, -1.0, 0.0], "maxit": 30, "toler": 1e-10, "verb": 0,
                              "realtime": 0.75, "kroot": cl(kr), "mu": cl(mu), "eigv": [cl(v) for v in ev],
                              "text": r.save_eigls(3, 4, 7, "mineigval", 32, [0.5, 3.0, -1.0, 0.0], 30, 1e-10, 0,
                                                   0.75, kr, mu, ev)}
    return [out]


if __name__ == "__main__":
    if "--chistogram-only" in sys.argv:
        # add or refresh only the mu-plane histogram cases of an existing reference_runs.json
        from oracle import Reference
        path = os.path.join(HERE, "reference_runs.json")
        with open(path) as f:
            runs = json.load(f)
        r = Reference()
        runs["cases"] = [c for c in runs["cases"] if c["kind"] not in ("chistogram", "imag_mu", "wavefunction_file",
                                                                       "logcut", "wfcut_stats",
                                                                       "wavefunction_cut_file", "diff_cross_section",
                                                                       "dat_sections")
                         and c.get("mtype") != "normalized"] + chistogram_cases(r) + logcut_cases(r) + wfcut_cases(r) + dcs_cases(r) + section_cases(r)
        with open(path, "w") as f:
            json.dump(runs, f, indent=0)
        sys.exit(0)
    with open(os.path.join(HERE, "reference_tests.json"), "w") as f:
        json.dump(reference_tests(), f)
    with open(os.path.join(HERE, "reference_runs.json"), "w") as f:
        json.dump(reference_runs(), f, indent=0)
    print("wrote", os.listdir(HERE))
