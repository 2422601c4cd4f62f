"""ln det M(k)/n on the GPU (FP64 engine) against the oracle, the reference's
runs and the reference's Mathematica goldens.  Tolerances: relative 1e-10 on
Re ln det (FP64 LU vs LAPACK on the same matrix, condition-limited), Im
modulo 2 pi / n (the reference's Im is sum Arg U_ii + pi[odd swaps])."""
import numpy as np
import pytest

from helpers import branch_distance, cplx, rel

pytestmark = pytest.mark.gpu


def test_reference_goldens(ms, ref_tests):
    g, m = ref_tests["tracelog"], ref_tests["medium"]
    med = ms.Medium(m["d"], g["n"], model=m["model"], params=m["params"], seed=m["seed"])
    got, st = ms.tracelog_batch([med], cplx(g["ks"]))
    want = cplx(g["expected"])
    assert np.all(st == 0)
    assert np.max(rel(got.real, want.real)) < 1e-9
    assert np.all(branch_distance(got.imag, want.imag, g["n"]) < 1e-9 * g["n"] * np.abs(want))


def test_reference_runs(ms, ref_runs):
    for c in ref_runs["cases"]:
        if c["kind"] != "tracelog":
            continue
        med = ms.Medium(c["d"], c["n"], model=c["model"], params=c.get("params", ()), seed=c["seed"])
        got, st = ms.tracelog_batch([med], cplx(c["ks"]))
        want = cplx(c["out"])
        assert np.all(st == 0)
        assert np.max(rel(got.real, want.real)) < 1e-10, (c["d"], c["n"], c["model"])
        assert np.max(branch_distance(got.imag, want.imag, c["n"])) < 1e-8 * c["n"]


@pytest.mark.parametrize("d,n", [(3, 2), (3, 3), (3, 31), (3, 32), (3, 33), (2, 65), (3, 100), (3, 257)])
def test_sizes_vs_oracle(ms, oracle, d, n):
    med = ms.Medium(d, n, seed=n)
    ks = np.array([0.6 - 0.01j, 1.7 - 0.3j, 2.9 - 0.05j])
    got, st = ms.tracelog_batch([med], ks)
    want, info = oracle.tracelog_batch(d, n, med.pos, ks)
    assert np.all(st == 0) and np.all(info == 0)
    assert np.max(rel(got.real, want.real)) < 1e-11
    # identical pivots give the identical branch
    assert np.max(branch_distance(got.imag, want.imag, n)) < 1e-9


def test_kplane_64_subset(ms, oracle):
    """d=3 N=64 complex map (64 x 64 over Re 0.5..3, Im -0.5..0), every 5th pixel."""
    med = ms.Medium(3, 64, seed=1)
    ks = ms.kplane_args(64, 64, 0.5, 3.0, -0.5, 0.0)[::5]
    got, st = ms.tracelog_batch([med], ks)
    want, _ = oracle.tracelog_batch(3, 64, med.pos, ks)
    assert np.all(st == 0)
    assert np.max(rel(got.real, want.real)) < 1e-11
    assert np.max(branch_distance(got.imag, want.imag, 64)) < 1e-9


def test_uneven_batch(ms, oracle):
    """Many media of uneven size in one job; results land in item order."""
    rng = np.random.default_rng(5)
    sizes = [100 + int(x) for x in rng.integers(0, 200, 9)]
    media = [ms.Medium(3, n, seed=i + 1) for i, n in enumerate(sizes)]
    item_med = np.repeat(np.arange(len(media)), 3).astype(np.int32)
    ks = np.tile([0.9 - 0.02j, 2.2 - 0.4j, 1.4 - 0.9j], len(media))
    got, st = ms.tracelog_batch(media, ks, item_med)
    assert np.all(st == 0)
    for i, m in enumerate(media):
        want, _ = oracle.tracelog_batch(3, m.n, m.pos, ks[3 * i:3 * i + 3])
        assert np.max(rel(got[3 * i:3 * i + 3].real, want.real)) < 1e-11


def test_models_and_d2(ms, oracle):
    for model, params in (("hardsphere", (0.4,)), ("softsphere", (0.1,)), ("resonant", (10.0, -0.1))):
        for d in (2, 3):
            med = ms.Medium(d, 40, model=model, params=params, seed=3)
            ks = np.array([1.0 - 0.3j, 4.0 - 0.05j, 7.5 - 1.0j])
            got, st = ms.tracelog_batch([med], ks)
            want, _ = oracle.tracelog_batch(d, 40, med.pos, ks, model, params)
            assert np.max(rel(got.real, want.real)) < 1e-11, (model, d)


def test_singular_and_nonfinite(ms):
    """Status words instead of aborts: a zero column is singular, NaN is non-finite."""
    n = 40
    a = np.eye(n, dtype=complex) + 0.1
    a[:, 7] = 0.0
    v, info = ms.tracelog_lu(a)
    assert info == 8 and v.real == -np.inf
    b = np.eye(n, dtype=complex)
    b[3, 5] = np.nan
    v, info = ms.tracelog_lu(b)
    assert not np.isfinite(v)


def test_single_matrix_path(ms, oracle):
    med = ms.Medium(3, 150, seed=9)
    k = 1.1 - 0.2j
    a = ms.build_ms_matrix(med, k)
    want = oracle.ms_matrix(3, 150, med.pos, k)
    assert np.max(np.abs(a - want)) <= 1e-14 * np.max(np.abs(want))
    da = ms.build_dk_ms_matrix(med, k)
    dwant = oracle.ms_matrix(3, 150, med.pos, k, deriv=True)
    assert np.max(np.abs(da - dwant)) <= 1e-13 * np.max(np.abs(dwant))
    v, info = ms.tracelog_lu(a)
    assert info == 0
    assert rel(v.real, oracle.tracelog_lu(want).real) < 1e-11


def test_run_tracelog_seed_average(ms, oracle):
    ks = ms.kcut_args(5, 0.5 - 0.05j, 3.0 - 0.05j)
    got, st = ms.run_tracelog(3, 60, ks, nseed=3)
    acc = np.zeros(ks.size, dtype=complex)
    for s in range(1, 4):
        pos = oracle.fill_medium(3, 60, s)
        v, _ = oracle.tracelog_batch(3, 60, pos, ks)
        acc = ((s - 1) * acc + v) / s
    assert np.max(rel(got.real, acc.real)) < 1e-11


def test_logcut_matches_reference(ms, ref_runs):
    """The [logkcut] task (run_tracelog_omp on init_logcut's mesh, ms_core.c:734-740):
    ln det/N at the log cut's points, approaching the real axis down to
    Im k = -1e-6, against the reference's run, both engines."""
    c = [c for c in ref_runs["cases"] if c["kind"] == "logcut"][0]
    med = ms.Medium(c["d"], c["n"], seed=c["seed"])
    ks = ms.logcut_args(c["ns"], c["rek"], c["imkmin"], c["imkmax"])
    want = cplx(c["values"])
    for precision, tol in (("fp64", 1e-10), ("mixed", 1e-8)):
        got, st = ms.tracelog_batch([med], ks, precision=precision)
        assert np.all(st == 0)
        assert np.max(np.abs(got.real - want.real) / np.abs(want.real)) < tol, precision


def test_sizes_at_panel_and_tile_edges(ms, oracle):
    """ln det and dlogf at n = 1, 2 and either side of the 32-column panel and
    the 128-row tensor-core tile, both engines, against the oracle: partial
    panels, partial tiles and the single-element matrix."""
    ks = np.array([1.3 - 0.1j, 2.6 - 0.02j])
    for n in (1, 2, 5, 31, 32, 33, 127, 128, 129):
        med = ms.Medium(3, n, seed=n)
        want, _ = oracle.tracelog_batch(3, n, med.pos, ks)
        wantd = oracle.dlogf_batch(3, n, med.pos, ks)
        for precision, tol, told in (("fp64", 1e-11, 1e-10), ("mixed", 1e-8, 1e-7)):
            got, st = ms.tracelog_batch([med], ks, precision=precision)
            assert np.all(st == 0), (n, precision)
            assert np.max(rel(got.real, want.real)) < tol, (n, precision)
            gd, sd = ms.dk_log_det_batch([med], ks, precision=precision)
            assert np.all(sd == 0), (n, precision)
            assert np.max(np.abs(gd - wantd) / np.abs(wantd)) < told, (n, precision)
