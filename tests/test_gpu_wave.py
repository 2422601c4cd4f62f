"""Wavefunction (run_wave_function_omp) against the reference's run and the
oracle: psi within 1e-10 of max|psi|, amplitudes relative 1e-10."""
import numpy as np
import pytest

from helpers import cplx, rel

pytestmark = pytest.mark.gpu


def test_wavefunction_reference_run(ms, ref_runs):
    c = [c for c in ref_runs["cases"] if c["kind"] == "wavefunction"][0]
    med = ms.Medium(c["d"], c["n"], seed=c["seed"])
    fun, den, psi, amps = ms.wave_function([med], complex(*c["k"]), c["nx"], c["ny"], c["dom"])
    want = cplx(c["psi"])
    assert np.max(np.abs(psi - want)) < 1e-10 * np.max(np.abs(want))
    assert np.max(rel(amps[0], cplx(c["amp"]))) < 1e-10
    assert np.allclose(fun, want.real, rtol=0, atol=1e-10 * np.max(np.abs(want)))
    assert np.allclose(den, np.abs(want) ** 2, rtol=1e-9, atol=1e-12)


def test_wavefunction_d2_seed_average(ms, oracle):
    d, n, k, nx, ny = 2, 60, 2.0 + 0.0j, 12, 10
    dom = [-6.0, 6.0, -5.0, 5.0]
    media = [ms.Medium(d, n, seed=s) for s in (1, 2, 3)]
    fun, den, psi, amps = ms.wave_function(media, k, nx, ny, dom)
    f_acc = np.zeros(nx * ny)
    d_acc = np.zeros(nx * ny)
    for i, m in enumerate(media):
        a, p = oracle.wavefunction(d, n, m.pos, k, nx, ny, dom)
        assert np.max(rel(amps[i], a)) < 1e-10
        if i == 0:
            assert np.max(np.abs(psi - p)) < 1e-10 * np.max(np.abs(p))
        f_acc += p.real
        d_acc += np.abs(p) ** 2
    assert np.max(np.abs(fun - f_acc / 3)) < 1e-10 * np.max(np.abs(f_acc))
    assert np.max(np.abs(den - d_acc / 3)) < 1e-9 * np.max(d_acc)


def test_wave_batch_equals_single_k(ms):
    """All (medium, k) solves in one job give the per-k results bit for bit."""
    media = [ms.Medium(3, 90, seed=s) for s in (1, 2)]
    ks = [1.1 + 0j, 2.2 - 0.1j, 0.7 + 0j]
    dom = [-3.0, 3.0, -2.5, 2.5]
    fb, db, pb, ab = ms.wave_function_batch(media, ks, 9, 7, dom)
    for i, k in enumerate(ks):
        f, d, p, a = ms.wave_function(media, k, 9, 7, dom)
        assert np.array_equal(f, fb[i]) and np.array_equal(d, db[i]) and np.array_equal(p, pb[i])
        for m in range(len(media)):
            assert np.array_equal(a[m], ab[m][i])


def _psi_fp64(pos, amps, k, nx, ny, dom):
    """psi = e^{ikx} + sum_i a_i G(k, r_i), G = -e^{ikr}/(4 pi r), FP64 numpy."""
    xs = dom[0] + (dom[1] - dom[0]) / (nx - 1) * (np.arange(nx * ny) % nx)
    ys = dom[3] - (dom[3] - dom[2]) / (ny - 1) * (np.arange(nx * ny) // nx)
    p = pos.reshape(-1, 3)
    r = np.sqrt((p[None, :, 0] - xs[:, None]) ** 2 + (p[None, :, 1] - ys[:, None]) ** 2 + p[None, :, 2] ** 2)
    g = -np.exp(1j * k * r) / (4 * np.pi * r)
    return np.exp(1j * k * xs) + g @ amps, np.abs(g) @ np.abs(amps)


@pytest.mark.parametrize("k", [1.5 + 0j, 2.9 + 0j, 0.8 - 0.4j, 2.0 + 0.3j])
def test_double_float_grid(ms, k):
    """d = 3 grid in double-float arithmetic (mixed precision): psi against an
    FP64 evaluation with the same amplitudes, within 1e-12 of sum |a_i G_i|."""
    n = 400
    med = ms.Medium(3, n, seed=3)
    rad = (n / (4.0 / 3.0 * np.pi)) ** (1.0 / 3.0)
    dom = [-1.2 * rad, 1.2 * rad, -rad, rad]
    _, _, psi, amps = ms.wave_function(med, k, 23, 19, dom, precision="mixed")
    want, scale = _psi_fp64(med.pos, amps[0], k, 23, 19, dom)
    err = np.max(np.abs(psi - want) / scale)
    assert err < 1e-12, err


def test_wave_singular_solve_is_reported(ms):
    """Two scatterers at the same point make M(k) non-finite (G(k, 0) diverges):
    the batch returns that solve's status bits instead of averaging it in silently."""
    med = ms.Medium(3, 40, seed=1)
    pos = med.pos.copy()
    pos[3:6] = pos[0:3]
    bad = ms.Medium(3, 40, pos=pos, seed=1)
    dom = [-2.0, 2.0, -2.0, 2.0]
    with pytest.warns(RuntimeWarning, match="status"):
        ms.wave_function_batch([bad], [1.5 + 0j], 8, 8, dom, want_psi=False)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        ms.wave_function_batch([med], [1.5 + 0j], 8, 8, dom, want_psi=False)


@pytest.mark.parametrize("d,precision", [(3, "fp64"), (3, "mixed"), (2, "fp64")])
def test_wave_cut_matches_oracle(ms, oracle, d, precision):
    """run_wave_function_cut_omp's samples: psi of every seed at the nbin points
    (xmin + i dx, 0, ...), against the oracle's psi on the y = 0 row of a grid;
    then the per-bin mean and quartiles of those samples."""
    n, k, nbin, xmin, xmax = 60, 1.5 - 0.01j, 33, -8.0, 8.0
    media = [ms.Medium(d, n, seed=s) for s in (1, 2, 3, 4)]
    psi = ms.wave_cut(media, k, nbin, xmin, xmax, precision)
    want = np.array([oracle.wavefunction(d, n, m.pos, k, nbin, 2, [xmin, xmax, -1.0, 0.0])[1][:nbin]
                     for m in media])
    assert psi.shape == (4, nbin)
    assert np.max(np.abs(psi - want)) < 1e-10 * np.max(np.abs(want))
    st = ms.run_wave_function_cut(media, k, nbin, xmin, xmax, precision)
    from msmodel_gb300.api import _mean_quartiles
    for key, v in (("repsi", want.real), ("impsi", want.imag), ("density", np.abs(want) ** 2)):
        ref = np.array([_mean_quartiles(v[:, i]) for i in range(nbin)])
        assert np.max(np.abs(st[key] - ref)) < 1e-9 * np.max(np.abs(ref)), key


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_diff_cross_section_matches_reference(ms, ref_runs, precision):
    """run_differential_cross_section_omp's samples (far-field amplitude of every
    seed at every angle) against the reference's own run, relative to the largest
    sample; then the statistics of the run_differential_cross_section path."""
    for c in [c for c in ref_runs["cases"] if c["kind"] == "diff_cross_section"]:
        media = [ms.Medium(c["d"], c["n"], seed=c["iseed"] + s) for s in range(c["nseed"])]
        want = np.array(c["samples"])
        got = ms.diff_cross_section(media, c["k"], c["nbin"], c["thmin"], c["thmax"], precision)
        assert got.shape == want.shape
        assert np.max(np.abs(got - want)) < 1e-10 * np.max(want), (c["d"], precision)
        st = ms.run_differential_cross_section(media, c["k"], c["nbin"], c["thmin"], c["thmax"], c["nq"], c["nc"],
                                               precision)
        for key in ("data", "mean", "curve"):
            assert np.max(np.abs(st[key] - np.array(c[key]))) < 1e-10 * np.max(want), key
