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
