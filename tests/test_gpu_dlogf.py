"""tr(M^-1 dM/dk) and the amplitude solve on the GPU against the oracle,
the reference's runs and goldens."""
import numpy as np
import pytest

from helpers import cplx, rel

pytestmark = pytest.mark.gpu


def test_dlogf_goldens(ms, ref_tests):
    g, m = ref_tests["dk_log_det"], ref_tests["medium"]
    med = ms.Medium(m["d"], g["n"], model=m["model"], params=m["params"], seed=m["seed"])
    ks = cplx(g["ks"])
    got, st = ms.dk_log_det_batch([med], ks)
    want = cplx(g["expected"])
    tol = np.where(np.abs(ks) < 0.5, 1e-4, 1e-6)  # finite-difference diagonal (ms_matrix_util.c:69-70)
    assert np.all(rel(got, want) < tol)


def test_dlogf_reference_runs(ms, ref_runs):
    for c in ref_runs["cases"]:
        if c["kind"] != "dlogf":
            continue
        med = ms.Medium(c["d"], c["n"], seed=c["seed"])
        got, st = ms.dk_log_det_batch([med], cplx(c["ks"]))
        assert np.all(st == 0)
        assert np.max(rel(got, cplx(c["out"]))) < 1e-10


@pytest.mark.parametrize("d,n", [(3, 2), (3, 33), (2, 70), (3, 129)])
def test_dlogf_vs_oracle(ms, oracle, d, n):
    med = ms.Medium(d, n, seed=2 * n)
    ks = np.array([0.8 - 0.1j, 2.5 - 0.02j])
    got, st = ms.dk_log_det_batch([med], ks)
    want = oracle.dlogf_batch(d, n, med.pos, ks)
    assert np.max(rel(got, want)) < 1e-10


def test_total_cross_section(ms, ref_tests, ref_runs):
    g, m = ref_tests["total_cross_section"], ref_tests["medium"]
    med = ms.Medium(m["d"], g["n"], model=m["model"], params=m["params"], seed=m["seed"])
    for k, want in zip(g["ks"], g["expected"]):
        assert rel(ms.total_cross_section(med, k), want) < 1e-10
    for c in ref_runs["cases"]:
        if c["kind"] == "total_cross_section":
            med = ms.Medium(c["d"], c["n"], seed=c["seed"])
            assert rel(ms.total_cross_section(med, c["k"]), c["out"]) < 1e-11


def test_amplitudes_vs_reference(ms, ref_runs):
    c = [c for c in ref_runs["cases"] if c["kind"] == "wavefunction"][0]
    med = ms.Medium(c["d"], c["n"], seed=c["seed"])
    sig, amps, st = ms.amplitude_batch([med], [complex(*c["k"])])
    assert np.all(st == 0)
    assert np.max(rel(amps[0], cplx(c["amp"]))) < 1e-10
