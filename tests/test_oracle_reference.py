"""The oracle against outputs of the reference itself (compiled from its
sources, fixtures in tests/golden/reference_runs.json) -- no GPU needed."""
import hashlib

import numpy as np
import pytest

from helpers import branch_distance, cplx, match_root_sets, rel


def _cases(ref_runs, kind):
    return [c for c in ref_runs["cases"] if c["kind"] == kind]


def test_medium_bit_exact(oracle, ref_runs):
    for c in _cases(ref_runs, "medium"):
        pos = oracle.fill_medium(c["d"], c["n"], c["seed"])
        assert hashlib.sha256(pos.astype("<f8").tobytes()).hexdigest() == c["sha256"], (c["d"], c["n"])


def test_realisation_sizes(oracle, ref_runs):
    c = _cases(ref_runs, "realisation_sizes")[0]
    st = np.zeros(4, dtype=np.uint64)
    oracle.L.orc_rng_init(st, c["seed"])
    sizes = [100 + int(501 * oracle.L.orc_rng_double(st)) for _ in range(len(c["sizes"]))]
    assert sizes == c["sizes"]


def test_tracelog_matches_reference(oracle, ref_runs):
    for c in _cases(ref_runs, "tracelog"):
        if c["n"] > 1100:
            continue  # the d=2 N=2048 points are checked on the GPU path
        pos = oracle.fill_medium(c["d"], c["n"], c["seed"])
        got, info = oracle.tracelog_batch(c["d"], c["n"], pos, cplx(c["ks"]), c["model"], c.get("params", ()))
        want = cplx(c["out"])
        assert np.all(info == 0)
        assert np.max(rel(got.real, want.real)) < 1e-11, c["model"]
        assert np.max(branch_distance(got.imag, want.imag, c["n"])) < 1e-9


def test_dlogf_matches_reference(oracle, ref_runs):
    for c in _cases(ref_runs, "dlogf"):
        pos = oracle.fill_medium(c["d"], c["n"], c["seed"])
        got = oracle.dlogf_batch(c["d"], c["n"], pos, cplx(c["ks"]))
        assert np.max(rel(got, cplx(c["out"]))) < 1e-10


def test_aberth_matches_reference(oracle, ref_runs):
    for c in _cases(ref_runs, "aberth"):
        pos = oracle.fill_medium(c["d"], c["n"], c["seed"])
        z0 = oracle.halton_points(c["dom"], c["nseed"])
        roots, _ = oracle.solve_aberth(c["d"], c["n"], pos, c["dom"], z0, nexpsup=c["nexpsup"], maxit=c["maxit"],
                                       toler=c["toler"])
        want = cplx(c["roots"])
        assert len(roots) == len(want)
        assert not match_root_sets(roots, want, 1e-8)


def test_wavefunction_matches_reference(oracle, ref_runs):
    c = _cases(ref_runs, "wavefunction")[0]
    pos = oracle.fill_medium(c["d"], c["n"], c["seed"])
    amp, psi = oracle.wavefunction(c["d"], c["n"], pos, complex(*c["k"]), c["nx"], c["ny"], c["dom"])
    assert np.max(rel(amp, cplx(c["amp"]))) < 1e-10
    assert np.max(np.abs(psi - cplx(c["psi"]))) < 1e-10 * np.max(np.abs(psi))


def test_total_cross_section_matches_reference(oracle, ref_runs):
    for c in _cases(ref_runs, "total_cross_section"):
        pos = oracle.fill_medium(c["d"], c["n"], c["seed"])
        assert rel(oracle.total_cross_section(c["d"], c["n"], pos, c["k"]), c["out"]) < 1e-11


def test_restated_lu_agrees_with_lapack(oracle):
    rng = np.random.default_rng(3)
    for n in (1, 2, 7, 33, 64):
        a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        l1, p1, i1 = oracle.lu(a, lapack=0)
        l2, p2, i2 = oracle.lu(a, lapack=1)
        assert np.array_equal(p1, p2) and i1 == i2 == 0
        assert np.max(np.abs(l1 - l2)) < 1e-12 * np.max(np.abs(l2))


def test_singular_matrix_info(oracle):
    a = np.ones((4, 4), dtype=complex)
    _, _, info = oracle.lu(a, lapack=0)
    assert info == 2
    _, _, info2 = oracle.lu(a, lapack=1)
    assert info2 == info


