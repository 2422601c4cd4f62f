"""The oracle against the known answers the reference's own tests hold
(src/test/test_ms_matrix.c, src/test/test_green_bessel_data.h, computed by the
reference author in Mathematica) -- no GPU needed."""
import numpy as np
import pytest

from helpers import branch_distance, cplx, rel


def _rows(ref_tests, name):
    return np.asarray(ref_tests[name], dtype=np.float64)


def test_green_goldens(oracle, ref_tests):
    # d in {-2..5, 10, 20}, r = 1; the reference's own test tolerance is 1e-12 (test_green_bessel.c:19)
    rows = _rows(ref_tests, "GREEN_DATA")
    errs = np.array([abs(oracle.free_green(int(r[0]), complex(r[1], r[2]), 1.0) / complex(r[3], r[4]) - 1)
                     for r in rows])
    assert np.median(errs) < 1e-14
    assert np.max(errs) < 1e-11


def test_dk_green_goldens(oracle, ref_tests):
    rows = _rows(ref_tests, "DK_GREEN_DATA")
    errs = np.array([abs(oracle.dk_free_green(int(r[0]), complex(r[1], r[2]), 1.0) / complex(r[3], r[4]) - 1)
                     for r in rows])
    assert np.median(errs) < 1e-14
    assert np.max(errs) < 1e-11


def test_bessel_k_goldens(oracle, ref_tests):
    rows = _rows(ref_tests, "BESSEL_K_DATA")
    errs = np.array([abs(oracle.bessel_k(int(np.floor(2 * r[0])), complex(r[1], r[2])) / complex(r[3], r[4]) - 1)
                     for r in rows])
    low = np.abs(rows[:, 0]) <= 2  # orders used by the d = 1..6 Green functions
    assert np.max(errs[low]) < 1e-11
    assert np.median(errs) < 1e-13


def test_green_imag_and_hyp0f1_goldens(oracle, ref_tests):
    rows = _rows(ref_tests, "GREEN_IMAG_DATA")
    errs = np.array([abs(oracle.free_green_imag(int(r[0]), complex(r[1], r[2]), 1.0) / complex(r[3], r[4]) - 1)
                     for r in rows])
    assert np.median(errs) < 1e-13
    rows = _rows(ref_tests, "HYP0F1_SERIES_DATA")
    errs = np.array([abs(oracle.hyp0f1(r[0], complex(r[1], r[2])) / complex(r[3], r[4]) - 1) for r in rows])
    assert np.median(errs) < 1e-13


@pytest.mark.parametrize("lapack", [0, 1])
def test_tracelog_goldens(oracle, ref_tests, lapack):
    g = ref_tests["tracelog"]
    m = ref_tests["medium"]
    pos = oracle.fill_medium(m["d"], g["n"], m["seed"])
    for k, want in zip(cplx(g["ks"]), cplx(g["expected"])):
        a = oracle.ms_matrix(m["d"], g["n"], pos, k, m["model"], m["params"])
        got = oracle.tracelog_lu(a, lapack=lapack)
        # the reference compares Re only (test_ms_matrix.c:69); Im agrees modulo 2 pi / n
        assert rel(got.real, want.real) < 1e-9
        # Im error measured relative to |ln det| (entries grow like e^{|Im k| r} at Im k = -6)
        assert branch_distance(got.imag, want.imag, g["n"]) < 1e-9 * g["n"] * abs(want)


def test_dk_log_det_goldens(oracle, ref_tests):
    g = ref_tests["dk_log_det"]
    m = ref_tests["medium"]
    pos = oracle.fill_medium(m["d"], g["n"], m["seed"])
    for k, want in zip(cplx(g["ks"]), cplx(g["expected"])):
        got = oracle.dk_log_det(m["d"], g["n"], pos, k, m["model"], m["params"])
        # the reference differentiates F^-1 by a central difference of step 1e-4
        # (ms_matrix_util.c:69-70): 5e-5 at k = 0.1, below 1e-6 elsewhere
        tol = 1e-4 if abs(k) < 0.5 else 1e-6
        assert rel(got, want) < tol


def test_total_cross_section_goldens(oracle, ref_tests):
    g = ref_tests["total_cross_section"]
    m = ref_tests["medium"]
    pos = oracle.fill_medium(m["d"], g["n"], m["seed"])
    for k, want in zip(g["ks"], g["expected"]):
        got = oracle.total_cross_section(m["d"], g["n"], pos, k, m["model"], m["params"])
        assert rel(got, want) < 1e-10


def test_psi_grid_is_the_wavefunction_grid(oracle):
    """The grid part alone (timed by the C5 CPU baseline) gives the combined
    solve-and-grid routine's psi bit for bit, from its amplitudes."""
    pos = oracle.fill_medium(3, 60, 1)
    dom = [-6.0, 6.0, -5.0, 5.0]
    amp, psi = oracle.wavefunction(3, 60, pos, 1.5 - 0.01j, 12, 10, dom)
    assert np.array_equal(oracle.psi_grid(3, 60, pos, 1.5 - 0.01j, 12, 10, dom, amp), psi)
