"""Device FP64 special functions against the reference's golden tables and
the oracle (which is itself pinned to them)."""
import numpy as np
import pytest

from helpers import cplx, rel

pytestmark = pytest.mark.gpu


def _rows(ref_tests, name):
    return np.asarray(ref_tests[name], dtype=np.float64)


@pytest.mark.parametrize("name,which", [("GREEN_DATA", 0), ("DK_GREEN_DATA", 1), ("GREEN_IMAG_DATA", 2)])
def test_green_tables(ms, ref_tests, name, which):
    # every dimension of the tables (d in -2..5, 10, 20), each bounded on its own
    rows = _rows(ref_tests, name)
    errs, worst = [], {}
    for d in np.unique(rows[:, 0]).astype(int):
        sel = rows[rows[:, 0] == d]
        got = ms.eval_special(which, int(d), sel[:, 1] + 1j * sel[:, 2], 1.0)
        e = rel(got, sel[:, 3] + 1j * sel[:, 4])
        worst[int(d)] = float(np.max(e))
        errs.append(e)
    e = np.concatenate(errs)
    assert np.median(e) < 1e-14
    assert max(worst.values()) < 1e-11, worst


def test_bessel_k_table(ms, ref_tests):
    rows = _rows(ref_tests, "BESSEL_K_DATA")
    low = rows[np.abs(rows[:, 0]) <= 2]
    for tw in np.unique(np.floor(2 * low[:, 0])).astype(int):
        sel = low[np.floor(2 * low[:, 0]).astype(int) == tw]
        got = ms.bessel_k(int(tw), sel[:, 1] + 1j * sel[:, 2])
        assert np.max(rel(got, sel[:, 3] + 1j * sel[:, 4])) < 1e-11, tw


@pytest.mark.parametrize("d", [1, 2, 3, 4, 5])
def test_green_vs_oracle_random(ms, oracle, d):
    rng = np.random.default_rng(d)
    ks = rng.uniform(0.05, 6, 400) + 1j * rng.uniform(-2, 0.3, 400)
    rs = rng.uniform(0.3, 60, 400)
    got = ms.free_green(d, ks, rs)
    want = np.array([oracle.free_green(d, k, r) for k, r in zip(ks, rs)])
    assert np.max(rel(got, want)) < 1e-12
    got = ms.dk_free_green(d, ks, rs)
    want = np.array([oracle.dk_free_green(d, k, r) for k, r in zip(ks, rs)])
    assert np.max(rel(got, want)) < 1e-12


@pytest.mark.parametrize("model,params", [("maximum", ()), ("hardsphere", (0.4,)), ("softsphere", (0.1,)),
                                          ("resonant", (10.0, -0.1))])
@pytest.mark.parametrize("d", [2, 3])
def test_invf_vs_oracle(ms, oracle, model, params, d):
    ks = np.array([0.3 - 0.1j, 1.0, 2.5 - 0.7j, 7.0 - 0.01j])
    got = ms.invf(d, ks, model, params)
    want = np.array([oracle.invf(d, k, model, params) for k in ks])
    assert np.max(rel(got, want)) < 1e-13
