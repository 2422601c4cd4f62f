"""Random functions (run_random_function_omp): total cross section and density
of states for seeds 1..nseed on the log-spaced real-k bins, every bin sorted,
against the reference's own run (fixture) -- FP64 within 1e-10 relative
(cross section) and 1e-9 of the largest |DOS|; the mixed form within 1e-10
(refined amplitudes) and 1e-6 of the largest |DOS|."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases(ref_runs):
    return [c for c in ref_runs["cases"] if c["kind"] == "random_function"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_random_function_reference_runs(ms, ref_runs, precision):
    cases = _cases(ref_runs)
    assert len(cases) == 3
    for c in cases:
        ks, data, st = ms.random_function(c["type"], c["d"], c["n"], c["nseed"], c["nbin"], c["xmin"], c["xmax"],
                                          precision=precision)
        want = np.asarray(c["data"])
        assert data.shape == want.shape and np.all(st == 0)
        assert np.all(np.diff(data, axis=1) >= 0)  # bins sorted
        if c["type"] == "crsec":
            tol = 1e-10
            assert np.max(np.abs(data - want) / np.abs(want)) < tol
        else:
            tol = 1e-9 if precision == "fp64" else 1e-6
            assert np.max(np.abs(data - want)) < tol * np.max(np.abs(want))


def test_random_function_layout(ms):
    """data[i, g] is the sorted sample of bin i over seeds g+1, k_i from the
    reference's grid formula (C libm through Python's math module)."""
    import math
    nseed, nbin, xmin, xmax = 3, 4, 0.3, 2.7
    ks, data, _ = ms.random_function("crsec", 3, 30, nseed, nbin, xmin, xmax)
    for i in range(nbin):
        k = xmin * math.exp(i * math.log(xmax / xmin) / (nbin - 1))
        col = sorted(ms.total_cross_section(ms.Medium(3, 30, seed=g + 1), k) for g in range(nseed))
        assert np.array_equal(data[i], col)
