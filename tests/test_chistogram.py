"""The mu-plane histogram binning (run_chistogram_omp, ms_core.c:173-232;
fill_chist, chistogram_util.c:253) against the reference's own binning of the
same eigenvalues (tests/golden/reference_runs.json, "chistogram" cases): the
2-D counts bit for bit, the log-binned marginal of Im mu, the moments and the
lost count.  Host-side; no GPU needed."""
import numpy as np

from helpers import cplx


def _cases(ref_runs):
    return [c for c in ref_runs["cases"] if c["kind"] == "chistogram"]


def test_chistogram_matches_reference(ref_runs):
    from msmodel_gb300 import chistogram
    cases = _cases(ref_runs)
    assert len(cases) == 2
    for c in cases:
        mus = [cplx(m) for m in c["mu"]]
        h = chistogram(mus, c["xbin"], c["ybin"], c["mbin"])
        info = c["info"]
        assert np.array_equal(h["data"].ravel(), np.asarray(c["data"]))
        assert np.allclose(h["mdata"], c["mdata"], rtol=1e-12, atol=0)
        assert h["dom"] == [info["xmin"], info["xmax"], info["ymin"], info["ymax"]]
        assert h["mrange"] == [info["mmin"], info["mmax"]]
        assert abs(h["avg"] - complex(info["avg_re"], info["avg_im"])) < 1e-14
        assert abs(h["sigma"] - complex(info["sigma_re"], info["sigma_im"])) < 1e-14
        assert h["lost"] == info["lost"]


def test_chistogram_domain_and_lost():
    """A given domain loses the values outside it, counted once per range missed."""
    from msmodel_gb300 import chistogram
    mu = np.array([0.1 + 0.2j, 0.5 + 0.9j, -3.0 + 0.5j, 0.3 + 0.4j])
    h = chistogram([mu], 4, 4, 3, dom=[0.0, 1.0, 0.0, 1.0], mrange=[0.1, 1.0])
    assert h["data"].sum() == 3 and h["lost"] == 1
    # pixel of 0.5+0.9i: ix = round(3 * 0.5) = 2, iy = round(3 * 0.1) = 0
    assert h["data"][0, 2] == 1
    np.testing.assert_allclose(np.sum(h["mdata"] * 0.1 * np.exp(np.log(10.0) / 2 * np.arange(3)) * np.log(10.0) / 2),
                               1.0, rtol=1e-12)
