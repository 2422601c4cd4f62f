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
    assert len(cases) == 3 and {c["mtype"] for c in cases} == {"msmatrix", "normalized"}
    for c in cases:
        mus = [cplx(m) for m in c["mu"]]
        h = chistogram(mus, c["xbin"], c["ybin"], c["mbin"])
        info = c["info"]
        assert np.array_equal(h["data"].ravel(), np.asarray(c["data"]))
        assert np.array_equal(h["mdata"], np.asarray(c["mdata"]))  # bits: the C library's log and exp
        assert h["dom"] == [info["xmin"], info["xmax"], info["ymin"], info["ymax"]]
        assert h["mrange"] == [info["mmin"], info["mmax"]]
        # the moments summed in the reference's order: its bits
        assert h["avg"] == complex(info["avg_re"], info["avg_im"])
        assert h["sigma"] == complex(info["sigma_re"], info["sigma_im"])
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


def test_muplane_section_matches_reference(ref_runs, tmp_path):
    """The [muplane] section (save_chistogram, chistogram_util.c:414-440) of each
    histogram, byte for byte the text the reference's own writer produced for
    the same eigenvalues, metadata and colour rule."""
    from msmodel_gb300 import chistogram
    from msmodel_gb300.datio import save_muplane
    for i, c in enumerate(_cases(ref_runs)):
        h = chistogram([cplx(m) for m in c["mu"]], c["xbin"], c["ybin"], c["mbin"])
        mp = c["muplane"]
        name, ctype, ctr, *rev = mp["color"].split()
        f = tmp_path / f"mu{i}.dat"
        save_muplane(str(f), h, complex(*c["k"]), c["nseed"], c["mtype"], mp["title"],
                     (name, ctype, float(ctr), bool(rev)), mp["realtime"])
        assert f.read_text() == mp["text"]
