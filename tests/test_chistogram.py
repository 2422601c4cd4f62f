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


def _case(ref_runs, kind):
    cases = [c for c in ref_runs["cases"] if c["kind"] == kind]
    assert len(cases) == 1
    return cases[0]


def test_imag_mu_task_matches_reference(ref_runs):
    """run_imag_mu_histogram_omp's arithmetic (ms_core.c:225-282) on the
    reference's eigenvalues: range from seed 1, log-binned density, exact mean
    and true variance, all the reference's bits.  The expected variance is
    Tr[G^+ G]/(4N) of M(k): the reference takes tracegtwo after zgeev has
    overwritten the matrix, so its figure is compared with M(k)'s here."""
    from msmodel_gb300 import imag_mu_task
    c = _case(ref_runs, "imag_mu")
    info = c["info"]
    h = imag_mu_task([cplx(m) for m in c["mu"]], c["nbin"], info["avgx"], c["trg2_of_m"])
    assert np.array_equal(h["data"], np.asarray(c["data"]))
    for key in ("xmin", "xmax", "avgx", "varx_true"):
        assert h[key] == info[key], key
    assert h["lost"] == info["lost"]
    assert abs(h["varx_expc"] - 0.25 * np.mean(c["trg2_of_m"])) < 1e-15


def test_imag_mu_and_wavefunction_sections_match_reference(ref_runs, tmp_path):
    """The [imag_mu] (save_ihist) and [wavefunction] (save_wfun) sections, byte
    for byte what the reference's writers produced for the same values."""
    from msmodel_gb300.datio import save_imag_mu, save_wavefunction
    c = _case(ref_runs, "imag_mu")
    h = {"data": np.asarray(c["data"]), **{k: c["info"][k] for k in ("xmin", "xmax", "avgx", "varx_true",
                                                                      "varx_expc")}}
    f = tmp_path / "imag_mu.dat"
    save_imag_mu(str(f), h, c["k"], c["nseed"], c["title"], c["realtime"])
    assert f.read_text() == c["text"]
    w = _case(ref_runs, "wavefunction_file")
    col = lambda a: (a.split()[0], a.split()[1], float(a.split()[2]), len(a.split()) > 3)
    f = tmp_path / "wave.dat"
    save_wavefunction(str(f), w["function"], w["density"], w["nx"], w["ny"], w["dom"], complex(*w["k"]), w["nseed"],
                      w["iseed"], "plane", w["realtime"], col(w["color1"]), col(w["color2"]))
    assert f.read_text() == w["text"]
