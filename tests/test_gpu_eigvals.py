"""Eigenvalues of M(k) (eigvals, zgeev) against the reference's own run: the
same n eigenvalues as sets, within 1e-10 of the largest |mu|."""
import numpy as np
import pytest

from helpers import cplx

pytestmark = pytest.mark.gpu


def test_eigvals_reference_runs(ms, ref_runs):
    cases = [c for c in ref_runs["cases"] if c["kind"] == "eigvals" and c.get("mtype", "msmatrix") == "msmatrix"]
    assert len(cases) == 2
    media = [ms.Medium(c["d"], c["n"], seed=c["seed"]) for c in cases]
    ks = [complex(*c["k"]) for c in cases]
    mus, st = ms.eigvals_batch(media, ks, item_med=[0, 1])
    assert np.all(st == 0)
    for c, mu in zip(cases, mus):
        want = list(cplx(c["mu"]))
        scale = max(abs(w) for w in want)
        assert len(mu) == len(want)
        for m in mu:  # greedy nearest matching, one to one
            j = int(np.argmin([abs(m - w) for w in want]))
            assert abs(m - want[j]) < 1e-10 * scale
            want.pop(j)


def _match_sets(mu, want, tol):
    want = list(want)
    scale = max(abs(w) for w in want)
    for m in mu:  # greedy nearest matching, one to one
        j = int(np.argmin([abs(m - w) for w in want]))
        assert abs(m - want[j]) < tol * scale
        want.pop(j)


def test_eigvals_larger_against_oracle_matrix(ms, oracle):
    """n = 200 (d = 3, complex k) and n = 129 (d = 2), a batch of three items on
    two media: the kernel's eigenvalues against LAPACK zgeev (numpy) of the
    oracle's M(k), within 1e-10 of the largest |mu|."""
    cases = [(3, 200, 2.0 - 0.3j), (2, 129, 1.1 + 0.0j), (3, 200, 0.7 - 0.02j)]
    media = [ms.Medium(3, 200, seed=4), ms.Medium(2, 129, seed=5)]
    mus, st = ms.eigvals_batch(media, [c[2] for c in cases], item_med=[0, 1, 0])
    assert np.all(st == 0)
    for (d, n, k), mu, med in zip(cases, mus, [media[0], media[1], media[0]]):
        assert len(mu) == n
        want = np.linalg.eigvals(oracle.ms_matrix(d, n, med.pos, k))
        _match_sets(mu, want, 1e-10)


def test_eigvals_normalized_reference_run(ms, ref_runs):
    """mtype=normalized: the eigenvalues of N(k) = i - G(k)/I(k,0)
    (build_normalized_matrix) against the reference's zgeev of its own N(k)."""
    cases = [c for c in ref_runs["cases"] if c["kind"] == "eigvals" and c.get("mtype") == "normalized"]
    assert len(cases) == 1
    c = cases[0]
    med = ms.Medium(c["d"], c["n"], seed=c["seed"])
    mus, st = ms.eigvals_batch([med], [complex(*c["k"])], item_med=[0], mtype="normalized")
    assert np.all(st == 0)
    _match_sets(mus[0], cplx(c["mu"]), 1e-10)


def test_eigvals_tiny_matrices(ms, oracle):
    """n = 1 (the QR returns the diagonal), 2 (no Householder step) and 3 (one),
    against LAPACK on the oracle's M(k)."""
    media = [ms.Medium(3, n, seed=7) for n in (1, 2, 3)]
    k = 0.9 - 0.1j
    mus, st = ms.eigvals_batch(media, [k] * 3, item_med=[0, 1, 2])
    assert np.all(st == 0)
    for n, mu, med in zip((1, 2, 3), mus, media):
        assert len(mu) == n
        _match_sets(mu, np.linalg.eigvals(oracle.ms_matrix(3, n, med.pos, k)), 1e-12)


def test_run_chistogram_matches_reference(ms, ref_runs):
    """run_chistogram_omp end to end: the eigenvalues of M(k) of seeds 1..nseed
    on the GPU, binned as the reference bins its own (zgeev) eigenvalues.  The
    eigen-solvers round differently (~1e-13), so a value on a bin edge may move:
    at most two counts differ, the moments agree to 1e-10."""
    for c in [c for c in ref_runs["cases"] if c["kind"] == "chistogram"]:
        media = [ms.Medium(c["d"], c["n"], seed=s) for s in range(1, c["nseed"] + 1)]
        h = ms.run_chistogram(media, complex(*c["k"]), c["xbin"], c["ybin"], c["mbin"], mtype=c["mtype"])
        assert np.all(h["status"] == 0)
        assert np.abs(h["data"].ravel() - np.asarray(c["data"])).sum() <= 2
        info = c["info"]
        assert abs(h["avg"] - complex(info["avg_re"], info["avg_im"])) < 1e-10
        assert abs(h["sigma"] - complex(info["sigma_re"], info["sigma_im"])) < 1e-10


def test_run_imag_mu_histogram_matches_reference(ms, ref_runs):
    """run_imag_mu_histogram_omp end to end on the GPU (eigenvalues and
    Tr[G^+ G]/N by the kernel) against the reference's run: the range, mean and
    true variance to 1e-12, the expected variance against Tr[G^+ G]/(4N) of M(k)
    (the reference evaluates it on zgeev's overwritten matrix), and the
    normalised histogram with at most two counts moved between bins."""
    c = [c for c in ref_runs["cases"] if c["kind"] == "imag_mu"][0]
    media = [ms.Medium(c["d"], c["n"], seed=s) for s in range(1, c["nseed"] + 1)]
    h = ms.run_imag_mu_histogram(media, c["k"], c["nbin"])
    assert np.all(h["status"] == 0)
    info = c["info"]
    for key in ("xmin", "xmax", "avgx", "varx_true"):
        assert abs(h[key] - info[key]) <= 1e-12 * abs(info[key]), key
    assert abs(h["varx_expc"] - 0.25 * np.mean(c["trg2_of_m"])) <= 1e-12 * h["varx_expc"]
    total = c["nseed"] * c["n"] - info["lost"]
    counts = lambda d: np.asarray(d) * h["centres"] * total * np.log(h["xmax"] / h["xmin"]) / c["nbin"]
    assert np.abs(np.round(counts(h["data"])) - np.round(counts(c["data"]))).sum() <= 2
