"""traceinv, inverse iteration (compute_eigenstates) and the Muller root
methods mineigval / invtraceinv against the reference's own runs (fixtures):
traceinv within 1e-11, eigenvalues within 1e-9 |M|, eigenvectors within 1e-8
(the phase is locked by the normalisation), invtraceinv root lists identical
within 1e-8 |k|, mineigval roots reference roots."""
import numpy as np
import pytest

from helpers import cplx, match_root_sets, rel

pytestmark = pytest.mark.gpu


def _cases(ref_runs, kind):
    return [c for c in ref_runs["cases"] if c["kind"] == kind]


def test_traceinv(ms, ref_runs):
    c = _cases(ref_runs, "traceinv")[0]
    med = ms.Medium(c["d"], c["n"], seed=c["seed"])
    out, st = ms.traceinv_batch([med], cplx(c["ks"]))
    assert np.all(st == 0)
    assert np.max(rel(out, cplx(c["out"]))) < 1e-11


def test_inverse_iteration(ms, ref_runs):
    cases = _cases(ref_runs, "inverse_iteration")
    assert len(cases) == 3
    med = ms.Medium(3, 100, seed=1)
    ks = [complex(*c["k"]) for c in cases]
    lam, vecs, st = ms.inverse_iteration_batch([med], ks)
    for i, c in enumerate(cases):
        want = complex(*c["lam"])
        conv = not (st[i] & 16)
        assert conv == bool(c["conv"])
        if c["conv"]:
            assert abs(lam[i] - want) < 1e-9
            assert np.max(np.abs(vecs[i] - cplx(c["vec"]))) < 1e-8
        else:  # 50 steps without convergence: the same iterate up to rounding
            assert abs(lam[i] - want) < 1e-6 * abs(want)


def test_invtraceinv_roots(ms, ref_runs):
    c = [c for c in _cases(ref_runs, "roots_muller") if c["method"] == "invtraceinv"][0]
    med = ms.Medium(c["d"], c["n"], seed=c["seed"])
    roots, ne = ms.find_roots_muller("invtraceinv", [med], c["dom"], cplx(c["z0"]), c["maxit"], c["toler"])
    want = cplx(c["roots"])
    assert len(roots[0]) == len(want) and ne > 0
    assert np.max(np.abs(roots[0] - want) / np.abs(want)) < 1e-8  # same list, same order


def test_mineigval_roots(ms, ref_runs):
    """Each realisation runs its roots in the reference's order with one
    eigenvector chained through every inverse iteration (each starts from the
    vector the previous call returned, ms_core.c:339-340): the reference's
    root list within 1e-8 |k|, in the same order."""
    c = [c for c in _cases(ref_runs, "roots_muller") if c["method"] == "mineigval"][0]
    med = ms.Medium(c["d"], c["n"], seed=c["seed"])
    roots, _ = ms.find_roots_muller("mineigval", [med], c["dom"], cplx(c["z0"]), c["maxit"], c["toler"])
    want = cplx(c["roots"])
    assert len(roots[0]) == len(want), (roots[0], want)
    assert np.max(np.abs(roots[0] - want) / np.abs(want)) < 1e-8


def test_mineigval_batched_over_media(ms, ref_runs):
    """Several realisations in one call: each one's chain of eigenvectors is
    its own, so every realisation gets the roots it gets alone."""
    c = [c for c in _cases(ref_runs, "roots_muller") if c["method"] == "mineigval"][0]
    media = [ms.Medium(c["d"], c["n"], seed=c["seed"]), ms.Medium(c["d"], c["n"] + 7, seed=c["seed"] + 1)]
    z0 = cplx(c["z0"])
    both, _ = ms.find_roots_muller("mineigval", media, c["dom"], z0, c["maxit"], c["toler"])
    for i, m in enumerate(media):
        one, _ = ms.find_roots_muller("mineigval", [m], c["dom"], z0, c["maxit"], c["toler"])
        assert len(one[0]) == len(both[i])
        assert np.max(np.abs(one[0] - both[i]), initial=0.0) < 1e-12


def test_eigenstates_at_roots(ms, oracle):
    """compute_eigenstates after the determinant search: at every root the
    eigenvalue of smallest modulus vanishes and M v = mu v holds."""
    med = ms.Medium(3, 80, seed=4)
    dom = [0.5, 3.0, -1.0, 0.0]
    roots, _, states = ms.find_eigenstates([med], dom, 16, eigenvectors=True)
    assert len(states[0]) == len(roots[0]) > 0
    for k, mu, v in states[0]:
        m = oracle.ms_matrix(3, 80, med.pos, k)
        assert abs(np.linalg.norm(v) - 1.0) < 1e-12
        assert np.linalg.norm(m @ v - mu * v) < 1e-9 * np.linalg.norm(m)
        assert abs(mu) < 1e-6 * np.linalg.norm(m)


def test_batched_roots_over_media(ms):
    """Many media in one call give each medium's own result."""
    media = [ms.Medium(3, n, seed=s) for s, n in ((1, 60), (2, 90))]
    dom = [0.5, 3.0, -1.0, 0.0]
    z0 = ms.halton_points(dom, 6)
    both, _ = ms.find_roots_muller("invtraceinv", media, dom, z0)
    for i, m in enumerate(media):
        one, _ = ms.find_roots_muller("invtraceinv", [m], dom, z0)
        assert np.array_equal(one[0], both[i])
