"""Batched resonance search against the reference's own root lists
(tests/golden/reference_runs.json, solve_aberth on dk_log_det_ms with 32 Halton
starting points, nexpsup 4, maxit 30, toler 1e-10) and the oracle.  Root sets
must match within |dk| <= 1e-8 |k| (set semantics of the reference's
assert_cvector_subset, src/test/assertion.c:136)."""
import numpy as np
import pytest

from helpers import cplx, match_root_sets

pytestmark = pytest.mark.gpu


def test_roots_match_reference(ms, ref_runs):
    cases = [c for c in ref_runs["cases"] if c["kind"] == "aberth"]
    media = [ms.Medium(c["d"], c["n"], seed=c["seed"]) for c in cases]
    z0 = ms.halton_points(cases[0]["dom"], cases[0]["nseed"])
    roots, ne = ms.solve_aberth_batch(media, cases[0]["dom"], z0, cases[0]["nexpsup"], cases[0]["maxit"],
                                      cases[0]["toler"])
    for r, c in zip(roots, cases):
        want = cplx(c["roots"])
        assert len(r) == len(want), (c["n"], len(r), len(want))
        assert not match_root_sets(r, want, 1e-8)
    assert ne > 24 * len(cases)


def test_roots_match_oracle_batch(ms, oracle):
    dom = [0.5, 3.0, -1.0, 0.0]
    sizes = [(3, 90, 5), (3, 120, 6), (2, 110, 7)]
    media = [ms.Medium(d, n, seed=s) for d, n, s in sizes]
    z0 = ms.halton_points(dom, 16)
    roots, _ = ms.solve_aberth_batch(media, dom, z0, 4, 30, 1e-10)
    for r, (d, n, s), m in zip(roots, sizes, media):
        want, _ = oracle.solve_aberth(d, n, m.pos, dom, z0)
        assert len(r) == len(want)
        assert not match_root_sets(r, want, 1e-8)


def test_mixed_precision_roots(ms, ref_runs):
    """Mixed-precision dlogf far from the roots, FP64 dlogf from a relative
    step of 1e-9 on, within the reference's budget of maxit sweeps per root:
    the reference's root lists within 1e-8 |k|, none missing, none extra."""
    for c in [c for c in ref_runs["cases"] if c["kind"] == "aberth"]:
        med = ms.Medium(c["d"], c["n"], seed=c["seed"])
        z0 = ms.halton_points(c["dom"], c["nseed"])
        roots, _ = ms.solve_aberth_batch([med], c["dom"], z0, 4, 30, 1e-10, precision="mixed")
        want = cplx(c["roots"])
        assert len(roots[0]) == len(want), (len(roots[0]), len(want))
        assert not match_root_sets(want, roots[0], 1e-8)


def test_mixed_precision_roots_larger(ms):
    """Realisations of the batched configuration (N from [100, 600]): the mixed
    search returns exactly the FP64 search's root lists."""
    sizes = ms.realisation_sizes(8, seed=0)
    media = [ms.Medium(3, n, seed=r + 1) for r, n in enumerate(sizes)]
    dom = [0.5, 3.0, -1.0, 0.0]
    z0 = ms.halton_points(dom, 32)
    r64, _ = ms.solve_aberth_batch(media, dom, z0, 4, 30, 1e-10, precision="fp64")
    rmx, _ = ms.solve_aberth_batch(media, dom, z0, 4, 30, 1e-10, precision="mixed")
    for i in range(len(media)):
        assert len(rmx[i]) == len(r64[i]), (i, len(rmx[i]), len(r64[i]))
        assert not match_root_sets(r64[i], rmx[i], 1e-8), i


def test_too_few_starting_points(ms):
    """Fewer than two starting points inside the domain: the reference gives up
    and returns the filtered guesses unchanged (root_finder.c:525-528)."""
    med = ms.Medium(3, 50, seed=1)
    roots, ne = ms.solve_aberth_batch([med], [0.5, 3.0, -1.0, 0.0], [1.0 - 0.5j, 5.0 - 0.5j], 4, 30, 1e-10)
    assert ne == 0 and len(roots[0]) == 1 and roots[0][0] == 1.0 - 0.5j
