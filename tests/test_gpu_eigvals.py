"""Eigenvalues of M(k) (eigvals, zgeev) against the reference's own run: the
same n eigenvalues as sets, within 1e-10 of the largest |mu|."""
import numpy as np
import pytest

from helpers import cplx

pytestmark = pytest.mark.gpu


def test_eigvals_reference_runs(ms, ref_runs):
    cases = [c for c in ref_runs["cases"] if c["kind"] == "eigvals"]
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
