"""Repeated runs give bit-identical results (the work queue deals items to
CTAs in a different order each time; each item's arithmetic must not depend
on it), for both engines."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_repeatable(ms, precision):
    med = ms.Medium(3, 300, seed=21)
    ks = 0.5 + 2.5 * np.arange(64) / 63 - 0.05j
    a, sa = ms.tracelog_batch([med], ks, precision=precision)
    b, sb = ms.tracelog_batch([med], ks, precision=precision)
    c, sc = ms.tracelog_batch([med], ks[::-1].copy(), precision=precision)
    assert np.all(sa == 0) and np.all(sb == 0) and np.all(sc == 0)
    assert np.array_equal(a, b)
    assert np.array_equal(a, c[::-1])
