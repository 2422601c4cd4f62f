"""Failure path of the mixed engine's bounded device waits, exercised without
faulting the GPU: the first operand wait of each trailing update is given a
limit of zero polls, so it runs out at once.  The engine must then issue no
MMA, let the bulk copy in flight land, report MSGPU_S_TIMEOUT (value NaN) for
every item of the run, free its tensor memory and return; the next run on the
same context must be correct."""
import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu

S_TIMEOUT = 8


def test_first_operand_wait_timeout(ms, oracle):
    med = ms.Medium(3, 200, seed=5)
    ks = np.array([0.9 - 0.05j, 1.7 - 0.2j, 2.6 - 0.01j])
    ms.debug_first_wait_limit(0)
    try:
        got, st = ms.tracelog_batch([med], ks, precision="mixed")
    finally:
        ms.debug_first_wait_limit(-1)
    assert np.all(st & S_TIMEOUT), st
    assert np.all(np.isnan(got.real))
    # the context is still usable and the normal limit is back
    got, st = ms.tracelog_batch([med], ks, precision="mixed")
    want, _ = oracle.tracelog_batch(3, 200, med.pos, ks)
    assert np.all(st == 0), st
    assert np.max(rel(got.real, want.real)) < 1e-8


def test_timeout_in_a_larger_batch_marks_every_item(ms):
    """More items than resident CTAs: the CTAs that time out take the rest of
    the queue and mark it, so no item keeps a stale result."""
    med = ms.Medium(3, 64, seed=2)
    ks = 0.5 + 2.5 * np.arange(1000) / 999 - 0.05j
    ms.debug_first_wait_limit(0)
    try:
        got, st = ms.tracelog_batch([med], ks, precision="mixed")
    finally:
        ms.debug_first_wait_limit(-1)
    assert np.all(st & S_TIMEOUT)
    got, st = ms.tracelog_batch([med], ks, precision="mixed")
    assert np.all(st == 0)
