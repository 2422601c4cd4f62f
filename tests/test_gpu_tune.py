"""Autotuning: the probe times every candidate launch, keeps the fastest, and
jobs created afterwards follow the choice -- with results that still meet the
requested precision (FP64 bit-identical to the untuned engine)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_and_follow(ms):
    med = ms.Medium(3, 64, seed=1)
    ks = ms.kplane_args(16, 16, 0.5, 3.0, -0.5, 0.0)
    base64, _ = ms.tracelog_batch([med], ks, precision="fp64")
    basemx, _ = ms.tracelog_batch([med], ks, precision="mixed")
    try:
        times, choice = ms.autotune("tracelog", "mixed", 3, 64, nitem=2 * ms.sm_count())
        assert set(times) == {"fp64 x1", "fp64 x2", "mixed x1", "mixed x2"} and all(t > 0 for t in times.values())
        best = min(times, key=times.get)
        assert choice == (best.split()[0], int(best[-1]))
        out, st = ms.tracelog_batch([med], ks, precision="mixed")
        assert np.all(st == 0)
        want = base64 if choice[0] == "fp64" else basemx
        assert np.array_equal(out, want)
        times64, choice64 = ms.autotune("tracelog", "fp64", 3, 64, nitem=ms.sm_count())
        assert choice64[0] == "fp64" and set(times64) == {"fp64 x1", "fp64 x2"}
        out64, _ = ms.tracelog_batch([med], ks, precision="fp64")
        assert np.array_equal(out64, base64)  # the grid size never changes an item's arithmetic
    finally:
        ms.tune_set("tracelog", "mixed", 64, None, 0)
        ms.tune_set("tracelog", "fp64", 64, None, 0)
    assert ms.tune_table() == []
