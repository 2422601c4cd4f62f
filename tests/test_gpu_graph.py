"""Resident jobs replayed as captured CUDA graphs and re-pointed with
set_points: every result bit-identical to a plain batched call on the same
points, in both engines, including after the shared workspace has moved
(which forces a recapture)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["tracelog", "dlogf", "amplitude"])
def test_graph_replay_and_set_points(ms, kind, precision):
    media = [ms.Medium(3, n, seed=s) for s, n in ((1, 70), (2, 130), (3, 45))]
    rng = np.random.default_rng(7)
    ks = rng.uniform(0.5, 3.0, 40) - 1j * rng.uniform(0.0, 0.6, 40)
    if kind == "amplitude":
        ks = ks.real + 0j
    im = rng.integers(0, 3, 40).astype(np.int32)
    batch = {"tracelog": ms.tracelog_batch, "dlogf": ms.dk_log_det_batch,
             "amplitude": lambda m, k, i, p: ms.amplitude_batch(m, k, i, p, want_amps=False)[::2]}[kind]
    want, _ = batch(media, ks, im, precision)
    job = ms.Job(kind, media, ks, item_med=im, precision=precision)
    job.use_graph(True)
    for _ in range(2):
        job.run()
        got, st = job.results()
        assert np.array_equal(got, want) and np.all(st == 0)
    # fewer, different points on the same job
    sub = np.arange(3, 40, 3)
    job.set_points(ks[sub][::-1], im[sub][::-1])
    job.run()
    got, _ = job.results()
    assert np.array_equal(got, want[sub][::-1])
    # a larger job grows the shared workspace; the first job recaptures
    big = ms.Job(kind, [ms.Medium(3, 700, seed=9)], ks[:2], precision=precision)
    big.run()
    big.results()
    job.set_points(ks, im)
    job.run()
    got, _ = job.results()
    assert np.array_equal(got, want)
    job.close()
    big.close()


def test_set_points_rejects_over_capacity(ms):
    job = ms.Job("tracelog", [ms.Medium(3, 20, seed=1)], [1.0 + 0j, 2.0 + 0j])
    with pytest.raises(ms.MsgpuError):
        job.set_points([1.0 + 0j] * 3)
    job.close()
