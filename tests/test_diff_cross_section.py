"""The differential cross section's host side (run_differential_cross_section_omp,
ms_core.c:526-594) against the reference's own run on one thread
(tests/golden/reference_runs.json, kind diff_cross_section): the statistics
formed from the reference's samples (curves, sorted quantiles at q/(nq-1), mean
summed in order) bit-exact, and the [diff_cross_section] section byte-identical
to save_diff_cross_section's.  No GPU needed."""
import numpy as np


def _cases(ref_runs):
    return [c for c in ref_runs["cases"] if c["kind"] == "diff_cross_section"]


def test_statistics_match_reference(ref_runs):
    from msmodel_gb300 import dcs_statistics
    cases = _cases(ref_runs)
    assert {c["d"] for c in cases} == {2, 3}
    for c in cases:
        st = dcs_statistics(np.array(c["samples"]), c["nq"], c["nc"])
        assert np.array_equal(st["data"], np.array(c["data"]))
        assert np.array_equal(st["mean"], np.array(c["mean"]))
        assert np.array_equal(st["curve"], np.array(c["curve"]))


def test_section_matches_reference(ref_runs, tmp_path):
    from msmodel_gb300.datio import save_diff_cross_section
    for c in _cases(ref_runs):
        f = tmp_path / f"dcs{c['d']}.dat"
        save_diff_cross_section(str(f), {"data": c["data"], "mean": c["mean"], "curve": c["curve"]}, c["k"],
                                c["nseed"], c["iseed"], c["thmin"], c["thmax"], c["title"], c["realtime"])
        assert f.read_text() == c["text"]
