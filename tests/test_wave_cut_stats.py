"""The wavefunction cut's statistics (run_wave_function_cut_omp's
store_data_wfcut, wave_function_cut_util.c:92-114) restated in
msmodel_gb300.api: the mean summed in order and the quartiles interpolated at
(n-1) q, against the reference's own output on seeded samples
(tests/golden/reference_runs.json, kind wfcut_stats): bit-exact, one seed, two
seeds and tied samples included.  No GPU needed."""
import numpy as np

from helpers import cplx


def test_mean_quartiles_match_reference(ref_runs):
    from msmodel_gb300.api import _mean_quartiles
    cases = [c for c in ref_runs["cases"] if c["kind"] == "wfcut_stats"]
    assert {c["nseed"] for c in cases} >= {1, 2}
    for c in cases:
        psi = np.array([cplx(row) for row in c["psi"]])
        for key, v in (("repsi", psi.real), ("impsi", psi.imag), ("density", psi.real ** 2 + psi.imag ** 2)):
            got = np.array([_mean_quartiles(v[:, i]) for i in range(c["nbin"])])
            assert np.array_equal(got, np.array(c[key])), (c["nseed"], key)


def test_wavefunction_cut_section_matches_reference(ref_runs, tmp_path):
    """save_wavefunction_cut writes the reference's save_wfcut section byte for byte."""
    from msmodel_gb300.datio import save_wavefunction_cut
    c = [c for c in ref_runs["cases"] if c["kind"] == "wavefunction_cut_file"][0]
    f = tmp_path / "cut.dat"
    save_wavefunction_cut(str(f), {key: c[key] for key in ("repsi", "impsi", "density")}, c["nbin"], c["xmin"],
                          c["xmax"], complex(*c["k"]), c["nseed"], c["iseed"], "plane", c["realtime"])
    assert f.read_text() == c["text"]
