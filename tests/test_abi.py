"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares; the product's host inputs are bit-exact with the oracle."""
import ctypes
import glob
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b([a-z_][a-z0-9_]*)\s*\(", txt, flags=re.M):
            name = m.group(1)
            if name not in ("if", "return", "typedef") and not txt[m.start():m.end()].lstrip().startswith("typedef"):
                names.add(name)
    return names


@pytest.fixture(scope="module")
def libpath():
    from msmodel_gb300 import build
    return build.build()


def test_exports_every_declared_symbol(libpath):
    L = ctypes.CDLL(libpath)
    names = _declared()
    assert "msgpu_tracelog_batch" in names and "tracelog_lu" in names and "run_tracelog_omp" in names
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


@pytest.mark.parametrize("prog", ["dropin_check", "dropin_roots_check"])
def test_dropin_c_program_links(libpath, tmp_path, prog):
    """The C callers of the drop-ins compile warning-free against the headers and link."""
    exe = tmp_path / prog
    src = os.path.join(ROOT, "tests", prog + ".c")
    r = subprocess.run(["gcc", "-O1", "-std=gnu11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src,
                        "-o", str(exe), libpath, "-Wl,-rpath," + os.path.dirname(libpath), "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_host_inputs_bit_exact(oracle):
    import msmodel_gb300 as ms
    for d, n, seed, shape, ratio in [(3, 1024, 1, "ball", 1.0), (2, 2048, 1, "ball", 1.0), (3, 100, 77, "cube", 1.0),
                                     (2, 50, 3, "gaussian", 2.5), (3, 27, 1, "lattice", 1.0), (1, 40, 5, "ball", 1.0)]:
        a = ms.fill_medium(d, n, seed, shape, ratio)
        b = oracle.fill_medium(d, n, seed, shape, ratio)
        assert np.array_equal(a, b), (d, n, shape)
    assert np.array_equal(ms.kplane_args(64, 64, 0.5, 3.0, -0.5, 0.0), oracle.kplane_args(64, 64, 0.5, 3.0, -0.5, 0.0))
    assert np.array_equal(ms.kcut_args(4096, 0.5 - 0.05j, 3.0 - 0.05j), oracle.kcut_args(4096, 0.5 - 0.05j, 3.0 - 0.05j))
    assert np.array_equal(ms.kcut_args(40, 6 - 0.0j, 6 - 0.2j), oracle.kcut_args(40, 6 - 0.0j, 6 - 0.2j))
    dom = (0.5, 3.0, -1.0, 0.0)
    assert np.array_equal(ms.halton_points(dom, 64), oracle.halton_points(dom, 64))


def test_cut_centre_samples_are_the_benchmark_grid():
    """The 4096-point cut k_j = 0.5 + 2.5 j/4095 - 0.05i equals the central
    samples data[3j+4] of a reference kcut with sample=4096."""
    import msmodel_gb300 as ms
    ks = ms.kcut_args(4096, 0.5 - 0.05j, 3.0 - 0.05j)
    centre = ks[4::3][:4096]
    want = 0.5 + 2.5 * np.arange(4096) / 4095 - 0.05j
    assert np.max(np.abs(centre - want)) < 1e-15


def test_realisation_sizes_match_reference(ref_runs):
    import msmodel_gb300 as ms
    c = [c for c in ref_runs["cases"] if c["kind"] == "realisation_sizes"][0]
    assert ms.realisation_sizes(len(c["sizes"]), seed=c["seed"]) == c["sizes"]


def test_tuning_table_host_side():
    """The launch-choice table is host state: set, query, save and load without a GPU."""
    import msmodel_gb300 as ms
    try:
        ms.tune_set("dlogf", "mixed", 300, "fp64", 1)
        assert ms.tune_get("dlogf", "mixed", 400) == ("fp64", 1)   # same bucket (256, 512]
        assert ms.tune_get("dlogf", "mixed", 600) == (None, 0)     # next bucket untouched
        with pytest.raises(ms.MsgpuError):
            ms.tune_set("tracelog", "fp64", 64, "mixed", 0)        # FP64 requests stay FP64
        rows = ms.tune_table()
        assert ("dlogf", "mixed", 512, "fp64", 1) in [tuple(r) for r in rows]
    finally:
        ms.tune_set("dlogf", "mixed", 300, None, 0)
    assert ms.tune_table() == []


def test_imag_mu_histogram_restates_reference_binning():
    """Log-spaced bins, samples outside (or with Im mu <= 0) lost, unit integral
    with each bin divided by its width (imag_mu_histogram_util.c:108-153)."""
    import msmodel_gb300 as ms
    mu = [np.array([1e-3j, 2e-2j, 0.5j, -1j, 3j, 0.9 + 0.2j])]
    dens, centres, lost = ms.imag_mu_histogram(mu, 4, 1e-3, 1.0)
    assert lost == 2
    width = np.log(1e3) / 4
    assert abs(np.sum(dens * centres * width) - 1.0) < 1e-14
    counts = dens * centres * 4 * width
    assert np.allclose(counts, [1, 1, 0, 2])  # bin edges 1e-3, 5.6e-3, 3.2e-2, 0.18, 1


def test_eigvals_entry_rejects_bad_arguments_without_a_gpu(libpath):
    """msgpu_eigvals_batch_mtype checks its arguments before it touches a device:
    an unknown matrix type is MSGPU_E_ARG, a matrix beyond the kernel's limit
    (n > 4097, the reflector lives in shared memory) MSGPU_E_SIZE."""
    import msmodel_gb300 as ms
    from msmodel_gb300 import api
    L = ms.lib()
    mu = np.zeros(2 * 4098)
    st = np.zeros(1, dtype=np.int32)
    ks = np.array([1.0, 0.0])
    small = ms.Medium(3, 10, pos=np.zeros(30), seed=1)
    big = ms.Medium(3, 4098, pos=np.zeros(3 * 4098), seed=1)
    im = np.zeros(1, dtype=np.int32)
    assert L.msgpu_eigvals_batch_mtype(7, 1, api._media_array([small]), 1, im, ks, mu, st, None) == -1
    assert L.msgpu_eigvals_batch_mtype(1, 1, api._media_array([big]), 1, im, ks, mu, st, None) == -4
    assert b"4097" in L.msgpu_last_error()
    assert L.msgpu_eigvals_batch_mtype(0, 0, api._media_array([small]), 1, im, ks, mu, st, None) == -1


def test_wave_cut_and_dcs_entries_reject_bad_arguments_without_a_gpu(libpath):
    """The cut and differential cross section entries check their arguments
    before any device work and say why in msgpu_last_error."""
    import msmodel_gb300 as ms
    from msmodel_gb300 import api
    L = ms.lib()
    a = ms.Medium(3, 10, pos=np.zeros(30), seed=1)
    b = ms.Medium(3, 11, pos=np.zeros(33), seed=1)
    k = np.array([1.0, 0.0])
    psi = np.zeros(2 * 2 * 8)
    assert L.msgpu_wave_cut(1, api._media_array([a]), k, 1, -1.0, 1.0, psi, None, 0) == -1
    assert b"nbin" in L.msgpu_last_error()
    assert L.msgpu_wave_cut(2, api._media_array([a, b]), k, 8, -1.0, 1.0, psi, None, 0) == -1
    assert b"same n" in L.msgpu_last_error()
    out = np.zeros(2 * 8)
    assert L.msgpu_diff_cross_section(1, api._media_array([a]), 1.0, 8, 0.0, 180.0, out, 0) == -1
    assert b"thmin" in L.msgpu_last_error()
    assert L.msgpu_diff_cross_section(70000, api._media_array([a]), 1.0, 8, 1.0, 180.0, out, 0) == -1


def test_host_entries_say_why_they_reject_arguments(libpath):
    """fill_medium, the two root searches and the random function check their
    arguments on the host and set msgpu_last_error before returning MSGPU_E_ARG."""
    import ctypes as C
    import msmodel_gb300 as ms
    from msmodel_gb300 import api
    L = ms.lib()
    pos = np.zeros(30)
    assert L.msgpu_fill_medium(0, 10, 1, 1.0, 1, pos) == -1
    assert b"fill_medium" in L.msgpu_last_error()
    assert L.msgpu_fill_medium(3, 10, 9, 1.0, 1, pos) == -1
    assert b"shape" in L.msgpu_last_error()
    a = ms.Medium(3, 10, pos=pos, seed=1)
    dom = np.array([0.5, 3.0, -1.0, 0.0])
    z0 = np.array([1.0, -0.5, 2.0, -0.5])
    roots = np.zeros(4)
    nr = np.zeros(1, dtype=np.int32)
    ne = C.c_int(0)
    assert L.msgpu_solve_aberth_batch(1, api._media_array([a]), dom, 2, z0, 17, 30, 1e-10, 0, roots, nr,
                                      C.byref(ne)) == -1
    assert b"nexpsup" in L.msgpu_last_error()
    assert L.msgpu_find_roots_muller_batch(5, 1, api._media_array([a]), dom, 2, z0, 30, 1e-10, 0, roots, nr,
                                           C.byref(ne)) == -1
    assert b"method" in L.msgpu_last_error()
    m = api._model()
    data = np.zeros(8)
    assert L.msgpu_random_function(4, 3, 10, 1, 1.0, C.byref(m), 2, 4, 0.5, 2.5, data, np.zeros(8, dtype=np.int32),
                                   0) == -1
    assert b"random_function" in L.msgpu_last_error()


def test_task_dropins_refuse_without_the_reference_helpers(libpath, tmp_path):
    """In a program without the reference's fill_chist, append_list_ihist,
    normalize_ihist, alloc/check_eigenstate_list and store_data_wfcut, the task
    drop-ins that hand their results to those functions print an error and
    return before any device work, as does a wavefunction with a spherical
    source; no GPU is touched, so this runs anywhere."""
    exe = tmp_path / "refusals"
    src = os.path.join(ROOT, "tests", "dropin_refusals_check.c")
    r = subprocess.run(["gcc", "-O1", "-std=gnu11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src,
                        "-o", str(exe), libpath, "-Wl,-rpath," + os.path.dirname(libpath), "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.splitlines()
    for name in ("run_chistogram_omp", "run_imag_mu_histogram_omp", "compute_eigenstates",
                 "run_wave_function_cut_omp"):
        assert any(l.startswith(f"[ERROR] {name}:") and "not linked in" in l for l in lines), (name, lines)
    assert any(l.startswith("[ERROR] run_wave_function_omp:") and "plane" in l for l in lines), lines
    assert "done chist" in lines and "done ihist 0" in lines and "done eigls 0" in lines
    assert "done wfcut 0" in lines and "done wfun 0" in lines
