"""The function-level drop-in inside the reference's own build.

Where the reference tree is present (MSMODEL_REF, default /root/reference;
where the tree is absent this test skips), compile every translation unit
of its src/core plus src/main/ms_main.c with the reference's own flags
(Makefile:28-31: -fms-extensions -fopenmp), ms_matrix_util.c with the -D
renames of the integration recipe, and link the result against libmsgpu.so and
a LAPACK (the OpenBLAS scipy bundles, through oracle/lapack_shim.c).  Then
check, with immediate binding at load time, that the relinked program binds
every hot-path symbol it calls to libmsgpu.so, and that the reference's own
copies survive only under their cpu_ names.  build_dk_ms_matrix has no caller
outside ms_matrix_util.c, so it is checked as exported by the library only.

The second test takes the other route, with no renames at all: the reference's
src/core built unchanged as a shared library (-fPIC keeps GCC's default
semantic interposition, so calls between its functions go through the PLT) and
ms_main.c linked against libmsgpu.so ahead of it.  The dynamic linker then binds
the core's calls of the hot-path functions and of the task drivers defined and
called inside ms_core.c (run_tracelog_omp, run_random_function_omp,
run_chistogram_omp, run_imag_mu_histogram_omp, run_wave_function_omp,
run_wave_function_cut_omp, run_differential_cross_section_omp,
find_eigenstates_serial_1/2/3, compute_eigenstates)
to libmsgpu.so, and libmsgpu's weak references to the reference's histogram,
eigenstate-list and cut-statistics functions back to the core.
No GPU is needed: the programs print their usage without touching the device."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

import pytest

from conftest import ROOT

REF = os.environ.get("MSMODEL_REF", "/root/reference")
LIB = os.path.join(ROOT, "msmodel_gb300", "libmsgpu.so")
HOT = ["build_ms_matrix", "build_dk_ms_matrix", "build_plane_wave", "tracelog_lu", "dk_log_det_ms",
       "total_cross_section"]
CALLED = ["build_ms_matrix", "build_plane_wave", "tracelog_lu", "dk_log_det_ms", "total_cross_section"]
DRIVERS = ["run_tracelog_omp", "run_random_function_omp", "run_chistogram_omp", "run_imag_mu_histogram_omp",
           "run_wave_function_omp", "run_wave_function_cut_omp", "run_differential_cross_section_omp",
           "find_eigenstates_serial_1", "find_eigenstates_serial_2",
           "find_eigenstates_serial_3", "compute_eigenstates"]
BACK = ["fill_chist", "append_list_ihist", "normalize_ihist", "alloc_eigenstate_list", "check_eigenstate_list",
        "store_data_wfcut"]


def _need():
    if not os.path.isdir(os.path.join(REF, "src", "core")):
        pytest.skip("reference tree absent")
    if not os.path.exists(LIB):
        pytest.skip("libmsgpu.so not built")
    if shutil.which("gcc") is None or shutil.which("nm") is None:
        pytest.skip("gcc/nm absent")


def _run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    assert r.returncode == 0, " ".join(cmd) + "\n" + r.stdout[-2000:] + r.stderr[-2000:]
    return r


def test_reference_relinks_against_library(tmp_path):
    _need()
    sys.path.insert(0, ROOT)
    from oracle.build_oracle import openblas_path
    ob = openblas_path()
    if ob is None:
        pytest.skip("no LAPACK to link the reference against")
    core = os.path.join(REF, "src", "core")
    rename = [f"-D{s}=cpu_{s}" for s in HOT]
    srcs = sorted(os.path.join(core, f) for f in os.listdir(core) if f.endswith(".c"))
    srcs.append(os.path.join(REF, "src", "main", "ms_main.c"))
    flags = ["gcc", "-O1", "-w", "-fms-extensions", "-fopenmp", "-I", core]

    def compile_one(src):
        obj = str(tmp_path / (os.path.basename(src)[:-2] + ".o"))
        extra = rename if os.path.basename(src) == "ms_matrix_util.c" else []
        _run(flags + extra + ["-c", src, "-o", obj])
        return obj

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, srcs))
    shim = str(tmp_path / "lapack_shim.o")
    _run(["gcc", "-O1", "-c", os.path.join(ROOT, "oracle", "lapack_shim.c"), "-o", shim])
    exe = str(tmp_path / "msmain")
    libdir = os.path.dirname(LIB)
    _run(["gcc", "-fopenmp"] + objs + [shim, "-L", libdir, "-lmsgpu", "-Wl,-rpath," + libdir, ob,
                                       "-Wl,-rpath," + os.path.dirname(ob), "-lm", "-o", exe])
    # the reference's own copies are still there, renamed; the hot-path names are left undefined
    defined = _run(["nm", "--defined-only", exe]).stdout
    undefined = _run(["nm", "-D", "--undefined-only", exe]).stdout
    for s in HOT:
        assert f" cpu_{s}\n" in defined, s
    for s in CALLED:
        assert f" {s}\n" in undefined, s
    exported = _run(["nm", "-D", "--defined-only", LIB]).stdout
    for s in HOT:
        assert f" T {s}\n" in exported, s
    # load the program with every symbol bound at start-up and read where each one went
    env = dict(os.environ, LD_BIND_NOW="1", LD_DEBUG="bindings")
    r = subprocess.run([exe], capture_output=True, text=True, env=env, cwd=str(tmp_path), timeout=120)
    assert "MSModel" in r.stdout, r.stdout[-500:] + r.stderr[-500:]
    for s in CALLED:
        lines = [l for l in r.stderr.splitlines() if l.rstrip().endswith(f"symbol `{s}'")]
        assert lines, s
        assert all(os.path.basename(LIB) in l for l in lines), lines


def _bindings(exe, cwd):
    """{(from, to, symbol)} of a start-up with every symbol bound immediately."""
    env = dict(os.environ, LD_BIND_NOW="1", LD_DEBUG="bindings")
    r = subprocess.run([exe], capture_output=True, text=True, env=env, cwd=cwd, timeout=120)
    assert "MSModel" in r.stdout, r.stdout[-500:] + r.stderr[-500:]
    out = set()
    for l in r.stderr.splitlines():
        f = l.split()
        if "binding" in f and "symbol" in f:
            i = f.index("binding")
            out.add((os.path.basename(f[i + 2]), os.path.basename(f[i + 5]), f[-1].strip("`'")))
    return out


def test_reference_core_library_interposed(tmp_path):
    _need()
    sys.path.insert(0, ROOT)
    from oracle.build_oracle import openblas_path
    ob = openblas_path()
    if ob is None:
        pytest.skip("no LAPACK to link the reference against")
    core = os.path.join(REF, "src", "core")
    srcs = sorted(os.path.join(core, f) for f in os.listdir(core) if f.endswith(".c"))
    flags = ["gcc", "-O2", "-w", "-fPIC", "-fms-extensions", "-fopenmp", "-I", core]

    def compile_one(src):
        obj = str(tmp_path / (os.path.basename(src)[:-2] + ".o"))
        _run(flags + ["-c", src, "-o", obj])
        return obj

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, srcs))
    shim = str(tmp_path / "lapack_shim.o")
    _run(["gcc", "-O1", "-fPIC", "-c", os.path.join(ROOT, "oracle", "lapack_shim.c"), "-o", shim])
    core_so = str(tmp_path / "libmscore.so")
    _run(["gcc", "-shared", "-fopenmp"] + objs + [shim, ob, "-Wl,-rpath," + os.path.dirname(ob), "-lm",
                                                  "-o", core_so])
    # the two libraries overlap in exactly the names libmsgpu replaces
    def names(so):
        return {l.split()[-1] for l in _run(["nm", "-D", "--defined-only", so]).stdout.splitlines() if l.strip()}

    assert names(core_so) & names(LIB) == set(HOT + DRIVERS)
    exe = str(tmp_path / "msmain")
    libdir = os.path.dirname(LIB)
    _run(["gcc", "-O1", "-w", "-fms-extensions", "-fopenmp", "-I", core, os.path.join(REF, "src", "main", "ms_main.c"),
          "-L", libdir, "-Wl,--no-as-needed", "-lmsgpu", "-Wl,--as-needed", "-L", str(tmp_path), "-lmscore",
          "-Wl,-rpath," + libdir, "-Wl,-rpath," + str(tmp_path), "-lm", "-o", exe])
    b = _bindings(exe, str(tmp_path))
    lib, core_name = os.path.basename(LIB), "libmscore.so"
    for s in CALLED + ["build_dk_ms_matrix"] + DRIVERS:
        assert (core_name, lib, s) in b, s
        assert (core_name, core_name, s) not in b, s
    for s in BACK:
        assert (lib, core_name, s) in b, s
