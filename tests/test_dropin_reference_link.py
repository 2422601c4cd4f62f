"""The function-level drop-in inside the reference's own build.

Where the reference tree is present (MSMODEL_REF, default /root/reference;
absent on GPU machines, where this test skips), compile every translation unit
of its src/core plus src/main/ms_main.c with the reference's own flags
(Makefile:28-31: -fms-extensions -fopenmp), ms_matrix_util.c with the -D
renames of the integration recipe, and link the result against libmsgpu.so and
a LAPACK (the OpenBLAS scipy bundles, through oracle/lapack_shim.c).  Then
check, with immediate binding at load time, that the relinked program binds
every hot-path symbol it calls to libmsgpu.so, and that the reference's own
copies survive only under their cpu_ names.  build_dk_ms_matrix has no caller
outside ms_matrix_util.c, so it is checked as exported by the library only.
No GPU is needed: the program prints its usage without touching the device."""
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
