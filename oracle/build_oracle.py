"""Build recipe for the CPU oracle (test infrastructure).

* ``oracle/liboracle.so`` -- the C restatement in ``msoracle.c`` (always).
* ``oracle/_ref/libmsref.so`` -- the reference MSModel sources compiled
  unmodified from ``$MSMODEL_REF/src/core`` (the reference tree, given by the
  environment variable MSMODEL_REF or ``--ref``; default ``/root/reference``)
  together with
  ``ref_driver.c`` and ``lapack_shim.c``; only where the reference tree
  exists (it is absent on GPU machines, where the oracle alone is used).

Outputs go only to ``oracle/`` and ``oracle/_ref/`` (both git-ignored).
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("MSMODEL_REF", "/root/reference")
# the reference's hot-path translation units (and what they pull in)
REF_SOURCES = [
    "ms_matrix_util.c", "green_bessel.c", "medium_util.c", "nru_random.c",
    "scattering_model_util.c", "real_vector_util.c", "complex_vector_util.c",
    "common_util.c", "root_finder.c", "domain_util.c", "complex_data_util.c",
    # the mu-plane histogram binning (chistogram_util.c) and what its unit pulls in
    "chistogram_util.c", "color_rule_util.c", "color_data_util.c", "tikz_util.c",
    # the Im mu histogram and the wave function with their .dat writers
    "imag_mu_histogram_util.c", "wave_function_util.c", "incident_wave_util.c",
    # the log cut's mesh and writer, and the incomplete gamma function its unit calls
    "log_cut_util.c", "incomplete_gamma.c", "classical_diffusion_util.c",
    # the wavefunction cut's statistics (store_data_wfcut)
    "wave_function_cut_util.c",
    # the differential cross section's angles and writer
    "diff_cross_section_util.c",
    # the writers of the map, cut, random function and eigenstate list sections
    "complex_map_util.c", "complex_cut_util.c", "random_function_util.c", "eigenstate_list_util.c",
    "eigenstate_util.c", "square_well_resonances.c",
]


def openblas_path():
    """Locate the OpenBLAS shipped inside the installed scipy wheel."""
    import scipy
    base = os.path.dirname(os.path.dirname(scipy.__file__))
    cands = sorted(glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas*.so*")))
    cands += sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__), ".libs", "libscipy_openblas*.so*")))
    return cands[0] if cands else None


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("oracle build failed")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle(force=False):
    out = os.path.join(HERE, "liboracle.so")
    src = [os.path.join(HERE, "msoracle.c"), os.path.join(HERE, "msoracle.h")]
    if force or _stale(out, src):
        _run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-o", out, src[0], "-ldl", "-lm"])
    return out


def build_ref(force=False, ref_root=None):
    core = os.path.join(ref_root or REF_ROOT, "src", "core")
    if not os.path.isdir(core):
        return None
    ob = openblas_path()
    if ob is None:
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libmsref.so")
    srcs = [os.path.join(core, s) for s in REF_SOURCES]
    mine = [os.path.join(HERE, "ref_driver.c"), os.path.join(HERE, "lapack_shim.c")]
    if force or _stale(out, mine):
        _run(["gcc", "-O2", "-fms-extensions", "-fopenmp", "-fPIC", "-shared", "-w", "-I", core, "-o", out]
             + srcs + mine
             + [ob, "-Wl,-rpath," + os.path.dirname(ob), "-lm"])
    return out


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference tree (default: $MSMODEL_REF or /root/reference)")
    a = ap.parse_args()
    print(build_oracle(force=True))
    print(build_ref(force=True, ref_root=a.ref))
