"""Build libmsgpu.so in-tree for GB300 (sm_103a).

nvcc compiles the CUDA translation units (one -gencode, compute_103a/sm_103a),
g++ the host inputs, gcc the C drop-in layer; the objects link into
``msmodel_gb300/libmsgpu.so`` (CUDA runtime linked statically).  Translation
units compile in parallel; a unit is rebuilt only when a source it includes
changed.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmsgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INC, "-I", CSRC,
                     "--expt-relaxed-constexpr"]


def _nvcc():
    for c in ("/usr/local/cuda/bin/nvcc", "nvcc"):
        if os.path.exists(c) or c == "nvcc":
            return c
    return "nvcc"


def _deps():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(
        os.path.join(INC, "*.h"))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def _compile(job):
    cmd, out = job
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return out


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    deps = _deps()
    jobs, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        out = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(out)
        if force or _stale(out, [src] + deps):
            jobs.append(([_nvcc()] + NVCC_FLAGS + ["-c", src, "-o", out], out))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        out = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(out)
        if force or _stale(out, [src] + deps):
            jobs.append((["g++", "-O2", "-std=c++17", "-fPIC", "-I", INC, "-c", src, "-o", out], out))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.c"))):
        out = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(out)
        if force or _stale(out, [src] + deps):
            jobs.append((["gcc", "-O2", "-std=gnu11", "-fPIC", "-I", INC, "-c", src, "-o", out], out))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for out in ex.map(_compile, jobs):
                if verbose:
                    print("built", out)
    if force or jobs or _stale(LIB, objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lm"]
        _compile((cmd, LIB))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
