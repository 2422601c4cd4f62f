"""The benchmark's reference arm runs on the host cores alone and prints the
contract's JSON line (no GPU needed): the reference algorithm on a bounded
sample of the same cut, with its cpu_baseline and e2e objects.  It loads no
library of this package: only the oracle is mapped into the process."""
import json
import os
import subprocess
import sys

from conftest import ROOT

_DRIVER = r"""
import json, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"]
sys.path.insert(0, ".")
import bench
rc = bench.main()
maps = open("/proc/self/maps").read()
libs = sorted({l.split()[-1] for l in maps.splitlines() if l.endswith(".so") and ROOT in l})
print(json.dumps({"rc": rc, "libs": libs, "package_imported": "msmodel_gb300" in sys.modules}))
"""


def test_reference_arm_line():
    out = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + _DRIVER], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = out.stdout.strip().splitlines()
    line, probe = json.loads(lines[-2]), json.loads(lines[-1])
    assert probe["rc"] == 0
    assert not probe["package_imported"], "the reference arm imported msmodel_gb300"
    assert all(os.path.basename(p) != "libmsgpu.so" for p in probe["libs"]), probe["libs"]
    assert line["impl"] == "reference" and line["unit"] == "evals/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["steps"] == 1
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "evals/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["natom"] == 1024 and line["config"]["nk"] == 4096


def test_strided_sample_spans_the_cut():
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench
    ks = np.arange(4096)
    s0 = bench.strided_sample(ks, 0, 32)
    assert list(s0) == list(range(0, 4096, 128))
    s1 = bench.strided_sample(ks, 5, 40)
    assert list(s1[:32]) == list(range(5, 4096, 128)) and list(s1[32:]) == list(range(6, 4096, 128))[:8]
