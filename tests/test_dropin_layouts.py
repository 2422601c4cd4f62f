"""Every struct msgpu_dropin.h mirrors has the reference's layout: a C unit
that includes the reference's own type headers (MSMODEL_REF, default
/root/reference; where the tree is absent this test skips) next to
msgpu_dropin.h must compile with a static assertion on the size of each pair
and on the offset of every field.  No GPU needed."""
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

REF = os.environ.get("MSMODEL_REF", "/root/reference")
PAIRS = {
    "msgpu_ref_scmodel": "ScatteringModel",
    "msgpu_ref_medium": "Medium",
    "msgpu_ref_cdata": "ComplexData",
    "msgpu_ref_rfun": "RandomFunction",
    "msgpu_ref_chist": "Chistogram",
    "msgpu_ref_ihist": "ImagMuHistogram",
    "msgpu_ref_domain": "Domain",
    "msgpu_ref_iwave": "IncidentWave",
    "msgpu_ref_wfun": "WaveFunction",
    "msgpu_ref_wfcut": "WaveFunctionCut",
    "msgpu_ref_dcs": "DiffCrossSection",
    "msgpu_ref_eigenstate": "Eigenstate",
    "msgpu_ref_eigls": "EigenstateList",
}
HEADERS = ["medium_type.h", "scattering_model_type.h", "complex_data_type.h", "random_function_type.h",
           "chistogram_type.h", "imag_mu_histogram_type.h", "domain_type.h", "incident_wave_type.h",
           "wave_function_type.h", "wave_function_cut_type.h", "diff_cross_section_type.h", "eigenstate_type.h",
           "eigenstate_list_type.h"]


def _fields():
    """{struct name: [field names]} of the msgpu_ref_* mirrors in msgpu_dropin.h."""
    with open(os.path.join(ROOT, "include", "msgpu_dropin.h")) as f:
        text = f.read()
    out = {}
    for m in re.finditer(r"typedef struct (msgpu_ref_\w+) \{(.*?)\} \1;", text, re.S):
        names = []
        for line in m.group(2).split(";"):
            line = re.sub(r"/\*.*?\*/", "", line).strip()
            if not line:
                continue
            fp = re.search(r"\(\*(\w+)\)", line)
            names.append(fp.group(1) if fp else re.search(r"(\w+)\s*(\[\d+\])?$", line).group(1))
        out[m.group(1)] = names
    return out


def test_mirrors_match_reference_layouts(tmp_path):
    if not os.path.isdir(os.path.join(REF, "src", "core")) or shutil.which("gcc") is None:
        pytest.skip("reference tree or gcc absent")
    fields = _fields()
    assert set(fields) == set(PAIRS), set(fields) ^ set(PAIRS)
    lines = ["#include <stddef.h>", "#include <stdint.h>", "#include <complex.h>"]
    lines += [f'#include "{h}"' for h in HEADERS] + ['#include "msgpu_dropin.h"']
    for mine, ref in PAIRS.items():
        lines.append(f'_Static_assert(sizeof({mine}) == sizeof({ref}), "size of {ref}");')
        for f in fields[mine]:
            lines.append(f'_Static_assert(offsetof({mine}, {f}) == offsetof({ref}, {f}), "{ref}.{f}");')
    src = tmp_path / "layouts.c"
    src.write_text("\n".join(lines) + "\n")
    r = subprocess.run(["gcc", "-std=gnu11", "-fms-extensions", "-c", "-I", os.path.join(REF, "src", "core"), "-I",
                        os.path.join(ROOT, "include"), str(src), "-o", str(tmp_path / "layouts.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert sum(len(v) for v in fields.values()) > 100
