"""The tensor-core operand layout: one bf16 product through the engine's
tcgen05 descriptors must be exact (small integers) and the negate bit must
negate.  Pins the layout the mixed-precision LU relies on."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _probe(ms, mode, A, B):
    L = ms.lib()
    fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
    L.msgpu_probe_umma.argtypes = [C.c_int, fp, fp, fp]
    D = np.zeros((128, 64), dtype=np.float32)
    rc = L.msgpu_probe_umma(mode, A, B, D)
    return rc, D


def test_umma_layout_exact(ms):
    rng = np.random.default_rng(0)
    A = rng.integers(-128, 129, (128, 32)).astype(np.float32)
    B = rng.integers(-128, 129, (64, 32)).astype(np.float32)
    want = A.astype(np.float64) @ B.astype(np.float64).T
    res = {}
    for mode in range(4):
        rc, D = _probe(ms, mode, A, B)
        res[mode] = (rc, float(np.max(np.abs(D - want))), float(np.max(np.abs(D + want))))
    print(res)
    assert res[0][0] == 0 and res[0][1] == 0.0, res
    assert res[2][0] == 0 and res[2][2] == 0.0, res
