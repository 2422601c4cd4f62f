"""The allocation-free entry point, msgpu_tracelog_batch_noalloc, for callers
that cannot call cudaMalloc (code under stream capture, a GPU whose memory
another allocator owns): called through the C ABI with device buffers the
test allocates itself, its results must match the regular entry point
msgpu_tracelog_batch within the tolerance the FP64 parity tests use
(relative 1e-11 on Re ln det, identical branch of Im), on two calls in a row
that share the library's fixed scratch array.  Kept in its own file that
pytest collects last."""
import ctypes as C

import numpy as np
import pytest

from helpers import branch_distance, rel

pytestmark = pytest.mark.gpu


class _Model(C.Structure):
    _fields_ = [("type", C.c_int), ("np", C.c_int), ("p", C.c_double * 2)]


def _noalloc(ms, torch, d, n, pos, ks):
    L = ms.lib()
    f = L.msgpu_tracelog_batch_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, _Model, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    dpos = torch.tensor(pos, dtype=torch.float64, device="cuda")
    dks = torch.tensor(np.ascontiguousarray(ks).view(np.float64), dtype=torch.float64, device="cuda")
    dout = torch.full((2 * len(ks),), float("nan"), dtype=torch.float64, device="cuda")
    dst = torch.full((len(ks),), -1, dtype=torch.int32, device="cuda")
    m = _Model()
    m.type, m.np = 3, 0  # maximum model
    stream = torch.cuda.current_stream()
    rc = f(d, n, dpos.data_ptr(), m, len(ks), dks.data_ptr(), dout.data_ptr(), dst.data_ptr(), stream.cuda_stream)
    assert rc == 0, ms.lib().msgpu_last_error()
    torch.cuda.synchronize()
    out = dout.cpu().numpy().view(np.complex128)
    return out, dst.cpu().numpy()


def test_noalloc_matches_batch(ms):
    torch = pytest.importorskip("torch")
    d, n = 3, 160
    med = ms.Medium(d, n, seed=4)
    ks1 = ms.kcut_args(12, 0.5 - 0.05j, 3.0 - 0.05j)[4::3][:12]
    ks2 = np.array([0.9 - 0.3j, 2.0 - 0.01j, 1.4 - 0.6j, 2.7 - 0.2j, 0.6 - 0.05j])
    for ks in (ks1, ks2):  # two calls in a row on the shared scratch array
        got, st = _noalloc(ms, torch, d, n, med.pos, ks)
        want, wst = ms.tracelog_batch([med], ks)
        assert np.all(st == 0) and np.all(wst == 0)
        assert np.max(rel(got.real, want.real)) < 1e-11
        assert np.max(branch_distance(got.imag, want.imag, n)) < 1e-9


def test_noalloc_rejects_oversize(ms):
    torch = pytest.importorskip("torch")
    L = ms.lib()
    f = L.msgpu_tracelog_batch_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, _Model, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    m = _Model()
    m.type = 3
    rc = f(3, 4096, buf.data_ptr(), m, 1, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), None)
    assert rc == -4  # MSGPU_E_SIZE: n beyond the stated maximum of 2048
