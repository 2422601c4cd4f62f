"""Python host mirror of MSModel's hot-path interface over libmsgpu.so.

Names follow the reference (src/core/ms_matrix_util.h, medium_util.h,
ms_core.c): ``Medium``/``fill_medium``, ``build_ms_matrix``, ``tracelog_lu``,
``dk_log_det_ms``, ``total_cross_section``, ``run_tracelog`` (the k-point
loop of run_tracelog_omp) and their batched forms.  Every numerical call
goes through the C ABI declared in include/msgpu.h; there is no CPU path:
if the CUDA library is missing or no GPU is present the calls raise.
"""
import ctypes as C
import warnings
import os

import math

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmsgpu.so")

MODELS = {"hardsphere": 0, "softsphere": 1, "resonant": 2, "maximum": 3}
SHAPES = {"cube": 0, "ball": 1, "lattice": 2, "gaussian": 3}
PRECISION = {"fp64": 0, "mixed": 1}
S_SINGULAR, S_NONFINITE = 1, 2


class MsgpuError(RuntimeError):
    pass


class _Model(C.Structure):
    _fields_ = [("type", C.c_int), ("np", C.c_int), ("p", C.c_double * 2)]


class _Medium(C.Structure):
    _fields_ = [("d", C.c_int), ("n", C.c_int), ("pos", C.POINTER(C.c_double)), ("model", _Model)]


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lib = None


def lib():
    """Load libmsgpu.so (built by __graft_entry__.build() / msmodel_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise MsgpuError("libmsgpu.so is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(LIB_PATH)
    L.msgpu_init.argtypes = [C.c_int]
    L.msgpu_last_error.restype = C.c_char_p
    L.msgpu_launch_count.restype = C.c_uint64
    L.msgpu_probe_fp64.argtypes = [C.POINTER(C.c_double)]
    L.msgpu_probe_fp64_mma.argtypes = [C.POINTER(C.c_double)]
    L.msgpu_fill_medium.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint64, _dp]
    L.msgpu_random_doubles.argtypes = [C.c_uint64, C.c_int, _dp]
    L.msgpu_kplane_args.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _dp]
    L.msgpu_kcut_args.argtypes = [C.c_int, _dp, _dp, _dp]
    L.msgpu_logcut_args.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, _dp]
    L.msgpu_halton_points.argtypes = [_dp, C.c_int, _dp]
    L.msgpu_eval_special.argtypes = [C.c_int, C.c_int, C.POINTER(_Model), C.c_int, _dp, C.c_void_p, _dp]
    L.msgpu_build_matrix.argtypes = [C.POINTER(_Medium), _dp, C.c_int, _dp]
    L.msgpu_tracelog_matrix.argtypes = [C.c_int, _dp, _dp, C.POINTER(C.c_int)]
    batch = [C.c_int, C.POINTER(_Medium), C.c_int, _ip, _dp, _dp, _ip, C.c_int]
    L.msgpu_tracelog_batch.argtypes = batch
    L.msgpu_dk_log_det_batch.argtypes = batch
    L.msgpu_amplitude_batch.argtypes = [C.c_int, C.POINTER(_Medium), C.c_int, _ip, _dp, _dp, C.c_void_p, _ip,
                                        C.c_int]
    L.msgpu_job_create.restype = C.c_void_p
    L.msgpu_job_create.argtypes = [C.c_int, C.c_int, C.POINTER(_Medium), C.c_int, _ip, _dp, C.c_int]
    L.msgpu_job_run.argtypes = [C.c_void_p, C.c_void_p]
    L.msgpu_job_results.argtypes = [C.c_void_p, _dp, _ip]
    L.msgpu_job_amplitudes.argtypes = [C.c_void_p, _dp]
    L.msgpu_job_set_points.argtypes = [C.c_void_p, C.c_int, C.c_void_p, _dp]
    L.msgpu_job_use_graph.argtypes = [C.c_void_p, C.c_int]
    L.msgpu_job_launches.argtypes = [C.c_void_p]
    L.msgpu_job_flops.argtypes = [C.c_void_p]
    L.msgpu_job_flops.restype = C.c_double
    L.msgpu_job_destroy.argtypes = [C.c_void_p]
    L.msgpu_engine_stats.argtypes = [_dp, C.c_int]
    L.msgpu_debug_first_wait_limit.argtypes = [C.c_int]
    L.msgpu_wave_function.argtypes = [C.c_int, C.POINTER(_Medium), _dp, C.c_int, C.c_int, _dp, _dp, _dp, C.c_void_p,
                                       C.c_void_p, C.c_int]
    L.msgpu_wave_function_batch.argtypes = [C.c_int, C.POINTER(_Medium), C.c_int, _dp, C.c_int, C.c_int, _dp, _dp,
                                             _dp, C.c_void_p, C.c_void_p, C.c_int]
    L.msgpu_wave_cut.argtypes = [C.c_int, C.POINTER(_Medium), _dp, C.c_int, C.c_double, C.c_double, _dp, C.c_void_p,
                                 C.c_int]
    L.msgpu_diff_cross_section.argtypes = [C.c_int, C.POINTER(_Medium), C.c_double, C.c_int, C.c_double, C.c_double,
                                           _dp, C.c_int]
    L.msgpu_random_function.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.POINTER(_Model), C.c_int,
                                         C.c_int, C.c_double, C.c_double, _dp, _ip, C.c_int]
    L.msgpu_traceinv_batch.argtypes = [C.c_int, C.POINTER(_Medium), C.c_int, _ip, _dp, _dp, _ip, C.c_int]
    L.msgpu_inverse_iteration_batch.argtypes = [C.c_int, C.POINTER(_Medium), C.c_int, _ip, _dp, _dp, C.c_void_p,
                                                _ip, C.c_int]
    L.msgpu_find_roots_muller_batch.argtypes = [C.c_int, C.c_int, C.POINTER(_Medium), _dp, C.c_int, _dp, C.c_int,
                                                C.c_double, C.c_int, _dp, _ip, C.POINTER(C.c_int)]
    L.msgpu_eigvals_batch.argtypes = [C.c_int, C.POINTER(_Medium), C.c_int, _ip, _dp, _dp, _ip]
    L.msgpu_eigvals_batch_mtype.argtypes = [C.c_int, C.c_int, C.POINTER(_Medium), C.c_int, _ip, _dp, _dp, _ip,
                                            C.c_void_p]
    L.msgpu_tune_set.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    L.msgpu_tune_get.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.msgpu_autotune.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp]
    L.msgpu_solve_aberth_batch.argtypes = [C.c_int, C.POINTER(_Medium), _dp, C.c_int, _dp, C.c_int, C.c_int,
                                           C.c_double, C.c_int, _dp, _ip, C.POINTER(C.c_int)]
    _lib = L
    return L


def _check(rc, what):
    if rc != 0:
        raise MsgpuError(f"{what} failed ({rc}): {lib().msgpu_last_error().decode()}")


def init(device=0):
    _check(lib().msgpu_init(device), "msgpu_init")


def launch_count():
    """Kernels launched by libmsgpu.so since it was loaded."""
    return int(lib().msgpu_launch_count())


def probe_fp64_tflops():
    """Measured FP64 FMA throughput (TFLOP/s) of the current device."""
    v = C.c_double(0.0)
    _check(lib().msgpu_probe_fp64(C.byref(v)), "probe_fp64")
    return v.value


def probe_fp64_mma_tflops():
    """Measured FP64 tensor-core throughput (warp-level m8n8k4 MMA, TFLOP/s)."""
    v = C.c_double(0.0)
    _check(lib().msgpu_probe_fp64_mma(C.byref(v)), "probe_fp64_mma")
    return v.value


def engine_stats():
    """Per-phase SM cycles of the last mixed-precision run made with the
    environment variable MSGPU_STATS set (None otherwise)."""
    out = np.zeros(8)
    n = lib().msgpu_engine_stats(out, 8)
    if n <= 0:
        return None
    names = ["assemble", "panel", "trsm", "slice", "tiles", "solve", "items"]
    return {k: float(v) for k, v in zip(names, out[:n])}


def debug_first_wait_limit(polls):
    """Poll limit of the first operand wait of each mixed trailing update
    (polls < 0: the normal limit); 0 makes that wait run out (failure-path tests)."""
    _check(lib().msgpu_debug_first_wait_limit(int(polls)), "debug_first_wait_limit")


def sm_count():
    return int(lib().msgpu_sm_count())


def _model(model="maximum", params=()):
    m = _Model()
    m.type = MODELS[model] if isinstance(model, str) else int(model)
    m.np = len(params)
    for i, v in enumerate(params):
        m.p[i] = float(v)
    return m


def _c2(z):
    z = complex(z)
    return np.array([z.real, z.imag], dtype=np.float64)


def _cplx(zs):
    zs = np.ascontiguousarray(np.atleast_1d(np.asarray(zs, dtype=np.complex128)))
    return zs.view(np.float64).reshape(-1).copy()


# --------------------------------------------------------------------------- media
def fill_medium(d, n, seed, shape="ball", ratio=1.0):
    """Seeded scatterers, bit-exact with the reference fill_medium (medium_util.c:164)."""
    pos = np.zeros(n * d)
    _check(lib().msgpu_fill_medium(d, n, SHAPES[shape] if isinstance(shape, str) else shape, ratio, seed, pos),
           "fill_medium")
    return pos


class Medium:
    """A scatterer set: d, n, atom-major positions and the scattering model
    (the reference Medium, src/core/medium_type.h:42-54)."""

    def __init__(self, d, n, pos=None, model="maximum", params=(), shape="ball", ratio=1.0, seed=None):
        self.d, self.n = int(d), int(n)
        self.model, self.params, self.shape, self.ratio = model, tuple(params), shape, ratio
        self.seed = seed
        if pos is None:
            pos = fill_medium(d, n, 1 if seed is None else seed, shape, ratio)
        self.pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        assert self.pos.size == self.n * self.d

    def fill(self, seed):
        """fill_medium(med, seed): redraw the positions with the given seed."""
        self.seed = seed
        self.pos = fill_medium(self.d, self.n, seed, self.shape, self.ratio)
        return self

    def _struct(self):
        m = _Medium()
        m.d, m.n = self.d, self.n
        m.pos = self.pos.ctypes.data_as(C.POINTER(C.c_double))
        m.model = _model(self.model, self.params)
        return m


def _media_array(media):
    arr = (_Medium * len(media))()
    for i, m in enumerate(media):
        arr[i] = m._struct()
    return arr


def random_doubles(seed, n):
    """n values of the reference generator from init_random(seed) (nru_random.c:39, :63)."""
    out = np.zeros(n)
    lib().msgpu_random_doubles(seed, n, out)
    return out


def realisation_sizes(count, nmin=100, nmax=600, seed=0):
    """Sizes of the batched realisations: N_r = nmin + floor((nmax-nmin+1) u_r), u_r drawn
    in order from init_random(seed)."""
    u = random_doubles(seed, count)
    return [nmin + int((nmax - nmin + 1) * x) for x in u]


# --------------------------------------------------------------------------- grids
def kplane_args(nx, ny, xmin, xmax, ymin, ymax):
    """k of every pixel of a complex map, get_arg_cmap order (complex_map_util.c:27)."""
    out = np.zeros(2 * nx * ny)
    lib().msgpu_kplane_args(nx, ny, xmin, xmax, ymin, ymax, out)
    return out.view(np.complex128).copy()


def kcut_args(ns, zmin, zmax):
    """k of every sample of a complex cut, get_arg_ccut order (complex_cut_util.c:32)."""
    out = np.zeros(2 * 3 * (ns + 2))
    lib().msgpu_kcut_args(ns, _c2(zmin), _c2(zmax), out)
    return out.view(np.complex128).copy()


def logcut_args(ns, rek, imkmin, imkmax):
    """k of every sample of a log cut (init_logcut, log_cut_util.c:93-96): the
    points run_tracelog evaluates for the reference's [logkcut] task."""
    if ns < 2 or imkmin >= 0 or imkmax >= 0:
        raise ValueError("logcut_args: ns >= 2 and negative end points (as init_logcut requires)")
    out = np.zeros(2 * ns)
    lib().msgpu_logcut_args(ns, float(rek), float(imkmin), float(imkmax), out)
    return out.view(np.complex128).copy()


def halton_points(dom, n):
    """First n Halton (2,3) points of dom = (xmin, xmax, ymin, ymax) (domain_util.c:180)."""
    out = np.zeros(2 * n)
    lib().msgpu_halton_points(np.asarray(dom, dtype=np.float64), n, out)
    return out.view(np.complex128).copy()


# --------------------------------------------------------------------------- device special functions
def eval_special(which, d, ks, rs=None, model="maximum", params=()):
    kk = _cplx(ks)
    n = kk.size // 2
    out = np.zeros(2 * n)
    m = _model(model, params)
    rr = None if rs is None else np.ascontiguousarray(np.broadcast_to(np.asarray(rs, dtype=np.float64), (n,)))
    _check(lib().msgpu_eval_special(which, d, C.byref(m), n, kk, None if rr is None else rr.ctypes.data, out),
           "eval_special")
    return out.view(np.complex128).copy()


def free_green(d, ks, rs=1.0):
    return eval_special(0, d, ks, rs)


def dk_free_green(d, ks, rs=1.0):
    return eval_special(1, d, ks, rs)


def free_green_imag(d, ks, rs=1.0):
    return eval_special(2, d, ks, rs)


def bessel_k(twonu, zs):
    return eval_special(3, twonu, zs)


def invf(d, ks, model="maximum", params=()):
    return eval_special(4, d, ks, None, model, params)


# --------------------------------------------------------------------------- single matrices
def build_ms_matrix(med, k, deriv=False):
    """M(k) (or dM/dk) assembled on the GPU; returned as an [row, col] array."""
    out = np.zeros(2 * med.n * med.n)
    s = med._struct()
    _check(lib().msgpu_build_matrix(C.byref(s), _c2(k), int(deriv), out), "build_ms_matrix")
    return out.view(np.complex128).reshape(med.n, med.n).T


def build_dk_ms_matrix(med, k):
    return build_ms_matrix(med, k, deriv=True)


def tracelog_lu(matrix):
    """ln det(M)/n of an [row, col] matrix, LU on the GPU (ms_matrix_util.c:185). Returns (value, info)."""
    a = np.asarray(matrix, dtype=np.complex128)
    n = a.shape[0]
    buf = np.ascontiguousarray(a.T).view(np.float64).reshape(-1).copy()
    out = np.zeros(2)
    info = C.c_int(0)
    _check(lib().msgpu_tracelog_matrix(n, buf, out, C.byref(info)), "tracelog_lu")
    return complex(out[0], out[1]), info.value


# --------------------------------------------------------------------------- batches
def _items(media, ks, item_med):
    kk = _cplx(ks)
    nitem = kk.size // 2
    if item_med is None:
        im = np.zeros(nitem, dtype=np.int32)
    else:
        im = np.ascontiguousarray(item_med, dtype=np.int32)
    assert im.size == nitem
    return kk, nitem, im


def tracelog_batch(media, ks, item_med=None, precision="fp64"):
    """ln det M(k)/n for every item (medium item_med[i], wave number ks[i])."""
    media = [media] if isinstance(media, Medium) else list(media)
    kk, nitem, im = _items(media, ks, item_med)
    out = np.zeros(2 * nitem)
    st = np.zeros(nitem, dtype=np.int32)
    arr = _media_array(media)
    _check(lib().msgpu_tracelog_batch(len(media), arr, nitem, im, kk, out, st, PRECISION[precision]),
           "tracelog_batch")
    return out.view(np.complex128).copy(), st


def dk_log_det_batch(media, ks, item_med=None, precision="fp64"):
    """tr(M^-1 dM/dk) for every item (dk_log_det_ms, ms_matrix_util.c:242)."""
    media = [media] if isinstance(media, Medium) else list(media)
    kk, nitem, im = _items(media, ks, item_med)
    out = np.zeros(2 * nitem)
    st = np.zeros(nitem, dtype=np.int32)
    arr = _media_array(media)
    _check(lib().msgpu_dk_log_det_batch(len(media), arr, nitem, im, kk, out, st, PRECISION[precision]),
           "dk_log_det_batch")
    return out.view(np.complex128).copy(), st


def amplitude_batch(media, ks, item_med=None, precision="fp64", want_amps=True):
    """a = M^-1 phi (plane wave along +x) and -Im(conj(phi).a)/k per item."""
    media = [media] if isinstance(media, Medium) else list(media)
    kk, nitem, im = _items(media, ks, item_med)
    out = np.zeros(2 * nitem)
    st = np.zeros(nitem, dtype=np.int32)
    ntot = sum(media[i].n for i in im)
    amps = np.zeros(2 * ntot) if want_amps else None
    arr = _media_array(media)
    _check(lib().msgpu_amplitude_batch(len(media), arr, nitem, im, kk, out,
                                       None if amps is None else amps.ctypes.data, st, PRECISION[precision]),
           "amplitude_batch")
    sig = out.view(np.complex128).copy()
    if amps is None:
        return sig, None, st
    amps = amps.view(np.complex128)
    parts, off = [], 0
    for i in im:
        parts.append(amps[off:off + media[i].n].copy())
        off += media[i].n
    return sig, parts, st


def dk_log_det_ms(med, k):
    """Scalar form of dk_log_det_ms (ms_matrix_util.c:242)."""
    v, st = dk_log_det_batch([med], [k])
    return complex(v[0])


def total_cross_section(med, k):
    """Optical-theorem total cross section at real k (ms_matrix_util.c:344)."""
    sig, _, _ = amplitude_batch([med], [k], want_amps=False)
    return float(sig[0].real)


RANDOM_FUNCTIONS = {"crsec": 0, "dos": 1}


def random_function(kind, d, n, nseed, nbin, xmin, xmax, model="maximum", params=(), shape="ball", ratio=1.0,
                    precision="fp64"):
    """run_random_function_omp (ms_core.c:476-519): total cross section
    ("crsec") or density of states ("dos") for seeds 1..nseed at the nbin
    log-spaced real k of get_arg_rfun (random_function_util.c:103), every bin
    sorted.  Returns (k[nbin], data[nbin, nseed], status[nbin*nseed])."""
    data = np.zeros(nseed * nbin)
    status = np.zeros(nseed * nbin, dtype=np.int32)
    m = _model(model, params)
    _check(lib().msgpu_random_function(RANDOM_FUNCTIONS[kind], d, n, SHAPES[shape] if isinstance(shape, str) else shape,
                                       ratio, C.byref(m), nseed, nbin, xmin, xmax, data, status,
                                       PRECISION[precision]), "random_function")
    ks = xmin * np.exp(np.arange(nbin) * np.log(xmax / xmin) / (nbin - 1))
    return ks, data.reshape(nbin, nseed), status


def run_tracelog(d, n, ks, nseed=1, model="maximum", params=(), shape="ball", ratio=1.0, precision="fp64"):
    """The k-point loop of run_tracelog_omp (ms_core.c:96-141): seeds 1..nseed,
    ln det/n at every k, averaged over seeds in seed order."""
    media = [Medium(d, n, model=model, params=params, shape=shape, ratio=ratio, seed=s) for s in range(1, nseed + 1)]
    ks = np.atleast_1d(np.asarray(ks, dtype=np.complex128))
    nk = ks.size
    allk = np.tile(ks, nseed)
    im = np.repeat(np.arange(nseed, dtype=np.int32), nk)
    out, st = tracelog_batch(media, allk, im, precision)
    data = np.zeros(nk, dtype=np.complex128)
    for s in range(1, nseed + 1):
        data = ((s - 1) * data + out[(s - 1) * nk:s * nk]) / s
    return data, st


def wave_function(media, k, nx, ny, dom, precision="fp64"):
    """run_wave_function_omp (ms_core.c:596): seed-averaged Re psi and |psi|^2 on
    the nx x ny grid, plus psi of the first medium and every medium's amplitudes."""
    fun, den, psi, amps = wave_function_batch(media, [k], nx, ny, dom, precision)
    return fun[0], den[0], psi[0], [a[0] for a in amps]


def wave_function_batch(media, ks, nx, ny, dom, precision="fp64", want_psi=True):
    """run_wave_function_omp at every k of ks, all solves in one batched job.
    Returns fun[nk, nx*ny], den[nk, nx*ny], psi[nk, nx*ny] of the first medium
    (None unless want_psi), amps[medium][k] (n complex each)."""
    media = [media] if isinstance(media, Medium) else list(media)
    ks = np.ascontiguousarray(np.asarray(ks, dtype=np.complex128))
    nk, n, npx = len(ks), media[0].n, nx * ny
    fun = np.zeros(nk * npx)
    den = np.zeros(nk * npx)
    psi = np.zeros(2 * nk * npx) if want_psi else None
    amps = np.zeros(2 * len(media) * nk * n)
    arr = _media_array(media)
    rc = lib().msgpu_wave_function_batch(len(media), arr, nk, ks.view(np.float64), nx, ny,
                                         np.asarray(dom, dtype=np.float64), fun, den,
                                         psi.ctypes.data if want_psi else None, amps.ctypes.data,
                                         PRECISION[precision])
    if rc < 0:
        _check(rc, "wave_function_batch")
    if rc > 0:
        warnings.warn(f"wave_function_batch: a solve returned status {rc:#x} "
                      f"(singular or non-finite amplitudes were averaged in)", RuntimeWarning, stacklevel=2)
    a = amps.view(np.complex128).reshape(len(media), nk, n)
    return (fun.reshape(nk, npx), den.reshape(nk, npx),
            psi.view(np.complex128).reshape(nk, npx) if want_psi else None, [a[m].copy() for m in range(len(media))])


def wave_cut(media, k, nbin, xmin, xmax, precision="fp64"):
    """psi of every medium at the nbin points (xmin + i dx, 0, ...) of the x axis,
    dx = (xmax - xmin)/(nbin - 1) (run_wave_function_cut_omp, ms_core.c:654-703;
    get_pos_wfcut, wave_function_cut_util.c:83), all solves in one batched job.
    Returns psi[nmed, nbin] (complex)."""
    media = [media] if isinstance(media, Medium) else list(media)
    psi = np.zeros(2 * len(media) * nbin)
    kk = np.array([complex(k).real, complex(k).imag])
    rc = lib().msgpu_wave_cut(len(media), _media_array(media), kk, nbin, float(xmin), float(xmax), psi, None,
                              PRECISION[precision])
    if rc < 0:
        _check(rc, "wave_cut")
    if rc > 0:
        warnings.warn(f"wave_cut: a solve returned status {rc:#x} (singular or non-finite amplitudes)",
                      RuntimeWarning, stacklevel=2)
    return psi.view(np.complex128).reshape(len(media), nbin)


def _quantile_sorted(x, q):
    """quantile (real_vector_util.c:121-134) of sorted samples x: linear
    interpolation at the continuous index (n-1) q."""
    n = x.size
    if n == 1 or q <= 0.0:
        return float(x[0])
    if q >= 1.0:
        return float(x[n - 1])
    idx = (n - 1) * q
    i = int(math.floor(idx))
    return float(x[i] + (idx - i) * (x[i + 1] - x[i]))


def _mean_sorted(x):
    """mean_vector (real_vector_util.c:139-147): the sum in order over n."""
    return float(np.cumsum(x)[-1]) / x.size


def _mean_quartiles(samples):
    """store_data_wfcut's statistics of one bin (wave_function_cut_util.c:92-114):
    the samples sorted, their mean summed in order (mean_vector) and the first
    and third quartiles (quantile)."""
    x = np.sort(np.asarray(samples, dtype=np.float64))
    return [_mean_sorted(x), _quantile_sorted(x, 0.25), _quantile_sorted(x, 0.75)]


def run_wave_function_cut(media, k, nbin, xmin, xmax, precision="mixed"):
    """run_wave_function_cut_omp (ms_core.c:654-703), plane wave, for the
    realisations of media: psi of every seed on the cut on the GPU (wave_cut),
    then per bin the mean and quartiles of Re psi, Im psi and |psi|^2 as
    store_data_wfcut forms them.  Returns dict(repsi, impsi, density) with rows
    [mean, q1/4, q3/4] per bin, and psi[nmed, nbin]."""
    psi = wave_cut(media, k, nbin, xmin, xmax, precision)
    out = {"psi": psi}
    for key, v in (("repsi", psi.real), ("impsi", psi.imag), ("density", psi.real ** 2 + psi.imag ** 2)):
        out[key] = np.array([_mean_quartiles(v[:, i]) for i in range(nbin)])
    return out


def diff_cross_section(media, k, nbin, thmin, thmax, precision="fp64"):
    """The differential cross section samples of run_differential_cross_section_omp
    (ms_core.c:526-594) at real k for every medium, all solves in one batched job:
    samples[i, m] = (k/2pi)^(d-3)/(16 pi^2) |b(th_i)^H a_m|^2 at the angles
    th_i = thmin exp(i log(thmax/thmin)/(nbin-1)) degrees (get_arg_dcs)."""
    media = [media] if isinstance(media, Medium) else list(media)
    out = np.zeros(len(media) * nbin)
    rc = lib().msgpu_diff_cross_section(len(media), _media_array(media), float(k), nbin, float(thmin), float(thmax),
                                        out, PRECISION[precision])
    if rc < 0:
        _check(rc, "diff_cross_section")
    if rc > 0:
        warnings.warn(f"diff_cross_section: a solve returned status {rc:#x} (singular or non-finite amplitudes)",
                      RuntimeWarning, stacklevel=2)
    return out.reshape(nbin, len(media))


def dcs_statistics(samples, nq, nc):
    """The statistics run_differential_cross_section_omp forms from samples[nbin,
    nseed] (ms_core.c:572-583): curve[i, s] the first nc seeds' samples, then per
    bin the samples sorted, data[i, q] their quantile at q/(nq-1) and mean[i]."""
    samples = np.asarray(samples, dtype=np.float64)
    nbin = samples.shape[0]
    curve = samples[:, :nc].copy()
    data = np.zeros((nbin, nq))
    mean = np.zeros(nbin)
    for i in range(nbin):
        x = np.sort(samples[i])
        data[i] = [_quantile_sorted(x, q / (nq - 1)) for q in range(nq)]
        mean[i] = _mean_sorted(x)
    return {"data": data, "mean": mean, "curve": curve}


def run_differential_cross_section(media, k, nbin, thmin, thmax, nq=5, nc=1, precision="mixed"):
    """run_differential_cross_section_omp for the realisations of media (seeds in
    order): the samples on the GPU (diff_cross_section), then dcs_statistics.
    Returns dict(samples, data, mean, curve)."""
    samples = diff_cross_section(media, k, nbin, thmin, thmax, precision)
    out = dcs_statistics(samples, nq, nc)
    out["samples"] = samples
    return out


def solve_aberth_batch(media, dom, z0, nexpsup=4, maxit=30, toler=1e-10, precision="fp64"):
    """solve_aberth on dlogf (root_finder.c:522) for every medium, starting from
    the same points z0.  Returns (list of root arrays sorted by Re, dlogf evaluations)."""
    media = [media] if isinstance(media, Medium) else list(media)
    z = _cplx(z0)
    nz = z.size // 2
    roots = np.zeros(2 * nz * len(media))
    nr = np.zeros(len(media), dtype=np.int32)
    ne = C.c_int(0)
    arr = _media_array(media)
    _check(lib().msgpu_solve_aberth_batch(len(media), arr, np.asarray(dom, dtype=np.float64), nz, z, nexpsup,
                                          maxit, toler, PRECISION[precision], roots, nr, C.byref(ne)),
           "solve_aberth_batch")
    rc = roots.view(np.complex128).reshape(len(media), max(nz, 1))
    return [rc[m, :nr[m]].copy() for m in range(len(media))], ne.value


def traceinv_batch(media, ks, item_med=None, precision="fp64"):
    """tr M(k)^-1 per item (traceinv, ms_matrix_util.c:319)."""
    media = [media] if isinstance(media, Medium) else list(media)
    kk, nitem, im = _items(media, ks, item_med)
    out = np.zeros(2 * nitem)
    st = np.zeros(nitem, dtype=np.int32)
    _check(lib().msgpu_traceinv_batch(len(media), _media_array(media), nitem, im, kk, out, st, PRECISION[precision]),
           "traceinv_batch")
    return out.view(np.complex128).copy(), st


def inverse_iteration_batch(media, ks, item_med=None, want_vecs=True):
    """inverse_iteration (ms_matrix_util.c:279) on M(k) from the constant unit
    vector (compute_eigenstates, ms_core.c:296): (lambda, eigenvectors, status)."""
    media = [media] if isinstance(media, Medium) else list(media)
    kk, nitem, im = _items(media, ks, item_med)
    lam = np.zeros(2 * nitem)
    st = np.zeros(nitem, dtype=np.int32)
    ntot = sum(media[i].n for i in im)
    vecs = np.zeros(2 * ntot) if want_vecs else None
    _check(lib().msgpu_inverse_iteration_batch(len(media), _media_array(media), nitem, im, kk, lam,
                                               None if vecs is None else vecs.ctypes.data, st, 0),
           "inverse_iteration_batch")
    parts = None
    if want_vecs:
        v = vecs.view(np.complex128)
        parts, off = [], 0
        for i in im:
            parts.append(v[off:off + media[i].n].copy())
            off += media[i].n
    return lam.view(np.complex128).copy(), parts, st


MTYPES = {"msmatrix": 0, "normalized": 1}


def eigvals_batch(media, ks, item_med=None, mtype="msmatrix", want_trg2=False):
    """The n eigenvalues per item (eigvals, ms_matrix_util.c:147) of M(k), or
    with mtype "normalized" of N(k) = i - G(k)/I(k,0) (build_normalized_matrix,
    ms_matrix_util.c:50): (list of arrays, status), and with want_trg2 also
    each item's Tr[G^+ G]/N (tracegtwo, ms_matrix_util.c:167)."""
    media = [media] if isinstance(media, Medium) else list(media)
    kk, nitem, im = _items(media, ks, item_med)
    mu = np.zeros(2 * sum(media[i].n for i in im))
    st = np.zeros(nitem, dtype=np.int32)
    trg = np.zeros(nitem) if want_trg2 else None
    _check(lib().msgpu_eigvals_batch_mtype(MTYPES[mtype], len(media), _media_array(media), nitem, im, kk, mu, st,
                                           trg.ctypes.data if want_trg2 else None), "eigvals_batch")
    mu = mu.view(np.complex128)
    out, off = [], 0
    for i in im:
        out.append(mu[off:off + media[i].n].copy())
        off += media[i].n
    return (out, st, trg) if want_trg2 else (out, st)


def imag_mu_histogram(mus, nbin, xmin, xmax):
    """Histogram of Im mu on log-spaced bins over [xmin, xmax] (0 < xmin), as
    run_imag_mu_histogram_omp builds it (imag_mu_histogram_util.c:108-153):
    bin floor(nbin (ln Im mu - ln xmin) / ln(xmax/xmin)), samples outside the
    range lost, then normalised to unit integral, bin i divided by x_i fac with
    fac = total ln(xmax/xmin)/nbin and x_i = xmin exp(ln(xmax/xmin)(i + 1/2)/nbin)
    the bin's centre; the C library's log and exp, in the reference's order of
    operations.  Returns (density, bin centres, lost count)."""
    x = np.concatenate([np.asarray(m).imag for m in mus])
    counts = np.zeros(nbin)
    lo, hi = _c_log(xmin), _c_log(xmax)
    with np.errstate(divide="ignore", invalid="ignore"):
        idx = np.floor(nbin * (np.array([_c_log(v) for v in x]) - lo) / (hi - lo))
    ok = np.isfinite(idx) & (idx >= 0) & (idx < nbin)
    np.add.at(counts, idx[ok].astype(int), 1.0)
    lost = int(x.size - ok.sum())
    lw = _c_log(xmax / xmin)
    centres = np.array([xmin * _c_exp(lw * (i + 0.5) / nbin) for i in range(nbin)])
    total = float(np.cumsum(counts)[-1]) if nbin else 0.0
    fac = total * lw / nbin
    dens = counts / (centres * fac) if total else counts
    return dens, centres, lost


def imag_mu_task(mus, nbin, avgx, trg2):
    """The arithmetic of run_imag_mu_histogram_omp (ms_core.c:225-282) from the
    eigenvalues of the realisations of seeds 1, 2, ... in order (mus[s-1]), the
    exact mean avgx = Re I(k, 0) of Im mu and each realisation's Tr[G^+ G]/N
    (trg2): the range from seed 1 (setup_domain_ihist: the smallest positive and
    the largest Im mu, halved and doubled), the histogram (imag_mu_histogram),
    the true variance sum (Im mu - avgx)^2 / (nseed n) and the expected one
    sum Tr[G^+ G]/(4 N) / nseed, summed in order as one thread of the reference
    does.  Returns dict(data, centres, xmin, xmax, avgx, varx_true, varx_expc,
    lost)."""
    y0 = np.asarray(mus[0]).imag
    xmin = xmax = float(y0[0])
    for v in y0[1:]:
        v = float(v)
        if v < xmin and v > 0.0:
            xmin = v
        if v > xmax:
            xmax = v
    xmin, xmax = xmin / 2.0, 2.0 * xmax
    data, centres, lost = imag_mu_histogram(mus, nbin, xmin, xmax)
    y = np.concatenate([np.asarray(m).imag for m in mus])
    varx_true = float(np.cumsum((y - avgx) * (y - avgx))[-1]) / (len(mus) * len(y0))
    varx_expc = float(np.cumsum(0.25 * np.asarray(trg2, dtype=np.float64))[-1]) / len(mus)
    return {"data": data, "centres": centres, "xmin": xmin, "xmax": xmax, "avgx": float(avgx),
            "varx_true": varx_true, "varx_expc": varx_expc, "lost": lost}


def run_imag_mu_histogram(media, k, nbin):
    """run_imag_mu_histogram_omp (ms_core.c:225-282) for the realisations of
    media (seeds 1, 2, ... in order) at real k: the eigenvalues and each
    Tr[G^+ G]/N on the GPU (eigvals_batch), I(k, 0) by the GPU's Green function,
    the rest by imag_mu_task.  Adds "status"."""
    media = [media] if isinstance(media, Medium) else list(media)
    mus, st, trg = eigvals_batch(media, np.full(len(media), complex(k)), np.arange(len(media), dtype=np.int32),
                                 want_trg2=True)
    avgx = complex(np.asarray(free_green_imag(media[0].d, [complex(k)], [0.0])).reshape(-1)[0]).real
    out = imag_mu_task(mus, nbin, avgx, trg)
    out["status"] = st
    return out

def _c_round(v):
    """C's round(): halves away from zero (numpy rounds them to even)."""
    v = np.asarray(v, dtype=np.float64)
    r = np.trunc(v)
    return r + np.where(np.abs(v - r) >= 0.5, np.sign(v), 0.0)


def _c_log(v):
    """The C library's log (math.log calls it), with its results for v <= 0."""
    v = float(v)
    if v > 0.0 or v != v:
        return math.log(v) if v == v else v
    return -math.inf if v == 0.0 else -math.nan


def _c_exp(v):
    v = float(v)
    try:
        return math.exp(v)
    except OverflowError:
        return math.inf


def chistogram(mus, xbin, ybin, mbin, dom=None, mrange=None):
    """The mu-plane histogram of run_chistogram_omp (ms_core.c:173-232) from the
    eigenvalues of every realisation, binned as fill_chist does
    (chistogram_util.c:103-264):
      * moments: the mean and the per-component standard deviation of mu,
        summed in order as the reference sums them;
      * domain {xmin, xmax, ymin, ymax}: given, or the extremes of the values;
        pixel (ix, iy) = (round((xbin-1)(Re mu - xmin)/(xmax - xmin)),
        round((ybin-1)(ymax - Im mu)/(ymax - ymin))), row-major from the top
        row, counts (not normalised, as the reference leaves them);
      * marginal of Im mu on mbin log-spaced bin centres over [mmin, mmax]
        (given, or the range of Im mu): bin round((mbin-1) ln(Im mu/mmin) /
        ln(mmax/mmin)), normalised to unit integral with the width fac x of
        each bin, fac = ln(mmax/mmin)/(mbin-1).
    Values outside a range are lost (counted once per range they miss).
    Returns dict(data[ybin, xbin], mdata[mbin], dom, mrange, avg, sigma, lost)."""
    z = np.concatenate([np.asarray(m, dtype=np.complex128).ravel() for m in mus])
    if z.size < 2:
        raise ValueError("chistogram: at least two values are needed to set up the domain")
    # stat_moments (chistogram_util.c:103-121): sums in order, as the reference
    # adds them (cumsum is sequential), so that the moments match its bits
    nz = z.size
    avg = complex(np.cumsum(z.real)[-1] / nz, np.cumsum(z.imag)[-1] / nz)
    dzr, dzi = z.real - avg.real, z.imag - avg.imag
    sigma = complex(np.sqrt(np.cumsum(dzr * dzr)[-1] / nz), np.sqrt(np.cumsum(dzi * dzi)[-1] / nz))
    if dom is None:
        dom = [float(z.real.min()), float(z.real.max()), float(z.imag.min()), float(z.imag.max())]
    if mrange is None:
        mrange = [float(z.imag.min()), float(z.imag.max())]
    xmin, xmax, ymin, ymax = dom
    with np.errstate(divide="ignore", invalid="ignore"):
        ix = _c_round((xbin - 1) * (z.real - xmin) / (xmax - xmin))
        iy = _c_round((ybin - 1) * (ymax - z.imag) / (ymax - ymin))
    ok = np.isfinite(ix) & np.isfinite(iy) & (ix >= 0) & (ix < xbin) & (iy >= 0) & (iy < ybin)
    data = np.zeros(xbin * ybin)
    np.add.at(data, (ix[ok] + iy[ok] * xbin).astype(np.int64), 1.0)
    lost = int(z.size - ok.sum())
    # the marginal with the C library's log and exp, as the reference's
    # append_to_marginal and normalize_marginal_chist (chistogram_util.c:210-249) call them
    mmin, mmax = mrange
    lmin, lmax = _c_log(mmin), _c_log(mmax)
    with np.errstate(divide="ignore", invalid="ignore"):
        im = _c_round((mbin - 1) * (np.array([_c_log(v) for v in z.imag]) - lmin) / (lmax - lmin))
    okm = np.isfinite(im) & (im >= 0) & (im < mbin)
    mdata = np.zeros(mbin)
    np.add.at(mdata, im[okm].astype(np.int64), 1.0)
    lost += int(z.size - okm.sum())
    total = float(np.cumsum(mdata)[-1])
    fac = _c_log(mmax / mmin) / (mbin - 1) if mmin != 0 else math.nan
    with np.errstate(divide="ignore", invalid="ignore"):
        for i in range(mbin):
            x = mmin * _c_exp(fac * i)
            mdata[i] = mdata[i] / (fac * x * total)
    return {"data": data.reshape(ybin, xbin), "mdata": mdata, "dom": dom, "mrange": mrange, "avg": avg,
            "sigma": sigma, "lost": lost}


def run_chistogram(media, k, xbin, ybin, mbin, dom=None, mrange=None, mtype="msmatrix"):
    """run_chistogram_omp (ms_core.c:173-232): the eigenvalues of M(k) (or of
    N(k), mtype "normalized") of every realisation on the GPU (eigvals_batch),
    binned by chistogram."""
    media = [media] if isinstance(media, Medium) else list(media)
    mus, st = eigvals_batch(media, np.full(len(media), complex(k)), np.arange(len(media), dtype=np.int32), mtype)
    out = chistogram(mus, xbin, ybin, mbin, dom, mrange)
    out["status"] = st
    return out


EIG_METHODS = {"determinant": 0, "mineigval": 1, "invtraceinv": 2}


def find_roots_muller(method, media, dom, z0, maxit=30, toler=1e-10, precision="fp64"):
    """find_eigenstates_serial_2/3 (ms_core.c:335-401) for every medium from the
    same starting points: (list of root arrays, function evaluations)."""
    media = [media] if isinstance(media, Medium) else list(media)
    z = _cplx(z0)
    nz = z.size // 2
    roots = np.zeros(2 * max(nz, 1) * len(media))
    nr = np.zeros(len(media), dtype=np.int32)
    ne = C.c_int(0)
    _check(lib().msgpu_find_roots_muller_batch(EIG_METHODS[method], len(media), _media_array(media),
                                               np.asarray(dom, dtype=np.float64), nz, z, maxit, toler,
                                               PRECISION[precision], roots, nr, C.byref(ne)), "find_roots_muller")
    r = roots.view(np.complex128)
    return [r[m * nz:m * nz + nr[m]].copy() for m in range(len(media))], ne.value


def find_eigenstates(media, dom, ntarget, maxit=30, toler=1e-10, precision="fp64", method="determinant",
                     eigenvectors=False):
    """run_eigenstate_list_serial (ms_core.c:407-435): ntarget Halton targets
    sorted by -Im, the chosen root method (Aberth with nexpsup = 4 on dlogf for
    "determinant", Muller for "mineigval" / "invtraceinv"), roots ordered by
    -Im.  With eigenvectors, also compute_eigenstates (ms_core.c:296): per
    medium a list of (root, mu, eigenvector) by inverse iteration at each root.
    Returns (roots per medium, function evaluations[, eigenstates])."""
    media = [media] if isinstance(media, Medium) else list(media)
    z0 = halton_points(dom, ntarget)
    z0 = z0[np.argsort(-z0.imag, kind="stable")]
    if method == "determinant":
        roots, ne = solve_aberth_batch(media, dom, z0, 4, maxit, toler, precision)
    else:
        roots, ne = find_roots_muller(method, media, dom, z0, maxit, toler, precision)
    roots = [r[np.argsort(-r.imag, kind="stable")] for r in roots]
    if not eigenvectors:
        return roots, ne
    ks = np.concatenate(roots) if any(len(r) for r in roots) else np.zeros(0, complex)
    states = [[] for _ in media]
    if ks.size:
        im = np.concatenate([np.full(len(r), m, dtype=np.int32) for m, r in enumerate(roots)])
        lam, vecs, _ = inverse_iteration_batch(media, ks, im)
        for q in range(ks.size):
            states[im[q]].append((ks[q], lam[q], vecs[q]))
    return roots, ne, states


# --------------------------------------------------------------------------- autotuning
KIND_CODES = {"tracelog": 0, "dlogf": 1, "amplitude": 2}
ENGINES = {-1: None, 0: "fp64", 1: "mixed"}


def tune_set(kind, precision, n, engine=None, ctas_per_sm=0):
    """Fix the launch choice for jobs of this kind and requested precision whose
    largest n falls in n's size bucket (engine None = the requested one)."""
    e = -1 if engine is None else PRECISION[engine]
    _check(lib().msgpu_tune_set(KIND_CODES[kind], PRECISION[precision], n, e, ctas_per_sm), "tune_set")


def tune_get(kind, precision, n):
    e, c = C.c_int(0), C.c_int(0)
    _check(lib().msgpu_tune_get(KIND_CODES[kind], PRECISION[precision], n, C.byref(e), C.byref(c)), "tune_get")
    return ENGINES[e.value], c.value


def autotune(kind, precision, d, n, nitem=None):
    """Time the candidate launches (engine x CTAs per SM) on a probe batch and
    keep the fastest for n's size bucket.  Returns {candidate: seconds} and the
    choice."""
    nitem = nitem or 2 * sm_count()
    t = np.full(4, -1.0)
    _check(lib().msgpu_autotune(KIND_CODES[kind], PRECISION[precision], d, n, nitem, t), "autotune")
    names = ["fp64 x1", "fp64 x2", "mixed x1", "mixed x2"]
    return {names[i]: float(t[i]) for i in range(4) if t[i] >= 0}, tune_get(kind, precision, n)


def tune_table():
    """Every non-default entry: [(kind, precision, bucket upper n, engine, ctas)]."""
    rows = []
    for kind in KIND_CODES:
        for prec in PRECISION:
            for b in range(17):
                e, c = tune_get(kind, prec, 1 << b)
                if e is not None or c:
                    rows.append((kind, prec, 1 << b, e, c))
    return rows


def tune_save(path):
    import json
    with open(path, "w") as f:
        json.dump(tune_table(), f)


def tune_load(path):
    import json
    with open(path) as f:
        for kind, prec, n, e, c in json.load(f):
            tune_set(kind, prec, n, e, c)


class Job:
    """A resident job: inputs on the device, run asynchronously on a stream
    (the handle of a CUDA stream, e.g. torch.cuda.current_stream().cuda_stream)."""

    KINDS = {"tracelog": 0, "dlogf": 1, "amplitude": 2}

    def __init__(self, kind, media, ks, item_med=None, precision="fp64"):
        media = [media] if isinstance(media, Medium) else list(media)
        self.media = media
        kk, self.nitem, im = _items(media, ks, item_med)
        self._keep = (kk, im)
        arr = _media_array(media)
        self.kind = self.KINDS[kind]
        self.h = lib().msgpu_job_create(self.kind, len(media), arr, self.nitem, im, kk, PRECISION[precision])
        if not self.h:
            raise MsgpuError("job_create failed: " + lib().msgpu_last_error().decode())
        self.item_med = im

    def run(self, stream=None):
        _check(lib().msgpu_job_run(self.h, stream), "job_run")

    def set_points(self, ks, item_med=None):
        """Replace the items (at most the count the job was created with); the
        media stay resident."""
        kk, nitem, im = _items(self.media, ks, item_med)
        _check(lib().msgpu_job_set_points(self.h, nitem, im.ctypes.data, kk), "job_set_points")
        self.nitem, self._keep, self.item_med = nitem, (kk, im), im

    def use_graph(self, on=True):
        """Replay the run as a captured CUDA graph."""
        _check(lib().msgpu_job_use_graph(self.h, int(on)), "job_use_graph")

    def results(self):
        out = np.zeros(2 * self.nitem)
        st = np.zeros(self.nitem, dtype=np.int32)
        _check(lib().msgpu_job_results(self.h, out, st), "job_results")
        return out.view(np.complex128).copy(), st

    @property
    def flops(self):
        return float(lib().msgpu_job_flops(self.h))

    @property
    def launches(self):
        return int(lib().msgpu_job_launches(self.h))

    def close(self):
        if self.h:
            lib().msgpu_job_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
