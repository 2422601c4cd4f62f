"""CPU oracle for the Foldy-Lax hot path (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` import this package, and only as
the reference results to compare with or the timed CPU baseline.  The product (``msmodel_gb300``)
never imports it.

``Oracle`` wraps ``liboracle.so`` (the C restatement, ``msoracle.c``);
``Reference`` wraps ``_ref/libmsref.so`` (the reference sources compiled
unmodified) when that was built.  Complex scalars are passed as two doubles.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle as _bo

HERE = os.path.dirname(os.path.abspath(__file__))

MODELS = {"hardsphere": 0, "softsphere": 1, "resonant": 2, "maximum": 3}
SHAPES = {"cube": 0, "ball": 1, "lattice": 2, "gaussian": 3}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class _Model(C.Structure):
    _fields_ = [("type", C.c_int), ("np", C.c_int), ("p", C.c_double * 2)]


def model_struct(model="maximum", params=()):
    m = _Model()
    m.type = MODELS[model] if isinstance(model, str) else int(model)
    m.np = len(params)
    for i, v in enumerate(params):
        m.p[i] = v
    return m


def _c2(z):
    z = complex(z)
    return np.array([z.real, z.imag], dtype=np.float64)


def _cplx_array(zs):
    zs = np.ascontiguousarray(np.asarray(zs, dtype=np.complex128))
    return zs.view(np.float64).reshape(-1).copy()


class Oracle:
    """ctypes view of liboracle.so."""

    def __init__(self, lapack=True):
        path = _bo.build_oracle()
        L = C.CDLL(path)
        self.L = L
        L.orc_set_lapack.argtypes = [C.c_char_p]
        L.orc_lapack_config.restype = C.c_char_p
        L.orc_fill_medium.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint64, _dp]
        L.orc_rng_init.argtypes = [np.ctypeslib.ndpointer(dtype=np.uint64), C.c_uint64]
        L.orc_rng_double.argtypes = [np.ctypeslib.ndpointer(dtype=np.uint64)]
        L.orc_rng_double.restype = C.c_double
        for f in ("orc_free_green", "orc_dk_free_green", "orc_free_green_imag"):
            getattr(L, f).argtypes = [C.c_int, _dp, C.c_double, _dp]
        L.orc_bessel_k.argtypes = [C.c_int, _dp, _dp]
        L.orc_hyp0f1.argtypes = [C.c_double, _dp, _dp]
        L.orc_invf.argtypes = [C.POINTER(_Model), C.c_int, _dp, _dp]
        L.orc_build_ms_matrix.argtypes = [C.c_int, C.c_int, _dp, C.POINTER(_Model), _dp, _dp]
        L.orc_build_dk_ms_matrix.argtypes = [C.c_int, C.c_int, _dp, C.POINTER(_Model), _dp, _dp]
        L.orc_lu.argtypes = [C.c_int, _dp, _ip, C.c_int]
        L.orc_tracelog_lu.argtypes = [C.c_int, _dp, C.c_int, _dp]
        L.orc_dk_log_det.argtypes = [C.c_int, C.c_int, _dp, C.POINTER(_Model), _dp, C.c_int, _dp]
        L.orc_total_cross_section.argtypes = [C.c_int, C.c_int, _dp, C.POINTER(_Model), C.c_double, C.c_int]
        L.orc_total_cross_section.restype = C.c_double
        L.orc_solve.argtypes = [C.c_int, _dp, _dp, C.c_int]
        L.orc_tracelog_batch.argtypes = [C.c_int, C.c_int, _dp, C.POINTER(_Model), C.c_int, _dp, _dp, _ip,
                                         C.c_int, C.c_int]
        L.orc_dlogf_batch.argtypes = [C.c_int, C.c_int, _dp, C.POINTER(_Model), C.c_int, _dp, _dp, C.c_int,
                                      C.c_int]
        L.orc_kplane_args.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _dp]
        L.orc_kcut_args.argtypes = [C.c_int, _dp, _dp, _dp]
        L.orc_halton_points.argtypes = [_dp, C.c_int, _dp]
        L.orc_solve_aberth.argtypes = [C.c_int, C.c_int, _dp, C.POINTER(_Model), _dp, C.c_int, _dp, C.c_int,
                                       C.c_int, C.c_double, C.c_int, C.POINTER(C.c_int)]
        L.orc_psi_grid.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int]
        L.orc_psi_grid.restype = None
        L.orc_wavefunction.argtypes = [C.c_int, C.c_int, _dp, C.POINTER(_Model), _dp, C.c_int, C.c_int, _dp, _dp,
                                       _dp, C.c_int, C.c_int]
        self.use_lapack = 0
        if lapack:
            ob = _bo.openblas_path()
            if ob is not None and L.orc_set_lapack(ob.encode()) == 0:
                self.use_lapack = 1

    def lapack_config(self):
        return self.L.orc_lapack_config().decode()

    # --- medium -----------------------------------------------------------
    def fill_medium(self, d, n, seed, shape="ball", ratio=1.0):
        pos = np.zeros(n * d)
        self.L.orc_fill_medium(d, n, SHAPES[shape] if isinstance(shape, str) else shape, ratio, seed, pos)
        return pos

    # --- scalar special functions ----------------------------------------
    def _c(self, fn, *args):
        out = np.zeros(2)
        fn(*args, out)
        return complex(out[0], out[1])

    def free_green(self, d, k, r=1.0):
        return self._c(self.L.orc_free_green, d, _c2(k), r)

    def dk_free_green(self, d, k, r=1.0):
        return self._c(self.L.orc_dk_free_green, d, _c2(k), r)

    def free_green_imag(self, d, k, r=1.0):
        return self._c(self.L.orc_free_green_imag, d, _c2(k), r)

    def bessel_k(self, twonu, z):
        return self._c(self.L.orc_bessel_k, twonu, _c2(z))

    def hyp0f1(self, a, z):
        return self._c(self.L.orc_hyp0f1, a, _c2(z))

    def invf(self, d, k, model="maximum", params=()):
        m = model_struct(model, params)
        return self._c(self.L.orc_invf, C.byref(m), d, _c2(k))

    # --- matrices ------------------------------------------------------------
    def ms_matrix(self, d, n, pos, k, model="maximum", params=(), deriv=False):
        m = model_struct(model, params)
        out = np.zeros(2 * n * n)
        fn = self.L.orc_build_dk_ms_matrix if deriv else self.L.orc_build_ms_matrix
        fn(d, n, np.ascontiguousarray(pos, dtype=np.float64), C.byref(m), _c2(k), out)
        return out.view(np.complex128).reshape(n, n).T  # column-major -> [row, col]

    def lu(self, a, lapack=None):
        """LU of the square complex matrix a ([row, col]); returns (lu, ipiv, info)."""
        n = a.shape[0]
        buf = np.ascontiguousarray(np.asarray(a, dtype=np.complex128).T).view(np.float64).reshape(-1).copy()
        ipiv = np.zeros(n, dtype=np.int32)
        info = self.L.orc_lu(n, buf, ipiv, self.use_lapack if lapack is None else int(lapack))
        return buf.view(np.complex128).reshape(n, n).T, ipiv, info

    def tracelog_lu(self, a, lapack=None):
        n = a.shape[0]
        buf = np.ascontiguousarray(np.asarray(a, dtype=np.complex128).T).view(np.float64).reshape(-1).copy()
        out = np.zeros(2)
        self.L.orc_tracelog_lu(n, buf, self.use_lapack if lapack is None else int(lapack), out)
        return complex(out[0], out[1])

    def dk_log_det(self, d, n, pos, k, model="maximum", params=(), lapack=None):
        m = model_struct(model, params)
        out = np.zeros(2)
        self.L.orc_dk_log_det(d, n, np.ascontiguousarray(pos, dtype=np.float64), C.byref(m), _c2(k),
                              self.use_lapack if lapack is None else int(lapack), out)
        return complex(out[0], out[1])

    def total_cross_section(self, d, n, pos, k, model="maximum", params=()):
        m = model_struct(model, params)
        return self.L.orc_total_cross_section(d, n, np.ascontiguousarray(pos, dtype=np.float64), C.byref(m),
                                              float(k), self.use_lapack)

    def tracelog_batch(self, d, n, pos, ks, model="maximum", params=(), nthreads=None, lapack=None):
        m = model_struct(model, params)
        kk = _cplx_array(ks)
        nk = kk.size // 2
        out = np.zeros(2 * nk)
        info = np.zeros(nk, dtype=np.int32)
        self.L.orc_tracelog_batch(d, n, np.ascontiguousarray(pos, dtype=np.float64), C.byref(m), nk, kk, out, info,
                                  nthreads or os.cpu_count(), self.use_lapack if lapack is None else int(lapack))
        return out.view(np.complex128).copy(), info

    def dlogf_batch(self, d, n, pos, ks, model="maximum", params=(), nthreads=None, lapack=None):
        m = model_struct(model, params)
        kk = _cplx_array(ks)
        nk = kk.size // 2
        out = np.zeros(2 * nk)
        self.L.orc_dlogf_batch(d, n, np.ascontiguousarray(pos, dtype=np.float64), C.byref(m), nk, kk, out,
                               nthreads or os.cpu_count(), self.use_lapack if lapack is None else int(lapack))
        return out.view(np.complex128).copy()

    # --- grids ---------------------------------------------------------------
    def kplane_args(self, nx, ny, xmin, xmax, ymin, ymax):
        out = np.zeros(2 * nx * ny)
        self.L.orc_kplane_args(nx, ny, xmin, xmax, ymin, ymax, out)
        return out.view(np.complex128).copy()

    def kcut_args(self, ns, zmin, zmax):
        out = np.zeros(2 * 3 * (ns + 2))
        self.L.orc_kcut_args(ns, _c2(zmin), _c2(zmax), out)
        return out.view(np.complex128).copy()

    def halton_points(self, dom, n):
        out = np.zeros(2 * n)
        self.L.orc_halton_points(np.asarray(dom, dtype=np.float64), n, out)
        return out.view(np.complex128).copy()

    # --- root finder / wavefunction -----------------------------------------
    def solve_aberth(self, d, n, pos, dom, z0, model="maximum", params=(), nexpsup=4, maxit=30, toler=1e-10,
                     lapack=None):
        m = model_struct(model, params)
        z = _cplx_array(z0)
        ne = C.c_int(0)
        nr = self.L.orc_solve_aberth(d, n, np.ascontiguousarray(pos, dtype=np.float64), C.byref(m),
                                     np.asarray(dom, dtype=np.float64), z.size // 2, z, nexpsup, maxit, toler,
                                     self.use_lapack if lapack is None else int(lapack), C.byref(ne))
        return z.view(np.complex128)[:nr].copy(), ne.value

    def wavefunction(self, d, n, pos, k, nx, ny, dom, model="maximum", params=(), nthreads=None):
        m = model_struct(model, params)
        amp = np.zeros(2 * n)
        psi = np.zeros(2 * nx * ny)
        self.L.orc_wavefunction(d, n, np.ascontiguousarray(pos, dtype=np.float64), C.byref(m), _c2(k), nx, ny,
                                np.asarray(dom, dtype=np.float64), amp, psi, nthreads or os.cpu_count(),
                                self.use_lapack)
        return amp.view(np.complex128).copy(), psi.view(np.complex128).copy()


    def psi_grid(self, d, n, pos, k, nx, ny, dom, amp, nthreads=None):
        """psi on the nx x ny grid of dom for given amplitudes amp (the grid part of
        wavefunction, without the solve)."""
        psi = np.zeros(2 * nx * ny)
        a = np.ascontiguousarray(np.asarray(amp, dtype=np.complex128)).view(np.float64)
        self.L.orc_psi_grid(d, n, np.ascontiguousarray(pos, dtype=np.float64), _c2(k), nx, ny,
                            np.asarray(dom, dtype=np.float64), a, psi, nthreads or os.cpu_count())
        return psi.view(np.complex128).copy()


class Reference:
    """ctypes view of oracle/_ref/libmsref.so (reference sources, unmodified)."""

    def __init__(self):
        path = _bo.build_ref()
        if path is None:
            raise FileNotFoundError("reference sources not present; oracle/_ref not built")
        L = C.CDLL(path)
        self.L = L
        med = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.c_int, C.c_double, C.c_ulong]
        L.ref_fill.argtypes = med + [_dp]
        L.ref_green.argtypes = [C.c_int, _dp, C.c_double, _dp]
        L.ref_dk_green.argtypes = [C.c_int, _dp, C.c_double, _dp]
        L.ref_bessel_k.argtypes = [C.c_int, _dp, _dp]
        L.ref_tracelog.argtypes = med + [C.c_int, _dp, _dp]
        L.ref_matrix.argtypes = med + [_dp, C.c_int, _dp]
        L.ref_dlogf.argtypes = med + [C.c_int, _dp, _dp]
        L.ref_total_cross_section.argtypes = med + [C.c_double]
        L.ref_total_cross_section.restype = C.c_double
        L.ref_aberth.argtypes = med + [_dp, C.c_int, _dp, C.c_int, C.c_int, C.c_double]
        L.ref_wavefunction.argtypes = med + [_dp, C.c_int, C.c_int, _dp, _dp, _dp]
        L.ref_save_cdata.argtypes = [C.c_int, _dp, C.c_char_p]
        L.ref_parse_cdata.argtypes = [C.c_int, C.c_char_p, _dp]
        L.ref_traceinv.argtypes = med + [C.c_int, _dp, _dp]
        L.ref_eigvals.argtypes = med + [_dp, _dp]
        L.ref_chistogram.argtypes = [C.c_int, _dp, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]
        L.ref_eigvals_normalized.argtypes = med + [_dp, _dp]
        L.ref_logcut.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_char_p, C.c_double,
                                 _dp, _dp, C.c_char_p]
        L.ref_save_wfun.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_ulong, C.c_double,
                                    C.c_char_p, C.c_char_p, _dp, _dp, C.c_char_p]
        L.ref_imag_mu.argtypes = med[:-1] + [C.c_double, C.c_int, C.c_int, C.c_char_p, C.c_double, C.c_char_p,
                                             _dp, _dp]
        L.ref_save_chistogram.argtypes = [C.c_int, _dp, C.c_int, _dp, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.c_char_p, C.c_char_p, C.c_double, C.c_char_p]
        L.ref_inverse_iteration.argtypes = med + [_dp, _dp, _dp]
        L.ref_roots_muller.argtypes = [C.c_int] + med + [_dp, C.c_int, _dp, C.c_int, C.c_double]
        L.ref_save_wfcut.argtypes = [C.c_int, C.c_double, C.c_double, _dp, C.c_int, C.c_int, C.c_ulong, C.c_double,
                                     _dp, _dp, _dp, C.c_char_p]
        L.ref_diff_cross_section.argtypes = med[:-1] + [C.c_double, C.c_int, C.c_ulong, C.c_int, C.c_double,
                                                        C.c_double, C.c_int, C.c_int, C.c_char_p, C.c_double,
                                                        C.c_char_p, _dp, _dp, _dp, _dp]
        L.ref_save_medium.argtypes = med[:-1] + [C.c_char_p]
        L.ref_save_kcut.argtypes = [C.c_int, _dp, _dp, C.c_int, C.c_char_p, C.c_double, _dp, C.c_char_p]
        L.ref_save_kplane.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                      C.c_char_p, C.c_double, C.c_char_p, _dp, C.c_char_p]
        L.ref_save_rfun.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_char_p, C.c_double, _dp,
                                    C.c_char_p]
        L.ref_save_eigls.argtypes = [C.c_int, C.c_int, C.c_ulong, C.c_int, C.c_int, _dp, C.c_int, C.c_double, C.c_int,
                                     C.c_double, C.c_int, _dp, _dp, _dp, C.c_char_p]
        L.ref_wfcut_stats.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp]
        L.ref_random_function.argtypes = [C.c_int] + med[:-1] + [C.c_int, C.c_int, C.c_double, C.c_double, _dp]

    @staticmethod
    def _med(d, n, model, params, shape, ratio, seed):
        p = np.zeros(2)
        p[:len(params)] = params
        return [d, n, MODELS[model], len(params), p, SHAPES[shape], ratio, seed]

    def fill_medium(self, d, n, seed, model="maximum", params=(), shape="ball", ratio=1.0):
        pos = np.zeros(n * d)
        self.L.ref_fill(*self._med(d, n, model, params, shape, ratio, seed), pos)
        return pos

    def free_green(self, d, k, r=1.0):
        out = np.zeros(2)
        self.L.ref_green(d, _c2(k), r, out)
        return complex(*out)

    def dk_free_green(self, d, k, r=1.0):
        out = np.zeros(2)
        self.L.ref_dk_green(d, _c2(k), r, out)
        return complex(*out)

    def bessel_k(self, twonu, z):
        out = np.zeros(2)
        self.L.ref_bessel_k(twonu, _c2(z), out)
        return complex(*out)

    def tracelog(self, d, n, seed, ks, model="maximum", params=(), shape="ball", ratio=1.0):
        kk = _cplx_array(ks)
        out = np.zeros_like(kk)
        self.L.ref_tracelog(*self._med(d, n, model, params, shape, ratio, seed), kk.size // 2, kk, out)
        return out.view(np.complex128).copy()

    def ms_matrix(self, d, n, seed, k, model="maximum", params=(), deriv=False, shape="ball", ratio=1.0):
        out = np.zeros(2 * n * n)
        self.L.ref_matrix(*self._med(d, n, model, params, shape, ratio, seed), _c2(k), int(deriv), out)
        return out.view(np.complex128).reshape(n, n).T

    def dlogf(self, d, n, seed, ks, model="maximum", params=(), shape="ball", ratio=1.0):
        kk = _cplx_array(ks)
        out = np.zeros_like(kk)
        self.L.ref_dlogf(*self._med(d, n, model, params, shape, ratio, seed), kk.size // 2, kk, out)
        return out.view(np.complex128).copy()

    def total_cross_section(self, d, n, seed, k, model="maximum", params=(), shape="ball", ratio=1.0):
        return self.L.ref_total_cross_section(*self._med(d, n, model, params, shape, ratio, seed), float(k))

    def eigvals(self, d, n, seed, k, model="maximum", params=(), shape="ball", ratio=1.0):
        mu = np.zeros(2 * n)
        self.L.ref_eigvals(*self._med(d, n, model, params, shape, ratio, seed), np.array([k.real, k.imag]), mu)
        return mu.view(np.complex128).copy()

    def eigvals_normalized(self, d, n, seed, k, model="maximum", params=(), shape="ball", ratio=1.0):
        """eigvals of the normalized MS matrix N(k) = i - G(k)/I(k,0) (build_normalized_matrix)."""
        mu = np.zeros(2 * n)
        self.L.ref_eigvals_normalized(*self._med(d, n, model, params, shape, ratio, seed),
                                      np.array([k.real, k.imag]), mu)
        return mu.view(np.complex128).copy()

    def save_chistogram(self, mu, normalized, k, nseed, xbin, ybin, mbin, title, color, realtime):
        """The text of the [muplane] section save_chistogram writes for the histogram of mu
        (fill_chist) with this metadata and colour rule argument."""
        import tempfile
        z = _cplx_array(mu)
        with tempfile.TemporaryDirectory() as tmp:
            fname = os.path.join(tmp, "muplane.dat")
            self.L.ref_save_chistogram(len(z) // 2, z, int(normalized), np.array([k.real, k.imag]), nseed, xbin,
                                       ybin, mbin, title.encode(), color.encode(), realtime, fname.encode())
            with open(fname) as f:
                return f.read()

    def save_wfun(self, nx, ny, dom, k, nseed, iseed, realtime, color1, color2, fun, den, spherical=False):
        """The text of the [wavefunction] section save_wfun writes for these values."""
        import tempfile
        with tempfile.TemporaryDirectory() as tmp:
            fname = os.path.join(tmp, "wfun.dat")
            self.L.ref_save_wfun(nx, ny, np.asarray(dom, dtype=np.float64), np.array([k.real, k.imag]),
                                 int(spherical), nseed, iseed, realtime, color1.encode(), color2.encode(),
                                 np.ascontiguousarray(fun, dtype=np.float64),
                                 np.ascontiguousarray(den, dtype=np.float64), fname.encode())
            with open(fname) as f:
                return f.read()

    def imag_mu(self, d, n, k, nseed, nbin, title="", realtime=0.0, model="maximum", params=(), shape="ball",
                ratio=1.0):
        """run_imag_mu_histogram_omp on one thread and save_ihist: (text of the [imag_mu]
        section, data[nbin], info dict)."""
        import tempfile
        data, info = np.zeros(nbin), np.zeros(6)
        with tempfile.TemporaryDirectory() as tmp:
            fname = os.path.join(tmp, "imag_mu.dat")
            self.L.ref_imag_mu(*self._med(d, n, model, params, shape, ratio, 1)[:-1], float(k), nseed, nbin,
                               title.encode(), realtime, fname.encode(), data, info)
            with open(fname) as f:
                text = f.read()
        keys = ["xmin", "xmax", "avgx", "varx_true", "varx_expc", "lost"]
        return text, data, dict(zip(keys, info.tolist()))

    def logcut(self, ns, rek, imkmin, imkmax, data=None, nseed=1, title="", realtime=0.0):
        """init_logcut's mesh (k[ns]) and, with data, the text of the [logkcut] section
        save_logcut writes: (k, text or None)."""
        import tempfile
        k = np.zeros(2 * ns)
        d = np.zeros(2 * ns) if data is None else _cplx_array(data)
        with tempfile.TemporaryDirectory() as tmp:
            fname = os.path.join(tmp, "logcut.dat")
            self.L.ref_logcut(ns, rek, imkmin, imkmax, nseed, title.encode(), realtime, d, k,
                              fname.encode() if data is not None else None)
            text = open(fname).read() if data is not None else None
        return k.view(np.complex128).copy(), text

    def chistogram(self, mu, xbin, ybin, mbin):
        """fill_chist of the complex values mu into a fresh xbin x ybin histogram with an
        mbin marginal: (data[ybin, xbin], mdata[mbin], info dict)."""
        z = _cplx_array(mu)
        data, mdata, info = np.zeros(xbin * ybin), np.zeros(mbin), np.zeros(11)
        self.L.ref_chistogram(len(z) // 2, z, xbin, ybin, mbin, data, mdata, info)
        keys = ["xmin", "xmax", "ymin", "ymax", "mmin", "mmax", "avg_re", "avg_im", "sigma_re", "sigma_im", "lost"]
        return data.reshape(ybin, xbin), mdata, dict(zip(keys, info.tolist()))

    def traceinv(self, d, n, seed, ks, model="maximum", params=(), shape="ball", ratio=1.0):
        kk = _cplx_array(ks)
        out = np.zeros_like(kk)
        self.L.ref_traceinv(*self._med(d, n, model, params, shape, ratio, seed), kk.size // 2, kk, out)
        return out.view(np.complex128).copy()

    def inverse_iteration(self, d, n, seed, k, model="maximum", params=(), shape="ball", ratio=1.0):
        lam = np.zeros(2)
        vec = np.zeros(2 * n)
        conv = self.L.ref_inverse_iteration(*self._med(d, n, model, params, shape, ratio, seed),
                                            np.array([k.real, k.imag]), lam, vec)
        return complex(lam[0], lam[1]), vec.view(np.complex128).copy(), conv

    def roots_muller(self, method, d, n, seed, dom, z0, maxit=30, toler=1e-10, model="maximum", params=(),
                     shape="ball", ratio=1.0):
        z = _cplx_array(z0)
        nr = self.L.ref_roots_muller({"mineigval": 1, "invtraceinv": 2}[method],
                                     *self._med(d, n, model, params, shape, ratio, seed),
                                     np.asarray(dom, dtype=float), z.size // 2, z, maxit, toler)
        return z.view(np.complex128)[:nr].copy()

    def save_wfcut(self, nbin, xmin, xmax, k, nseed, iseed, realtime, re, im, den, spherical=False):
        """The text of the [wavefunction_cut] section save_wfcut writes for these statistics."""
        import tempfile
        with tempfile.TemporaryDirectory() as tmp:
            fname = os.path.join(tmp, "wfcut.dat")
            arr = [np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1)) for v in (re, im, den)]
            self.L.ref_save_wfcut(nbin, xmin, xmax, np.array([k.real, k.imag]), int(spherical), nseed, iseed,
                                  realtime, *arr, fname.encode())
            with open(fname) as f:
                return f.read()

    def diff_cross_section(self, d, n, k, nseed, iseed, nbin, thmin, thmax, nq, nc, title="", realtime=0.0,
                           model="maximum", params=(), shape="ball", ratio=1.0):
        """run_differential_cross_section_omp's arithmetic on one thread with the
        reference's functions: (samples[nbin, nseed], data[nbin, nq], mean[nbin],
        curve[nbin, nc], the [diff_cross_section] section text)."""
        import tempfile
        smp, data, mean, curve = np.zeros(nseed * nbin), np.zeros(nbin * nq), np.zeros(nbin), np.zeros(nbin * nc)
        with tempfile.TemporaryDirectory() as tmp:
            fname = os.path.join(tmp, "dcs.dat")
            self.L.ref_diff_cross_section(*self._med(d, n, model, params, shape, ratio, 1)[:-1], float(k), nseed,
                                          iseed, nbin, thmin, thmax, nq, nc, title.encode(), realtime,
                                          fname.encode(), smp, data, mean, curve)
            with open(fname) as f:
                text = f.read()
        return smp.reshape(nbin, nseed), data.reshape(nbin, nq), mean, curve.reshape(nbin, nc), text

    @staticmethod
    def _section(call):
        """The text a reference writer appends to a fresh file."""
        import tempfile
        with tempfile.TemporaryDirectory() as tmp:
            fname = os.path.join(tmp, "section.dat")
            call(fname.encode())
            with open(fname) as f:
                return f.read()

    def save_medium(self, d, n, model="maximum", params=(), shape="ball", ratio=1.0):
        return self._section(lambda f: self.L.ref_save_medium(*self._med(d, n, model, params, shape, ratio, 1)[:-1],
                                                              f))

    def save_kcut(self, ns, zmin, zmax, nseed, title, realtime, data):
        z = _cplx_array(data)
        return self._section(lambda f: self.L.ref_save_kcut(ns, _c2(zmin), _c2(zmax), nseed, title.encode(),
                                                            realtime, z, f))

    def save_kplane(self, nx, ny, xmin, xmax, ymin, ymax, nseed, title, realtime, color, data):
        z = _cplx_array(data)
        return self._section(lambda f: self.L.ref_save_kplane(nx, ny, xmin, xmax, ymin, ymax, nseed, title.encode(),
                                                              realtime, color.encode(), z, f))

    def save_rfun(self, kind, nseed, nbin, xmin, xmax, title, realtime, data):
        v = np.ascontiguousarray(np.asarray(data, dtype=np.float64).reshape(-1))
        return self._section(lambda f: self.L.ref_save_rfun({"crsec": 0, "dos": 1}[kind], nseed, nbin, xmin, xmax,
                                                            title.encode(), realtime, v, f))

    def save_eigls(self, d, n, seed, method, ntarget, dom, maxit, toler, verb, realtime, kroot, mu, eigv):
        kr, m, ev = _cplx_array(kroot), _cplx_array(mu), _cplx_array(np.asarray(eigv).reshape(-1))
        meth = {"determinant": 0, "mineigval": 1, "invtraceinv": 2}[method]
        return self._section(lambda f: self.L.ref_save_eigls(d, n, seed, meth, ntarget,
                                                             np.asarray(dom, dtype=np.float64), maxit, toler, verb,
                                                             realtime, len(kr) // 2, kr, m, ev, f))

    def wfcut_stats(self, psi):
        """store_data_wfcut on psi[nseed, nbin]: (repsi, impsi, density) rows
        [mean, q1/4, q3/4] per bin, the reference's own arithmetic."""
        psi = np.asarray(psi, dtype=np.complex128)
        ns, nb = psi.shape
        cols = [np.ascontiguousarray(v.T.reshape(-1)) for v in (psi.real, psi.imag, psi.real ** 2 + psi.imag ** 2)]
        outs = [np.zeros(3 * nb) for _ in range(3)]
        self.L.ref_wfcut_stats(ns, nb, *cols, *outs)
        return tuple(o.reshape(nb, 3) for o in outs)

    def save_cdata(self, values, fname):
        z = np.ascontiguousarray(np.asarray(values, dtype=np.complex128))
        assert self.L.ref_save_cdata(z.size, z.view(np.float64), fname.encode()) == 0

    def parse_cdata(self, text, n):
        out = np.zeros(2 * n)
        self.L.ref_parse_cdata(n, text.encode(), out)
        return out.view(np.complex128)

    def random_function(self, kind, d, n, nseed, nbin, xmin, xmax, model="maximum", params=(), shape="ball",
                        ratio=1.0):
        data = np.zeros(nseed * nbin)
        args = self._med(d, n, model, params, shape, ratio, 1)[:-1]
        self.L.ref_random_function({"crsec": 0, "dos": 1}[kind], *args, nseed, nbin, xmin, xmax, data)
        return data.reshape(nbin, nseed)

    def solve_aberth(self, d, n, seed, dom, z0, model="maximum", params=(), nexpsup=4, maxit=30, toler=1e-10,
                     shape="ball", ratio=1.0):
        z = _cplx_array(z0)
        nr = self.L.ref_aberth(*self._med(d, n, model, params, shape, ratio, seed), np.asarray(dom, dtype=float),
                               z.size // 2, z, nexpsup, maxit, toler)
        return z.view(np.complex128)[:nr].copy()

    def wavefunction(self, d, n, seed, k, nx, ny, dom, model="maximum", params=(), shape="ball", ratio=1.0):
        amp = np.zeros(2 * n)
        psi = np.zeros(2 * nx * ny)
        self.L.ref_wavefunction(*self._med(d, n, model, params, shape, ratio, seed), _c2(k), nx, ny,
                                np.asarray(dom, dtype=float), amp, psi)
        return amp.view(np.complex128).copy(), psi.view(np.complex128).copy()
