"""Output files in the reference's ".dat" format, so that results computed here
can be plotted and re-read by the reference's own tools.

The reference appends INI-like sections to one output file; each writer here
appends the section it names with the same keys, order and number formats:

  [medium]           save_medium           src/core/medium_util.c:420-429
                     (model line: save_scmodel, scattering_model_util.c:174-181)
  [kplane]           save_complexmap       src/core/complex_map_util.c:236-249
                     (color line: save_colorrule, color_rule_util.c:276-282)
  [kcut]             save_complexcut       src/core/complex_cut_util.c:106-117
  [logkcut]          save_logcut           src/core/log_cut_util.c:122-134
  [random_function]  save_random_function  src/core/random_function_util.c:178-193
  [eigenstate_list]  save_eigenstate_list  src/core/eigenstate_list_util.c:296-314
                     (domain: save_domain, domain_util.c:83; states: save_eigenstate,
                     eigenstate_util.c:202-213)
  [muplane]          save_chistogram       src/core/chistogram_util.c:414-440
                     (domain: save_domain; color line: save_colorrule)
  [imag_mu]          save_ihist            src/core/imag_mu_histogram_util.c:195-213
  [wavefunction]     save_wfun             src/core/wave_function_util.c:228-245
                     (k and source: save_iwave, incident_wave_util.c:101;
                     function=/density=: save_real_data, real_vector_util.c:166)
  [wavefunction_cut] save_wfcut            src/core/wave_function_cut_util.c:211-226
  [diff_cross_section] save_diff_cross_section  src/core/diff_cross_section_util.c:259-284
  data= line         save_cdata            src/core/complex_data_util.c:21-28

`parse_cdata` reads a data= line back (parse_complex_data,
src/core/complex_vector_util.c:215-231).  Numbers go through C-style printf
conversions (%g, %.16g, %+.16g), which Python's % operator reproduces except
for the sign glibc writes on a NaN ("-nan", "+nan"), which _gfmt adds.
"""
import math

import numpy as np

__all__ = ["format_cdata", "parse_cdata", "save_medium", "save_complexmap", "save_complexcut",
           "save_random_function", "save_eigenstate_list", "save_muplane", "save_imag_mu", "save_wavefunction",
           "save_wavefunction_cut", "save_diff_cross_section", "save_logcut"]

MODEL_NAMES = ("hardsphere", "softsphere", "resonant", "maximum")
SHAPE_NAMES = ("cube", "ball", "lattice", "gaussian")


def _gfmt(v, prec=16, plus=False):
    """%.<prec>g (or %+.<prec>g) as glibc's printf writes it: Python drops a
    NaN's sign, glibc writes it ("-nan", and "+nan" under the plus flag)."""
    v = float(v)
    if v != v:
        return "-nan" if math.copysign(1.0, v) < 0 else ("+nan" if plus else "nan")
    return ("%+.*g" if plus else "%.*g") % (prec, v)


def _cfmt(z, prec=16):
    """A complex value as "%.<prec>g%+.<prec>gi" (save_cdata, save_eigenstate)."""
    z = complex(z)
    return _gfmt(z.real, prec) + _gfmt(z.imag, prec, True) + "i"


def format_cdata(data):
    """The data= line of save_cdata: every value as "%.16lg%+.16lgi " then a newline."""
    z = np.asarray(data, dtype=np.complex128).reshape(-1)
    return "data=" + "".join(_cfmt(v) + " " for v in z) + "\n"


def parse_cdata(line, n=None):
    """Complex values of a data= line (or of the text after "data=")."""
    text = line.split("=", 1)[1] if line.startswith("data=") else line
    out = []
    for tok in text.split():
        if not tok.endswith("i"):
            raise ValueError(f"data corruption at {tok[:20]!r}")
        body = tok[:-1]
        # the imaginary part starts at the last sign that is not an exponent sign
        cut = max(j for j in range(1, len(body)) if body[j] in "+-" and body[j - 1] not in "eE")
        out.append(complex(float(body[:cut]), float(body[cut:])))
        if n is not None and len(out) == n:
            break
    return np.asarray(out, dtype=np.complex128)


def _g16(v):
    """%.16g as glibc's printf writes it, NaN with its sign ("-nan") included."""
    return _gfmt(v)


def _append(fname, text):
    with open(fname, "a") as f:
        f.write(text)


def save_medium(fname, d, n, model="maximum", params=(), shape="ball", ratio=1.0):
    name = model if isinstance(model, str) else MODEL_NAMES[model]
    shp = shape if isinstance(shape, str) else SHAPE_NAMES[shape]
    line = "model=" + name + "".join(" %.16g" % p for p in params)
    _append(fname, "[medium]\ndimension=%d\nnatom=%d\n%s\nshape=%s\nratio=%g\n\n" % (d, n, line, shp, ratio))


def save_complexmap(fname, data, nx, ny, xrange, yrange, title="", realtime=0.0, nseed=1,
                    color=("magma", "seq", 3.0, False)):
    """A [kplane] section; data in get_arg_cmap order (row-major from the top row)."""
    cname, ctype, ctr, rev = color
    text = ("[kplane]\ntitle=%s\nrealtime=%g\nnseed=%d\nxsample=%d\nysample=%d\nxrange=%g:%g\nyrange=%g:%g\n"
            % (title, realtime, nseed, nx, ny, xrange[0], xrange[1], yrange[0], yrange[1]))
    text += "color=%s %s %g%s\n" % (cname, ctype, ctr, " rev" if rev else "")
    _append(fname, text + format_cdata(data) + "\n")


def save_complexcut(fname, data, ns, kmin, kmax, title="", realtime=0.0, nseed=1):
    """A [kcut] section; data in get_arg_ccut order (3 (ns+2) values)."""
    kmin, kmax = complex(kmin), complex(kmax)
    text = ("[kcut]\ntitle=%s\nrealtime=%g\nnseed=%d\nsample=%d\nkmin=%s\nkmax=%s\n"
            % (title, realtime, nseed, ns, _cfmt(kmin, 12), _cfmt(kmax, 12)))
    _append(fname, text + format_cdata(data) + "\n")


def save_logcut(fname, data, ns, rek, imkmin, imkmax, title="", realtime=0.0, nseed=1):
    """A [logkcut] section; data at logcut_args' points (ns values)."""
    text = ("[logkcut]\ntitle=%s\nrealtime=%g\nnseed=%d\nsample=%d\nrek=%.12g\nimkmin=%.12g\nimkmax=%.12g\n"
            % (title, realtime, nseed, ns, rek, imkmin, imkmax))
    _append(fname, text + format_cdata(data) + "\n")


def save_random_function(fname, kind, data, xmin, xmax, title="", realtime=0.0):
    """A [random_function] section; data[nbin, nseed] (bin-major, as computed)."""
    data = np.asarray(data, dtype=np.float64)
    nbin, nseed = data.shape
    text = ("[random_function]\ntitle=%s\ntype=%s\nnseed=%d\nnbin=%d\nxmin=%.16g\nxmax=%.16g\nrealtime=%.16g\n"
            % (title, kind, nseed, nbin, xmin, xmax, realtime))
    text += "data=" + "".join(_g16(v) + " " for v in data.reshape(-1)) + "\n\n"
    _append(fname, text)


def save_eigenstate_list(fname, states, seed, method, ntarget, dom, maxit, toler, realtime=0.0, verb=0):
    """An [eigenstate_list] section; states = [(kroot, mu, eigenvector)] as
    find_eigenstates(..., eigenvectors=True) returns them for one medium."""
    text = ("[eigenstate_list]\nseed=%d\nmethod=%s\nntarget=%d\nnstate=%d\n"
            % (seed, method, ntarget, len(states)))
    text += "xrange=%.16g:%.16g\nyrange=%.16g:%.16g\n" % (dom[0], dom[1], dom[2], dom[3])
    text += "maxit=%d\ntoler=%g\nverb=%d\nrealtime=%g\n" % (maxit, toler, verb, realtime)
    for i, (k, mu, v) in enumerate(states):
        k, mu = complex(k), complex(mu)
        text += "st%d_kroot=%s\n" % (i, _cfmt(k))
        text += "st%d_mu=%s\n" % (i, _cfmt(mu))
        text += "st%d_eigv=" % i + "".join(_cfmt(z) + " " for z in np.asarray(v)) + "\n"
    _append(fname, text + "\n")


def save_muplane(fname, hist, k, nseed, mtype="msmatrix", title="", color=("magma", "seq", 3.0, False),
                 realtime=0.0):
    """A [muplane] section for the mu-plane histogram hist (the dict chistogram /
    run_chistogram return) of the eigenvalues of M(k) (mtype "msmatrix") or of
    N(k) (mtype "normalized") over nseed realisations.  color = (map name, "seq"
    or "div", contrast, reversed), the reference's default being magma seq 3."""
    k = complex(k)
    xmin, xmax, ymin, ymax = hist["dom"]
    name, ctype, ctr, rev = color
    text = "[muplane]\ntitle=%s\nmtype=%s\nk=%s\nnseed=%d\n" % (title, mtype, _cfmt(k), nseed)
    data = np.asarray(hist["data"]).reshape(-1)
    ybin, xbin = np.asarray(hist["data"]).shape
    text += "xbin=%d\nybin=%d\n" % (xbin, ybin)
    text += "xrange=%.16g:%.16g\nyrange=%.16g:%.16g\n" % (xmin, xmax, ymin, ymax)
    avg, sig = complex(hist["avg"]), complex(hist["sigma"])
    text += "avgz=%s\nsigmaz=%s\n" % (_cfmt(avg), _cfmt(sig))
    text += "realtime=%g\ncolor=%s %s %g%s\n" % (realtime, name, ctype, ctr, " rev" if rev else "")
    text += "data=" + "".join(_g16(v) + " " for v in data) + "\n"
    mdata = np.asarray(hist["mdata"])
    text += "mbin=%d\nmrange=%.16g:%.16g\n" % (mdata.size, hist["mrange"][0], hist["mrange"][1])
    text += "mdata=" + "".join(_g16(v) + " " for v in mdata) + "\n\n"
    _append(fname, text)


def _colorrule(key, color):
    name, ctype, ctr, rev = color
    return "%s=%s %s %g%s\n" % (key, name, ctype, ctr, " rev" if rev else "")


def _real_data(key, values):
    return key + "=" + "".join(_g16(v) + " " for v in np.asarray(values, dtype=np.float64).reshape(-1)) + "\n"


def save_imag_mu(fname, hist, k, nseed, title="", realtime=0.0):
    """An [imag_mu] section for the Im mu histogram hist (the dict imag_mu_task /
    run_imag_mu_histogram return) at real k over nseed realisations."""
    text = "[imag_mu]\ntitle=%s\nk=%g\nnseed=%d\nnbin=%d\n" % (title, k, nseed, len(hist["data"]))
    text += "xmin=%s\nxmax=%s\navgx=%s\n" % (_g16(hist["xmin"]), _g16(hist["xmax"]), _g16(hist["avgx"]))
    text += "varx_true=%s\nvarx_expc=%s\nrealtime=%g\n" % (_g16(hist["varx_true"]), _g16(hist["varx_expc"]),
                                                              realtime)
    text += "data=" + "".join(_g16(v) + " " for v in hist["data"]) + "\n\n"
    _append(fname, text)


def save_wavefunction(fname, function, density, nx, ny, dom, k, nseed, iseed=1, source="plane", realtime=0.0,
                      color1=("magma", "seq", 3.0, False), color2=("magma", "seq", 3.0, False)):
    """A [wavefunction] section: the seed-averaged Re psi (function) and |psi|^2
    (density) on the nx x ny grid over dom = (xmin, xmax, ymin, ymax), row-major
    from the top row (wave_function / wave_function_batch return them so), for
    the incident wave of wave number k ("plane" or "spherical")."""
    k = complex(k)
    text = "[wavefunction]\nnseed=%d\niseed=%d\nnx=%d\nny=%d\n" % (nseed, iseed, nx, ny)
    text += "xrange=%.16g:%.16g\nyrange=%.16g:%.16g\n" % tuple(dom)
    text += "k=%.16g%+.16gi\nsource=%s\nrealtime=%g\n" % (k.real, k.imag, source, realtime)
    text += _colorrule("color1", color1) + _colorrule("color2", color2)
    text += _real_data("function", function) + _real_data("density", density) + "\n"
    _append(fname, text)


def save_wavefunction_cut(fname, stats, nbin, xmin, xmax, k, nseed, iseed=1, source="plane", realtime=0.0):
    """A [wavefunction_cut] section: per bin of the cut the mean, first and third
    quartiles of Re psi, Im psi and |psi|^2 over the seeds (stats as
    run_wave_function_cut returns it: "repsi", "impsi", "density", nbin rows of
    three), for the incident wave of wave number k."""
    k = complex(k)
    text = "[wavefunction_cut]\nnseed=%d\niseed=%d\nnbin=%d\n" % (nseed, iseed, nbin)
    text += "xrange=%.16g:%.16g\n" % (xmin, xmax)
    text += "k=%.16g%+.16gi\nsource=%s\nrealtime=%g\n" % (k.real, k.imag, source, realtime)
    for key in ("repsi", "impsi", "density"):
        text += _real_data(key, np.asarray(stats[key], dtype=np.float64).reshape(-1))
    _append(fname, text + "\n")


def save_diff_cross_section(fname, dcs, k, nseed, iseed, thmin, thmax, title="", realtime=0.0):
    """A [diff_cross_section] section: per bin the nq quantiles (data, rows of
    nq), the mean and the first nc seeds' curves (curve, rows of nc), as
    run_differential_cross_section returns them, at wave number k over the
    angles thmin..thmax degrees."""
    data = np.asarray(dcs["data"], dtype=np.float64)
    curve = np.asarray(dcs["curve"], dtype=np.float64)
    nbin, nq = data.shape
    text = "[diff_cross_section]\ntitle=%s\nnseed=%d\niseed=%d\nk=%g\n" % (title, nseed, iseed, k)
    text += "thmin=%s\nthmax=%s\nnbin=%d\nnq=%d\nrealtime=%s\n" % (_g16(thmin), _g16(thmax), nbin, nq,
                                                                     _g16(realtime))
    text += "data=" + "".join(_g16(v) + " " for v in data.reshape(-1))
    text += "\nmean=" + "".join(_g16(v) + " " for v in np.asarray(dcs["mean"], dtype=np.float64))
    text += "\nnc=%d\ncurve=" % curve.shape[1] + "".join(_g16(v) + " " for v in curve.reshape(-1)) + "\n\n"
    _append(fname, text)
