"""The .dat writers and reader against the reference's own save_cdata and
parse_cdata (compiled from its sources): byte-identical data= lines, values
read back bit for bit; the section layouts as the reference's save_* write them."""
import os

import numpy as np
import pytest

from msmodel_gb300 import datio


@pytest.fixture(scope="module")
def ref():
    from oracle import Reference
    try:
        return Reference()
    except OSError:
        pytest.skip("reference build absent")


def _values():
    rng = np.random.default_rng(4)
    v = rng.standard_normal(40) * 10.0 ** rng.integers(-12, 12, 40) + 1j * rng.standard_normal(40)
    return np.concatenate([v, [0.0, -0.0 + 1j, 1e300 - 1e-300j, -2.5e-7 + 3j, 123456789.125 - 0j]])


def test_cdata_line_is_byte_identical(ref, tmp_path):
    z = _values()
    fname = str(tmp_path / "ref.dat")
    ref.save_cdata(z, fname)
    assert open(fname).read() == datio.format_cdata(z)


def test_cdata_reads_back(ref):
    z = _values()
    line = datio.format_cdata(z)
    mine = datio.parse_cdata(line)
    theirs = ref.parse_cdata(line[len("data="):], z.size)
    assert np.array_equal(mine, theirs)
    # %.16g keeps 16 significant digits (an exact round trip needs 17)
    assert np.all(np.abs(mine.real - z.real) <= 1e-15 * np.abs(z.real))
    assert np.all(np.abs(mine.imag - z.imag) <= 1e-15 * np.abs(z.imag))


def test_sections(tmp_path):
    f = str(tmp_path / "out.dat")
    datio.save_medium(f, 3, 1024, "maximum", (), "ball", 1.0)
    datio.save_complexcut(f, [1 + 2j, 3 - 4j, 0.5 + 0j], 1, 0.5 - 0.05j, 3 - 0.05j, title="Trace-log", realtime=1.5)
    datio.save_random_function(f, "dos", [[1.0, 2.0], [3.0, 4.5]], 0.4, 3.5, title="DOS", realtime=2.0)
    datio.save_complexmap(f, [1j, 2, 3, 4], 2, 2, (0.5, 3), (-0.5, 0), title="Map")
    text = open(f).read()
    assert text.startswith("[medium]\ndimension=3\nnatom=1024\nmodel=maximum\nshape=ball\nratio=1\n\n[kcut]\n")
    assert "kmin=0.5-0.05i\nkmax=3-0.05i\ndata=1+2i 3-4i 0.5+0i \n\n" in text
    assert "[random_function]\ntitle=DOS\ntype=dos\nnseed=2\nnbin=2\nxmin=0.4\nxmax=3.5\nrealtime=2\n" \
           "data=1 2 3 4.5 \n\n" in text
    assert "xrange=0.5:3\nyrange=-0.5:0\ncolor=magma seq 3\ndata=0+1i 2+0i 3+0i 4+0i \n\n" in text


def test_eigenstate_list_section(tmp_path):
    f = str(tmp_path / "eig.dat")
    states = [(1.5 - 0.02j, 1e-12 + 2e-13j, np.array([0.6 + 0j, 0.8j])), (2.25 - 0.5j, complex(0.0, -3e-11), np.array([1, 0]))]
    datio.save_eigenstate_list(f, states, 7, "determinant", 32, (0.5, 3, -1, 0), 30, 1e-10)
    text = open(f).read()
    assert text.startswith("[eigenstate_list]\nseed=7\nmethod=determinant\nntarget=32\nnstate=2\n"
                           "xrange=0.5:3\nyrange=-1:0\nmaxit=30\ntoler=1e-10\nverb=0\nrealtime=0\n")
    assert "st0_kroot=1.5-0.02i\nst0_mu=1e-12+2e-13i\nst0_eigv=0.6+0i 0+0.8i \n" in text
    assert "st1_kroot=2.25-0.5i\nst1_mu=0-3e-11i\nst1_eigv=1+0i 0+0i \n\n" in text
    assert datio.parse_cdata("data=" + text.split("st0_eigv=")[1].split("\n")[0]).tolist() == [0.6, 0.8j]


def test_logcut_mesh_and_section_match_reference(ref_runs, tmp_path):
    """The log cut: init_logcut's mesh bit for bit (logcut_args, the C library's
    log and exp) and the [logkcut] section byte for byte what save_logcut wrote
    for the reference's own ln det values there."""
    import msmodel_gb300 as ms
    from helpers import cplx
    c = [c for c in ref_runs["cases"] if c["kind"] == "logcut"][0]
    k = ms.logcut_args(c["ns"], c["rek"], c["imkmin"], c["imkmax"])
    assert np.array_equal(k, cplx(c["k"]))
    f = tmp_path / "logcut.dat"
    datio.save_logcut(str(f), cplx(c["values"]), c["ns"], c["rek"], c["imkmin"], c["imkmax"], c["title"],
                      c["realtime"])
    assert f.read_text() == c["text"]
    with pytest.raises(ValueError):
        ms.logcut_args(10, 2.5, 1e-6, -0.4)


def test_sections_match_reference_writers(ref_runs, tmp_path):
    """[medium], [kcut], [kplane], [random_function] and [eigenstate_list] byte for
    byte as the reference's own writers append them (tests/golden, kind
    dat_sections), signed zeros, signed NaNs, infinities and extreme exponents
    included."""
    c = [c for c in ref_runs["cases"] if c["kind"] == "dat_sections"][0]

    def bits_c(b):  # the fixture keeps the values' IEEE bit patterns
        return np.array(b, dtype=np.uint64).view(np.complex128)

    def written(fn):
        f = tmp_path / "s.dat"
        if f.exists():
            f.unlink()
        fn(str(f))
        return f.read_text()

    for m in c["medium"]:
        assert written(lambda f: datio.save_medium(f, m["d"], m["n"], m["model"], m["params"], m["shape"],
                                                   m["ratio"])) == m["text"]
    k = c["kcut"]
    assert written(lambda f: datio.save_complexcut(f, bits_c(k["data"]), k["ns"], complex(*k["zmin"]),
                                                   complex(*k["zmax"]), k["title"], k["realtime"],
                                                   k["nseed"])) == k["text"]
    p = c["kplane"]
    col = p["color"].split()
    assert written(lambda f: datio.save_complexmap(f, bits_c(p["data"]), p["nx"], p["ny"], p["xrange"], p["yrange"],
                                                   p["title"], p["realtime"], p["nseed"],
                                                   (col[0], col[1], float(col[2]), len(col) > 3))) == p["text"]
    r = c["random_function"]
    data = np.array(r["data"], dtype=np.uint64).view(np.float64).reshape(r["nbin"], r["nseed"])
    assert written(lambda f: datio.save_random_function(f, r["kind"], data, r["xmin"], r["xmax"], r["title"],
                                                        r["realtime"])) == r["text"]
    e = c["eigenstate_list"]
    states = list(zip(bits_c(e["kroot"]), bits_c(e["mu"]), [bits_c(v) for v in e["eigv"]]))
    assert written(lambda f: datio.save_eigenstate_list(f, states, e["seed"], e["method"], e["ntarget"], e["dom"],
                                                        e["maxit"], e["toler"], e["realtime"],
                                                        e["verb"])) == e["text"]
