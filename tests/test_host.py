"""Host-side logic of the library (CPU only): the C ABI loads and exports
every declared symbol, option defaults and parsing follow the reference,
bin expressions compile, and the workloads are deterministic."""
import hashlib
import sys
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from pyradiance_gb300 import _lib
    return _lib


def test_c_abi_exports_every_declared_symbol(lib):
    import ctypes
    hdr = (ROOT / "include" / "gbrad.h").read_text()
    names = re.findall(r"^[a-z][^(\n]*?\b(gb_[a-z_0-9]+)\s*\(", hdr, re.M)
    assert len(names) >= 15
    L = ctypes.CDLL(str(lib._LIBPATH))
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_option_defaults(lib):
    o, used = lib.parse_opts([], lib.GB_PROG_RTRACE)
    assert (o.ab, o.ad, o.lr, o.aa, o.lw, o.dj, o.ds, o.dt, o.st, o.u) == (0, 1024, -10, 0.1, 1e-4, 0.0, 0.2, 0.03,
                                                                            0.15, 1)
    o, used = lib.parse_opts([], lib.GB_PROG_RCONTRIB)
    assert (o.ab, o.ad, o.lw, o.dj, o.dt, o.st, o.c, o.V) == (1, 350, 2e-3, 0.9, 0.0, 0.02, 1, 0)


def test_option_parsing(lib):
    o, used = lib.parse_opts(["-I+", "-ab", "3", "-ad", "1024", "-lw", "1e-4", "-c", "4", "-u-", "-faf",
                              "-av", "1", "2", "3", "-m", "sky"], lib.GB_PROG_RCONTRIB)
    assert used == 15 and o.I == 1 and o.ab == 3 and o.ad == 1024 and o.lw == 1e-4 and o.c == 4 and o.u == 0
    assert (o.fin, o.fout) == (b"a", b"f") and list(o.av) == [1, 2, 3]
    o, used = lib.parse_opts(["-h", "-ovs", "-I", "-dj", ".5"], lib.GB_PROG_RTRACE)
    assert o.h == 0 and o.outspec == b"vs" and o.I == 1 and o.dj == 0.5
    with pytest.raises(lib.GbError):
        lib.parse_opts(["-qq"], lib.GB_PROG_RTRACE)
    with pytest.raises(lib.GbError):
        lib.parse_opts(["-me", "1", "1", "1"], lib.GB_PROG_RTRACE)


def test_trace_list_options(lib, tmp_path):
    """-ti/-te take the modifier as the next argument and -tI/-tE a file
    that must open (rt/rtmain.c:210-260); the single-argument form that
    pyradiance's rtrace wrapper builds (src/pyradiance/rt.py:342-349) is a
    command line error, as it is for the reference's rtrace."""
    o, used = lib.parse_opts(["-ti", "glass", "-te", "light", "-t", "10", "-ab", "1"], lib.GB_PROG_RTRACE)
    assert used == 8 and o.ab == 1
    f = tmp_path / "mods.txt"
    f.write_text("glass light\n")
    _, used = lib.parse_opts(["-tI", str(f), "-tE", str(f)], lib.GB_PROG_RTRACE)
    assert used == 4
    for bad in (["-teglass"], ["-tI", str(tmp_path / "none.txt")], ["-ti"], ["-tx", "a"]):
        with pytest.raises(lib.GbError):
            lib.parse_opts(bad, lib.GB_PROG_RTRACE)
    import pyradiance_gb300 as gb
    with pytest.raises(RuntimeError):
        gb.rtrace(b"0 0 0 0 0 1\n", b"", trace_exclude="glass")


def nbins(lib, mods):
    arr = (lib.GbModspec * len(mods))()
    keep = []
    for i, m in enumerate(mods):
        v = {k: (m[k].encode() if m.get(k) else None) for k in ("modifier", "binv", "nbins", "params", "calfile",
                                                                 "expr")}
        keep.append(v)
        arr[i] = lib.GbModspec(v["modifier"], v["binv"], v["nbins"], v["params"], v["calfile"], v["expr"])
    n = lib.C.c_int(0)
    lib.check(lib.lib().gb_rcontrib_nbins(arr, len(mods), lib.C.byref(n)))
    return n.value


def test_bin_expressions(lib):
    assert nbins(lib, [dict(modifier="g")]) == 1
    assert nbins(lib, [dict(modifier="s", calfile="reinhartb.cal", params="MF=1", binv="rbin",
                            nbins="Nrbins")]) == 145
    assert nbins(lib, [dict(modifier="s", calfile="reinhartb.cal", params="MF=2", binv="rbin",
                            nbins="Nrbins")]) == 577
    assert nbins(lib, [dict(modifier="s", binv="if(-Dx*0-Dy*0-Dz*-1,0,-1)", nbins="1")]) == 1
    assert nbins(lib, [dict(modifier="s", expr="b=floor(Dz*10)", binv="b", nbins="10")]) == 10
    # general calcomp: functions with arguments, recursion on constants, built-ins
    cal = str(ROOT / "tests" / "golden" / "patchbins.cal")
    assert nbins(lib, [dict(modifier="s", calfile=cal, binv="pbin", nbins="Npbins")]) == 81
    assert nbins(lib, [dict(modifier="s", expr="f(x,n)=floor(x*n)+n*0;k(r):if(r-.5,r+k(r-1),0)",
                            binv="min(f(Dz+1,k(3)),5)", nbins="k(3)")]) == 6
    assert nbins(lib, [dict(modifier="s", binv="floor(4*(sin(Dx)+1)/2.01)", nbins="4")]) == 4
    for bad in ("rand(Dx)", "g(Dx)", "select(Dx)", "q"):
        with pytest.raises(lib.GbError):
            nbins(lib, [dict(modifier="s", binv=bad, nbins="4")])
    with pytest.raises(lib.GbError):                          # unbounded recursion on the ray
        nbins(lib, [dict(modifier="s", expr="r(x)=if(x,r(x-1),0)", binv="r(Dz)", nbins="2")])
    with pytest.raises(lib.GbError):
        nbins(lib, [dict(modifier="s", binv="3")])          # non-zero constant bin
    with pytest.raises(lib.GbError):
        nbins(lib, [dict(modifier="s", binv="Dz")])         # no bin count


def test_workloads_are_deterministic():
    from pyradiance_gb300 import workloads as w
    h = hashlib.sha256(w.window_room(ntri=500).encode()).hexdigest()
    assert h == hashlib.sha256(w.window_room(ntri=500).encode()).hexdigest()
    g = w.sensor_grid(64, 64)
    assert g.shape == (4096, 6) and np.allclose(g[:, 5], 1.0) and np.allclose(g[:, 2], 0.8)
    dc, sky = w.dc_sky(64, 100, 200)
    assert dc.dtype == np.float32 and (dc == 0).all(axis=2).mean() > 0.2
    assert (sky == 0).all(axis=(0, 2)).mean() > 0.3


def test_read_rays_formats():
    import pyradiance_gb300 as gb
    r = np.arange(12, dtype=np.float64).reshape(2, 6)
    np.testing.assert_array_equal(gb.read_rays(b"0 1 2 3 4 5\n6 7 8 9 10 11\n", "a"), r)
    np.testing.assert_array_equal(gb.read_rays(r.astype(np.float32).tobytes(), "f"), r)
    np.testing.assert_array_equal(gb.read_rays(r.tobytes(), "d"), r)


def test_rfluxmtx_receiver_arguments(tmp_path):
    """Receiver directives give the rcontrib modifier arguments the reference
    rfluxmtx passes on (its -v report for these files: util/rfluxmtx.c:427-582);
    directives and options it rejects raise."""
    from pyradiance_gb300 import rflux
    from pyradiance_gb300 import workloads as w
    f = w.flux_files(ntri=10)
    for k, v in f.items():
        (tmp_path / f"{k}.rad").write_text(v)
    sky = rflux._receivers(tmp_path / "sky.rad")
    assert [(m["modifier"], m["calfile"], m["params"], m["nbins"], m["binv"]) for m in sky] == [
        ("groundglow", None, None, "1", "0"),
        ("skyglow", "reinhartb.cal", "MF=1,rNx=0,rNy=0,rNz=-1,Ux=0,Uy=1,Uz=0,RHS=+1", "Nrbins", "rbin")]
    kf = rflux._receivers(tmp_path / "window_kf.rad")
    assert [(m["modifier"], m["calfile"], m["params"], m["nbins"], m["binv"]) for m in kf] == [
        ("windowglow", "klems_full.cal", "RHS=+1", "Nkbins", "kbin(0,1,0,0,0,1)")]
    (tmp_path / "cie.rad").write_text("#@rfluxmtx h=cie\nvoid glow g\n0\n0\n4 1 1 1 0\n\n"
                                      "g polygon p\n0\n0\n9 0 0 0 1 0 0 0 1 0\n")
    cie = rflux._receivers(tmp_path / "cie.rad")        # the reference's -v: -f cieskyscan.cal -p ... -b cbin
    assert [(m["modifier"], m["calfile"], m["params"], m["nbins"], m["binv"]) for m in cie] == [
        ("g", "cieskyscan.cal", "rNx=0,rNy=0,rNz=1,Ux=0,Uy=1,Uz=0,RHS=+1", "Ncbins", "cbin")]
    (tmp_path / "bad.rad").write_text("#@rfluxmtx h=xyz\nvoid glow g\n0\n0\n4 1 1 1 0\n\n"
                                      "g polygon p\n0\n0\n9 0 0 0 1 0 0 0 1 0\n")
    with pytest.raises(Exception):
        rflux._receivers(tmp_path / "bad.rad")
    assert rflux._screen(["-bj", ".5"])[-1] == ".5"      # bin jitter: JTR among the bin parameters
    assert rflux._receivers(tmp_path / "cie.rad", ".5")[0]["params"].endswith(",RHS=+1,JTR=.5")
    assert rflux._receivers(tmp_path / "window_kf.rad", ".5")[0]["params"] == "RHS=+1,JTR=.5"
    rc, fmt, xres, yres, cnt, iropt, ld, jit = rflux._screen(["-v", "-ab", "2", "-ff", "-c", "30", "-I+", "-y", "4",
                                                         "-av", "1", "1", "1", "-ld-"])
    assert rc == ["-ab", "2", "-av", "1", "1", "1"] and fmt == ["f", "f"] and cnt == 30 and iropt == "-I+"
    assert yres == "4" and ld == "-ld-"
    p = rflux._sender(tmp_path / "window_send.rad")
    rays, nb = rflux._sender_rays(p, 50, np.random.default_rng(1))
    assert nb == 145 and rays.shape == (145 * 50, 6)
    assert (rays[:, 4] < 0).all()                       # leaving the window away from its normal (+y)
    assert np.allclose(rays[:, 1], 0) and (rays[:, 0] >= 3.5).all() and (rays[:, 0] <= 6.5).all()


def rmtxop_chain(gb, g, chain: str, outform: str = "d"):
    """An Rmtxop built from a recorded rmtxop command line (options before
    each matrix, operators between them), matrices as bytes or paths."""
    import tempfile
    w = chain.split()
    rm = gb.Rmtxop(outform=outform)
    kw, op, i = {}, ".", 0
    tmp = Path(tempfile.mkdtemp())
    while i < len(w):
        t = w[i]
        if t == "-s":
            kw["scale"] = float(w[i + 1])
            i += 2
        elif t == "-t":
            kw["transpose"] = True
            i += 1
        elif t == "-c":
            j = i + 1
            while j < len(w) and w[j][0] in ".0123456789":
                j += 1
            kw["transform"] = [float(x) for x in w[i + 1:j]]
            i = j
        elif t in (".", "+", "*", "/"):
            op = t
            i += 1
        else:
            m = g[t]
            f = tmp / f"{t}.mtx"
            f.write_bytes(f"#?RADIANCE\nNROWS={m.shape[0]}\nNCOLS={m.shape[1]}\nNCOMP={m.shape[2]}\n"
                          "BigEndian=0\nFORMAT=double\n\n".encode() + m.astype("<f8").tobytes())
            rm.add_input(f, op=op, **kw)
            kw, op = {}, "."
            i += 1
    return rm


def test_rmtxop_elementwise_chains():
    """Rmtxop (util/rmtxop.c:383-525) chains of sums, element-wise products
    and quotients (zeros in the divisor give zeros, a one-component divisor
    is inverted first), with per-matrix scales and transforms: sums and
    products equal to the reference program's output, quotients within two
    single-precision ulps (the reference is built with -ffast-math, whose
    divisions round differently from IEEE division).  Chains with matrix
    products run on the GPU (tests/test_gpu_rmtxop.py)."""
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import rmtx
    g = np.load(ROOT / "tests" / "golden" / "rmtxop_chains.npz")
    n = 0
    for i, chain in enumerate(g["chains"]):
        chain = str(chain)
        if " . " in f" {chain} ":
            continue
        a = rmtx.read_rmatrix(rmtxop_chain(gb, g, chain)())
        np.testing.assert_allclose(a, g[f"out{i}"], rtol=3e-7 if "/" in chain else 0, atol=0, err_msg=chain)
        n += 1
    assert n == 6
    rm = gb.Rmtxop().add_input(b"x")
    with pytest.raises(gb.GbError, match="unknown operation"):
        rm.add_input("y.mtx", op="-")
    with pytest.raises(ValueError, match="stdin"):
        rm.add_input(b"y", op="+")
    with pytest.raises(gb.GbError):
        gb.Rmtxop(color="XYZ")


def test_rmtxop_against_reference():
    """rmtxop's single-matrix operations (util/rmtxop.c:288-381: transform with
    the scale folded in, else scale, then transpose) equal the reference
    program's output for each recorded option set."""
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import rmtx
    g = np.load(ROOT / "tests" / "golden" / "rmtxop.npz")
    m = g["m"]
    src = b"#?RADIANCE\nNROWS=5\nNCOLS=7\nNCOMP=3\nBigEndian=0\nFORMAT=double\n\n" + m.astype("<f8").tobytes()
    for i, case in enumerate(g["cases"]):
        w = str(case).split()
        kw = {}
        if "-t" in w:
            kw["transpose"] = True
        if "-s" in w:
            kw["scale"] = float(w[w.index("-s") + 1])
        if "-c" in w:
            kw["transform"] = [float(x) for x in w[w.index("-c") + 1:]]
        out = gb.rmtxop(src, outform="d", **kw)
        a = rmtx.read_rmatrix(out)
        np.testing.assert_allclose(a.ravel(), g[f"out{i}"], rtol=1e-7, err_msg=str(case))
        back = rmtx.read_rmatrix(gb.rmtxop(src, outform="a", **kw))
        np.testing.assert_allclose(back, a, rtol=1e-6)
    with pytest.raises(RuntimeError):
        gb.rmtxop(src, transform=[1, 2])


def test_btdf_matrices_against_reference(tmp_path):
    """Klems matrix BSDFs read as dctimestep reads a transmission matrix
    (util/cmbsdf.c:146-181 cm_loadBTDF over common/bsdf_m.c): front and back
    transmission by columns; back transmission only, by rows, turned
    around by reciprocity, with a floor taken out as a Lambertian part; the
    Klems half basis; no transmission data (the reference's Lambertian
    fallback, util/cmbsdf.c:122-143: zeros).  Equal to the reference
    dctimestep's matrices to
    within 3.5e-7 (the reference's RGB conversion of the Lambertian part
    rounds some values by a single-precision ulp or two)."""
    from pyradiance_gb300 import bsdf, workloads as w
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from make_golden import BTDF_CASES
    g = np.load(ROOT / "tests" / "golden" / "btdf.npz")
    for k, kw in BTDF_CASES.items():
        xml = tmp_path / f"{k}.xml"
        xml.write_text(w.klems_bsdf_xml(**kw))
        T = bsdf.load_btdf(xml)
        ref = g[f"{k}_T"]
        assert T.shape == ref.shape + (3,), k
        for c in range(3):
            np.testing.assert_allclose(T[..., c], ref, rtol=3.5e-7, atol=0, err_msg=k)
    bad = tmp_path / "tree.xml"
    bad.write_text(w.klems_bsdf_xml(seed=1).replace("<IncidentDataStructure>Columns", "<IncidentDataStructure>TensorTree3"))
    with pytest.raises(RuntimeError, match="unsupported BSDF"):
        bsdf.load_btdf(bad)


def test_ascii_rows_formatted_by_the_library():
    """gb_format_rows (the byte surface's ASCII output, host threads) gives
    the text of a sequential %e loop, for ragged shapes, zeros of both
    signs, subnormals, infinities and huge values; an output buffer that is
    too small is reported, not overrun."""
    import ctypes as C
    from pyradiance_gb300 import _ascii_block, _ascii_rows, _lib
    rng = np.random.default_rng(3)
    for shape in ((1, 1), (7, 3), (513, 146 * 3), (2, 0)):
        v = rng.lognormal(-3, 6, shape) * rng.choice([-1.0, 1.0, 0.0], shape)
        if v.size >= 5:
            v.flat[:5] = [-0.0, 5e-324, 1e300, np.inf, -np.inf]
        for sep, end in (("\t", "\t\n"), (" ", "\n")):
            assert _ascii_block(v, sep, end) == "".join(_ascii_rows(v, sep, end)).encode()
    v = np.ones((4, 3))
    buf = C.create_string_buffer(8)
    n = C.c_int64(0)
    rc = _lib.lib().gb_format_rows(v.ctypes.data, 4, 3, b"\t", b"\n", buf, 8, C.byref(n))
    assert rc == -6 and n.value == len("".join(_ascii_rows(v, "\t", "\n")))
