"""The drop-in functions' bytes against pyradiance's own functions run on
the reference programs (needs a GB300).

tests/golden/bytes_surface.npz holds what src/pyradiance/rt.py rtrace and
Rcontrib and src/pyradiance/util.py dctimestep returned, with the reference
programs built from the reference sources, for: the direct-irradiance
workload (ASCII and binary double, headers on; first-hit names), rays
leaving the window room through its glass at -ab 0 (deterministic: each
reaches the sky or the ground through the window), once with the sky's
columns sent to a file (add_modifier(output=...)), and dctimestep of a
small matrix pair.  The frozen octrees are in the fixture, so both sides
copy the same octree header.

Headers must be line for line the reference's but for the lines that
carry the software version and the time (SOFTWARE=, CAPDATE=, GMT=),
trailing padding, and the directories of matrix files on a dctimestep
command line.  ASCII bodies must have the reference's layout exactly (with
every number replaced by a mark the texts are equal: separators, line
ends, number format) and numbers within 1e-5 relative; binary bodies the
same length and values within 1e-5; names equal as text.
"""
import re

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
VARIABLE = ("SOFTWARE=", "CAPDATE=", "GMT=")
NUM = re.compile(rb"-?\d\.\d{6}e[+-]\d{2,3}")


@pytest.fixture(scope="module")
def env(tmp_path_factory):
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import _lib
    _lib.lib()
    g = golden("bytes_surface.npz")
    d = tmp_path_factory.mktemp("bytes")
    (d / "c1_ref.oct").write_bytes(g["c1_oct"].tobytes())
    (d / "c2s_ref.oct").write_bytes(g["c2_oct"].tobytes())
    return gb, g, d


def split(b: bytes):
    i = b.find(b"\n\n")
    return b[:i].decode().split("\n"), b[i + 2:]


def norm_header(lines):
    out = []
    for ln in lines:
        if ln.startswith(VARIABLE):
            continue
        toks = [t.rsplit("/", 1)[-1] if t.endswith(".mtx") else t for t in ln.split(" ")]
        out.append(" ".join(toks).rstrip())
    return out


def check_ascii(ours: bytes, ref: bytes, rtol=1e-5, atol=1e-9):
    assert NUM.sub(b"#", ours) == NUM.sub(b"#", ref)
    a = np.array(NUM.findall(ours), dtype=float)
    b = np.array(NUM.findall(ref), dtype=float)
    np.testing.assert_allclose(a, b, rtol=rtol, atol=atol)


def compare(ours: bytes, ref: bytes, binary=None, **tol):
    h1, b1 = split(ours)
    h2, b2 = split(ref)
    assert norm_header(h1) == norm_header(h2)
    if binary:
        assert len(b1) == len(b2)
        np.testing.assert_allclose(np.frombuffer(b1, binary), np.frombuffer(b2, binary),
                                   rtol=tol.get("rtol", 1e-5), atol=tol.get("atol", 1e-9))
    else:
        check_ascii(b1, b2, **tol)
    return b2


def test_rtrace_irradiance_ascii_and_double(env):
    gb, g, d = env
    from pyradiance_gb300 import workloads as w
    rays = g["rays1"]
    params = [str(x) for x in g["params1"]]
    out = gb.rtrace(w.rays_ascii(rays), str(d / "c1_ref.oct"), irradiance=True, params=params)
    compare(out, g["c1_a"].tobytes())
    out = gb.rtrace(rays.astype("<f8").tobytes(), str(d / "c1_ref.oct"), irradiance=True, inform="d",
                    outform="d", params=params)
    compare(out, g["c1_d"].tobytes(), binary="<f8")


def test_rtrace_hit_names_text(env):
    gb, g, d = env
    from pyradiance_gb300 import workloads as w
    out = gb.rtrace(w.rays_ascii(g["rays1"]), str(d / "c1_ref.oct"), outspec="s", params=["-ab", "0"])
    h1, b1 = split(out)
    h2, b2 = split(g["c1_s"].tobytes())
    assert norm_header(h1) == norm_header(h2)
    assert b1 == b2


def _rc(gb, g, d, output=None):
    from pyradiance_gb300 import workloads as w
    rc = gb.Rcontrib(w.rays_ascii(g["rays2"]), str(d / "c2s_ref.oct"), params=[str(x) for x in g["rcp"]])
    rc.add_modifier(modifier="groundglow")
    kw = dict(modifier="skyglow", calfile="reinhartb.cal", param="MF=1", binv="rbin", nbins="Nrbins")
    if output:
        kw["output"] = output
    rc.add_modifier(**kw)
    return rc


def test_rcontrib_bytes(env):
    gb, g, d = env
    ref = compare(_rc(gb, g, d)(), g["c2_out"].tobytes())
    assert (np.array(NUM.findall(ref), dtype=float) > 0).sum() > 100      # rays reach the sky and ground


def test_rcontrib_modifier_output_file(env, monkeypatch):
    """add_modifier(output="sky_%s.mtx"): the sky's 145 columns go to the
    file named for the modifier, with its own header (MODIFIER=, NCOLS=),
    and the returned bytes keep the ground's column; a second run does not
    overwrite the file (an error, as rcontrib without -fo)."""
    gb, g, d = env
    wd = d / "out"
    wd.mkdir(exist_ok=True)
    monkeypatch.chdir(wd)
    compare(_rc(gb, g, d, output="sky_%s.mtx")(), g["c2_split"].tobytes())
    compare((wd / "sky_skyglow.mtx").read_bytes(), g["c2_file"].tobytes())
    with pytest.raises(RuntimeError):
        _rc(gb, g, d, output="sky_%s.mtx")()


def test_rcontrib_per_bin_output_files(env, monkeypatch):
    """add_modifier(output="bin_%s_%03d.mtx") (rt/rc2.c:41-97 ofname): one
    file per sky bin, named with the modifier and the bin, each with its
    own header (MODIFIER=, BIN=, NCOLS=1) and its column; the returned
    bytes keep the ground's column."""
    gb, g, d = env
    wd = d / "bins"
    wd.mkdir(exist_ok=True)
    monkeypatch.chdir(wd)
    compare(_rc(gb, g, d, output="bin_%s_%03d.mtx")(), g["c2_binsplit"].tobytes())
    ref = dict(part.split(b"\n", 1) for part in g["c2_bins"].tobytes().split(b"\0"))
    ours = sorted(wd.glob("bin_skyglow_*.mtx"))
    assert [f.name.encode() for f in ours] == sorted(ref)
    for f in ours:
        compare(f.read_bytes(), ref[f.name.encode()])


def test_dctimestep_bytes(env):
    gb, g, d = env
    m = golden("dct_small.npz")
    paths = []
    for name, a in (("D", m["dc"]), ("S", m["sky"])):
        p = d / f"{name}.mtx"
        p.write_bytes((f"#?RADIANCE\nNROWS={a.shape[0]}\nNCOLS={a.shape[1]}\nNCOMP=3\nBigEndian=0\n"
                       "FORMAT=float\n\n").encode() + a.astype("<f4").tobytes())
        paths.append(str(p))
    atol = 1e-6 * float(np.abs(m["out"]).max())
    compare(gb.dctimestep(*paths), g["dct_a"].tobytes(), atol=atol)
    compare(gb.dctimestep(*paths, outform="d"), g["dct_d"].tobytes(), binary="<f8", atol=atol)
