"""Edge cases of the GPU path (needs a GB300): empty inputs, rays with no
direction, rays along the axes and from outside the scene cube, rays aimed
exactly at polygon edges and corners (the tie rules of rt/raytrace.c:536-575
and the edge cases of common/face.c:121-161), and rcontrib's -c records with
a trailing partial record.  Hit objects are compared with the oracle."""
import numpy as np
import pytest

from conftest import MODS_C2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(scene_dir):
    import pyradiance_gb300 as gb
    from oracle import pyoracle as po
    from pyradiance_gb300 import _lib
    _lib.lib()
    return gb, _lib, po, gb.Scene(rad_files=[scene_dir / "c1.rad"]), po.Scene(scene_dir / "c1.rad"), scene_dir


def cast(_lib, sc, rays):
    o, _ = _lib.parse_opts(["-ab", "0"], _lib.GB_PROG_RTRACE)
    rays = np.ascontiguousarray(rays, dtype=np.float64)
    hid = np.zeros(len(rays), dtype=np.int32)
    ht = np.zeros(len(rays))
    _lib.check(_lib.lib().gb_rtrace(sc.handle, o, _lib.ptr(rays), len(rays), None, _lib.ptr(hid), _lib.ptr(ht)))
    return hid, ht


def oracle_cast(po, osc, rays):
    o = po.default_opts("rtrace", ab=0)
    _, hid, ht, _ = po.rtrace(osc, o, rays, values=False)
    return hid, ht


def test_empty_inputs(env):
    gb, _lib, po, sc, osc, _ = env
    o, _ = _lib.parse_opts(["-I+", "-ab", "1"], _lib.GB_PROG_RTRACE)
    z = np.zeros((0, 6))
    _lib.check(_lib.lib().gb_rtrace(sc.handle, o, _lib.ptr(z), 0, None, None, None))
    out = gb.rtrace(b"", sc, params=["-ab", "0"], header=False)
    assert out == b""
    rc = gb.Rcontrib(b"", sc, params=["-ab", "1"])
    for m in MODS_C2:
        rc.add_modifier(**{{"expr": "expression", "params": "param"}.get(k, k): v for k, v in m.items()})
    assert rc.run_array(z).shape == (0, 146, 3)
    with pytest.raises(_lib.GbError):
        gb.dctimestep_array(np.zeros((0, 4, 3)), np.zeros((4, 2, 3)))


def test_zero_direction_rays_give_zero_values(env):
    gb, _lib, po, sc, osc, _ = env
    text = b"5 4 1 0 0 0\n5 4 1 0 0 1\n"
    out = gb.rtrace(text, sc, params=["-ab", "0", "-ds", "0"], header=False, outform="d")
    vals = np.frombuffer(out, dtype=np.float64).reshape(-1, 3)
    assert vals.shape == (2, 3)
    np.testing.assert_array_equal(vals[0], 0.0)


def test_axis_rays_and_rays_from_outside(env):
    gb, _lib, po, sc, osc, _ = env
    rng = np.random.default_rng(8)
    org = rng.uniform((0.5, 0.5, 0.3), (9.5, 7.5, 2.7), size=(300, 3))
    rays = []
    for d in np.vstack([np.eye(3), -np.eye(3)]):
        rays.append(np.hstack([org, np.tile(d, (len(org), 1))]))
    out = rng.uniform((-20, -20, -20), (30, 30, 20), size=(600, 3))
    tgt = rng.uniform((0, 0, 0), (10, 8, 3), size=(600, 3))
    dirs = tgt - out
    rays.append(np.hstack([out, dirs / np.linalg.norm(dirs, axis=1, keepdims=True)]))
    rays = np.vstack(rays)
    g_id, g_t = cast(_lib, sc, rays)
    o_id, o_t = oracle_cast(po, osc, rays)
    np.testing.assert_array_equal(g_id, o_id)
    hit = o_id >= 0
    np.testing.assert_allclose(g_t[hit], o_t[hit], rtol=1e-5, atol=2e-6)   # FP32 positions, scene of ~10 m


def _polygons(rad_text):
    """vertices of every polygon in a scene text"""
    toks = rad_text.split()
    polys, i = [], 0
    while i + 2 < len(toks):
        if toks[i + 1] == "polygon":
            j = i + 3
            ns = int(toks[j]); j += 1 + ns
            ni = int(toks[j]); j += 1 + ni
            nr = int(toks[j])
            v = np.array(toks[j + 1:j + 1 + nr], dtype=float).reshape(-1, 3)
            polys.append(v)
            i = j + 1 + nr
        else:
            i += 1
    return polys


def _aimed_rays(polys, inset, seed=9):
    """rays from random points of the room to a vertex and an edge midpoint
    of each of 400 box faces, moved `inset` metres towards the face centre;
    also the cosine between each ray and its face's normal"""
    rng = np.random.default_rng(seed)
    pts, nrm = [], []
    for v in polys[6:406]:                        # box faces (the room shell first)
        k = rng.integers(0, len(v))
        c = v.mean(0)
        n = np.cross(v[1] - v[0], v[2] - v[1])
        for q in (v[k], 0.5 * (v[k] + v[(k + 1) % len(v)])):
            u = c - q
            pts.append(q + inset * u / np.linalg.norm(u))
            nrm.append(n / np.linalg.norm(n))
    pts = np.array(pts)
    org = np.clip(pts + rng.normal(size=pts.shape) * 2.0, (0.05, 0.05, 0.05), (9.95, 7.95, 2.95))
    d = pts - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.hstack([org, d]), np.abs((d * np.array(nrm)).sum(1))


def test_rays_near_edges_and_corners(env):
    """Aimed 0.1 mm inside box faces next to a vertex or an edge midpoint,
    where the walk crosses leaf boundaries and tests neighbouring faces.
    The ray also crosses the plane of the face on the other side of that
    edge close to the edge, sometimes within FTINY plus the FP32 rounding of
    the hit point, where the two arithmetics can decide the edge rule of
    common/face.c:121-161 differently (measured: 1 ray in 800 on the GPU,
    none on the host build of the same code).  Bound: 99.5%."""
    gb, _lib, po, sc, osc, scene_dir = env
    rays, _ = _aimed_rays(_polygons((scene_dir / "c1.rad").read_text()), 1e-4)
    g_id, g_t = cast(_lib, sc, rays)
    o_id, o_t = oracle_cast(po, osc, rays)
    assert (g_id == o_id).mean() >= 0.995, np.nonzero(g_id != o_id)


def test_rays_exactly_at_edges_and_corners(env):
    """Aimed exactly at a vertex or an edge midpoint.  There both faces
    meeting at the edge, or neither, pass the FTINY edge rules of
    common/face.c:121-161 depending on the last bits of the hit point, which
    FP32 and the reference's FP64 round differently (measured: about 3% of
    these rays pick the other face or the object behind).  Bound: 95%
    agreement; off the edges the walk agrees exactly (sensor grids, axis
    rays, rays from outside the scene above)."""
    gb, _lib, po, sc, osc, scene_dir = env
    rays, _ = _aimed_rays(_polygons((scene_dir / "c1.rad").read_text()), 0.0)
    g_id, _ = cast(_lib, sc, rays)
    o_id, _ = oracle_cast(po, osc, rays)
    assert (g_id == o_id).mean() >= 0.95, np.nonzero(g_id != o_id)


def test_rcontrib_records_of_c_rays(env, scene_dir):
    """-c 4: each record is the mean of its four rays' coefficients (the
    same sensors draw the same streams), and a trailing partial record is
    not returned (rt/rc2.c:294-357)."""
    gb, _lib, po, sc, osc, _ = env
    sc2 = gb.Scene(rad_files=[scene_dir / "c2.rad"])
    rays = np.repeat(np.array([[5.0, 4.0, 0.8, 0, 0, 1], [3.0, 2.0, 0.8, 0, 0, 1]]), [6, 4], axis=0)
    def run(c):
        rc = gb.Rcontrib(b"", sc2, params=["-I+", "-ab", "1", "-ad", "64", "-lw", "1e-4", "-c", str(c), "-u-"])
        for m in MODS_C2:
            rc.add_modifier(**{{"expr": "expression", "params": "param"}.get(k, k): v for k, v in m.items()})
        rc.seed = 77
        return rc.run_array(rays)
    one, four = run(1), run(4)
    assert one.shape[0] == 10 and four.shape[0] == 2
    np.testing.assert_allclose(four, one[:8].reshape(2, 4, *one.shape[1:]).mean(1), rtol=1e-6, atol=1e-12)
