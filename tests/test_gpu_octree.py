"""The octree built on the GPU against the host builder and the reference's
oconv (needs a GB300).

gb_scene_load_rad builds the octree of a scene of polygons and spheres on
the GPU; every tree must equal the host builder's (the oracle's digest of
the same scene text) and, for the scenes the reference's oconv was run on,
the reference's.  Scenes with cones fall back to the host builder.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def info(sc):
    from pyradiance_gb300 import _lib
    n, s, d, dev = C.c_int64(), C.c_int64(), C.c_uint64(), C.c_int()
    _lib.check(_lib.lib().gb_scene_octree_info(sc.handle, C.byref(n), C.byref(s), C.byref(d), C.byref(dev)))
    return [n.value, s.value, d.value], dev.value


@pytest.fixture(scope="module")
def gb():
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import _lib
    _lib.lib()
    return gb


@pytest.mark.parametrize("name", ["c1", "c2", "zoo"])
def test_reference_scenes(gb, scene_dir, name):
    g = golden("octree_ref.npz")
    sc = gb.Scene(rad_files=[scene_dir / f"{name}.rad"])
    digest, dev = info(sc)
    assert digest == [int(x) for x in g[name]], name
    assert dev == (0 if name == "zoo" else 1), "cones are built on the host, polygons on the device"


@pytest.mark.parametrize("kw", [dict(seed=4, ntri=200000, nmat=64, nwin=4, tessellated=True),
                                dict(seed=5, ntri=60000, nmat=8),
                                dict(seed=6, ntri=3000, nwin=8)])
def test_device_tree_equals_host_tree(gb, tmp_path, kw):
    """Dense and sparse rooms of random triangles, several windows: the
    device builder's tree equals the host builder's."""
    from oracle import pyoracle as po
    from pyradiance_gb300 import workloads as w
    p = tmp_path / "room.rad"
    p.write_text(w.window_room(**kw))
    sc = gb.Scene(rad_files=[p])
    digest, dev = info(sc)
    assert dev == 1
    assert digest == po.octree_digest(p), kw


def test_spheres_on_the_device(gb, tmp_path):
    """The glossy room's spheres (ot/sphere.c cube test) and the minimum
    cube size: small objlim and resolution force deep trees."""
    from oracle import pyoracle as po
    from pyradiance_gb300 import workloads as w
    from pyradiance_gb300 import _lib
    p = tmp_path / "glossy.rad"
    p.write_text(w.glossy_room())
    sc = gb.Scene(rad_files=[p])
    digest, dev = info(sc)
    assert dev == 1 and digest == po.octree_digest(p)
    # objlim 2, resolution 64: the host and device builders on the same text
    for objlim, resolu in ((2, 64), (1, 16384)):
        h = C.c_void_p()
        arr = (C.c_char_p * 1)(str(p).encode())
        _lib.check(_lib.lib().gb_scene_load_rad(arr, 1, objlim, resolu, C.byref(h)))
        try:
            n, s, d, dv = C.c_int64(), C.c_int64(), C.c_uint64(), C.c_int()
            _lib.check(_lib.lib().gb_scene_octree_info(h, C.byref(n), C.byref(s), C.byref(d), C.byref(dv)))
            assert dv.value == 1
            assert [n.value, s.value, d.value] == po.octree_digest(p, objlim=objlim, resolu=resolu)
        finally:
            _lib.lib().gb_scene_free(h)
