"""The CPU oracle against the golden vectors of the reference programs.

These pin the oracle (and the host scene loader and octree builder it
shares with the library) before it is used to check the GPU.  CPU only.
"""
import os
from pathlib import Path

import numpy as np
import pytest

from conftest import MODS_C2, golden, reference_tree, zscores
from oracle import pyoracle as po
from pyradiance_gb300 import workloads as w

_TREE = reference_tree()
REF_TRACE = _TREE / "tests" / "Resources" / "trace.oct" if _TREE else Path("/nonexistent")


@pytest.fixture(scope="module")
def oscenes(scene_dir):
    return {k: po.Scene(scene_dir / f"{k}.rad") for k in ("c1", "c2", "zoo", "glossy", "c2e")}


def test_octree_builder_matches_reference(scene_dir):
    g = golden("octree_ref.npz")
    for name in ("c1", "c2", "zoo"):
        assert po.octree_digest(scene_dir / f"{name}.rad") == [int(x) for x in g[name]], name


def test_c1_direct_irradiance_and_hits(oscenes):
    g = golden("c1_direct.npz")
    sc = oscenes["c1"]
    o = po.default_opts("rtrace", I=1, ab=0, dj=0, ds=0, dr=0, u=0)
    rgb, hid, ht, _ = po.rtrace(sc, o, g["rays"])
    ref = g["irradiance"]
    lit = ref[:, 0] > 0
    assert lit.mean() > 0.05
    np.testing.assert_array_equal(rgb[~lit], 0.0)
    rel = np.abs(rgb[lit] - ref[lit]) / ref[lit]
    assert rel.max() < 1e-6, rel.max()
    names = np.array([sc.object_name(i) if i >= 0 else "*" for i in hid])
    assert (names == g["hit_name"]).all()
    np.testing.assert_allclose(ht, g["hit_dist"], rtol=1e-7)  # frozen-octree float precision


def test_c1_partitioned_source(oscenes):
    """-ds 0.2: the light split into pieces as rt/srcsamp.c:260-330 does
    (many near the 2.5 m grid); -dt 0, every piece's shadow tested."""
    g = golden("c1_partitioned.npz")
    o = po.default_opts("rtrace", I=1, ab=0, dj=0, ds=0.2, dr=0, dt=0, u=0)
    rgb, _, _, _ = po.rtrace(oscenes["c1"], o, g["rays"], hits=False, threads=8)
    ref = g["irradiance"]
    lit = ref[:, 0] > 0
    np.testing.assert_array_equal(rgb[~lit], 0.0)
    assert (np.abs(rgb[lit] - ref[lit]) / ref[lit]).max() < 1e-6


def test_glossy_direct_lobe(oscenes):
    """Rough plastic and metal with every lobe below -st 1: the direct
    Gaussian specular term of rt/normal.c:142-170 plus diffuse, no
    sampling (deterministic)."""
    g = golden("glossy.npz")
    o = po.default_opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, st=1, u=0)
    rgb, _, _, _ = po.rtrace(oscenes["glossy"], o, g["rays"], hits=False, threads=8)
    np.testing.assert_allclose(rgb, g["radiance_st1"], rtol=1e-6, atol=1e-9)


def glossy_sampled(sc, g, K, **kw):
    """per-ray mean and standard error of K replicas (independent streams:
    replicas are different sensors)"""
    n = len(g["rays"])
    o = po.default_opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, u=0, **kw)
    rgb, _, _, _ = po.rtrace(sc, o, np.repeat(g["rays"], K, axis=0), hits=False, threads=8)
    a = rgb.reshape(n, K, 3)
    return a.mean(1), a.std(1, ddof=1) / np.sqrt(K)


@pytest.mark.parametrize("key,kw", [("st0", {"st": 0}), ("ss3", {"ss": 3})])
def test_glossy_sampled_lobe(oscenes, key, kw):
    """The rough specular lobe sampled (rt/normal.c:364-440 gaussamp): one
    sample per hit with -st 0, several with the W-G-M-D weighting with
    -ss 3.  Per-ray means of 256 replicas against the reference's 1,024:
    z-scores of every ray and channel within 5, their mean within 4
    standard errors of zero, the overall mean within 0.5%.  Rays whose
    value has no random part (matte surfaces) are compared at 1e-6."""
    g = golden("glossy.npz")
    m, se = glossy_sampled(oscenes["glossy"], g, 256, **kw)
    rm = g[f"{key}_mean"]
    z = (m - rm) / np.sqrt(se ** 2 + g[f"{key}_se"] ** 2 + (1e-6 * np.abs(rm) + 1e-9) ** 2)
    assert np.abs(z).max() < 5, np.abs(z).max()
    assert abs(z.mean()) < 4 / np.sqrt(len(z)), z.mean()
    assert abs(m.mean() / g[f"{key}_mean"].mean() - 1) < 5e-3


@pytest.mark.parametrize("key", ["c1", "c2e"])
def test_surface_irradiance(oscenes, key):
    """-i: primary hits on non-light materials shaded as a Lambertian of
    reflectance pi, glass passed through (rt/raytrace.c:211-236)."""
    g = golden("surface_irradiance.npz")
    o = po.default_opts("rtrace", i=1, ab=0, dj=0, ds=0, dr=0, dt=0, u=0)
    rgb, _, _, _ = po.rtrace(oscenes[key], o, g[f"{key}_rays"], hits=False, threads=8)
    np.testing.assert_allclose(rgb, g[f"{key}_irr"], rtol=1e-6, atol=1e-9)


def test_surface_irradiance_one_bounce(oscenes):
    """-i -ab 1 -ad 256: per-ray means of 256 replicas against the
    reference's (-u+), z-scores within 5, their mean within 4 standard
    errors of zero."""
    g = golden("surface_irradiance.npz")
    K, n = 256, len(g["ab1_rays"])
    o = po.default_opts("rtrace", i=1, ab=1, ad=256, lw=1e-4, dj=0, ds=0, dr=0, dt=0, u=0, aa=0)
    rgb, _, _, _ = po.rtrace(oscenes["c1"], o, np.repeat(g["ab1_rays"], K, axis=0), hits=False, threads=8)
    a = rgb.reshape(n, K, 3)
    m, se = a.mean(1), a.std(1, ddof=1) / np.sqrt(K)
    z = (m - g["ab1_mean"]) / np.sqrt(se ** 2 + g["ab1_se"] ** 2 + (1e-6 * np.abs(g["ab1_mean"]) + 1e-9) ** 2)
    assert np.abs(z).max() < 5 and abs(z.mean()) < 4 / np.sqrt(n), (np.abs(z).max(), z.mean())


@pytest.mark.parametrize("key,asn", [("as512", 512), ("as0", 0)])
def test_supersampled_first_hemisphere(oscenes, key, asn):
    """rtrace -I -ab 2 -aa 0 -ad 256 with ambient super-sampling (-as 512,
    rtrace's default; rt/ambcomp.c:256-346) and without: per-sensor means of
    96 replicas against the reference's 512 (-u+), z-scores within 5, their
    mean within 4 standard errors of zero.  (Without the super-sampling the
    -as 512 means differ from the reference's by up to 1.5% on single
    sensors, many standard errors.)"""
    g = golden("supersampled.npz")
    K, n = 96, 40
    o = po.default_opts("rtrace", I=1, ab=2, aa=0, ad=256, lw=1e-4, dj=0, ds=0, dr=0, dt=0, u=0)
    o.as_ = asn
    rgb, _, _, _ = po.rtrace(oscenes["c1"], o, np.repeat(g["rays"][:n], K, axis=0), hits=False, threads=16)
    a = rgb.reshape(n, K, 3)
    m, se = a.mean(1), a.std(1, ddof=1) / np.sqrt(K)
    rm, rse = g[f"{key}_mean"][:n], g[f"{key}_se"][:n]
    z = (m - rm) / np.sqrt(se ** 2 + rse ** 2 + (1e-6 * np.abs(rm) + 1e-9) ** 2)
    assert np.abs(z).max() < 5 and abs(z.mean()) < 4 / np.sqrt(n), (np.abs(z).max(), z.mean())


CAL = Path(__file__).resolve().parent / "golden" / "patchbins.cal"
MODS_PATCH = [dict(modifier=m, calfile=str(CAL), binv="pbin", nbins="Npbins") for m in ("skyglow", "groundglow")]


def test_general_bin_expressions(oscenes):
    """A function file of our own (recursion on constant arguments, select,
    if, asin, atan2, floor, sqrt, max, min, ^) compiled to the bin byte
    code: rcontrib -ab 0 radiance-mode rays leaving through the window each
    land in the reference's bin, with its value."""
    g = golden("general_bins.npz")
    o = po.default_opts("rcontrib", I=0, ab=0, c=1, u=0)
    out, _ = po.rcontrib(oscenes["c2e"], o, MODS_PATCH, g["rays"], threads=8)
    got = out[..., 0]
    np.testing.assert_array_equal(got > 0, g["bins"] > 0)
    np.testing.assert_allclose(got, g["bins"], rtol=1e-6, atol=1e-9)


def test_cie_sky_scanner_bins(tmp_path):
    """The CIE sky scanner bins of util/cieskyscan.cal (cbin, Ncbins) built
    into the bin compiler: rays in every direction in a scene of the sky and
    ground glows land in the reference's bin, for the default frame and one
    turned a quarter round."""
    g = golden("cie_bins.npz")
    (tmp_path / "sky.rad").write_text(w.SKY_GLOW)
    sc = po.Scene(tmp_path / "sky.rad")
    o = po.default_opts("rcontrib", I=0, ab=0, c=1, u=0)
    for key, params in (("default", None), ("upx", "Ux=1,Uy=0,Uz=0")):
        mods = [dict(modifier=m, calfile="cieskyscan.cal", binv="cbin", nbins="Ncbins", **(
            {"params": params} if params else {})) for m in ("skyglow", "groundglow")]
        out, _ = po.rcontrib(sc, o, mods, g["rays"], threads=8)
        got = out[..., 0]
        np.testing.assert_array_equal(got > 0, g[key] > 0, err_msg=key)
        np.testing.assert_allclose(got, g[key], rtol=1e-6, atol=1e-9, err_msg=key)


def test_translucent(tmp_path):
    """The trans material: -I irradiance through the diffuser and radiance
    of view rays with -ab 0 -st 1, 1e-6; aimed view rays with -ab 1 -st 0
    (ambient from both sides, both lobes sampled): means of 256 replicas
    within 5 standard errors of the reference's."""
    from pyradiance_gb300 import workloads as w
    g = golden("translucent.npz")
    (tmp_path / "trans.rad").write_text(w.trans_room())
    sc = po.Scene(tmp_path / "trans.rad")
    o = po.default_opts("rtrace", I=1, ab=0, dj=0, ds=0, dr=0, dt=0, st=1, u=0)
    rgb, _, _, _ = po.rtrace(sc, o, g["grid"], hits=False, threads=8)
    np.testing.assert_allclose(rgb, g["irradiance"], rtol=1e-6, atol=1e-9)
    o.I = 0
    rgb, _, _, _ = po.rtrace(sc, o, g["view"], hits=False, threads=8)
    np.testing.assert_allclose(rgb, g["radiance"], rtol=1e-6, atol=1e-9)
    K, n = 256, len(g["aimed"])
    o = po.default_opts("rtrace", ab=1, aa=0, ad=256, lw=1e-4, dj=0, ds=0, dr=0, dt=0, st=0, u=0)
    o.as_ = 0
    rgb, _, _, _ = po.rtrace(sc, o, np.repeat(g["aimed"], K, axis=0), hits=False, threads=8)
    a = rgb.reshape(n, K, 3)
    m, se = a.mean(1), a.std(1, ddof=1) / np.sqrt(K)
    z = (m - g["ab1_mean"]) / np.sqrt(se ** 2 + g["ab1_se"] ** 2 + (1e-6 * np.abs(g["ab1_mean"]) + 1e-9) ** 2)
    assert np.abs(z).max() < 5 and abs(z.mean()) < 4 / np.sqrt(n), (np.abs(z).max(), z.mean())


@pytest.mark.parametrize("room,fixture", [("lamp_room", "circular_sources.npz"),
                                          ("tube_room", "cylinder_sources.npz")])
def test_circular_sources(scene_dir, tmp_path, room, fixture):
    """Sphere and disk lights, and cylinder lights (partitioned along their
    axis, rt/srcsamp.c:187-273): -I direct irradiance with -ds 0 and with the
    disk partitioned (-ds 0.2, pieces trimmed to the circle), 1e-6; with
    jittered samples (-dj 0.9) per-sensor means of 256 replicas within 5
    standard errors of the reference's."""
    from pyradiance_gb300 import workloads as w
    g = golden(fixture)
    (tmp_path / "lamp.rad").write_text(getattr(w, room)())
    sc = po.Scene(tmp_path / "lamp.rad")
    for key, ds in (("ds0", 0.0), ("ds2", 0.2)):
        o = po.default_opts("rtrace", I=1, ab=0, dj=0, ds=ds, dr=0, dt=0, u=0)
        rgb, _, _, _ = po.rtrace(sc, o, g["rays"], hits=False, threads=8)
        np.testing.assert_allclose(rgb, g[key], rtol=1e-6, atol=1e-9, err_msg=key)
    K, n = 256, len(g["dj_rays"])
    o = po.default_opts("rtrace", I=1, ab=0, dj=0.9, ds=0.2, dr=0, dt=0, u=0)
    rgb, _, _, _ = po.rtrace(sc, o, np.repeat(g["dj_rays"], K, axis=0), hits=False, threads=8)
    a = rgb.reshape(n, K, 3)
    m, se = a.mean(1), a.std(1, ddof=1) / np.sqrt(K)
    z = (m - g["dj_mean"]) / np.sqrt(se ** 2 + g["dj_se"] ** 2 + (1e-6 * np.abs(g["dj_mean"]) + 1e-9) ** 2)
    assert np.abs(z).max() < 5 and abs(z.mean()) < 4 / np.sqrt(n), (np.abs(z).max(), z.mean())


def test_spotlights(tmp_path):
    """Spotlights: -I direct irradiance (samples outside a cone dropped,
    the solid angle seen from the focus) and view rays at the lights (lit
    only from inside the cones), 1e-6."""
    from pyradiance_gb300 import workloads as w
    g = golden("spotlights.npz")
    (tmp_path / "spot.rad").write_text(w.spot_room())
    sc = po.Scene(tmp_path / "spot.rad")
    o = po.default_opts("rtrace", I=1, ab=0, dj=0, ds=0, dr=0, dt=0, u=0)
    rgb, _, _, _ = po.rtrace(sc, o, g["grid"], hits=False, threads=8)
    np.testing.assert_allclose(rgb, g["irradiance"], rtol=1e-6, atol=1e-9)
    o.I = 0
    rgb, _, _, _ = po.rtrace(sc, o, g["view"], hits=False, threads=8)
    np.testing.assert_allclose(rgb, g["radiance"], rtol=1e-6, atol=1e-9)


def test_mirrors(tmp_path):
    """Mirrors with -dr 0: -I irradiance (mirrors block shadow rays) and
    view rays through mirror chains, 1e-6."""
    from pyradiance_gb300 import workloads as w
    g = golden("mirrors.npz")
    (tmp_path / "mirror.rad").write_text(w.mirror_room())
    sc = po.Scene(tmp_path / "mirror.rad")
    o = po.default_opts("rtrace", I=1, ab=0, dj=0, ds=0, dr=0, dt=0, u=0)
    rgb, _, _, _ = po.rtrace(sc, o, g["grid"], hits=False, threads=8)
    np.testing.assert_allclose(rgb, g["irradiance"], rtol=1e-6, atol=1e-9)
    o.I = 0
    rgb, _, _, _ = po.rtrace(sc, o, g["view"], hits=False, threads=8)
    np.testing.assert_allclose(rgb, g["radiance"], rtol=1e-6, atol=1e-9)


def flux_close(a, b, n):
    """Sender matrices: each entry is a mean over n rays of a coefficient in
    [0, 1]; both within 5 combined standard errors (plus a 1.5/n floor)."""
    tol = 5 * np.sqrt((a * (1 - a) + b * (1 - b)) / n) + 1.5 / n
    bad = np.abs(a - b) > tol
    assert bad.mean() <= 2e-3, (bad.sum(), np.argwhere(bad)[:5])
    np.testing.assert_allclose(a.sum(axis=1), b.sum(axis=1), atol=0.05)


def test_flux_matrices(tmp_path):
    """rfluxmtx (util/rfluxmtx.c): the receiver directives become the
    reference's rcontrib modifier arguments, which the oracle traces to the
    reference's pass-through matrices (sky in Reinhart bins through the glass,
    the window opening in Klems bins; 1e-6), and the host's Klems sender rays
    give the reference's sender matrix within sampling error."""
    from pyradiance_gb300 import rflux
    from pyradiance_gb300 import workloads as w
    g = golden("flux_matrices.npz")
    f = w.flux_files()
    for k, v in f.items():
        (tmp_path / f"{k}.rad").write_text(v)
    o = po.default_opts("rcontrib", ab=0, u=0)
    for key, recv, scene in (("sky", "sky", "system"), ("window_kf", "window_kf", "interior")):
        specs = rflux._receivers(tmp_path / f"{recv}.rad")
        (tmp_path / "all.rad").write_text(f[scene] + f[recv])
        out, _ = po.rcontrib(po.Scene(tmp_path / "all.rad"), o, specs, g["rays"], threads=8)
        np.testing.assert_allclose(out, g[key], rtol=1e-6, atol=1e-9)
    n = int(g["send_count"])
    rays, nb = rflux._sender_rays(rflux._sender(tmp_path / "window_send.rad"), n, np.random.default_rng(0))
    assert nb == 145 and rays.shape == (145 * n, 6)
    o.c = n
    (tmp_path / "all.rad").write_text(f["obstruction"] + f["sky"])
    out, _ = po.rcontrib(po.Scene(tmp_path / "all.rad"), o, rflux._receivers(tmp_path / "sky.rad"), rays,
                         threads=8)
    flux_close(out[:, :, 0], g["send"][:, :, 0], n)


def test_flux_shirchiu(tmp_path):
    """Shirley-Chiu bases (h=sc4, util/disk2square.cal) in rfluxmtx: the
    window opening as a receiver, view rays passed through (1e-6), and the
    window as a sender within sampling error."""
    from pyradiance_gb300 import rflux
    from pyradiance_gb300 import workloads as w
    g = golden("flux_shirchiu.npz")
    f = w.flux_files()
    (tmp_path / "recv.rad").write_text(f["window_kf"].replace("h=kf u=Z", "h=sc4 u=Z"))
    (tmp_path / "send.rad").write_text(f["window_send"].replace("h=kf u=Z", "h=sc4 u=Z"))
    (tmp_path / "sky.rad").write_text(f["sky"])
    o = po.default_opts("rcontrib", ab=0, u=0)
    (tmp_path / "all.rad").write_text(f["interior"] + f["window_kf"])
    out, _ = po.rcontrib(po.Scene(tmp_path / "all.rad"), o, rflux._receivers(tmp_path / "recv.rad"), g["rays"],
                         threads=8)
    np.testing.assert_allclose(out, g["window_sc"], rtol=1e-6, atol=1e-9)
    n = int(g["send_count"])
    rays, nb = rflux._sender_rays(rflux._sender(tmp_path / "send.rad"), n, np.random.default_rng(0))
    assert nb == 16
    o.c = n
    (tmp_path / "all.rad").write_text(f["obstruction"] + f["sky"])
    out, _ = po.rcontrib(po.Scene(tmp_path / "all.rad"), o, rflux._receivers(tmp_path / "sky.rad"), rays,
                         threads=8)
    flux_close(out[:, :, 0], g["send"][:, :, 0], n)


def test_instances():
    """Instanced octrees (rt/o_instance.c:15-71, common/instance.c,
    common/xf.c): the furniture octree 12 times in the room, rotated,
    scaled, mirrored, some with their own material.  Hit surfaces by name
    (the instance's when it has a modifier), distances, -ab 0 radiance and
    -I irradiance."""
    g = golden("instances.npz")
    sc = po.Scene(Path(__file__).resolve().parent / "golden" / "inst_main.oct")
    o = po.default_opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, u=0)
    rgb, hid, ht, _ = po.rtrace(sc, o, g["rays"], threads=8)
    names = np.array([sc.object_name(i) if i >= 0 else "*" for i in hid])
    assert (names == g["hit_name"]).all(), np.nonzero(names != g["hit_name"])
    hit = g["hit_dist"] < 1e9
    np.testing.assert_allclose(ht[hit], g["hit_dist"][hit], rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(rgb, g["radiance"], rtol=1e-6, atol=1e-9)
    o.I = 1
    irr, _, _, _ = po.rtrace(sc, o, g["rays"], hits=False, threads=8)
    np.testing.assert_allclose(irr, g["irradiance"], rtol=1e-6, atol=1e-9)


def test_meshes():
    """Compiled meshes (rt/o_mesh.c, common/mesh.c, common/readmesh.c):
    the reference obj2mesh's mesh of a sphere and a bumpy sheet, 10 times in
    the room, rotated, scaled, mirrored, some with their own material.  Hit
    surfaces by name (the mesh's when it has a modifier, else the
    reference's triangle pseudo object "M-Tri"), distances, -ab 0 radiance
    and -I irradiance."""
    g = golden("meshes.npz")
    sc = po.Scene(Path(__file__).resolve().parent / "golden" / "mesh_room.oct")
    o = po.default_opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, u=0)
    rgb, hid, ht, _ = po.rtrace(sc, o, g["rays"], threads=8)
    names = np.array([sc.object_name(i) if i >= 0 else "*" for i in hid])
    assert (names == g["hit_name"]).all(), np.nonzero(names != g["hit_name"])
    assert (names == "M-Tri").sum() > 100 and np.char.startswith(names, "mesh").sum() > 100
    hit = g["hit_dist"] < 1e9
    np.testing.assert_allclose(ht[hit], g["hit_dist"][hit], rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(rgb, g["radiance"], rtol=1e-6, atol=1e-9)
    o.I = 1
    irr, _, _, _ = po.rtrace(sc, o, g["rays"], hits=False, threads=8)
    np.testing.assert_allclose(irr, g["irradiance"], rtol=1e-6, atol=1e-9)


def test_mesh_with_vertex_normals_refused_by_the_oracle():
    """A mesh whose vertices carry normals (rt/o_mesh.c:198-206 perturbs the
    shading normal with them) is read by the scene reader, but the oracle
    does not restate that shading and refuses the scene; the GPU path is
    checked against the reference's own output for it."""
    with pytest.raises(RuntimeError, match="normals are not supported by the oracle"):
        po.Scene(Path(__file__).resolve().parent / "golden" / "mesh_normals.oct")


def test_zoo_cast_and_direct(oscenes):
    g = golden("zoo.npz")
    sc = oscenes["zoo"]
    o = po.default_opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, u=0)
    rgb, hid, ht, _ = po.rtrace(sc, o, g["rays"])
    names = np.array([sc.object_name(i) if i >= 0 else "*" for i in hid])
    assert (names == g["hit_name"]).mean() == 1.0
    # the reference read a frozen octree (31-bit mantissas); near-tangent
    # hits on curved surfaces amplify that to a few 1e-6
    np.testing.assert_allclose(ht, g["hit_dist"], rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(rgb, g["radiance"], rtol=1e-5, atol=1e-9)
    o.I = 1
    irr, _, _, _ = po.rtrace(sc, o, g["rays"], hits=False)
    np.testing.assert_allclose(irr, g["irradiance"], rtol=1e-6, atol=1e-9)


@pytest.mark.skipif(not REF_TRACE.exists(), reason="reference test fixture not present")
def test_reference_fixture_trace_oct():
    g = golden("ref_trace_oct.npz")
    sc = po.Scene(REF_TRACE)
    o = po.default_opts("rtrace", ab=0, u=0)
    _, hid, ht, _ = po.rtrace(sc, o, g["rays"], values=False)
    names = np.array([sc.object_name(i) if i >= 0 else "*" for i in hid])
    assert (names == g["hit_name"]).all()
    np.testing.assert_allclose(ht, g["hit_dist"], rtol=1e-8)


def test_dctimestep_oracle():
    g = golden("dct_small.npz")
    out = po.dctimestep(g["dc"], g["sky"])
    np.testing.assert_array_equal(out, g["out"])


def test_dctimestep_four_matrix_oracle():
    """V x T x D x sky as the reference multiplies it (D x sky, then T, then
    V, float intermediates): the oracle's product chain within 1e-6."""
    g = golden("dct_four.npz")
    out = po.dctimestep(g["V"], po.dctimestep(g["T"], po.dctimestep(g["D"], g["S"])))
    np.testing.assert_allclose(out, g["out"], rtol=1e-6, atol=1e-12)


def check_c2_statistics(a, g, K):
    """a: (sensors, K, 146) samples of channel 0.  Compares with the golden
    reference statistics: per-sensor totals, per-sensor altitude-row groups
    and the individual bins that both sides sample often enough for a
    normal approximation (z-scores of the difference of means)."""
    from conftest import ROW_EDGES
    zt = zscores(a.sum(2).mean(1), a.sum(2).std(1, ddof=1) / np.sqrt(K), g["total_mean"], g["total_se"])
    assert np.abs(zt).max() < 4.5, zt
    assert abs(zt.mean()) < 1.0, zt
    grp = np.stack([a[:, :, e0:e1].sum(2) for e0, e1 in zip(ROW_EDGES[:-1], ROW_EDGES[1:])], 2)
    gm, gs = grp.mean(1), grp.std(1, ddof=1) / np.sqrt(K)
    gn = (grp > 0).sum(1)
    ok = (gn >= 10) & (g["group_se"] > 0)
    zg = (gm - g["group_mean"])[ok] / np.sqrt(gs ** 2 + g["group_se"] ** 2)[ok]
    assert len(zg) >= 20
    assert abs(zg.mean()) < 0.5 and zg.std() < 1.5 and np.abs(zg).max() < 5, (zg.mean(), zg.std())
    nz = (a > 0).sum(1)
    okb = (nz >= 10) & (g["nnz"] >= 10 * g["K"] // K)
    zb = (a.mean(1) - g["mean"])[okb] / np.sqrt((a.std(1, ddof=1) / np.sqrt(K)) ** 2 + g["se"] ** 2)[okb]
    if len(zb) >= 20:
        assert abs(zb.mean()) < 0.5 and zb.std() < 1.5 and (np.abs(zb) > 4).mean() < 0.01, (zb.mean(), zb.std())
    return zt, zg, zb


def headline_stats(a, g):
    """a: (sensors, K, 146) samples of channel 0 of the headline rcontrib
    workload; g: the reference's statistics of the same 256 sensors (64
    replicas of 1,024 first-hemisphere samples).  Returns
      z   the z-scores (difference of means over the combined standard
          error) of every sensor x bin that both sides sample in at least
          two replicas;
      zg  the same for each sensor's sums over the Reinhart altitude rows
          (and the ground bin), where both sides sample the row in a
          quarter of their replicas or more;
      p   for every sensor x bin that either side samples, the two-sided
          p-value of its replica counts under equal rates (given the total
          count, this side's count is binomial with probability K/(K+Kr)).
    Most sensor x bin pairs are sampled by neither side (sensors under
    boxes, bins no path reaches)."""
    from scipy.stats import binom
    from conftest import ROW_EDGES
    K, Kr = a.shape[1], int(g["K"])
    m, se, nn = a.mean(1), a.std(1, ddof=1) / np.sqrt(K), (a > 0).sum(1)
    rm, rse, rn = g["mean"].astype(np.float64), g["se"].astype(np.float64), g["nnz"].astype(np.int64)
    both = (nn >= 2) & (rn >= 2)
    z = (m - rm)[both] / np.sqrt(se ** 2 + rse ** 2)[both]
    grp = np.stack([a[:, :, e0:e1].sum(2) for e0, e1 in zip(ROW_EDGES[:-1], ROW_EDGES[1:])], 2)
    gm, gs, gn = grp.mean(1), grp.std(1, ddof=1) / np.sqrt(K), (grp > 0).sum(1)
    ok = (gn * 4 >= K) & (g["group_se"] > 0)
    zg = (gm - g["group_mean"])[ok] / np.sqrt(gs ** 2 + g["group_se"] ** 2)[ok]
    any_ = (nn > 0) | (rn > 0)
    x, t = nn[any_], (nn + rn)[any_]
    q = K / (K + Kr)
    p = np.minimum(1.0, 2 * np.minimum(binom.cdf(x, t, q), binom.sf(x - 1, t, q)))
    return z, zg, p


def within_normal_rate(z, zmax):
    """The share of |z| beyond 3 may exceed its rate under equal means
    (0.27%) by at most four binomial standard deviations; no |z| beyond
    zmax."""
    n, p3 = len(z), 0.0027
    share = (np.abs(z) > 3).mean()
    assert share <= p3 + 4 * np.sqrt(p3 * (1 - p3) / n), (share, n)
    assert np.abs(z).max() <= zmax, np.sort(np.abs(z))[-5:]


def check_headline_bins(a, g):
    """Every sensor x bin mean that both sides sample twice or more within
    the reference's at the rate a normal variable allows, none beyond 5.5
    standard errors (probability about 1e-3 over these bins under equal
    means); every sensor's altitude-row sums likewise, none beyond 5, their
    mean z within four standard errors of 0; the sampling rate of every bin
    that either side reaches consistent with the reference's (count
    p-values: at most 0.27% below 0.0027 plus four binomial standard
    deviations, none below 1e-3 / the number of bins)."""
    z, zg, p = headline_stats(a, g)
    assert len(z) >= 1000 and len(zg) >= 300 and len(p) >= 2000, (len(z), len(zg), len(p))
    within_normal_rate(z, 5.5)
    within_normal_rate(zg, 5.0)
    assert abs(zg.mean()) < 4 / np.sqrt(len(zg)), zg.mean()
    n, p3 = len(p), 0.0027
    assert (p < p3).mean() <= p3 + 4 * np.sqrt(p3 * (1 - p3) / n), ((p < p3).mean(), n)
    assert p.min() * n >= 1e-3, np.sort(p)[:5]
    return z, zg, p


def test_headline_rcontrib_bins_vs_reference(oscenes):
    """The oracle at 64 replicas of the headline workload's 256 sensors
    against the reference's 64 independent replicas (2^16 first-hemisphere
    samples per sensor on each side): per sensor x bin.  Equal replica
    counts keep the comparison symmetric: the mean of a few skewed samples
    falls below the true mean more often than above, and unequal counts
    would shift the z-scores."""
    g = golden("c2_headline.npz")
    K = int(g["K"])
    rays = np.repeat(g["rays"], K, axis=0)
    o = po.default_opts("rcontrib", I=1, ab=3, ad=1024, lw=1e-4, c=1, u=0, seed=97)
    out, _ = po.rcontrib(oscenes["c2"], o, MODS_C2, rays, threads=os.cpu_count() or 1)
    z, zg, p = check_headline_bins(out[..., 0].reshape(len(g["rays"]), K, 146), g)
    print("oracle vs reference: %d bins, share |z|>3 %.4f, max %.2f; %d row sums, max %.2f; %d counts, "
          "min p %.2g" % (len(z), (np.abs(z) > 3).mean(), np.abs(z).max(), len(zg), np.abs(zg).max(), len(p),
                          p.min()))


@pytest.mark.parametrize("ab,K", [(1, 128), (3, 48)])
def test_c2_rcontrib_statistics(oscenes, ab, K):
    """Sample means of the oracle agree with the reference's -u+ runs within
    their standard errors."""
    g = golden(f"c2_stats_ab{ab}.npz")
    sc = oscenes["c2"]
    rays = np.repeat(g["rays"], K, axis=0)
    o = po.default_opts("rcontrib", I=1, ab=ab, ad=1024, lw=1e-4, c=1, u=0, seed=12345)
    out, nr = po.rcontrib(sc, o, MODS_C2, rays, threads=8)
    check_c2_statistics(out[..., 0].reshape(len(g["rays"]), K, 146), g, K)
