"""GPU path against the golden vectors and the CPU oracle (needs a GB300).

Every call goes through the C ABI of libgbrad.so (ctypes).
Tolerances: bit-exact first-hit objects; FP32 traversal and shading give
values within 1e-5 relative of the reference for the deterministic direct
cases (the bar of the deterministic rtrace workload), 1e-4 for distances
and for radiance chains through mirrors; Monte Carlo results are compared
with the oracle sample for sample (same random streams) and with the
reference statistically.
"""
import numpy as np
import pytest

from conftest import MODS_C2, golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import _lib
    _lib.lib()
    return gb


@pytest.fixture(scope="module")
def scenes(gb, scene_dir):
    return {k: gb.Scene(rad_files=[scene_dir / f"{k}.rad"]) for k in ("c1", "c2", "zoo", "c2e", "glossy")}


def opts(prog, **kw):
    from pyradiance_gb300 import _lib
    o, _ = _lib.parse_opts([], _lib.GB_PROG_RCONTRIB if prog == "rcontrib" else _lib.GB_PROG_RTRACE)
    for k, v in kw.items():
        setattr(o, "as_" if k == "as" else k, v)
    return o


def rtrace_c(gb, sc, o, rays, values=True):
    from pyradiance_gb300 import _lib
    rays = np.ascontiguousarray(rays, dtype=np.float64)
    n = len(rays)
    rgb = np.zeros((n, 3)) if values else None
    hid = np.zeros(n, dtype=np.int32)
    ht = np.zeros(n)
    _lib.check(_lib.lib().gb_rtrace(sc.handle, o, _lib.ptr(rays), n, _lib.ptr(rgb), _lib.ptr(hid), _lib.ptr(ht)))
    return rgb, hid, ht


def rcontrib_c(gb, sc, o, rays, mods=MODS_C2):
    rc = gb.Rcontrib(b"", sc)
    for m in mods:
        rc.add_modifier(**{{"expr": "expression", "params": "param"}.get(k, k): v for k, v in m.items()})
    rc.args = []
    rc.seed = int(o.seed)
    from pyradiance_gb300 import _lib
    out_opts = o

    # run through the C ABI with exactly these options
    specs, keep = rc._specs()
    nb = _lib.C.c_int(0)
    _lib.check(_lib.lib().gb_rcontrib_nbins(specs, len(rc.mods), _lib.C.byref(nb)))
    rays = np.ascontiguousarray(rays, dtype=np.float64)
    out = np.zeros((len(rays) // max(1, out_opts.c), nb.value, 3))
    cnt = _lib.C.c_int64(0)
    _lib.check(_lib.lib().gb_rcontrib(sc.handle, out_opts, specs, len(rc.mods), _lib.ptr(rays), len(rays),
                                      _lib.ptr(out), _lib.C.byref(cnt)))
    return out, cnt.value


def names_of(sc, hid):
    return np.array([sc.object_name(int(i)) if i >= 0 else "*" for i in hid])


def test_c1_hit_ids_bit_exact(gb, scenes):
    g = golden("c1_direct.npz")
    sc = scenes["c1"]
    _, hid, ht = rtrace_c(gb, sc, opts("rtrace", ab=0, u=0), g["rays"], values=False)
    assert (names_of(sc, hid) == g["hit_name"]).all()
    np.testing.assert_allclose(ht, g["hit_dist"], rtol=1e-5)


def test_c1_direct_irradiance(gb, scenes):
    g = golden("c1_direct.npz")
    sc = scenes["c1"]
    rgb, _, _ = rtrace_c(gb, sc, opts("rtrace", I=1, ab=0, dj=0, ds=0, dr=0, u=0), g["rays"])
    ref = g["irradiance"]
    lit = ref[:, 0] > 0
    np.testing.assert_array_equal(rgb[~lit], 0.0)
    rel = np.abs(rgb[lit] - ref[lit]) / ref[lit]
    assert rel.max() < 1e-5, rel.max()


def test_c1_partitioned_source(gb, scenes):
    """-ds 0.2 (rtrace's default): the light split into pieces by distance
    (rt/srcsamp.c:260-330), every piece's shadow tested (-dt 0).  Where a
    sensor's distance to a piece's centre sits within FP32 rounding of the
    splitting threshold the GPU may split differently from the reference,
    which changes that sensor's estimate by the quadrature difference of
    the two splits: at least 99.5% of the lit sensors within 1e-5 relative,
    all within 1e-2."""
    g = golden("c1_partitioned.npz")
    rgb, _, _ = rtrace_c(gb, scenes["c1"], opts("rtrace", I=1, ab=0, dj=0, ds=0.2, dr=0, dt=0, u=0), g["rays"])
    ref = g["irradiance"]
    lit = ref[:, 0] > 0
    np.testing.assert_array_equal(rgb[~lit], 0.0)
    rel = np.abs(rgb[lit] - ref[lit]).max(1) / ref[lit].max(1)
    print("partitioned source: max rel %.3g, share above 1e-5 %.4f" % (rel.max(), (rel > 1e-5).mean()))
    assert (rel <= 1e-5).mean() >= 0.995 and rel.max() < 1e-2


def test_glossy_direct_lobe(gb, scenes):
    """Rough plastic and metal below -st 1: diffuse plus the direct Gaussian
    specular term, deterministic.  Paths through the pure-metal boxes are
    mirror chains (1e-4, as for the shape zoo); a ray whose mirror chain
    meets an edge within FP32 rounding may end on another surface."""
    g = golden("glossy.npz")
    rgb, _, _ = rtrace_c(gb, scenes["glossy"], opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, st=1, u=0), g["rays"])
    ref = g["radiance_st1"]
    rel = np.abs(rgb - ref).max(1) / np.maximum(np.abs(ref).max(1), 1e-9)
    assert (rel <= 1e-4).mean() >= 0.99 and np.median(rel) < 1e-5, (np.median(rel), np.sort(rel)[-5:])


@pytest.mark.parametrize("kw", [{"st": 0}, {"ss": 3}])
def test_glossy_lobe_matches_oracle_sample_for_sample(gb, scenes, scene_dir, kw):
    """The sampled specular lobe (rt/normal.c:364-440) with the same random
    streams on the GPU (FP32) and in the oracle (FP64): the same trials are
    taken and rejected, so values agree closely ray for ray; a sample that
    grazes an edge can end on another surface."""
    from oracle import pyoracle as po
    g = golden("glossy.npz")
    rays = np.repeat(g["rays"], 4, axis=0)
    o = opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, u=0, seed=99, **kw)
    rgb, _, _ = rtrace_c(gb, scenes["glossy"], o, rays)
    oo = po.default_opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, u=0, seed=99, **kw)
    ref, _, _, _ = po.rtrace(po.Scene(scene_dir / "glossy.rad"), oo, rays, hits=False, threads=8)
    rel = np.abs(rgb - ref).max(1) / np.maximum(np.abs(ref).max(1), 1e-9)
    assert np.median(rel) < 1e-5 and (rel <= 1e-3).mean() >= 0.98, (np.median(rel), (rel > 1e-3).mean())


@pytest.mark.parametrize("key,kw", [("st0", {"st": 0}), ("ss3", {"ss": 3})])
def test_glossy_lobe_statistics_vs_reference(gb, scenes, key, kw):
    """Per-ray means of 1,024 replicas against the reference's 1,024 (-u+):
    z-scores within 5, their mean within 4 standard errors of zero."""
    g = golden("glossy.npz")
    n, K = len(g["rays"]), 1024
    rgb, _, _ = rtrace_c(gb, scenes["glossy"], opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, u=0, seed=5, **kw),
                         np.repeat(g["rays"], K, axis=0))
    a = rgb.reshape(n, K, 3)
    m, se = a.mean(1), a.std(1, ddof=1) / np.sqrt(K)
    rm = g[f"{key}_mean"]
    z = (m - rm) / np.sqrt(se ** 2 + g[f"{key}_se"] ** 2 + (1e-5 * np.abs(rm) + 1e-9) ** 2)
    print("glossy %s: max |z| %.2f, mean z %.3f" % (key, np.abs(z).max(), z.mean()))
    assert np.abs(z).max() < 5 and abs(z.mean()) < 4 / np.sqrt(n)


def test_first_hit_normals(gb, scenes, tmp_path):
    """rtrace -oN and -on (rt/rtrace.c:787-820) through the drop-in: the
    surface's own normal at the first hit (FP64 casts) and the shading
    normal, turned toward the ray where plastic, metal, trans or glass meet
    a surface from behind, for every primitive of the shape zoo and for rays
    through the window glass from both sides: the reference's within 1e-6."""
    from pyradiance_gb300 import workloads as w
    g = golden("normals.npz")
    (tmp_path / "win.rad").write_text(w.window_room(ntri=0))
    for key, sc in (("zoo", scenes["zoo"]), ("win", gb.Scene(rad_files=[tmp_path / "win.rad"]))):
        rays = g[f"{key}_rays"]
        out = gb.rtrace(rays.astype("<f8").tobytes(), sc, params=["-ab", "0"], inform="d", outform="d",
                        outspec="Nn", header=False)
        v = np.frombuffer(out, dtype="<f8").reshape(-1, 6)
        np.testing.assert_allclose(v[:, :3], g[f"{key}_N"], rtol=1e-6, atol=1e-6, err_msg=key)
        np.testing.assert_allclose(v[:, 3:], g[f"{key}_n"], rtol=1e-6, atol=1e-6, err_msg=key)
    # -oV and -oW of primary rays (rt/rtrace.c:734-743, 847-860): the contribution is the value, the
    # coefficient one, as in the reference's output
    ref = g["zoo_VWv"]
    assert (ref[:, :3] == ref[:, 6:]).all() and (ref[:, 3:6] == 1).all()
    out = gb.rtrace(g["zoo_rays"][:500].astype("<f8").tobytes(), scenes["zoo"], inform="d", outform="d",
                    outspec="VWv", header=False, params=["-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0"])
    v = np.frombuffer(out, dtype="<f8").reshape(-1, 9)
    assert (v[:, :3] == v[:, 6:]).all() and (v[:, 3:6] == 1).all()
    rel = np.abs(v[:, 6:] - ref[:, 6:]).max(1) / np.maximum(np.abs(ref[:, 6:]).max(1), 1e-9)
    assert (rel <= 1e-4).mean() >= 0.99


def test_zoo_all_primitives(gb, scenes):
    g = golden("zoo.npz")
    sc = scenes["zoo"]
    o = opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, u=0)
    rgb, hid, ht = rtrace_c(gb, sc, o, g["rays"])
    names = names_of(sc, hid)
    match = names == g["hit_name"]
    assert match.all(), np.nonzero(~match)                    # first hits cast in FP64
    ok = match & (g["hit_dist"] < 1e9)
    np.testing.assert_allclose(ht[ok], g["hit_dist"][ok], rtol=1e-6, atol=1e-7)  # distances stored in FP32
    np.testing.assert_allclose(rgb[match], g["radiance"][match], rtol=1e-4, atol=1e-6)
    o.I = 1
    irr, _, _ = rtrace_c(gb, sc, o, g["rays"])
    # -I at the ray origin: the value is proportional to the cosine between
    # the sensor direction and the direction to the light's centre (the one
    # sample of -ds 0).  That direction is formed in FP32 from positions of
    # a few metres, an angular error of about 1e-6 rad, so the relative
    # error is bounded by 1e-5 + 1e-6 / cosine: grazing sensors amplify it.
    rays = g["rays"]
    to_light = np.array([5.0, 4.0, 2.99]) - rays[:, :3]
    to_light /= np.linalg.norm(to_light, axis=1, keepdims=True)
    cosine = np.abs((rays[:, 3:] / np.linalg.norm(rays[:, 3:], axis=1, keepdims=True) * to_light).sum(1))
    bound = (1e-5 + 1e-6 / np.maximum(cosine, 1e-3))[:, None] * np.abs(g["irradiance"]) + 1e-6
    err = np.abs(irr - g["irradiance"])
    assert (err <= bound).all(), (np.nonzero((err > bound).any(1))[0], err.max())
    # isotropic directions: about 5% of the rays are within 0.05 of grazing
    assert (cosine < 0.05).mean() < 0.08


def test_c2_matches_oracle_sample_for_sample(gb, scenes, scene_dir):
    """Same random streams on the GPU (FP32) and in the oracle (FP64):
    per-record sums agree closely; a path that diverges near an edge moves
    at most one sample's coefficient."""
    from oracle import pyoracle as po
    rays = np.repeat(golden("c2_stats_ab3.npz")["rays"][:8], 4, axis=0)
    o = opts("rcontrib", I=1, ab=3, ad=1024, lw=1e-4, c=1, u=0, seed=777)
    out, nr = rcontrib_c(gb, scenes["c2"], o, rays)
    osc = po.Scene(scene_dir / "c2.rad")
    oo = po.default_opts("rcontrib", I=1, ab=3, ad=1024, lw=1e-4, c=1, u=0, seed=777)
    ref, onr = po.rcontrib(osc, oo, MODS_C2, rays, threads=8)
    ta, tb = out.sum((1, 2)), ref.sum((1, 2))
    rel = np.abs(ta - tb) / np.maximum(tb, 1e-12)
    assert np.median(rel) < 1e-4, rel
    assert (rel < 2e-2).all(), rel
    assert abs(nr - onr) / onr < 1e-3, (nr, onr)
    assert abs(out.sum() - ref.sum()) / ref.sum() < 2e-3


@pytest.mark.parametrize("ab,K", [(1, 256), (3, 256)])
def test_c2_statistics_vs_reference(gb, scenes, ab, K):
    from test_oracle_golden import check_c2_statistics
    g = golden(f"c2_stats_ab{ab}.npz")
    rays = np.repeat(g["rays"], K, axis=0)
    o = opts("rcontrib", I=1, ab=ab, ad=1024, lw=1e-4, c=1, u=0, seed=4242)
    out, _ = rcontrib_c(gb, scenes["c2"], o, rays)
    check_c2_statistics(out[..., 0].reshape(len(g["rays"]), K, 146), g, K)


def test_c2_headline_bins_vs_reference(gb, scenes):
    """The headline rcontrib workload (-I+ -ab 3 -ad 1024 -lw 1e-4 -c 1)
    at 2^16 first-hemisphere samples per sensor: 256 evenly spaced sensors
    of its 64 x 64 grid, 64 replicas each, every sensor x bin mean against
    the reference's 64 independent replicas (z-scores of the difference;
    the bounds of check_headline_bins)."""
    from test_oracle_golden import check_headline_bins
    g = golden("c2_headline.npz")
    K = int(g["K"])
    rays = np.repeat(g["rays"], K, axis=0)
    o = opts("rcontrib", I=1, ab=3, ad=1024, lw=1e-4, c=1, u=0, seed=20261204)
    out, _ = rcontrib_c(gb, scenes["c2"], o, rays)
    z, zg, p = check_headline_bins(out[..., 0].reshape(len(g["rays"]), K, 146), g)
    print("GPU vs reference: %d bins, share |z|>3 %.4f, max %.2f; %d row sums, max %.2f; %d counts, min p %.2g"
          % (len(z), (np.abs(z) > 3).mean(), np.abs(z).max(), len(zg), np.abs(zg).max(), len(p), p.min()))


def test_c2_headline_matches_oracle_sample_for_sample(gb, scenes, scene_dir):
    """The same 256 sensors with the bench's seed, one path set each, on the
    GPU (FP32) and in the oracle (FP64) from the same random streams: every
    record's sum, and the bins summed over all sensors, agree closely."""
    from oracle import pyoracle as po
    rays = golden("c2_headline.npz")["rays"]
    o = opts("rcontrib", I=1, ab=3, ad=1024, lw=1e-4, c=1, u=0, seed=20261203)
    out, nr = rcontrib_c(gb, scenes["c2"], o, rays)
    oo = po.default_opts("rcontrib", I=1, ab=3, ad=1024, lw=1e-4, c=1, u=0, seed=20261203)
    ref, onr = po.rcontrib(po.Scene(scene_dir / "c2.rad"), oo, MODS_C2, rays, threads=16)
    ta, tb = out.sum((1, 2)), ref.sum((1, 2))
    lit = tb > 0
    rel = np.abs(ta - tb)[lit] / tb[lit]
    assert (ta[~lit] == 0).all()
    assert np.median(rel) < 1e-4 and (rel < 2e-2).all(), np.sort(rel)[-5:]
    bins_a, bins_b = out.sum(0)[:, 0], ref.sum(0)[:, 0]
    relb = np.abs(bins_a - bins_b) / np.maximum(bins_b, 1e-300)
    assert np.median(relb[bins_b > 0]) < 1e-3, np.median(relb[bins_b > 0])
    assert abs(nr - onr) / onr < 1e-3, (nr, onr)


def fp32_fp64_convergence(out32, out64, S, K, ks=(1, 4, 16, 64)):
    """Per sensor x bin, the difference of the FP32 and FP64 means over the
    first k replicas against the standard error of the FP64 mean (the FP64
    replicas' spread / sqrt(k)), over bins with at least 10 non-zero
    replicas: the median and 99th percentile of |d| / se, and the median
    relative difference, for each k."""
    a = out32[..., 0].reshape(S, K, -1)
    b = out64[..., 0].reshape(S, K, -1)
    rich = (b > 0).sum(1) >= 10
    rows = []
    for k in ks:
        ma, mb = a[:, :k].mean(1), b[:, :k].mean(1)
        se = b.std(1, ddof=1) / np.sqrt(k)
        d = np.abs(ma - mb)[rich]
        r = d / se[rich]
        pos = mb[rich] > 0
        rel = d[pos] / mb[rich][pos]
        rows.append((k, float(np.median(r)), float(np.quantile(r, 0.99)), float(np.median(rel)),
                     float(np.quantile(rel, 0.99))))
    return rows


def test_c2_fp32_converges_to_fp64(gb, scenes, scene_dir):
    """The headline rcontrib workload on 64 of its sensors, 64 path sets
    each: the GPU's FP32 path against the oracle's FP64 restatement of the
    same paths (same random streams).  At every number of path sets the
    FP32 - FP64 difference of each sensor x bin mean is at the level of FP32
    rounding (measured: 1e-7 relative, 99th percentile) and some 1e6 times
    smaller than the Monte Carlo standard error: FP32 arithmetic adds no
    error that sampling at 2^16 samples per sensor could reveal."""
    from oracle import pyoracle as po
    S, K = 64, 64
    rays = np.repeat(golden("c2_headline.npz")["rays"][::4][:S], K, axis=0)
    o = opts("rcontrib", I=1, ab=3, ad=1024, lw=1e-4, c=1, u=0, seed=20261205)
    out, _ = rcontrib_c(gb, scenes["c2"], o, rays)
    oo = po.default_opts("rcontrib", I=1, ab=3, ad=1024, lw=1e-4, c=1, u=0, seed=20261205)
    ref, _ = po.rcontrib(po.Scene(scene_dir / "c2.rad"), oo, MODS_C2, rays, threads=16)
    rows = fp32_fp64_convergence(out, ref, S, K)
    for k, med, p99, rmed, r99 in rows:
        print("k=%2d path sets: |FP32-FP64|/se median %.2e p99 %.2e; relative median %.2e p99 %.2e"
              % (k, med, p99, rmed, r99))
    for k, med, p99, rmed, r99 in rows:
        assert p99 < 1e-3 and r99 < 1e-5, (k, p99, r99)


def test_c2_full_grid_bins_equal_irradiance(gb, scenes):
    """Size-independent property at the full 64 x 64 grid: the sky and
    ground glows have radiance 1, so each sensor's coefficients summed over
    all 146 bins equal its rtrace -I irradiance from the same random
    streams."""
    from pyradiance_gb300 import workloads as w
    rays = w.sensor_grid(64, 64)
    o = opts("rcontrib", I=1, ab=3, ad=1024, lw=1e-4, c=1, u=0, seed=99)
    out, nr = rcontrib_c(gb, scenes["c2"], o, rays)
    ort = opts("rtrace", I=1, ab=3, ad=1024, lw=1e-4, aa=0, as_=0, u=0, seed=99, dj=0.9, ds=0.2, st=0.02, dt=0)
    rgb, _, _ = rtrace_c(gb, scenes["c2"], ort, rays)
    np.testing.assert_allclose(out.sum(1)[:, 0], rgb[:, 0], rtol=1e-5, atol=1e-12)
    assert nr > 4096 * 5000


def test_supersampled_matches_oracle_sample_for_sample(gb, scenes, scene_dir):
    """rtrace -I -ab 2 -aa 0 -ad 256 with -as 512 (rtrace's default): the
    16 x 16 first hemispheres get 512 extra samples each after the first
    pass, placed by their strata's brightness differences.  Same streams on
    the GPU and in the oracle: the extra samples' placement depends on
    FP32 versus FP64 values only where a stratum's share rounds differently,
    so sensors agree closely."""
    from oracle import pyoracle as po
    g = golden("supersampled.npz")
    rays = np.repeat(g["rays"][:40], 3, axis=0)
    o = opts("rtrace", I=1, ab=2, aa=0, ad=256, lw=1e-4, dj=0, ds=0, dr=0, dt=0, u=0, seed=12)
    assert o.as_ == 512
    rgb, _, _ = rtrace_c(gb, scenes["c1"], o, rays)
    oo = po.default_opts("rtrace", I=1, ab=2, aa=0, ad=256, lw=1e-4, dj=0, ds=0, dr=0, dt=0, u=0, seed=12)
    ref, _, _, _ = po.rtrace(po.Scene(scene_dir / "c1.rad"), oo, rays, hits=False, threads=16)
    rel = np.abs(rgb - ref).max(1) / np.maximum(np.abs(ref).max(1), 1e-9)
    print("super-sampled vs oracle: median rel %.3g, share above 1e-3 %.3f, max %.3g" %
          (np.median(rel), (rel > 1e-3).mean(), rel.max()))
    assert np.median(rel) < 1e-4 and (rel <= 1e-3).mean() >= 0.9 and rel.max() < 5e-2


@pytest.mark.parametrize("key,asn", [("as512", 512), ("as0", 0)])
def test_supersampled_statistics_vs_reference(gb, scenes, key, asn):
    """Per-sensor means of 512 replicas against the reference's 512 (-u+),
    with and without super-sampling: z-scores within 5, their mean within 4
    standard errors of zero."""
    g = golden("supersampled.npz")
    n, K = len(g["rays"]), 512
    o = opts("rtrace", I=1, ab=2, aa=0, ad=256, lw=1e-4, dj=0, ds=0, dr=0, dt=0, u=0, seed=77, as_=asn)
    rgb, _, _ = rtrace_c(gb, scenes["c1"], o, np.repeat(g["rays"], K, axis=0))
    a = rgb.reshape(n, K, 3)
    m, se = a.mean(1), a.std(1, ddof=1) / np.sqrt(K)
    rm = g[f"{key}_mean"]
    z = (m - rm) / np.sqrt(se ** 2 + g[f"{key}_se"] ** 2 + (1e-5 * np.abs(rm) + 1e-9) ** 2)
    print("super-sampling %s: max |z| %.2f, mean z %.3f" % (key, np.abs(z).max(), z.mean()))
    assert np.abs(z).max() < 5 and abs(z.mean()) < 4 / np.sqrt(n)


@pytest.mark.parametrize("key", ["c1", "c2e"])
def test_surface_irradiance(gb, scenes, key):
    """-i (rt/raytrace.c:211-236): primary hits on non-light materials as a
    Lambertian of reflectance pi, glass passed through; deterministic with
    -ab 0.  The hit point is FP32, so a sensor near a shadow edge may differ
    by the share of the light it sees from there."""
    g = golden("surface_irradiance.npz")
    rgb, _, _ = rtrace_c(gb, scenes[key], opts("rtrace", i=1, ab=0, dj=0, ds=0, dr=0, dt=0, u=0), g[f"{key}_rays"])
    ref = g[f"{key}_irr"]
    rel = np.abs(rgb - ref).max(1) / np.maximum(np.abs(ref).max(1), 1e-9)
    assert np.median(rel) < 1e-5 and (rel <= 1e-4).mean() >= 0.99, (np.median(rel), (rel > 1e-4).mean())


def test_surface_irradiance_one_bounce(gb, scenes):
    g = golden("surface_irradiance.npz")
    n, K = len(g["ab1_rays"]), 256
    o = opts("rtrace", i=1, ab=1, aa=0, as_=0, ad=256, lw=1e-4, dj=0, ds=0, dr=0, dt=0, u=0, seed=3)
    rgb, _, _ = rtrace_c(gb, scenes["c1"], o, np.repeat(g["ab1_rays"], K, axis=0))
    a = rgb.reshape(n, K, 3)
    m, se = a.mean(1), a.std(1, ddof=1) / np.sqrt(K)
    z = (m - g["ab1_mean"]) / np.sqrt(se ** 2 + g["ab1_se"] ** 2 + (1e-5 * np.abs(g["ab1_mean"]) + 1e-9) ** 2)
    print("-i -ab 1: max |z| %.2f, mean z %.3f" % (np.abs(z).max(), z.mean()))
    assert np.abs(z).max() < 5 and abs(z.mean()) < 4 / np.sqrt(n)


def test_general_bin_expressions(gb, scenes):
    """Bins from a function file of our own (recursion on constant
    arguments, select, if, asin, atan2, floor, sqrt, max, min, ^), compiled
    to the device byte code: rcontrib -ab 0 radiance-mode rays leaving
    through the window each land in the reference's bin (FP32 directions:
    a ray within rounding of a bin edge may land beside it), values within
    1e-5."""
    from test_oracle_golden import MODS_PATCH
    g = golden("general_bins.npz")
    out, _ = rcontrib_c(gb, scenes["c2e"], opts("rcontrib", I=0, ab=0, c=1, u=0), g["rays"], mods=MODS_PATCH)
    got = out[..., 0]
    same = ((got > 0) == (g["bins"] > 0)).all(1)
    assert same.mean() >= 0.999, np.nonzero(~same)
    np.testing.assert_allclose(got[same], g["bins"][same], rtol=1e-5, atol=1e-9)


def test_cie_sky_scanner_bins(gb, tmp_path):
    """CIE sky scanner bins (util/cieskyscan.cal cbin) built into the
    device byte code: rays in every direction through a scene of the sky
    and ground glows land in the reference's bin (FP32 directions: a ray
    within rounding of a bin edge may land beside it), for the default and
    a quarter-turned frame."""
    from pyradiance_gb300 import workloads as w
    g = golden("cie_bins.npz")
    (tmp_path / "sky.rad").write_text(w.SKY_GLOW)
    sc = gb.Scene(rad_files=[tmp_path / "sky.rad"])
    for key, params in (("default", None), ("upx", "Ux=1,Uy=0,Uz=0")):
        mods = [dict(modifier=m, calfile="cieskyscan.cal", binv="cbin", nbins="Ncbins", **(
            {"params": params} if params else {})) for m in ("skyglow", "groundglow")]
        out, _ = rcontrib_c(gb, sc, opts("rcontrib", I=0, ab=0, c=1, u=0), g["rays"], mods=mods)
        got = out[..., 0]
        same = ((got > 0) == (g[key] > 0)).all(1)
        assert same.mean() >= 0.999, (key, np.nonzero(~same))
        np.testing.assert_allclose(got[same], g[key][same], rtol=1e-5, atol=1e-9, err_msg=key)


def test_translucent(gb, tmp_path, scene_dir):
    """The trans material (rt/normal.c, MAT_TRANS): -I irradiance through
    the diffuser (shadow rays continue through its specular transmission)
    and radiance of view rays with -ab 0 -st 1 against the reference
    (99% within 1e-4: view rays through the diffuser continue as
    transmitted rays); aimed view rays with -ab 1 -st 0 (ambient from both
    sides, both lobes sampled) ray for ray against the oracle on the same
    streams, and means of 256 replicas within 5 standard errors of the
    reference's."""
    from oracle import pyoracle as po
    from pyradiance_gb300 import workloads as w
    g = golden("translucent.npz")
    (tmp_path / "trans.rad").write_text(w.trans_room())
    sc = gb.Scene(rad_files=[tmp_path / "trans.rad"])
    for key, rays, I in (("irradiance", g["grid"], 1), ("radiance", g["view"], 0)):
        rgb, _, _ = rtrace_c(gb, sc, opts("rtrace", I=I, ab=0, dj=0, ds=0, dr=0, dt=0, st=1, u=0), rays)
        rel = np.abs(rgb - g[key]).max(1) / np.maximum(np.abs(g[key]).max(1), 1e-9)
        assert (rel <= 1e-4).mean() >= 0.99 and np.median(rel) < 1e-5, (key, np.sort(rel)[-5:])
    kw = dict(ab=1, aa=0, as_=0, ad=256, lw=1e-4, dj=0, ds=0, dr=0, dt=0, st=0, u=0)
    rays = np.repeat(g["aimed"], 4, axis=0)
    rgb, _, _ = rtrace_c(gb, sc, opts("rtrace", seed=5, **kw), rays)
    oo = po.default_opts("rtrace", seed=5, **{k: v for k, v in kw.items() if k != "as_"})
    oo.as_ = 0
    ref, _, _, _ = po.rtrace(po.Scene(tmp_path / "trans.rad"), oo, rays, hits=False, threads=16)
    rel = np.abs(rgb - ref).max(1) / np.maximum(np.abs(ref).max(1), 1e-9)
    print("trans vs oracle: median rel %.3g, share above 1e-3 %.3f" % (np.median(rel), (rel > 1e-3).mean()))
    assert np.median(rel) < 1e-4 and (rel <= 1e-3).mean() >= 0.95
    n, K = len(g["aimed"]), 256
    rgb, _, _ = rtrace_c(gb, sc, opts("rtrace", seed=6, **kw), np.repeat(g["aimed"], K, axis=0))
    a = rgb.reshape(n, K, 3)
    m, se = a.mean(1), a.std(1, ddof=1) / np.sqrt(K)
    z = (m - g["ab1_mean"]) / np.sqrt(se ** 2 + g["ab1_se"] ** 2 + (1e-5 * np.abs(g["ab1_mean"]) + 1e-9) ** 2)
    print("trans -ab 1: max |z| %.2f, mean z %.3f" % (np.abs(z).max(), z.mean()))
    assert np.abs(z).max() < 5 and abs(z.mean()) < 4 / np.sqrt(n)


@pytest.mark.parametrize("room,fixture", [("lamp_room", "circular_sources.npz"),
                                          ("tube_room", "cylinder_sources.npz")])
def test_circular_sources(gb, tmp_path, room, fixture):
    """Sphere and disk lights (rt/srcsupp.c sphsetsrc, rsetsrc), and
    cylinder lights (cylsetsrc, cylpart, scylform): -I direct
    irradiance with -ds 0 and with the disk partitioned (-ds 0.2, pieces
    trimmed to the circle) within 1e-5 for 99.5% of the sensors (a sensor
    whose distance to a piece sits on the splitting threshold within FP32
    rounding may split differently), and jittered (-dj 0.9) per-sensor
    means of 256 replicas within 5 standard errors of the reference's."""
    from pyradiance_gb300 import workloads as w
    g = golden(fixture)
    (tmp_path / "lamp.rad").write_text(getattr(w, room)())
    sc = gb.Scene(rad_files=[tmp_path / "lamp.rad"])
    for key, ds in (("ds0", 0.0), ("ds2", 0.2)):
        rgb, _, _ = rtrace_c(gb, sc, opts("rtrace", I=1, ab=0, dj=0, ds=ds, dr=0, dt=0, u=0), g["rays"])
        ref = g[key]
        rel = np.abs(rgb - ref).max(1) / np.maximum(np.abs(ref).max(1), 1e-9)
        print("%s: max rel %.3g, share above 1e-5 %.4f" % (key, rel.max(), (rel > 1e-5).mean()))
        assert (rel <= 1e-5).mean() >= 0.995 and rel.max() < 1e-2, key
    n, K = len(g["dj_rays"]), 256
    rgb, _, _ = rtrace_c(gb, sc, opts("rtrace", I=1, ab=0, dj=0.9, ds=0.2, dr=0, dt=0, u=0, seed=21),
                         np.repeat(g["dj_rays"], K, axis=0))
    a = rgb.reshape(n, K, 3)
    m, se = a.mean(1), a.std(1, ddof=1) / np.sqrt(K)
    z = (m - g["dj_mean"]) / np.sqrt(se ** 2 + g["dj_se"] ** 2 + (1e-5 * np.abs(g["dj_mean"]) + 1e-9) ** 2)
    print("jittered circular sources: max |z| %.2f, mean z %.3f" % (np.abs(z).max(), z.mean()))
    assert np.abs(z).max() < 5 and abs(z.mean()) < 4 / np.sqrt(n)


def test_spotlights(gb, tmp_path):
    """Spotlights (rt/srcsupp.c makespot, spotout): -I direct irradiance
    and view rays at the lights within 1e-5 for 99.5% (a sample on a cone's
    edge within FP32 rounding may fall on the other side)."""
    from pyradiance_gb300 import workloads as w
    g = golden("spotlights.npz")
    (tmp_path / "spot.rad").write_text(w.spot_room())
    sc = gb.Scene(rad_files=[tmp_path / "spot.rad"])
    for key, rays, I in (("irradiance", g["grid"], 1), ("radiance", g["view"], 0)):
        rgb, _, _ = rtrace_c(gb, sc, opts("rtrace", I=I, ab=0, dj=0, ds=0, dr=0, dt=0, u=0), rays)
        rel = np.abs(rgb - g[key]).max(1) / np.maximum(np.abs(g[key]).max(1), 1e-9)
        assert (rel <= 1e-5).mean() >= 0.995, (key, np.sort(rel)[-5:])


def test_mirrors(gb, tmp_path):
    """Mirrors (rt/m_mirror.c) with -dr 0: -I irradiance and view rays
    through mirror chains (1e-4 for 99.5%, as for mirror chains in the
    shape zoo); with -dr above 0 the virtual sources of flat mirrors are
    refused."""
    from pyradiance_gb300 import workloads as w
    from pyradiance_gb300 import _lib
    g = golden("mirrors.npz")
    (tmp_path / "mirror.rad").write_text(w.mirror_room())
    sc = gb.Scene(rad_files=[tmp_path / "mirror.rad"])
    for key, rays, I in (("irradiance", g["grid"], 1), ("radiance", g["view"], 0)):
        rgb, _, _ = rtrace_c(gb, sc, opts("rtrace", I=I, ab=0, dj=0, ds=0, dr=0, dt=0, u=0), rays)
        rel = np.abs(rgb - g[key]).max(1) / np.maximum(np.abs(g[key]).max(1), 1e-9)
        assert (rel <= 1e-4).mean() >= 0.995, (key, np.sort(rel)[-5:])
    with pytest.raises(_lib.GbError):
        rtrace_c(gb, sc, opts("rtrace", ab=0, dr=2, u=0), g["view"][:4])


def test_rfluxmtx(gb, tmp_path):
    """rfluxmtx end to end on the GPU against the reference program: view
    rays passed through to the sky receiver (glass in between) and to the
    window opening in Klems bins (1e-4 for 99.5% of the rows), the window as
    a Klems sender towards the sky behind an exterior block (sampling
    error), and the matrix header."""
    from pyradiance_gb300 import workloads as w
    from test_oracle_golden import flux_close
    g = golden("flux_matrices.npz")
    f = w.flux_files()
    for k, v in f.items():
        (tmp_path / f"{k}.rad").write_text(v)
    rb = g["rays"].astype("<f8").tobytes()
    for key, recv, scene in (("sky", "sky", "system"), ("window_kf", "window_kf", "interior")):
        out = gb.rfluxmtx(tmp_path / f"{recv}.rad", rays=rb, params=["-h", "-ab", "0", "-u-", "-fd"],
                          scene=[tmp_path / f"{scene}.rad"])
        a = np.frombuffer(out, dtype="<f8").reshape(g[key].shape)
        rel = np.abs(a - g[key]).max(axis=(1, 2)) / np.maximum(np.abs(g[key]).max(axis=(1, 2)), 1e-9)
        assert (rel <= 1e-4).mean() >= 0.995, (key, np.sort(rel)[-5:])
    n = int(g["send_count"])
    out = gb.rfluxmtx(tmp_path / "sky.rad", surface=tmp_path / "window_send.rad",
                      params=["-h", "-ab", "0", "-u-", "-fd", "-c", str(n)], scene=[tmp_path / "obstruction.rad"])
    a = np.frombuffer(out, dtype="<f8").reshape(g["send"].shape)
    flux_close(a[:, :, 0], g["send"][:, :, 0], n)
    out = gb.rfluxmtx(tmp_path / "sky.rad", surface=tmp_path / "window_send.rad", params=["-ab", "0", "-c", "4"],
                      scene=[tmp_path / "obstruction.rad"])
    head = out.split(b"\n\n")[0].decode()
    assert "NROWS=145" in head and "NCOLS=146" in head and "NCOMP=3" in head and "FORMAT=ascii" in head
    body = out.split(b"\n\n", 1)[1].decode().split("\n")
    assert len([ln for ln in body if ln.strip()]) == 145 and len(body[0].split()) == 146 * 3
    with pytest.raises(RuntimeError):
        gb.rfluxmtx(tmp_path / "sky.rad", surface=tmp_path / "window_send.rad", params=["-I", "-c", "4"])
    # o= on the sky receiver: its 145 columns go to a file, the ground's to stdout
    (tmp_path / "sky_o.rad").write_text(f["sky"].replace("#@rfluxmtx h=r1 u=Y", "#@rfluxmtx h=r1 u=Y o=%s.mtx"))
    import os
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        out = gb.rfluxmtx(tmp_path / "sky_o.rad", rays=rb, params=["-h", "-ab", "0", "-u-", "-fd"],
                          scene=[tmp_path / "system.rad"])
        sky = np.frombuffer((tmp_path / "skyglow.mtx").read_bytes(), dtype="<f8").reshape(-1, 145, 3)
    finally:
        os.chdir(cwd)
    ground = np.frombuffer(out, dtype="<f8").reshape(-1, 1, 3)
    a = np.concatenate([ground, sky], axis=1)
    rel = np.abs(a - g["sky"]).max(axis=(1, 2)) / np.maximum(np.abs(g["sky"]).max(axis=(1, 2)), 1e-9)
    assert (rel <= 1e-4).mean() >= 0.995


def test_rfluxmtx_shirchiu(gb, tmp_path):
    """Shirley-Chiu bases (h=sc4) end to end on the GPU: receiver bins of the
    window opening (1e-4 for 99.5% of the rows) and the window as a sender
    (sampling error) against the reference program."""
    from pyradiance_gb300 import workloads as w
    from test_oracle_golden import flux_close
    g = golden("flux_shirchiu.npz")
    f = w.flux_files()
    (tmp_path / "recv.rad").write_text(f["window_kf"].replace("h=kf u=Z", "h=sc4 u=Z"))
    (tmp_path / "send.rad").write_text(f["window_send"].replace("h=kf u=Z", "h=sc4 u=Z"))
    for k in ("sky", "interior", "obstruction"):
        (tmp_path / f"{k}.rad").write_text(f[k])
    out = gb.rfluxmtx(tmp_path / "recv.rad", rays=g["rays"].astype("<f8").tobytes(),
                      params=["-h", "-ab", "0", "-u-", "-fd"], scene=[tmp_path / "interior.rad"])
    a = np.frombuffer(out, dtype="<f8").reshape(g["window_sc"].shape)
    rel = np.abs(a - g["window_sc"]).max(axis=(1, 2)) / np.maximum(np.abs(g["window_sc"]).max(axis=(1, 2)), 1e-9)
    assert (rel <= 1e-4).mean() >= 0.995, np.sort(rel)[-5:]
    n = int(g["send_count"])
    out = gb.rfluxmtx(tmp_path / "sky.rad", surface=tmp_path / "send.rad",
                      params=["-h", "-ab", "0", "-u-", "-fd", "-c", str(n)], scene=[tmp_path / "obstruction.rad"])
    flux_close(np.frombuffer(out, dtype="<f8").reshape(g["send"].shape)[:, :, 0], g["send"][:, :, 0], n)


def test_instances(gb):
    """Instanced octrees (rt/o_instance.c:15-71): the furniture octree 12
    times in the room, rotated, scaled, mirrored, some with their own
    material, read from the reference oconv's octrees.  First hits are cast
    in FP64 (the ray carried into each instance's coordinates as
    rt/o_instance.c does): every hit name is the reference's.  Radiance and
    irradiance (FP32 shading, entering the instances in FP32) as for the
    shape zoo."""
    from pathlib import Path
    g = golden("instances.npz")
    sc = gb.Scene(str(Path(__file__).resolve().parent / "golden" / "inst_main.oct"))
    rgb, hid, ht = rtrace_c(gb, sc, opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, u=0), g["rays"])
    names = names_of(sc, hid)
    match = names == g["hit_name"]
    inst = np.array([not n.startswith(("floor", "ceiling", "north", "south", "east", "west", "light", "*"))
                     for n in g["hit_name"]])
    print("instances: %d of %d instanced hits named alike, %d of %d overall" %
          ((match & inst).sum(), inst.sum(), match.sum(), len(match)))
    assert match.all(), np.nonzero(~match)
    ok = match & (g["hit_dist"] < 1e9)
    np.testing.assert_allclose(ht[ok], g["hit_dist"][ok], rtol=1e-6, atol=1e-7)
    rel = np.abs(rgb - g["radiance"]).max(1) / np.maximum(np.abs(g["radiance"]).max(1), 1e-9)
    assert (rel[match] <= 1e-4).mean() >= 0.99, np.sort(rel[match])[-5:]
    o = opts("rtrace", I=1, ab=0, dj=0, ds=0, dr=0, dt=0, u=0)
    irr, _, _ = rtrace_c(gb, sc, o, g["rays"])
    rel = np.abs(irr - g["irradiance"]).max(1) / np.maximum(np.abs(g["irradiance"]).max(1), 1e-9)
    assert (rel <= 1e-4).mean() >= 0.99, np.sort(rel)[-5:]


def test_meshes(gb):
    """Compiled meshes (rt/o_mesh.c): the reference obj2mesh's mesh 10 times
    in the room, read from the reference oconv's octree; each mesh is an
    instance of its triangles.  First hits cast in FP64: every hit name is
    the reference's (the mesh's, or "M-Tri" for a mesh without its own
    modifier).  Radiance and irradiance as for the instances."""
    from pathlib import Path
    g = golden("meshes.npz")
    sc = gb.Scene(str(Path(__file__).resolve().parent / "golden" / "mesh_room.oct"))
    rgb, hid, ht = rtrace_c(gb, sc, opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, u=0), g["rays"])
    names = names_of(sc, hid)
    match = names == g["hit_name"]
    print("meshes: %d of %d hits named alike" % (match.sum(), len(match)))
    assert match.all(), np.nonzero(~match)
    ok = g["hit_dist"] < 1e9
    np.testing.assert_allclose(ht[ok], g["hit_dist"][ok], rtol=1e-6, atol=1e-7)
    rel = np.abs(rgb - g["radiance"]).max(1) / np.maximum(np.abs(g["radiance"]).max(1), 1e-9)
    assert (rel <= 1e-4).mean() >= 0.99, np.sort(rel)[-5:]
    o = opts("rtrace", I=1, ab=0, dj=0, ds=0, dr=0, dt=0, u=0)
    irr, _, _ = rtrace_c(gb, sc, o, g["rays"])
    rel = np.abs(irr - g["irradiance"]).max(1) / np.maximum(np.abs(g["irradiance"]).max(1), 1e-9)
    assert (rel <= 1e-4).mean() >= 0.99, np.sort(rel)[-5:]


def test_smooth_meshes(gb):
    """Meshes with vertex normals (rt/o_mesh.c:185-206; the reference
    obj2mesh's mesh, placed 10 times, one mirrored, some scaled, some with
    a plastic or rough metal of their own).  First hits cast in FP64: names
    and distances; the surface normal and the shading normal (-oNn, the
    vertex normals interpolated at the hit and oriented as the reference's
    raynormal does) within 1e-6 of the reference's.  -ab 0 -st 1 radiance
    (direct light through the shading normal, the rough lobes' direct
    Gaussian term) within 1e-4 on 99% of the rays, mesh hits among them.
    rcontrib -ab 1 contributions of the ceiling light on rays that meet a
    mesh (hemisphere about the surface normal, rough specular about the
    shading normal, samples rejected below the surface): every ray's mean
    over K replicas within 4 combined standard errors of the reference's.
    rtrace with ambient bounces on these surfaces is refused (their ambient
    texture factor is not formed), and so is a glass over them.  With
    texture coordinates, -oc within 1e-6 of the reference's."""
    from pathlib import Path
    from pyradiance_gb300 import _lib
    g = golden("smooth_meshes.npz")
    sc = gb.Scene(str(Path(__file__).resolve().parent / "golden" / "mesh_smooth_room.oct"))
    rgb, hid, ht = rtrace_c(gb, sc, opts("rtrace", ab=0, dj=0, ds=0, dr=0, dt=0, st=1.0, u=0), g["rays"])
    names = names_of(sc, hid)
    assert (names == g["hit_name"]).all(), np.nonzero(names != g["hit_name"])
    ok = g["hit_dist"] < 1e9
    np.testing.assert_allclose(ht[ok], g["hit_dist"][ok], rtol=1e-6, atol=1e-7)
    out = gb.rtrace(g["rays"].astype("<f8").tobytes(), sc, params=["-ab", "0"], inform="d", outform="d",
                    outspec="Nn", header=False)
    v = np.frombuffer(out, dtype="<f8").reshape(-1, 6)
    np.testing.assert_allclose(v[:, :3], g["N"], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(v[:, 3:], g["n"], rtol=1e-6, atol=1e-6)
    mesh = np.array([n == "M-Tri" or n.startswith("mesh") for n in g["hit_name"]])
    assert mesh.sum() > 300 and (np.abs(g["N"] - g["n"]).max(1)[mesh] > 1e-3).mean() > 0.9
    rel = np.abs(rgb - g["radiance"]).max(1) / np.maximum(np.abs(g["radiance"]).max(1), 1e-9)
    assert (rel <= 1e-4).mean() >= 0.99, np.sort(rel)[-5:]
    assert (rel[mesh] <= 1e-4).mean() >= 0.98, np.sort(rel[mesh])[-5:]
    K = int(g["K"])
    o = opts("rcontrib", ab=1, ad=256, lw=1e-4, u=0, seed=777)
    st, _ = rcontrib_c(gb, sc, o, np.repeat(g["stat_rays"], K, axis=0), mods=[dict(modifier="light_mat")])
    st = st.reshape(len(g["stat_rays"]), K, 3)
    mean, se = st.mean(1), st.std(1, ddof=1) / np.sqrt(K)
    z = np.abs(mean - g["mean"]) / np.sqrt(se ** 2 + g["se"] ** 2 + 1e-30)
    print("smooth meshes rcontrib: max z %.2f, mean z %.2f" % (z.max(), z.mean()))
    assert z.max() < 4.0 and z.mean() < 1.2, z
    with pytest.raises(_lib.GbError, match="vertex normals"):
        rtrace_c(gb, sc, opts("rtrace", ab=1, u=0), g["rays"][:8])
    # texture coordinates too (rt/rtrace.c:766-772 -oc): the vertex (u,v) interpolated at the hit, FP64 casts
    uvsc = gb.Scene(str(Path(__file__).resolve().parent / "golden" / "mesh_uv_room.oct"))
    out = gb.rtrace(g["rays"].astype("<f8").tobytes(), uvsc, params=["-ab", "0"], inform="d", outform="d",
                    outspec="cn", header=False)
    v = np.frombuffer(out, dtype="<f8").reshape(-1, 5)
    assert (np.abs(g["uv_c"]).sum(1) > 0).sum() > 300
    np.testing.assert_allclose(v[:, :2], g["uv_c"], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(v[:, 2:], g["uv_n"], rtol=1e-6, atol=1e-6)
    glassy = gb.Scene(str(Path(__file__).resolve().parent / "golden" / "mesh_smooth_glass.oct"))
    with pytest.raises(_lib.GbError, match="vertex normals"):
        rtrace_c(gb, glassy, opts("rtrace", ab=0, u=0), g["rays"][:8])


def test_dctimestep_fp32_fp64(gb):
    g = golden("dct_small.npz")
    r64 = gb.dctimestep_array(g["dc"], g["sky"], mode="fp64")
    np.testing.assert_allclose(r64, g["out"], rtol=1e-6, atol=1e-30)
    r32 = gb.dctimestep_array(g["dc"], g["sky"], mode="fp32")
    np.testing.assert_allclose(r32, g["out"], rtol=1e-4, atol=1e-6 * np.abs(g["out"]).max())


def test_dctimestep_four_matrix(gb, tmp_path):
    """dctimestep V T D sky (util/dctimestep.c:243-264) through the drop-in:
    matrix files in, the reference program's output within 1e-5; a
    missing XML BSDF transmission raises."""
    g = golden("dct_four.npz")
    paths = []
    for n in "VTDS":
        m = g[n]
        hdr = (f"#?RADIANCE\nNROWS={m.shape[0]}\nNCOLS={m.shape[1]}\nNCOMP=3\nBigEndian=0\n"
               "FORMAT=float\n\n").encode()
        (tmp_path / f"{n}.mtx").write_bytes(hdr + m.astype("<f4").tobytes())
        paths.append(tmp_path / f"{n}.mtx")
    out = gb.dctimestep(*paths, header=False, outform="d")
    r = np.frombuffer(out, dtype="<f8").reshape(g["out"].shape)
    np.testing.assert_allclose(r, g["out"], rtol=1e-5, atol=1e-6 * np.abs(g["out"]).max())
    with pytest.raises(RuntimeError):
        gb.dctimestep(paths[0], tmp_path / "T.xml", paths[2], paths[3])
    with pytest.raises(RuntimeError):
        gb.dctimestep(paths[0], paths[0], paths[2], paths[3])


def test_dctimestep_xml_transmission(gb, tmp_path):
    """dctimestep V T.xml D sky with Klems matrix BSDFs for T
    (util/dctimestep.c:250-254 cm_loadBTDF): the synthetic XML files
    of tests/golden/btdf.npz, each product on the GPU: the reference
    program's output within 1e-5."""
    import sys
    from pathlib import Path
    from pyradiance_gb300 import workloads as w
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from make_golden import BTDF_CASES
    g = golden("btdf.npz")
    for k, kw in BTDF_CASES.items():
        (tmp_path / f"{k}.xml").write_text(w.klems_bsdf_xml(**kw))
        paths = []
        for n in "VDS":
            m = g[f"{k}_{n}"]
            hdr = (f"#?RADIANCE\nNROWS={m.shape[0]}\nNCOLS={m.shape[1]}\nNCOMP=3\nBigEndian=0\n"
                   "FORMAT=float\n\n").encode()
            (tmp_path / f"{k}_{n}.mtx").write_bytes(hdr + m.astype("<f4").tobytes())
            paths.append(tmp_path / f"{k}_{n}.mtx")
        out = gb.dctimestep(paths[0], tmp_path / f"{k}.xml", paths[1], paths[2], header=False, outform="d")
        ref = g[f"{k}_R"]
        r = np.frombuffer(out, dtype="<f8").reshape(ref.shape)
        np.testing.assert_allclose(r, ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max(), err_msg=k)


def test_errors_are_reported(gb, scenes):
    from pyradiance_gb300 import _lib
    with pytest.raises(_lib.GbError) as e:
        _lib.parse_opts(["-ab", "1", "-zz"], _lib.GB_PROG_RTRACE)
    assert e.value.code == -1
    o = opts("rtrace", ab=1, aa=0.1)
    with pytest.raises(_lib.GbError) as e:
        rtrace_c(gb, scenes["c1"], o, np.array([[1, 1, 1, 0, 0, 1.0]]))
    assert e.value.code == -3
    with pytest.raises(RuntimeError):
        gb.rtrace(b"1 1 1 0 0 1\n", "/nonexistent.oct")
