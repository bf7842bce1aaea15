"""Generates the golden vectors in tests/golden from the reference programs.

Runs the reference rtrace, rcontrib, oconv and dctimestep compiled from the
reference sources by oracle/build_ref.mk (into oracle/_ref/) on the seeded
scenes of pyradiance_gb300.workloads, and stores their outputs as small .npz
fixtures.  Only this script runs the reference; the tests read the fixtures.

    make -f oracle/build_ref.mk REF=/root/reference -j8
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from pyradiance_gb300 import workloads as w  # noqa: E402

REF = ROOT / "oracle" / "_ref"
BIN = REF / "bin"
OUT = Path(__file__).resolve().parent
REFERENCE_TREE = Path(os.environ.get("GB_REFERENCE", "/root/reference"))


def run(args, inp: bytes | None = None, cwd=None) -> bytes:
    env = dict(os.environ, RAYPATH=f".:{REF / 'lib'}", PATH=f"{BIN}:{os.environ.get('PATH', '')}")
    p = subprocess.run([str(BIN / args[0]), *map(str, args[1:])], input=inp, capture_output=True, env=env,
                       cwd=cwd)
    if p.returncode != 0:
        raise RuntimeError(f"{args[0]} failed: {p.stderr.decode()}")
    return p.stdout


def run_independent(args, rays: np.ndarray, shards: int | None = None, cwd=None) -> bytes:
    """A -u+ (time-seeded) rcontrib or rtrace run over many rays in parallel
    with independent random streams: `shards` separate single-process runs
    over contiguous parts of the rays, started more than a second apart.
    The reference seeds its generator once per process with the time in
    seconds (rt/rcmain.c:330-336), and the workers of -n N are forked after
    that seeding, so they draw identical random sequences: replicas of one
    sensor handled by different workers come out equal.  Outputs are
    concatenated in ray order."""
    import time
    shards = shards or (os.cpu_count() or 1)
    env = dict(os.environ, RAYPATH=f".:{REF / 'lib'}", PATH=f"{BIN}:{os.environ.get('PATH', '')}")
    parts = np.array_split(np.ascontiguousarray(rays, dtype="<f8"), shards)
    procs = []
    with tempfile.TemporaryDirectory() as td:
        for i, part in enumerate(parts):
            fin = Path(td) / f"in{i}"
            fin.write_bytes(part.tobytes())
            if i:
                time.sleep(1.1)
            with open(fin, "rb") as fi, open(Path(td) / f"out{i}", "wb") as fo, \
                    open(Path(td) / f"err{i}", "wb") as fe:
                procs.append(subprocess.Popen([str(BIN / args[0]), *map(str, args[1:])], stdin=fi, stdout=fo,
                                              stderr=fe, env=env, cwd=cwd))
        outs = []
        for i, p in enumerate(procs):
            if p.wait() != 0:
                raise RuntimeError(f"{args[0]} failed: {(Path(td) / f'err{i}').read_text()}")
            outs.append((Path(td) / f"out{i}").read_bytes())
    return b"".join(outs)


def oconv(rad_text: str, tmp: Path, name: str) -> Path:
    rad = tmp / f"{name}.rad"
    rad.write_text(rad_text)
    oct_path = tmp / f"{name}.oct"
    oct_path.write_bytes(run(["oconv", "-f", rad]))
    return oct_path


def names(out: bytes) -> np.ndarray:
    return np.array([ln.split("\t")[0] for ln in out.decode().splitlines()])


def c1_direct(tmp: Path) -> None:
    """Deterministic direct irradiance (rtrace -I -ab 0 -dj 0 -ds 0 -dr 0)
    and first-hit surfaces on the 100 x 100 sensor grid."""
    octp = oconv(w.daylight_room(), tmp, "c1")
    rays = w.sensor_grid(100, 100)
    inp = rays.astype("<f8").tobytes()
    irr = np.frombuffer(run(["rtrace", "-h", "-u-", "-I", "-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0",
                             "-fdd", "-ov", octp], inp), dtype="<f8").reshape(-1, 3)
    hit = names(run(["rtrace", "-h", "-u-", "-ab", "0", "-fda", "-os", octp], inp))
    dist = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", "-fdd", "-oL", octp], inp), dtype="<f8")
    np.savez_compressed(OUT / "c1_direct.npz", rays=rays, irradiance=irr, hit_name=hit, hit_dist=dist,
                        cmd="rtrace -h -u- -I -ab 0 -dj 0 -ds 0 -dr 0 -fdd -ov | -ab 0 -os | -ab 0 -oL")
    print("c1_direct: lit fraction %.4f" % (irr[:, 0] > 0).mean())


def c1_partitioned(tmp: Path) -> None:
    """Direct irradiance with the light partitioned (rtrace -I -ab 0 -dj 0
    -ds 0.2 -dr 0 -dt 0): the 100 x 100 grid at 0.8 m and a 50 x 50 grid at
    2.5 m, half a metre below the light, where it splits into many pieces.
    -dt 0 tests every partition's shadow (the default -dt estimates untested
    ones from run-wide statistics)."""
    octp = oconv(w.daylight_room(), tmp, "c1p")
    rays = np.vstack([w.sensor_grid(100, 100), w.sensor_grid(50, 50, z=2.5)])
    inp = rays.astype("<f8").tobytes()
    irr = np.frombuffer(run(["rtrace", "-h", "-u-", "-I", "-ab", "0", "-dj", "0", "-ds", "0.2", "-dr", "0",
                             "-dt", "0", "-fdd", "-ov", octp], inp), dtype="<f8").reshape(-1, 3)
    np.savez_compressed(OUT / "c1_partitioned.npz", rays=rays, irradiance=irr,
                        cmd="rtrace -h -u- -I -ab 0 -dj 0 -ds 0.2 -dr 0 -dt 0 -fdd -ov")
    print("c1_partitioned: lit fraction %.4f" % (irr[:, 0] > 0).mean())


def zoo(tmp: Path) -> None:
    """Every primitive type: first-hit surface and distance of random rays,
    and deterministic -ab 0 radiance (direct + mirror reflections)."""
    octp = oconv(w.shape_zoo(), tmp, "zoo")
    rays = w.random_rays(4000, seed=3)
    inp = rays.astype("<f8").tobytes()
    hit = names(run(["rtrace", "-h", "-u-", "-ab", "0", "-fda", "-os", octp], inp))
    dist = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", "-fdd", "-oL", octp], inp), dtype="<f8")
    val = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0",
                             "-fdd", "-ov", octp], inp), dtype="<f8").reshape(-1, 3)
    irr = np.frombuffer(run(["rtrace", "-h", "-u-", "-I", "-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0",
                             "-dt", "0", "-fdd", "-ov", octp], inp), dtype="<f8").reshape(-1, 3)
    np.savez_compressed(OUT / "zoo.npz", rays=rays, hit_name=hit, hit_dist=dist, radiance=val, irradiance=irr,
                        cmd="rtrace -h -u- -ab 0 [-I] -dj 0 -ds 0 -dr 0 -dt 0")
    print("zoo: %d hits on curved surfaces" % sum(not n.startswith(("floor", "ceiling", "north", "south", "east",
                                                                   "west", "light")) for n in hit))


def normals(tmp: Path) -> None:
    """First-hit normals (rt/rtrace.c:787-820 oputN, oputn): the surface's
    own normal (-oN) and the shading normal turned toward the ray by the
    material (-on) of random rays in the shape zoo (every primitive, plastic
    and metal), the instances room (transformed octrees) and rays through
    the window room's glass from both sides."""
    out = {}
    rng = np.random.default_rng(21)
    x0, x1, z0, z1 = w.WINDOW
    tgt = np.column_stack([rng.uniform(x0 + .05, x1 - .05, 400), np.zeros(400), rng.uniform(z0 + .05, z1 - .05, 400)])
    org = np.vstack([rng.uniform((1.0, 1.0, 0.5), (9.0, 5.0, 2.5), (200, 3)),
                     rng.uniform((1.0, -6.0, 0.5), (9.0, -1.0, 2.5), (200, 3))])
    d = tgt - org
    cases = {"zoo": (oconv(w.shape_zoo(), tmp, "nzoo"), w.random_rays(3000, seed=4)),
             "win": (oconv(w.window_room(ntri=0), tmp, "nwin"), np.hstack([org, d / np.linalg.norm(d, axis=1,
                                                                                          keepdims=True)]))}
    for key, (octp, rays) in cases.items():
        inp = rays.astype("<f8").tobytes()
        v = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", "-fdd", "-oNn", octp], inp),
                          dtype="<f8").reshape(-1, 6)
        out[f"{key}_rays"], out[f"{key}_N"], out[f"{key}_n"] = rays, v[:, :3], v[:, 3:]
        print("normals %s: %d rays, %d flipped" % (key, len(rays), (np.abs(v[:, :3] + v[:, 3:]).sum(1) < 1e-9).sum()
                                                     - (np.abs(v[:, :3]).sum(1) == 0).sum()))
    zoo_oct, zoo_rays = cases["zoo"]
    vw = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0",
                            "-fdd", "-oVWv", zoo_oct], zoo_rays[:500].astype("<f8").tobytes()), dtype="<f8")
    out["zoo_VWv"] = vw.reshape(-1, 9)
    np.savez_compressed(OUT / "normals.npz", **out, cmd="rtrace -h -u- -ab 0 -fdd -oNn | -dj 0 -ds 0 -dr 0 -dt 0 -oVWv")


def glossy(tmp: Path, n: int = 300, K: int = 1024) -> None:
    """Rough specular plastic and metal (glossy_room), radiance of view rays
    from random interior points: deterministic with -st 1 (every rough lobe
    below the specular threshold: direct Gaussian term only, no sampling),
    and with the lobe sampled (-st 0 one sample; -ss 3 several per hit) as
    per-ray means and standard errors over K replicas of each ray.  The
    sampled runs use -u+ (the reference's default): with -u- the replicas'
    first trials come from successive entries of one urand table shared by
    every bounce of the path, and their mean is off by up to 1% on some
    rays (measured against -u+ runs)."""
    octp = oconv(w.glossy_room(), tmp, "glossy")
    rays = w.random_rays(n, seed=5)
    base = ["rtrace", "-h", "-u-", "-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0", "-fdd", "-ov"]
    det = np.frombuffer(run([*base, "-st", "1", octp], rays.astype("<f8").tobytes()), dtype="<f8").reshape(-1, 3)
    rep = np.repeat(rays, K, axis=0).astype("<f8").tobytes()
    stats = {}
    for key, extra in (("st0", ["-st", "0"]), ("ss3", ["-ss", "3"])):
        a = np.frombuffer(run([*base, "-u+", *extra, octp], rep), dtype="<f8").reshape(n, K, 3)
        stats[f"{key}_mean"] = a.mean(1)
        stats[f"{key}_se"] = a.std(1, ddof=1) / np.sqrt(K)
    np.savez_compressed(OUT / "glossy.npz", rays=rays, K=K, radiance_st1=det, **stats,
                        cmd=" ".join(base[1:]) + " with -st 1 | -u+ -st 0 | -u+ -ss 3 (K replicas)")
    print("glossy: mean radiance st1 %.4g, st0 %.4g, ss3 %.4g" % (det.mean(), stats["st0_mean"].mean(),
                                                                  stats["ss3_mean"].mean()))


def surface_irradiance(tmp: Path, K: int = 256) -> None:
    """rtrace -i (irradiance at the surface each ray hits): deterministic
    with -ab 0 in the box room and in the empty window room (rays pass
    through the glass, those leaving through the window see the sky and
    ground glows), and with
    one diffuse bounce (-ab 1 -aa 0 -as 0 -ad 256) as per-ray means and standard errors
    of K replicas (-u+)."""
    det = ["rtrace", "-h", "-u-", "-i", "-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0", "-fdd", "-ov"]
    out = {}
    for key, text, seed in (("c1", w.daylight_room(), 7), ("c2e", w.window_room(ntri=0), 8)):
        octp = oconv(text, tmp, f"irr_{key}")
        rays = w.random_rays(2000, seed=seed)
        if key == "c2e":                         # half of them aimed at the window
            rng = np.random.default_rng(seed)
            x0, x1, z0, z1 = w.WINDOW
            tgt = np.stack([rng.uniform(x0, x1, 1000), np.zeros(1000), rng.uniform(z0, z1, 1000)], 1)
            d = tgt - rays[:1000, :3]
            rays[:1000, 3:] = d / np.linalg.norm(d, axis=1, keepdims=True)
        out[f"{key}_rays"] = rays
        out[f"{key}_irr"] = np.frombuffer(run([*det, octp], rays.astype("<f8").tobytes()),
                                          dtype="<f8").reshape(-1, 3)
    octp = tmp / "irr_c1.oct"
    rays = w.random_rays(100, seed=9)
    a = np.frombuffer(run(["rtrace", "-h", "-u+", "-i", "-ab", "1", "-aa", "0", "-as", "0", "-ad", "256", "-lw", "1e-4",
                           "-dj", "0",
                           "-ds", "0", "-dr", "0", "-dt", "0", "-fdd", "-ov", octp],
                          np.repeat(rays, K, axis=0).astype("<f8").tobytes()), dtype="<f8").reshape(100, K, 3)
    np.savez_compressed(OUT / "surface_irradiance.npz", **out, ab1_rays=rays, K=K, ab1_mean=a.mean(1),
                        ab1_se=a.std(1, ddof=1) / np.sqrt(K),
                        cmd="rtrace -h -u- -i -ab 0 -dj 0 -ds 0 -dr 0 -dt 0 | -u+ -i -ab 1 -aa 0 -as 0 -ad 256 -lw 1e-4")
    print("surface_irradiance: c1 lit %.3f, c2e nonzero %.3f, ab1 mean %.4g" % (
        (out["c1_irr"][:, 0] > 0).mean(), (out["c2e_irr"][:, 0] > 0).mean(), a.mean()))


def supersampled_irradiance(tmp: Path, n: int = 100, K: int = 512) -> None:
    """rtrace -I with ambient super-sampling (-as 512, rtrace's default;
    -ab 2 -aa 0 -ad 256: 16 x 16 first hemispheres get 512 extra samples
    placed by the strata's brightness differences, rt/ambcomp.c:256-346):
    per-sensor means and standard errors of K replicas (-u+), with the same
    run at -as 0 beside it."""
    octp = oconv(w.daylight_room(), tmp, "ss_c1")
    rays = w.random_rays(n, seed=9)
    rep = np.repeat(rays, K, axis=0).astype("<f8").tobytes()
    out = {}
    for key, extra in (("as512", []), ("as0", ["-as", "0"])):
        a = np.frombuffer(run(["rtrace", "-h", "-u+", "-I", "-ab", "2", "-aa", "0", "-ad", "256", "-lw", "1e-4",
                               "-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0", *extra, "-fdd", "-ov", octp], rep),
                          dtype="<f8").reshape(n, K, 3)
        out[f"{key}_mean"] = a.mean(1)
        out[f"{key}_se"] = a.std(1, ddof=1) / np.sqrt(K)
    np.savez_compressed(OUT / "supersampled.npz", rays=rays, K=K, **out,
                        cmd="rtrace -h -u+ -I -ab 2 -aa 0 -ad 256 -lw 1e-4 -dj 0 -ds 0 -dr 0 -dt 0 [-as 0]")
    print("supersampled: mean %.4g (as 512) vs %.4g (as 0)" % (out["as512_mean"].mean(), out["as0_mean"].mean()))


def spotlights(tmp: Path) -> None:
    """Spotlights (rt/srcsupp.c makespot, spotout; rt/source.c:246-252 and
    782): -I direct irradiance on grids at 0.8 m and 2.3 m, and the
    radiance of view rays aimed at the lights' centres from random points
    (lit only from inside the cones), deterministic (-ab 0 -dj 0 -ds 0)."""
    octp = oconv(w.spot_room(), tmp, "spot")
    grid = np.vstack([w.sensor_grid(40, 40), w.sensor_grid(20, 20, z=2.3)])
    rng = np.random.default_rng(19)
    org = rng.uniform((0.3, 0.3, 0.1), (9.7, 7.7, 2.0), size=(1000, 3))
    tgt = np.array([[3.5, 4.0, 2.985], [7.0, 4.0, 2.4]])[np.arange(1000) % 2]
    d = tgt - org
    view = np.hstack([org, d / np.linalg.norm(d, axis=1, keepdims=True)])
    base = ["rtrace", "-h", "-u-", "-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0", "-fdd", "-ov"]
    irr = np.frombuffer(run([*base, "-I", octp], grid.astype("<f8").tobytes()), dtype="<f8").reshape(-1, 3)
    rad = np.frombuffer(run([*base, octp], view.astype("<f8").tobytes()), dtype="<f8").reshape(-1, 3)
    np.savez_compressed(OUT / "spotlights.npz", grid=grid, irradiance=irr, view=view, radiance=rad,
                        cmd="rtrace -h -u- -ab 0 -dj 0 -ds 0 -dr 0 -dt 0 -fdd -ov [-I]")
    print("spotlights: lit %.3f, irradiance mean %.4g, view lit %.3f" % ((irr[:, 0] > 0).mean(), irr.mean(),
                                                                        (rad[:, 0] > 50).mean()))


def mirrors(tmp: Path) -> None:
    """The mirror material (rt/m_mirror.c without virtual sources, -dr 0):
    -I direct irradiance (mirrors block shadow rays) and the radiance of
    random view rays (mirror chains), deterministic."""
    octp = oconv(w.mirror_room(), tmp, "mirror")
    grid = w.sensor_grid(40, 40)
    view = w.random_rays(2000, seed=23)
    base = ["rtrace", "-h", "-u-", "-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0", "-fdd", "-ov"]
    irr = np.frombuffer(run([*base, "-I", octp], grid.astype("<f8").tobytes()), dtype="<f8").reshape(-1, 3)
    rad = np.frombuffer(run([*base, octp], view.astype("<f8").tobytes()), dtype="<f8").reshape(-1, 3)
    np.savez_compressed(OUT / "mirrors.npz", grid=grid, irradiance=irr, view=view, radiance=rad,
                        cmd="rtrace -h -u- -ab 0 -dj 0 -ds 0 -dr 0 -dt 0 -fdd -ov [-I]")
    print("mirrors: irradiance mean %.4g, radiance mean %.4g" % (irr.mean(), rad.mean()))


def flux_matrices(tmp: Path) -> None:
    """rfluxmtx (util/rfluxmtx.c) in its two modes, -ab 0: view rays passed
    through to a sky receiver (ground uniform, sky Reinhart MF:1) seen through
    the glass, and to the window opening binned by the Klems full basis
    (deterministic); and the window as a Klems sender towards the sky behind an
    exterior block (2000 samples per sender bin; a statistical fixture)."""
    f = w.flux_files()
    for k, v in f.items():
        (tmp / f"{k}.rad").write_text(v)
    rng = np.random.default_rng(31)
    org = rng.uniform((0.2, 0.2, 0.2), (9.8, 7.8, 2.8), size=(1500, 3))
    tgt = np.stack([rng.uniform(3.5, 6.5, 1500), np.zeros(1500), rng.uniform(0.5, 2.5, 1500)], axis=1)
    d = tgt - org
    rays = np.hstack([org, d / np.linalg.norm(d, axis=1, keepdims=True)])      # aimed at the window
    rb = rays.astype("<f8").tobytes()
    base = ["rfluxmtx", "-h", "-ab", "0", "-u-", "-fd"]
    sky = np.frombuffer(run([*base, "-", tmp / "sky.rad", tmp / "system.rad"], rb, cwd=tmp),
                        dtype="<f8").reshape(len(rays), -1, 3)
    kf = np.frombuffer(run([*base, "-", tmp / "window_kf.rad", tmp / "interior.rad"], rb, cwd=tmp),
                       dtype="<f8").reshape(len(rays), -1, 3)
    send = np.frombuffer(run(["rfluxmtx", "-h", "-ab", "0", "-u-", "-fd", "-c", "2000", tmp / "window_send.rad",
                              tmp / "sky.rad", tmp / "obstruction.rad"], cwd=tmp), dtype="<f8").reshape(145, -1, 3)
    np.savez_compressed(OUT / "flux_matrices.npz", rays=rays, sky=sky, window_kf=kf, send=send, send_count=2000,
                        cmd="rfluxmtx -h -ab 0 -u- -fd [-c 2000] sender receiver scene")
    print("flux: rows reaching the sky %.3f, the window %.3f; sender row mean %.4f" % (
        (sky.sum(axis=(1, 2)) > 0).mean(), (kf.sum(axis=(1, 2)) > 0).mean(), send[:, :, 0].sum(1).mean()))


def flux_shirchiu(tmp: Path) -> None:
    """rfluxmtx with Shirley-Chiu bases (h=sc4, util/disk2square.cal), -ab 0:
    view rays passed through to the window opening binned as a receiver
    (deterministic), and the window as a sender towards the sky behind an
    exterior block (2000 samples per bin)."""
    f = w.flux_files()
    f["window_sc"] = f["window_kf"].replace("h=kf u=Z", "h=sc4 u=Z")
    f["send_sc"] = f["window_send"].replace("h=kf u=Z", "h=sc4 u=Z")
    for k, v in f.items():
        (tmp / f"{k}.rad").write_text(v)
    rays = np.load(OUT / "flux_matrices.npz")["rays"]
    base = ["rfluxmtx", "-h", "-ab", "0", "-u-", "-fd"]
    recv = np.frombuffer(run([*base, "-", tmp / "window_sc.rad", tmp / "interior.rad"], rays.astype("<f8").tobytes(),
                             cwd=tmp), dtype="<f8").reshape(len(rays), -1, 3)
    send = np.frombuffer(run([*base, "-c", "2000", tmp / "send_sc.rad", tmp / "sky.rad", tmp / "obstruction.rad"],
                             cwd=tmp), dtype="<f8").reshape(16, -1, 3)
    np.savez_compressed(OUT / "flux_shirchiu.npz", rays=rays, window_sc=recv, send=send, send_count=2000,
                        cmd="rfluxmtx -h -ab 0 -u- -fd [-c 2000] sender receiver scene (h=sc4)")
    print("flux sc: rows reaching the window %.3f, bins used %d; sender row mean %.4f" % (
        (recv.sum(axis=(1, 2)) > 0).mean(), (recv.sum(axis=(0, 2)) > 0).sum(), send[:, :, 0].sum(1).mean()))


def general_bins(tmp: Path) -> None:
    """General bin expressions: the sky subdivision of
    tests/golden/patchbins.cal (recursion, select, if, asin, atan2, floor,
    sqrt, max, min, ^) with rcontrib -ab 0 in radiance mode: rays from
    inside the empty window room aimed out of the window reach the sky or
    the ground glow through the glass, so each record has the one bin of
    its ray's direction (deterministic)."""
    import shutil
    octp = oconv(w.window_room(ntri=0), tmp, "bins")
    shutil.copy(OUT / "patchbins.cal", tmp / "patchbins.cal")
    rng = np.random.default_rng(17)
    org = rng.uniform((1.0, 1.0, 0.5), (9.0, 5.0, 2.5), size=(3000, 3))
    x0, x1, z0, z1 = w.WINDOW
    tgt = np.column_stack([rng.uniform(x0 + .05, x1 - .05, 3000), np.zeros(3000), rng.uniform(z0 + .05, z1 - .05, 3000)])
    d = tgt - org
    rays = np.hstack([org, d / np.linalg.norm(d, axis=1, keepdims=True)])
    out = run(["rcontrib", "-h", "-u-", "-ab", "0", "-fdd", "-f", "patchbins.cal", "-b", "pbin", "-bn", "Npbins",
               "-m", "skyglow", "-m", "groundglow", octp.name], rays.astype("<f8").tobytes(), cwd=tmp)
    a = np.frombuffer(out, dtype="<f8").reshape(len(rays), -1, 3)
    np.savez_compressed(OUT / "general_bins.npz", rays=rays, bins=a[..., 0].astype(np.float32),
                        cmd="rcontrib -h -u- -ab 0 -fdd -f patchbins.cal -b pbin -bn Npbins -m skyglow -m groundglow")
    hit = a[..., 0] > 0
    print("general_bins: %d bins, %d rays with a bin, %d distinct bins hit" % (a.shape[1], hit.any(1).sum(),
                                                                                hit.any(0).sum()))


def cie_bins(tmp: Path) -> None:
    """CIE sky scanner bins (util/cieskyscan.cal, cbin) with rcontrib -ab 0
    in radiance mode: rays in random directions in a scene of the sky and
    ground glows alone (every direction meets the sky or the ground), for
    the default frame and one turned a quarter round (up +X)."""
    octp = oconv(w.SKY_GLOW, tmp, "cbins")
    rng = np.random.default_rng(19)
    d = rng.normal(size=(4000, 3))
    rays = np.hstack([np.zeros((4000, 3)), d / np.linalg.norm(d, axis=1, keepdims=True)])
    res = {}
    for key, p in (("default", []), ("upx", ["-p", "Ux=1,Uy=0,Uz=0"])):
        out = run(["rcontrib", "-h", "-u-", "-ab", "0", "-fdd", "-f", "cieskyscan.cal", *p, "-b", "cbin", "-bn",
                   "Ncbins", "-m", "skyglow", "-m", "groundglow", octp.name], rays.astype("<f8").tobytes(), cwd=tmp)
        res[key] = np.frombuffer(out, dtype="<f8").reshape(len(rays), -1, 3)[..., 0].astype(np.float32)
        print("cie_bins %s: %d bins, %d distinct bins hit" % (key, res[key].shape[1], (res[key] > 0).any(0).sum()))
    np.savez_compressed(OUT / "cie_bins.npz", rays=rays, **res,
                        cmd="rcontrib -h -u- -ab 0 -fdd -f cieskyscan.cal [-p Ux=1,Uy=0,Uz=0] -b cbin -bn Ncbins -m skyglow -m groundglow")


def translucent(tmp: Path, K: int = 256) -> None:
    """The trans material (rt/normal.c, MAT_TRANS): -I irradiance on a grid
    at 0.8 m (the light seen through the diffuser: shadow rays pass its
    specular transmission) and radiance of random view rays, deterministic
    with -ab 0 -st 1 (no lobe sampling); and radiance of view rays aimed at
    the translucent surfaces with -ab 1 -aa 0 -as 0 -st 0 (ambient from both
    sides, transmitted and reflected lobes sampled) as per-ray means and
    standard errors of K replicas (-u+)."""
    octp = oconv(w.trans_room(), tmp, "trans")
    grid = w.sensor_grid(40, 40)
    view = w.random_rays(1000, seed=13)
    base = ["rtrace", "-h", "-u-", "-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0", "-st", "1", "-fdd", "-ov"]
    irr = np.frombuffer(run([*base[:2], *base[2:3], "-I", *base[3:], octp], grid.astype("<f8").tobytes()),
                        dtype="<f8").reshape(-1, 3)
    rad = np.frombuffer(run([*base, octp], view.astype("<f8").tobytes()), dtype="<f8").reshape(-1, 3)
    rng = np.random.default_rng(13)
    org = rng.uniform((0.5, 0.5, 0.3), (9.5, 7.5, 2.0), size=(60, 3))
    X, Y = 10.0, 8.0
    tgt = np.column_stack([rng.uniform(X / 2 - 1.8, X / 2 + 1.8, 60), rng.uniform(Y / 2 - 1.3, Y / 2 + 1.3, 60),
                           np.full(60, 2.2)])
    tgt[30:] = rng.uniform((1, 1, 0.3), (9, 7, 1.7), size=(30, 3))       # towards the panels' region
    d = tgt - org
    aimed = np.hstack([org, d / np.linalg.norm(d, axis=1, keepdims=True)])
    a = np.frombuffer(run(["rtrace", "-h", "-u+", "-ab", "1", "-aa", "0", "-as", "0", "-ad", "256", "-lw", "1e-4",
                           "-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0", "-st", "0", "-fdd", "-ov", octp],
                          np.repeat(aimed, K, axis=0).astype("<f8").tobytes()), dtype="<f8").reshape(60, K, 3)
    np.savez_compressed(OUT / "translucent.npz", grid=grid, irradiance=irr, view=view, radiance=rad, aimed=aimed,
                        K=K, ab1_mean=a.mean(1), ab1_se=a.std(1, ddof=1) / np.sqrt(K),
                        cmd="rtrace -h -u- -ab 0 -dj 0 -ds 0 -dr 0 -dt 0 -st 1 [-I] | -u+ -ab 1 -aa 0 -as 0 -ad 256 "
                            "-lw 1e-4 -st 0")
    print("translucent: irradiance mean %.4g, radiance mean %.4g, ab1 mean %.4g" % (irr.mean(), rad.mean(), a.mean()))


def circular_sources(tmp: Path, K: int = 256) -> None:
    """Sphere and disk lights (rt/srcsupp.c sphsetsrc, rsetsrc; the
    circular trims of rt/srcsamp.c:85-109), and cylinder lights (cylsetsrc,
    cylpart, scylform) in a second room: -I direct irradiance on a grid
    at 0.8 m and one at 2.3 m (close to the lights), deterministic with
    -dj 0 -ds 0 and with -ds 0.2 (the disk split into pieces), and with
    -dj 0.9 (jittered and trimmed samples) as per-sensor means and standard
    errors of K replicas (-u+)."""
    _circular(tmp, K, "lamp", w.lamp_room(), "circular_sources.npz")
    _circular(tmp, K, "tube", w.tube_room(), "cylinder_sources.npz")


def _circular(tmp: Path, K: int, name: str, text: str, fixture: str) -> None:
    octp = oconv(text, tmp, name)
    rays = np.vstack([w.sensor_grid(40, 40), w.sensor_grid(20, 20, z=2.3)])
    inp = rays.astype("<f8").tobytes()
    base = ["rtrace", "-h", "-u-", "-I", "-ab", "0", "-dr", "0", "-dt", "0", "-fdd", "-ov"]
    ds0 = np.frombuffer(run([*base, "-dj", "0", "-ds", "0", octp], inp), dtype="<f8").reshape(-1, 3)
    ds2 = np.frombuffer(run([*base, "-dj", "0", "-ds", "0.2", octp], inp), dtype="<f8").reshape(-1, 3)
    sub = rays[::8]
    a = np.frombuffer(run([*base[:2], "-u+", *base[3:], "-dj", "0.9", "-ds", "0.2", octp],
                          np.repeat(sub, K, axis=0).astype("<f8").tobytes()), dtype="<f8").reshape(len(sub), K, 3)
    np.savez_compressed(OUT / fixture, rays=rays, ds0=ds0, ds2=ds2, dj_rays=sub, K=K,
                        dj_mean=a.mean(1), dj_se=a.std(1, ddof=1) / np.sqrt(K),
                        cmd="rtrace -h -u- -I -ab 0 -dr 0 -dt 0 -dj 0 [-ds 0 | -ds 0.2] | -u+ -dj 0.9 -ds 0.2")
    print("%s: lit %.3f, ds0 mean %.4g, ds2 mean %.4g, dj mean %.4g" % (
        fixture, (ds0[:, 0] > 0).mean(), ds0.mean(), ds2.mean(), a.mean()))


def instances(tmp: Path) -> None:
    """Instances (rt/o_instance.c, common/instance.c): the furniture octree
    placed 12 times in the room, rotated, scaled, one mirrored, some with an
    overriding material.  Both octrees (frozen, made by the reference oconv)
    are kept as fixtures beside the vectors; the room octree names the
    furniture octree by its file name.  Random interior rays: first-hit
    surfaces and distances, deterministic -ab 0 radiance and -I
    irradiance."""
    (tmp / "inst_sub.rad").write_text(w.furniture())
    (tmp / "inst_sub.oct").write_bytes(run(["oconv", "-f", "inst_sub.rad"], cwd=tmp))
    (tmp / "inst_main.rad").write_text(w.instance_room("inst_sub.oct"))
    (tmp / "inst_main.oct").write_bytes(run(["oconv", "-f", "inst_main.rad"], cwd=tmp))
    rays = w.random_rays(4000, seed=11)
    rng = np.random.default_rng(11)                # half of them aimed low, where the furniture stands
    tgt = rng.uniform((0.5, 0.5, 0.0), (9.5, 7.5, 1.2), size=(2000, 3))
    d = tgt - rays[:2000, :3]
    rays[:2000, 3:] = d / np.linalg.norm(d, axis=1, keepdims=True)
    inp = rays.astype("<f8").tobytes()
    det = ["-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0"]
    hit = names(run(["rtrace", "-h", "-u-", "-ab", "0", "-fda", "-os", "inst_main.oct"], inp, cwd=tmp))
    dist = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", "-fdd", "-oL", "inst_main.oct"], inp, cwd=tmp),
                         dtype="<f8")
    val = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", *det, "-fdd", "-ov", "inst_main.oct"], inp, cwd=tmp),
                        dtype="<f8").reshape(-1, 3)
    irr = np.frombuffer(run(["rtrace", "-h", "-u-", "-I", "-ab", "0", *det, "-fdd", "-ov", "inst_main.oct"], inp,
                            cwd=tmp), dtype="<f8").reshape(-1, 3)
    for f in ("inst_sub.oct", "inst_main.oct"):
        (OUT / f).write_bytes((tmp / f).read_bytes())
    np.savez_compressed(OUT / "instances.npz", rays=rays, hit_name=hit, hit_dist=dist, radiance=val,
                        irradiance=irr, cmd="rtrace -h -u- -ab 0 -os | -oL | [-I] -dj 0 -ds 0 -dr 0 -dt 0 -ov")
    print("instances: %d of %d rays hit instanced surfaces" % (
        sum(not n.startswith(("floor", "ceiling", "north", "south", "east", "west", "light", "*")) for n in hit),
        len(hit)))


def meshes(tmp: Path) -> None:
    """Compiled meshes (rt/o_mesh.c, common/mesh.c, common/readmesh.c): a
    sphere and a bumpy sheet of triangles with two materials, compiled by
    the reference obj2mesh, placed 10 times in the room, rotated, scaled,
    mirrored, some with their own material.  The mesh file and the room's
    octree (frozen, by the reference oconv; it names the mesh by its file
    name) are kept beside the vectors.  Random interior rays: first-hit
    surfaces and distances, deterministic -ab 0 radiance and -I
    irradiance."""
    (tmp / "mesh.obj").write_text(w.mesh_obj())
    (tmp / "mesh_mat.rad").write_text(w.mesh_materials())
    run(["obj2mesh", "-a", "mesh_mat.rad", "mesh.obj", "mesh_parts.rtm"], b"", cwd=tmp)
    (tmp / "mesh_room.rad").write_text(w.mesh_room("mesh_parts.rtm"))
    (tmp / "mesh_room.oct").write_bytes(run(["oconv", "-f", "mesh_room.rad"], b"", cwd=tmp))
    rays = w.random_rays(4000, seed=12)
    rng = np.random.default_rng(12)                # half of them aimed low, where the meshes stand
    tgt = rng.uniform((0.5, 0.5, 0.0), (9.5, 7.5, 1.1), size=(2000, 3))
    d = tgt - rays[:2000, :3]
    rays[:2000, 3:] = d / np.linalg.norm(d, axis=1, keepdims=True)
    inp = rays.astype("<f8").tobytes()
    det = ["-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0"]
    hit = names(run(["rtrace", "-h", "-u-", "-ab", "0", "-fda", "-os", "mesh_room.oct"], inp, cwd=tmp))
    dist = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", "-fdd", "-oL", "mesh_room.oct"], inp, cwd=tmp),
                         dtype="<f8")
    val = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", *det, "-fdd", "-ov", "mesh_room.oct"], inp,
                            cwd=tmp), dtype="<f8").reshape(-1, 3)
    irr = np.frombuffer(run(["rtrace", "-h", "-u-", "-I", "-ab", "0", *det, "-fdd", "-ov", "mesh_room.oct"], inp,
                            cwd=tmp), dtype="<f8").reshape(-1, 3)
    # a mesh with vertex normals (refused: their shading perturbation is not built)
    (tmp / "mesh_vn.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nvn 0 0.1 1\nvn 0.1 0 1\n"
                                     "usemtl mesh_red\nf 1//1 2//2 3//3\n")
    run(["obj2mesh", "-a", "mesh_mat.rad", "mesh_vn.obj", "mesh_normals.rtm"], b"", cwd=tmp)
    (tmp / "mesh_normals.rad").write_text("void mesh smooth\n1 mesh_normals.rtm\n0\n0\n")
    (tmp / "mesh_normals.oct").write_bytes(run(["oconv", "-f", "mesh_normals.rad"], b"", cwd=tmp))
    for f in ("mesh_parts.rtm", "mesh_room.oct", "mesh_normals.rtm", "mesh_normals.oct"):
        (OUT / f).write_bytes((tmp / f).read_bytes())
    np.savez_compressed(OUT / "meshes.npz", rays=rays, hit_name=hit, hit_dist=dist, radiance=val,
                        irradiance=irr, cmd="rtrace -h -u- -ab 0 -os | -oL | [-I] -dj 0 -ds 0 -dr 0 -dt 0 -ov")
    print("meshes: %d of %d rays hit mesh triangles" % (
        sum(n == "M-Tri" or n.startswith("mesh") for n in hit), len(hit)))


def smooth_meshes(tmp: Path, nstat: int = 24, K: int = 256) -> None:
    """Meshes with vertex normals (rt/o_mesh.c:185-206): the sphere and
    sheet of `meshes` with a normal at every vertex, compiled by the
    reference obj2mesh and placed 10 times in the room (one mirrored, some
    scaled, some with a plastic or a rough metal of their own).  Random
    interior rays, half aimed at the meshes: first-hit names and distances,
    the surface normal and the shading normal (-oNn), and deterministic
    -ab 0 -st 1 radiance (direct light through the shading normal, the
    rough lobes' direct Gaussian term only, none sampled); and, for
    `nstat` rays that meet a mesh, rcontrib -ab 1 contributions of the
    ceiling light as means and standard errors over K replicas (-u+,
    independent processes)."""
    (tmp / "mesh_vn.obj").write_text(w.mesh_obj(normals=True))
    (tmp / "mesh_mat.rad").write_text(w.mesh_materials())
    run(["obj2mesh", "-a", "mesh_mat.rad", "mesh_vn.obj", "mesh_smooth.rtm"], b"", cwd=tmp)
    (tmp / "mesh_smooth_room.rad").write_text(w.mesh_room("mesh_smooth.rtm", metal=True))
    (tmp / "mesh_smooth_room.oct").write_bytes(run(["oconv", "-f", "mesh_smooth_room.rad"], b"", cwd=tmp))
    rays = w.random_rays(3000, seed=13)
    rng = np.random.default_rng(13)
    tgt = rng.uniform((0.5, 0.5, 0.0), (9.5, 7.5, 1.1), size=(2000, 3))
    d = tgt - rays[:2000, :3]
    rays[:2000, 3:] = d / np.linalg.norm(d, axis=1, keepdims=True)
    inp = rays.astype("<f8").tobytes()
    octn = "mesh_smooth_room.oct"
    det = ["-dj", "0", "-ds", "0", "-dr", "0", "-dt", "0"]
    hit = names(run(["rtrace", "-h", "-u-", "-ab", "0", "-fda", "-os", octn], inp, cwd=tmp))
    dist = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", "-fdd", "-oL", octn], inp, cwd=tmp), dtype="<f8")
    nn = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", "-fdd", "-oNn", octn], inp, cwd=tmp),
                       dtype="<f8").reshape(-1, 6)
    val = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", *det, "-st", "1", "-fdd", "-ov", octn], inp,
                            cwd=tmp), dtype="<f8").reshape(-1, 3)
    smooth = np.abs(nn[:, :3] - nn[:, 3:]).max(1) > 1e-6
    onmesh = np.array([n == "M-Tri" or n.startswith("mesh") for n in hit])
    pick = np.nonzero(onmesh[:2000] & (dist[:2000] < 1e9))[0][:: max(1, int(onmesh[:2000].sum()) // nstat)][:nstat]
    srays = rays[pick]
    out = run_independent(["rcontrib", "-h", "-u+", "-ab", "1", "-ad", "256", "-lw", "1e-4", "-fdd", "-m", "light_mat",
                           octn], np.repeat(srays, K, axis=0), cwd=tmp)
    a = np.frombuffer(out, dtype="<f8").reshape(len(srays), K, 3)
    # the mesh with texture coordinates too: -oc (rt/rtrace.c:766-772) and -on of every ray
    (tmp / "mesh_uv.obj").write_text(w.mesh_obj(normals=True, uv=True))
    run(["obj2mesh", "-a", "mesh_mat.rad", "mesh_uv.obj", "mesh_uv.rtm"], b"", cwd=tmp)
    (tmp / "mesh_uv_room.rad").write_text(w.mesh_room("mesh_uv.rtm", seed=1))
    (tmp / "mesh_uv_room.oct").write_bytes(run(["oconv", "-f", "mesh_uv_room.rad"], b"", cwd=tmp))
    cn = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", "-fdd", "-ocn", "mesh_uv_room.oct"], inp, cwd=tmp),
                       dtype="<f8").reshape(-1, 5)
    # the same mesh under a glass of its own (refused: glass is not shaded through vertex normals here)
    (tmp / "mesh_smooth_glass.rad").write_text("void glass smooth_glass\n0\n0\n3 0.9 0.9 0.9\n\n"
                                               "smooth_glass mesh glassy\n1 mesh_smooth.rtm\n0\n0\n")
    (tmp / "mesh_smooth_glass.oct").write_bytes(run(["oconv", "-f", "mesh_smooth_glass.rad"], b"", cwd=tmp))
    for f in ("mesh_smooth.rtm", "mesh_smooth_room.oct", "mesh_smooth_glass.oct", "mesh_uv.rtm", "mesh_uv_room.oct"):
        (OUT / f).write_bytes((tmp / f).read_bytes())
    np.savez_compressed(OUT / "smooth_meshes.npz", rays=rays, hit_name=hit, hit_dist=dist, N=nn[:, :3], n=nn[:, 3:],
                        radiance=val, stat_rays=srays, K=K, mean=a.mean(1), se=a.std(1, ddof=1) / np.sqrt(K),
                        uv_c=cn[:, :2], uv_n=cn[:, 2:],
                        cmd="rtrace -h -u- -ab 0 -os | -oL | -oNn | -dj 0 -ds 0 -dr 0 -dt 0 -st 1 -ov; "
                            "rcontrib -h -u+ -ab 1 -ad 256 -lw 1e-4 -m light_mat (independent -n 1 processes); "
                            "mesh_uv_room: rtrace -h -u- -ab 0 -ocn")
    print("smooth meshes: %d of %d rays hit mesh triangles, %d with a perturbed normal; %d stat rays" % (
        onmesh.sum(), len(hit), smooth.sum(), len(srays)))


# bin groups of the 146 columns: ground, then the 8 Reinhart MF:1 altitude rows
ROW_EDGES = [0, 1, 31, 61, 85, 109, 127, 139, 145, 146]

MODS = ["-m", "groundglow", "-f", "reinhartb.cal", "-p", "MF=1", "-b", "rbin", "-bn", "Nrbins", "-m", "skyglow"]


def c2_stats(tmp: Path, nsens: int = 32, K: int = 256, ab: int = 3) -> None:
    """rcontrib daylight coefficients on a subset of the 64 x 64 grid, each
    sensor replicated K times with uncorrelated sampling (-u+, the
    reference's default) in independent processes: per-sensor, per-bin
    sample mean and standard error of channel 0 (the scene is gray)."""
    octp = oconv(w.window_room(), tmp, "c2")
    grid = w.sensor_grid(64, 64)
    idx = np.linspace(0, len(grid) - 1, nsens).astype(int)
    rays = grid[idx]
    rep = np.repeat(rays, K, axis=0)
    out = run_independent(["rcontrib", "-h", "-u+", "-I+", "-ab", str(ab), "-ad", "1024", "-lw", "1e-4", "-c", "1",
                           "-fdd", *MODS, octp], rep)
    a = np.frombuffer(out, dtype="<f8").reshape(nsens, K, 146, 3)
    assert (a[..., 0] == a[..., 1]).all() and (a[..., 0] == a[..., 2]).all()
    a = a[..., 0]
    check_independent(a)
    grp = np.stack([a[:, :, e0:e1].sum(2) for e0, e1 in zip(ROW_EDGES[:-1], ROW_EDGES[1:])], 2)
    np.savez_compressed(OUT / f"c2_stats_ab{ab}.npz", sensor_index=idx, rays=rays, K=K,
                        mean=a.mean(1), se=a.std(1, ddof=1) / np.sqrt(K), nnz=(a > 0).sum(1),
                        group_mean=grp.mean(1), group_se=grp.std(1, ddof=1) / np.sqrt(K),
                        total_mean=a.sum(2).mean(1), total_se=a.sum(2).std(1, ddof=1) / np.sqrt(K),
                        cmd="rcontrib -h -u+ -I+ -ab %d -ad 1024 -lw 1e-4 -c 1 " % ab + " ".join(MODS)
                        + " (independent -n 1 processes)")
    print("c2_stats ab%d: mean total %.4g" % (ab, a.sum(2).mean()))


def check_independent(a: np.ndarray) -> None:
    """No two replicas of a sensor that reach ten bins or more may be equal
    (equal replicas mean shared random streams; records of a few sky
    samples through the window can coincide by chance)."""
    for s in range(a.shape[0]):
        rich = a[s][(a[s] > 0).sum(1) >= 10]
        if len(rich) > 1:
            assert len(np.unique(rich, axis=0)) == len(rich), f"sensor {s}: replicas repeat"


def c2_headline(tmp: Path, nsens: int = 256, K: int = 64) -> None:
    """The headline rcontrib workload (the window room, -I+ -ab 3 -ad 1024
    -lw 1e-4 -c 1, Reinhart MF:1 + ground) on 256 evenly spaced sensors of
    its 64 x 64 grid, each replicated 64 times with -u+ in independent
    processes: 64 x 1,024 = 2^16 first-hemisphere samples per sensor.
    Per-sensor, per-bin mean and standard error of channel 0 (the scene is
    gray), float32."""
    octp = oconv(w.window_room(), tmp, "c2")
    grid = w.sensor_grid(64, 64)
    idx = np.linspace(0, len(grid) - 1, nsens).astype(int)
    rays = grid[idx]
    rep = np.repeat(rays, K, axis=0)
    out = run_independent(["rcontrib", "-h", "-u+", "-I+", "-ab", "3", "-ad", "1024", "-lw", "1e-4", "-c", "1",
                           "-fdd", *MODS, octp], rep)
    a = np.frombuffer(out, dtype="<f8").reshape(nsens, K, 146, 3)
    assert (a[..., 0] == a[..., 1]).all() and (a[..., 0] == a[..., 2]).all()
    a = a[..., 0]
    check_independent(a)
    grp = np.stack([a[:, :, e0:e1].sum(2) for e0, e1 in zip(ROW_EDGES[:-1], ROW_EDGES[1:])], 2)
    np.savez_compressed(OUT / "c2_headline.npz", sensor_index=idx, rays=rays, K=K,
                        mean=a.mean(1).astype(np.float32), se=(a.std(1, ddof=1) / np.sqrt(K)).astype(np.float32),
                        nnz=(a > 0).sum(1).astype(np.int16),
                        group_mean=grp.mean(1), group_se=grp.std(1, ddof=1) / np.sqrt(K),
                        total_mean=a.sum(2).mean(1), total_se=a.sum(2).std(1, ddof=1) / np.sqrt(K),
                        cmd="rcontrib -h -u+ -I+ -ab 3 -ad 1024 -lw 1e-4 -c 1 " + " ".join(MODS)
                        + " (64 replicas per sensor in independent -n 1 processes)")
    print("c2_headline: mean total %.4g, lit sensors %d" % (a.sum(2).mean(), (a.sum((1, 2)) > 0).sum()))


def grad_fd(tmp: Path, nx: int = 32) -> None:
    """Differenced reference runs for the gradients: the window room with
    its 20,000 triangles in 64 plastic materials and the glass window,
    rtrace -u- -I -ab 2 -ad 1024 -aa 0 -as 0 -lw 1e-6 at a 32 x 32 grid of
    sensors, with one parameter at a time moved by -delta and +delta: the
    gray reflectance of three materials (irradiance is quadratic in each at
    two bounces, so the central difference is exact for the reference's
    fixed-seed estimate), and the window's transmissivity.  With -lw 1e-6
    no ray's fate depends on the weights, so the two runs of a pair draw
    the same random numbers (common random numbers).  The sensors run in
    eight fixed shards (the same in every run), one process each."""
    import re
    base = w.window_room(seed=0, ntri=20000, nmat=64)
    rays = w.sensor_grid(nx, nx)
    args = ["rtrace", "-h", "-u-", "-I", "-ab", "2", "-ad", "1024", "-aa", "0", "-as", "0", "-lw", "1e-6",
            "-fdd", "-ov"]
    # the glass step is small: at 0.02 the reference's central difference
    # is 8% above its value at 0.005, which the oracle's differences (same
    # at 0.02 and 0.005) and the path-replay gradient agree with
    params = [("tri_mat3", 0.05), ("tri_mat17", 0.05), ("tri_mat40", 0.05), ("window_glass", 0.005)]

    def with_value(name, dv):
        def mat(m):
            vals = [float(v) for v in m.group(2).split()]
            if name == "window_glass":
                vals = [v + dv for v in vals]
            else:
                vals = [v + dv for v in vals[:3]] + vals[3:]
            return m.group(1) + " ".join("%.9g" % v for v in vals) + "\n"
        pat = r"(void (?:plastic|glass) " + re.escape(name) + r"\n0\n0\n\d+ )([^\n]*)\n"
        out, k = re.subn(pat, mat, base)
        assert k == 1, name
        return out

    def irradiance(text, tag):
        octp = oconv(text, tmp, f"g_{tag}")
        parts = np.array_split(rays, 8)
        env = dict(os.environ, RAYPATH=f".:{REF / 'lib'}")
        procs = []
        for i, part in enumerate(parts):
            fi = tmp / f"g_{tag}_{i}.in"
            fi.write_bytes(part.astype("<f8").tobytes())
            procs.append(subprocess.Popen([str(BIN / args[0]), *args[1:], str(octp)], stdin=open(fi, "rb"),
                                          stdout=open(tmp / f"g_{tag}_{i}.out", "wb"), env=env))
        for p in procs:
            assert p.wait() == 0
        return np.concatenate([np.frombuffer((tmp / f"g_{tag}_{i}.out").read_bytes(), dtype="<f8")
                               for i in range(8)]).reshape(-1, 3)

    e0 = irradiance(base, "base")
    fd = []
    for name, d in params:
        ep = irradiance(with_value(name, +d), name + "p")
        em = irradiance(with_value(name, -d), name + "m")
        fd.append((ep - em) / (2 * d))
    fd = np.stack(fd, 0)                                   # params x sensors x 3
    np.savez_compressed(OUT / "grad_fd.npz", rays=rays, e0=e0, fd=fd,
                        names=np.array([p[0] for p in params]), deltas=np.array([p[1] for p in params]),
                        cmd=" ".join(args[1:]) + " (central differences of the parameters, 8 fixed shards)")
    print("grad_fd: mean irradiance %.4g; mean derivatives %s" % (e0[:, 0].mean(), fd[:, :, 0].mean(1)))


def reference_wrappers():
    """The reference's own Python functions (src/pyradiance/rt.py rtrace and
    Rcontrib, util.py dctimestep), loaded from the reference tree with their
    program path pointed at the reference programs built here.  The modules
    they import that need the reference's compiled extensions (bsdf, the
    scene model, ray parameters) are not used by these functions and are
    stood in for by empty modules.  Nothing is written into the reference
    tree (no bytecode)."""
    import importlib.util
    import types
    sys.dont_write_bytecode = True
    src = REFERENCE_TREE / "src" / "pyradiance"
    pkg = types.ModuleType("refpyradiance")
    pkg.__path__ = [str(src)]
    sys.modules["refpyradiance"] = pkg
    stubs = {"bsdf": ("spec_xyz", "xyz_rgb"), "model": ("Primitive", "Scene"),
             "rad_params": ("View", "RayParams", "get_ray_params_args", "get_view_args"),
             "ot": ("getbbox",), "px": ("pvaluer",), "cal": ("cnt",)}
    for name, attrs in stubs.items():
        m = types.ModuleType(f"refpyradiance.{name}")
        for a in attrs:
            setattr(m, a, type(a, (), {}))
        sys.modules[f"refpyradiance.{name}"] = m
    mods = {}
    for name in ("anci", "rt", "util"):
        spec = importlib.util.spec_from_file_location(f"refpyradiance.{name}", src / f"{name}.py")
        m = importlib.util.module_from_spec(spec)
        sys.modules[f"refpyradiance.{name}"] = m
        spec.loader.exec_module(m)
        m.BINPATH = BIN
        mods[name] = m
    os.environ["RAYPATH"] = f".:{REF / 'lib'}"
    return mods["rt"], mods["util"]


def bytes_surface(tmp: Path) -> None:
    """The bytes pyradiance's own functions return, run on the reference
    programs: rtrace of the direct-irradiance workload at 200 of its sensors
    (ASCII and binary double, with headers; first-hit names), rcontrib of
    rays leaving the small window room through its glass (deterministic at
    -ab 0: each ray reaches the sky or the ground through the window), once
    with the sky's columns sent to a file (add_modifier(output=...)), and
    dctimestep of a small matrix pair.  The frozen octrees are kept in the
    fixture so that the drop-in reads the same files (their headers are
    copied into the outputs)."""
    rt, util = reference_wrappers()
    (tmp / "c1b.rad").write_text(w.daylight_room())
    (tmp / "c2b.rad").write_text(w.window_room(seed=2, ntri=2000))
    c1oct, c2oct = tmp / "c1_ref.oct", tmp / "c2s_ref.oct"
    c1oct.write_bytes(run(["oconv", "-f", tmp / "c1b.rad"]))
    c2oct.write_bytes(run(["oconv", "-f", tmp / "c2b.rad"]))
    rays1 = w.sensor_grid(100, 100)[::50]
    params1 = ["-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0"]
    c1_a = rt.rtrace(w.rays_ascii(rays1), str(c1oct), irradiance=True, params=params1)
    c1_d = rt.rtrace(rays1.astype("<f8").tobytes(), str(c1oct), irradiance=True, inform="d", outform="d",
                     params=params1)
    c1_s = rt.rtrace(w.rays_ascii(rays1), str(c1oct), outspec="s", params=["-ab", "0"])
    rng = np.random.default_rng(12)
    org = np.column_stack([rng.uniform(4.0, 6.0, 64), rng.uniform(0.8, 1.5, 64), rng.uniform(1.0, 2.0, 64)])
    d = np.column_stack([rng.uniform(-0.4, 0.4, 64), -np.ones(64), rng.uniform(-0.3, 0.6, 64)])
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays2 = np.column_stack([org, d])
    rcp = ["-ab", "0", "-dj", "0", "-lw", "1e-4"]
    sky = dict(modifier="skyglow", calfile="reinhartb.cal", param="MF=1", binv="rbin", nbins="Nrbins")
    cwd = os.getcwd()
    os.chdir(tmp)
    try:
        rc = rt.Rcontrib(w.rays_ascii(rays2), str(c2oct), params=rcp)
        rc.add_modifier(modifier="groundglow").add_modifier(**sky)
        c2_out = rc()
        rc = rt.Rcontrib(w.rays_ascii(rays2), str(c2oct), params=rcp)
        rc.add_modifier(modifier="groundglow").add_modifier(**sky, output="sky_%s.mtx")
        c2_split = rc()
        c2_file = (tmp / "sky_skyglow.mtx").read_bytes()
        rc = rt.Rcontrib(w.rays_ascii(rays2), str(c2oct), params=rcp)
        rc.add_modifier(modifier="groundglow").add_modifier(**sky, output="bin_%s_%03d.mtx")
        c2_binsplit = rc()
        bin_files = sorted(tmp.glob("bin_skyglow_*.mtx"))
        c2_bins = b"\0".join(f.name.encode() + b"\n" + f.read_bytes() for f in bin_files)
    finally:
        os.chdir(cwd)
    g = np.load(OUT / "dct_small.npz")
    for name, m in (("D", g["dc"]), ("S", g["sky"])):
        (tmp / f"{name}.mtx").write_bytes((f"#?RADIANCE\nNROWS={m.shape[0]}\nNCOLS={m.shape[1]}\nNCOMP=3\n"
                                            "BigEndian=0\nFORMAT=float\n\n").encode() + m.astype("<f4").tobytes())
    dct_a = util.dctimestep(str(tmp / "D.mtx"), str(tmp / "S.mtx"))
    dct_d = util.dctimestep(str(tmp / "D.mtx"), str(tmp / "S.mtx"), outform="d")
    u8 = lambda b: np.frombuffer(b, dtype=np.uint8)
    np.savez_compressed(OUT / "bytes_surface.npz", c1_oct=u8(c1oct.read_bytes()), c2_oct=u8(c2oct.read_bytes()),
                        rays1=rays1, rays2=rays2, c1_a=u8(c1_a), c1_d=u8(c1_d), c1_s=u8(c1_s), c2_out=u8(c2_out),
                        c2_split=u8(c2_split), c2_file=u8(c2_file), c2_binsplit=u8(c2_binsplit),
                        c2_bins=u8(c2_bins), dct_a=u8(dct_a), dct_d=u8(dct_d),
                        params1=np.array(params1), rcp=np.array(rcp))
    print("bytes_surface: rtrace %d/%d/%d bytes, rcontrib %d (+ %d in a file), dctimestep %d/%d bytes" %
          (len(c1_a), len(c1_d), len(c1_s), len(c2_out), len(c2_file), len(dct_a), len(dct_d)))


def edge_rays(tmp: Path) -> None:
    """First-hit names of rays aimed at the edges and corners of the
    direct-irradiance room's box faces (exactly, and 0.1 mm inside), from
    the reference rtrace -ab 0 -os: where the FTINY edge rules of
    common/face.c and the ties of rt/raytrace.c decide."""
    text = w.daylight_room()
    octp = oconv(text, tmp, "c1e")
    polys = w.polygons(text)
    out = {}
    for key, inset in (("near", 1e-4), ("exact", 0.0)):
        rays, _ = w.aimed_rays(polys, inset)
        out[key + "_rays"] = rays
        out[key + "_names"] = names(run(["rtrace", "-h", "-u-", "-ab", "0", "-fda", "-os", octp],
                                        rays.astype("<f8").tobytes(), cwd=octp.parent))
    np.savez_compressed(OUT / "edges.npz", cmd="rtrace -h -u- -ab 0 -fda -os", **out)
    print("edges: %d + %d rays" % (len(out["near_rays"]), len(out["exact_rays"])))


def dct_four() -> None:
    """dctimestep's four-matrix form (util/dctimestep.c:243-264): view
    (sensors x 145 Klems), transmission (145 x 145), daylight (145 x 146) and
    sky (146 x 12 hours), random non-negative values with zeros."""
    rng = np.random.default_rng(9)
    mats = {}
    for name, shp, zf in (("V", (40, 145), .3), ("T", (145, 145), .5), ("D", (145, 146), .3), ("S", (146, 12), .2)):
        m = rng.lognormal(-2, 1, size=(*shp, 3)).astype(np.float32)
        m[rng.random(shp) < zf] = 0
        mats[name] = m
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        for name, m in mats.items():
            hdr = (f"#?RADIANCE\nNROWS={m.shape[0]}\nNCOLS={m.shape[1]}\nNCOMP=3\nBigEndian=0\n"
                   "FORMAT=float\n\n").encode()
            (td / f"{name}.mtx").write_bytes(hdr + m.astype("<f4").tobytes())
        out = run(["dctimestep", "-h", "-od", *(td / f"{n}.mtx" for n in "VTDS")])
    res = np.frombuffer(out, dtype="<f8").reshape(40, 12, 3)
    np.savez_compressed(OUT / "dct_four.npz", out=res, cmd="dctimestep -h -od V.mtx T.mtx D.mtx S.mtx",
                        **mats)
    print("dct_four: max %.4g" % res.max())


def rmtxop_cases() -> None:
    """rmtxop (util/rmtxop.c) on one 5 x 7 x 3 matrix: transpose, scale,
    component transform with and without a folded scale, both together."""
    rng = np.random.default_rng(13)
    m = rng.lognormal(-1, 1, size=(5, 7, 3))
    cases = [[], ["-t"], ["-s", "2.5"], ["-c", ".265", ".67", ".065"], ["-s", "3", "-c", ".2", ".3", ".5"],
             ["-t", "-s", "0.5", "-c", "1", "0", "0", "0", "0", "1"]]
    outs = {}
    with tempfile.TemporaryDirectory() as td:
        f = Path(td) / "m.mtx"
        f.write_bytes(b"#?RADIANCE\nNROWS=5\nNCOLS=7\nNCOMP=3\nBigEndian=0\nFORMAT=double\n\n" +
                      m.astype("<f8").tobytes())
        for i, c in enumerate(cases):
            outs[f"out{i}"] = np.frombuffer(run(["rmtxop", "-fd", *c, f]).split(b"\n\n", 1)[1], dtype="<f8")
    np.savez_compressed(OUT / "rmtxop.npz", m=m, cases=np.array([" ".join(c) for c in cases]), **outs)
    print("rmtxop: %d cases" % len(cases))


def rmtxop_chains() -> None:
    """rmtxop (util/rmtxop.c:383-525) on several matrices: products (a
    three-matrix chain whose rightmost matrix is a column, evaluated right
    to left), sums, element-wise products and quotients (with zeros, and by
    a one-component matrix), each matrix with its own scale, transform or
    transpose."""
    rng = np.random.default_rng(14)
    mats = {"A": rng.lognormal(-1, 1, (6, 9, 3)), "B": rng.lognormal(-1, 1, (9, 5, 3)),
            "Bt": rng.lognormal(-1, 1, (5, 9, 3)), "C": rng.lognormal(-1, 1, (5, 1, 3)),
            "D": rng.lognormal(-1, 1, (6, 9, 3)), "E": rng.lognormal(-1, 1, (6, 9, 1)),
            "F": rng.lognormal(-1, 1, (9, 9, 3))}
    mats["D"][rng.random((6, 9, 3)) < 0.2] = 0
    mats["E"][rng.random((6, 9, 1)) < 0.2] = 0
    chains = [["A", ".", "B"], ["A", ".", "B", ".", "C"], ["-s", "2", "A", ".", "-t", "Bt"],
              ["A", "+", "D"], ["A", "*", "D"], ["A", "/", "D"], ["A", "*", "E"], ["A", "/", "E"],
              ["A", ".", "F", ".", "B"], ["-c", ".3", ".6", ".1", "A", "*", "-c", ".3", ".6", ".1", "D"],
              ["A", "+", "-s", "0.5", "D", ".", "B"]]
    outs = {}
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        for k, m in mats.items():
            (td / f"{k}.mtx").write_bytes(
                f"#?RADIANCE\nNROWS={m.shape[0]}\nNCOLS={m.shape[1]}\nNCOMP={m.shape[2]}\nBigEndian=0\n"
                "FORMAT=double\n\n".encode() + m.astype("<f8").tobytes())
        for i, c in enumerate(chains):
            args = [a + ".mtx" if a in mats else a for a in c]
            out = run(["rmtxop", "-fd", *args], b"", cwd=td)
            head, body = out.split(b"\n\n", 1)
            dims = {ln.split("=")[0]: int(ln.split("=")[1]) for ln in head.decode().splitlines()
                    if ln.startswith(("NROWS=", "NCOLS=", "NCOMP="))}
            outs[f"out{i}"] = np.frombuffer(body, dtype="<f8").reshape(dims["NROWS"], dims["NCOLS"], dims["NCOMP"])
    np.savez_compressed(OUT / "rmtxop_chains.npz", chains=np.array([" ".join(c) for c in chains]), **mats, **outs)
    print("rmtxop chains: %d" % len(chains))


BTDF_CASES = {"fb_cols": dict(seed=1, basis="full", front=True, back=True, rows=False),
              "back_rows": dict(seed=2, basis="full", front=False, back=True, rows=True, base=0.01),
              "half_front": dict(seed=3, basis="half", front=True, back=False, rows=False, base=0.05),
              "no_trans": dict(seed=4, basis="full", front=False, back=False, rows=False)}


def btdf_matrices() -> None:
    """Klems matrix BSDFs (util/cmbsdf.c cm_loadBTDF, common/bsdf_m.c) as
    the reference dctimestep converts them: three synthetic XML files
    (workloads.klems_bsdf_xml, regenerated from their arguments by the
    tests): front and back transmission by columns, back transmission only
    by rows (reciprocity) with a floor taken out as a Lambertian part, and
    the Klems half basis, and a file without transmission data (the
    reference's Lambertian fallback: zeros).  Each transmission matrix is read through
    dctimestep with identity view, daylight and sky matrices; and one
    four-matrix product V T D sky per file."""
    def mtx(path, m):
        path.write_bytes(f"#?RADIANCE\nNROWS={m.shape[0]}\nNCOLS={m.shape[1]}\nNCOMP=3\nBigEndian=0\n"
                         "FORMAT=float\n\n".encode() + np.ascontiguousarray(m, dtype="<f4").tobytes())
    rng = np.random.default_rng(15)
    out = {}
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        for k, kw in BTDF_CASES.items():
            xml = td / f"{k}.xml"
            xml.write_text(w.klems_bsdf_xml(**kw))
            n = 145 if kw["basis"] == "full" else 77
            eye = np.repeat(np.eye(n)[:, :, None], 3, axis=2)
            mtx(td / "I.mtx", eye)
            T = np.frombuffer(run(["dctimestep", "-h", "-of", td / "I.mtx", xml, td / "I.mtx", td / "I.mtx"]),
                              dtype="<f4").reshape(n, n, 3)
            V = rng.lognormal(-3, 1, (4, n, 3))
            D = rng.lognormal(-4, 1, (n, 20, 3))
            S = rng.lognormal(1, 1, (20, 5, 3))
            for name, m in (("V", V), ("D", D), ("S", S)):
                mtx(td / f"{name}.mtx", m)
            R = np.frombuffer(run(["dctimestep", "-h", "-of", td / "V.mtx", xml, td / "D.mtx", td / "S.mtx"]),
                              dtype="<f4").reshape(4, 5, 3)
            out.update({f"{k}_T": T[..., 0].copy(), f"{k}_V": V.astype(np.float32), f"{k}_D": D.astype(np.float32),
                        f"{k}_S": S.astype(np.float32), f"{k}_R": R})
            print("btdf %s: T %s max %.4g, channels equal %s" % (k, T.shape, T.max(),
                                                                 bool((T[..., 0] == T[..., 1]).all())))
    np.savez_compressed(OUT / "btdf.npz", cases=np.array(list(BTDF_CASES)), **out)


def dct_small() -> None:
    """dctimestep on small matrices with the annual workload's value
    distributions (DC lognormal with zeros, sky spikes and night columns)."""
    dc, sky = w.dc_sky(48, 145, 40, seed=5)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        for name, m in (("dc", dc), ("sky", sky)):
            hdr = (f"#?RADIANCE\nNROWS={m.shape[0]}\nNCOLS={m.shape[1]}\nNCOMP=3\nBigEndian=0\n"
                   "FORMAT=float\n\n").encode()
            (td / f"{name}.mtx").write_bytes(hdr + m.astype("<f4").tobytes())
        out = run(["dctimestep", "-h", "-of", td / "dc.mtx", td / "sky.mtx"])
    res = np.frombuffer(out, dtype="<f4").reshape(48, 40, 3)
    np.savez_compressed(OUT / "dct_small.npz", dc=dc, sky=sky, out=res, cmd="dctimestep -h -of dc.mtx sky.mtx")
    print("dct_small: max %.4g" % res.max())


def octree_digests(tmp: Path) -> None:
    """Digest (node count, set count, pre-order hash of the tree and its
    leaf sets) of the reference oconv octree of each workload, read with the
    oracle's loader; the octree builder test rebuilds them from scene text."""
    sys.path.insert(0, str(ROOT))
    from oracle import pyoracle as po
    rows = {}
    for name, text in (("c1", w.daylight_room()), ("c2", w.window_room()), ("zoo", w.shape_zoo())):
        octp = oconv(text, tmp, name + "_d")
        rows[name] = np.array(po.octree_digest(octp), dtype=np.uint64)
    np.savez_compressed(OUT / "octree_ref.npz", **rows)
    print("octree digests:", {k: v.tolist() for k, v in rows.items()})


def ref_fixture_trace() -> None:
    """The reference's own test scene (tests/Resources/trace.oct, polygons,
    a cone and a sphere): first hits and distances of the two rays of its
    rtrace test (tests/test_rtrace.py:52-59) and of a fan of rays."""
    octp = REFERENCE_TREE / "tests" / "Resources" / "trace.oct"
    if not octp.exists():
        print("reference tree not found; skipping trace.oct vectors")
        return
    base = np.array([[1.0, 2.0, 3.0, 0.0, 0.0, 1.0], [4.0, 5.0, 6.0, 0.0, 1.0, 0.0]])
    rng = np.random.default_rng(11)
    o = rng.uniform((-2, 1, -15), (40, 4, 3), size=(2000, 3))
    d = rng.normal(size=(2000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.vstack([base, np.hstack([o, d])])
    inp = rays.astype("<f8").tobytes()
    hit = names(run(["rtrace", "-h", "-u-", "-ab", "0", "-fda", "-os", octp], inp, cwd=octp.parent))
    dist = np.frombuffer(run(["rtrace", "-h", "-u-", "-ab", "0", "-fdd", "-oL", octp], inp, cwd=octp.parent),
                         dtype="<f8")
    np.savez_compressed(OUT / "ref_trace_oct.npz", rays=rays, hit_name=hit, hit_dist=dist,
                        cmd="rtrace -h -u- -ab 0 -os | -oL  tests/Resources/trace.oct")
    print("ref_trace_oct: %d of %d rays hit" % ((hit != "*").sum(), len(hit)))


def main() -> None:
    if not (BIN / "rtrace").exists():
        sys.exit("reference programs missing: make -f oracle/build_ref.mk REF=/root/reference -j8")
    parts = {"octree": octree_digests, "c1": c1_direct, "c1p": c1_partitioned, "zoo": zoo, "glossy": glossy, "irr": surface_irradiance,
             "ss": supersampled_irradiance, "normals": normals, "inst": instances, "mesh": meshes, "meshvn": smooth_meshes, "circ": circular_sources,
             "trans": translucent, "bins": general_bins, "cbins": cie_bins,
             "spot": spotlights, "mirror": mirrors, "flux": flux_matrices, "flux_sc": flux_shirchiu,
             "dct": lambda tmp: dct_small(), "dct4": lambda tmp: dct_four(), "rmtxop": lambda tmp: rmtxop_cases(), "rmtxop_chains": lambda tmp: rmtxop_chains(), "btdf": lambda tmp: btdf_matrices(), "trace_oct": lambda tmp: ref_fixture_trace(),
             "c2ab1": lambda tmp: c2_stats(tmp, ab=1, K=256), "c2ab3": lambda tmp: c2_stats(tmp, ab=3, K=256),
             "c2head": c2_headline, "gradfd": grad_fd, "bytes": bytes_surface,
             "edges": edge_rays}
    only = sys.argv[1:] or list(parts)         # e.g. make_golden.py c1p
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        for name in only:
            parts[name](tmp)


if __name__ == "__main__":
    main()
