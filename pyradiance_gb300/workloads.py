"""Seeded synthetic scenes, sensor grids and matrices for the hot path.

Every generator is a pure function of its arguments (numpy ``default_rng``
seeded explicitly), so the same scene text, sensor file or matrix is produced
on any machine.  The scene text is plain Radiance scene description (``.rad``)
that the reference ``oconv`` and this package's own octree builder both read.

Workloads (sizes are the defaults):

* ``daylight_room`` -- 10 x 8 x 3 m closed room of 6 polygons (gray plastic
  0.5); 200 axis-aligned boxes (1,200 quads) with sizes U[0.2, 1.5] m and
  reflectance U[0.2, 0.7], standing 2-20 mm above the floor (bottoms that
  are coplanar with the floor and with each other, where boxes overlap,
  make oconv subdivide to its resolution limit); one 1 x 1 m ``light`` polygon of
  radiance 100 at the ceiling centre, coplanar with the ceiling and facing
  down.  Its modifier is defined last, so under Radiance's tie rule ("later
  modifier wins", rt/raytrace.c:573) the light, not the ceiling, is the
  surface hit where the two coincide.
* ``window_room`` -- the same room shell with a 3 x 2 m glass window
  (transmissivity 0.6) cut into the south (y = 0) wall, 20,000 random
  interior triangles (two edges of length U[0.05, 0.5] m from a random
  vertex, reflectance U[0.1, 0.8], one material each), and the glow sky and
  ground of the reference's own test fixture (tests/Resources/skyglow.rad).
* ``glossy_room`` -- the room with rough specular plastic and metal
  (the specular-lobe sampling workload).
* ``lamp_room`` -- the room lit by a sphere and a disk light (circular
  source shapes); ``tube_room`` -- lit by two cylinder lights;
  ``spot_room`` -- lit by two spotlights; ``mirror_room`` -- with mirrors.
* ``trans_room`` -- the room with translucent diffuser and frosted panels.
* ``furniture``, ``instance_room`` -- an object octree and a room holding
  transformed instances of it (the instance workload).
* ``sensor_grid`` -- cell-centred n x m grid at z = 0.8 facing +z.
* ``dc_sky`` -- daylight-coefficient and sky matrices with the value
  distributions of the annual dctimestep workload.
"""
from __future__ import annotations

import numpy as np

ROOM = (10.0, 8.0, 3.0)


def _poly(mod: str, name: str, verts) -> str:
    flat = " ".join(f"{v:.9g}" for p in verts for v in p)
    return f"{mod} polygon {name}\n0\n0\n{3 * len(verts)} {flat}\n\n"


def _mat_plastic(name: str, rho) -> str:
    r, g, b = rho
    return f"void plastic {name}\n0\n0\n5 {r:.9g} {g:.9g} {b:.9g} 0 0\n\n"


def _room_shell(mod: str, window=None) -> str:
    """Six inward-facing polygons; with ``window`` = (x0, x1, z0, z1) the
    south wall is split into four polygons around that opening."""
    X, Y, Z = ROOM
    out = []
    out.append(_poly(mod, "floor", [(0, 0, 0), (X, 0, 0), (X, Y, 0), (0, Y, 0)]))
    out.append(_poly(mod, "ceiling", [(0, 0, Z), (0, Y, Z), (X, Y, Z), (X, 0, Z)]))
    out.append(_poly(mod, "north", [(0, Y, 0), (X, Y, 0), (X, Y, Z), (0, Y, Z)]))
    out.append(_poly(mod, "west", [(0, 0, 0), (0, Y, 0), (0, Y, Z), (0, 0, Z)]))
    out.append(_poly(mod, "east", [(X, 0, 0), (X, 0, Z), (X, Y, Z), (X, Y, 0)]))
    if window is None:
        out.append(_poly(mod, "south", [(0, 0, 0), (0, 0, Z), (X, 0, Z), (X, 0, 0)]))
    elif isinstance(window, list):               # several openings side by side
        xl = 0.0
        for i, (x0, x1, z0, z1) in enumerate(window):
            out.append(_poly(mod, f"south_s{i}", [(xl, 0, 0), (xl, 0, Z), (x0, 0, Z), (x0, 0, 0)]))
            out.append(_poly(mod, f"south_b{i}", [(x0, 0, 0), (x0, 0, z0), (x1, 0, z0), (x1, 0, 0)]))
            out.append(_poly(mod, f"south_t{i}", [(x0, 0, z1), (x0, 0, Z), (x1, 0, Z), (x1, 0, z1)]))
            xl = x1
        out.append(_poly(mod, "south_r", [(xl, 0, 0), (xl, 0, Z), (X, 0, Z), (X, 0, 0)]))
    else:
        x0, x1, z0, z1 = window
        out.append(_poly(mod, "south_l", [(0, 0, 0), (0, 0, Z), (x0, 0, Z), (x0, 0, 0)]))
        out.append(_poly(mod, "south_r", [(x1, 0, 0), (x1, 0, Z), (X, 0, Z), (X, 0, 0)]))
        out.append(_poly(mod, "south_b", [(x0, 0, 0), (x0, 0, z0), (x1, 0, z0), (x1, 0, 0)]))
        out.append(_poly(mod, "south_t", [(x0, 0, z1), (x0, 0, Z), (x1, 0, Z), (x1, 0, z1)]))
    return "".join(out)


def _box(mod: str, name: str, o, s) -> str:
    """Axis-aligned box as 6 outward-facing quads."""
    x0, y0, z0 = o
    x1, y1, z1 = o[0] + s[0], o[1] + s[1], o[2] + s[2]
    q = []
    q.append(_poly(mod, f"{name}.bot", [(x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (x1, y0, z0)]))
    q.append(_poly(mod, f"{name}.top", [(x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)]))
    q.append(_poly(mod, f"{name}.s", [(x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1)]))
    q.append(_poly(mod, f"{name}.n", [(x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (x1, y1, z0)]))
    q.append(_poly(mod, f"{name}.w", [(x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0)]))
    q.append(_poly(mod, f"{name}.e", [(x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1)]))
    return "".join(q)


SKY_GLOW = """void glow skyglow
0
0
4 1 1 1 0

void glow groundglow
0
0
4 1 1 1 0

skyglow source sky
0
0
4 0 0 1 180

groundglow source ground
0
0
4 0 0 -1 180

"""


def daylight_room(seed: int = 0, nboxes: int = 200, light: bool = True) -> str:
    """Room + floor-standing boxes + ceiling light (the direct-irradiance
    workload).  Returns Radiance scene text."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    out = [_mat_plastic("room_mat", (0.5, 0.5, 0.5)), _room_shell("room_mat")]
    sizes = rng.uniform(0.2, 1.5, size=(nboxes, 3))
    fx = rng.uniform(0.0, 1.0, size=nboxes)
    fy = rng.uniform(0.0, 1.0, size=nboxes)
    rho = rng.uniform(0.2, 0.7, size=nboxes)
    lift = rng.uniform(0.002, 0.02, size=nboxes)
    for i in range(nboxes):
        s = sizes[i]
        o = (fx[i] * (X - s[0]), fy[i] * (Y - s[1]), lift[i])
        out.append(_mat_plastic(f"box_mat{i}", (rho[i],) * 3))
        out.append(_box(f"box_mat{i}", f"box{i}", o, s))
    if light:
        out.append("void light light_mat\n0\n0\n3 100 100 100\n\n")
        cx, cy = X / 2, Y / 2
        out.append(_poly("light_mat", "light", [(cx - .5, cy - .5, Z), (cx - .5, cy + .5, Z),
                                                (cx + .5, cy + .5, Z), (cx + .5, cy - .5, Z)]))
    return "".join(out)


WINDOW = (3.5, 6.5, 0.5, 2.5)


def window_room(seed: int = 0, ntri: int = 20000, nmat: int | None = None, nwin: int = 1,
                tessellated: bool = False) -> str:
    """Room shell with glass windows in the south wall (one 2 x 3 m window,
    or ``nwin`` of 1..8 smaller ones side by side), random interior
    triangles and the glow sky/ground.  ``nmat`` groups the triangles into
    that many materials (default: one material per triangle).  Triangle
    edges are 0.05..0.5 m; with ``tessellated`` they shrink as
    sqrt(20000 / ntri), so that any count covers the area of 20,000 such
    triangles, as a finer tessellation of the same furniture would."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    x0, x1, z0, z1 = WINDOW
    if nwin <= 1:
        wins = [WINDOW]
    else:
        w = (x1 - x0) * 2.0 / (2 * nwin - 1) if nwin <= 4 else 8.0 / (2 * nwin - 1)
        xs = (X - (2 * nwin - 1) * w) / 2
        wins = [(xs + 2 * i * w, xs + 2 * i * w + w, z0, z1) for i in range(nwin)]
    out = [_mat_plastic("room_mat", (0.5, 0.5, 0.5)), _room_shell("room_mat", wins if nwin > 1 else WINDOW)]
    out.append("void glass window_glass\n0\n0\n3 .6 .6 .6\n\n")
    for i, (a0, a1, b0, b1) in enumerate(wins):
        out.append(_poly("window_glass", "window" if i == 0 else f"window{i}",
                         [(a0, 0, b0), (a0, 0, b1), (a1, 0, b1), (a1, 0, b0)]))
    margin = 0.05
    v0 = rng.uniform((margin, margin, margin), (X - margin, Y - margin, Z - margin), size=(ntri, 3))
    scale = np.sqrt(20000.0 / ntri) if tessellated and ntri > 20000 else 1.0
    lens = rng.uniform(0.05, 0.5, size=(ntri, 2)) * scale
    dirs = rng.normal(size=(ntri, 2, 3))
    dirs /= np.linalg.norm(dirs, axis=2, keepdims=True)
    v1 = v0 + lens[:, 0:1] * dirs[:, 0]
    v2 = v0 + lens[:, 1:2] * dirs[:, 1]
    lo, hi = np.array([1e-3] * 3), np.array([X - 1e-3, Y - 1e-3, Z - 1e-3])
    v1 = np.clip(v1, lo, hi)
    v2 = np.clip(v2, lo, hi)
    nm = ntri if nmat is None else nmat
    rho = rng.uniform(0.1, 0.8, size=nm)
    for m in range(nm):
        out.append(_mat_plastic(f"tri_mat{m}", (rho[m],) * 3))
    fmt = "tri_mat%d polygon tri%d\n0\n0\n9 " + " ".join(["%.9g"] * 9) + "\n\n"   # as _poly formats
    idx = np.arange(ntri)
    rows = np.column_stack([idx % nm, idx, v0, v1, v2]).tolist()
    out.append("".join([fmt % (int(r[0]), int(r[1]), *r[2:]) for r in rows]))
    out.append(SKY_GLOW)
    return "".join(out)


def flux_files(ntri: int = 2000, seed: int = 0) -> dict:
    """Scene text for flux-matrix (rfluxmtx) runs around ``window_room``:
    ``system`` (the room without its sky), ``interior`` (the room without
    sky or glass), ``sky`` (receiver: ground as one uniform bin, sky in
    Reinhart MF:1 bins), ``window_kf`` (receiver: the window opening as a
    glow facing into the room, Klems full bins, up +Z), ``window_send``
    (sender: the window facing into the room, Klems full, up +Z) and
    ``obstruction`` (an exterior block south of the window)."""
    room = window_room(seed=seed, ntri=ntri)
    assert room.endswith(SKY_GLOW)
    system = room[:-len(SKY_GLOW)]
    x0, x1, z0, z1 = WINDOW
    win = [(x0, 0, z0), (x0, 0, z1), (x1, 0, z1), (x1, 0, z0)]
    glass = "void glass window_glass\n0\n0\n3 .6 .6 .6\n\n" + _poly("window_glass", "window", win)
    assert glass in system
    interior = system.replace(glass, "")
    sky = ("#@rfluxmtx h=u u=Y\nvoid glow groundglow\n0\n0\n4 1 1 1 0\n\n"
           "groundglow source ground\n0\n0\n4 0 0 -1 180\n\n"
           "#@rfluxmtx h=r1 u=Y\nvoid glow skyglow\n0\n0\n4 1 1 1 0\n\n"
           "skyglow source skydome\n0\n0\n4 0 0 1 180\n\n")
    window_kf = "#@rfluxmtx h=kf u=Z\nvoid glow windowglow\n0\n0\n4 1 1 1 0\n\n" + _poly("windowglow", "wrecv", win)
    window_send = "#@rfluxmtx h=kf u=Z\nvoid polygon wsend\n0\n0\n12 " + " ".join(
        "%.9g %.9g %.9g" % v for v in win) + "\n\n"
    obstruction = _mat_plastic("block_mat", (0.3, 0.3, 0.3)) + _box("block_mat", "block", (-5.0, -14.0, 0.0),
                                                                   (20.0, 4.0, 9.0))
    return dict(system=system, interior=interior, sky=sky, window_kf=window_kf, window_send=window_send,
                obstruction=obstruction)


def glossy_room(seed: int = 0, nboxes: int = 40, nspheres: int = 8) -> str:
    """The room of ``daylight_room`` with rough specular surfaces: a rough
    metal floor (specularity 0.5, roughness 0.08), rough plastic walls and
    ceiling (0.04, 0.12), floor-standing boxes cycling through rough plastic
    (0.06, 0.2), rough metal (0.8, 0.04), pure metal (0.9, 0) and matte
    plastic, rough metal spheres (0.7, 0.1), and the ceiling light."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    out = ["void metal floor_mat\n0\n0\n5 .7 .65 .6 .5 .08\n\n",
           "void plastic wall_mat\n0\n0\n5 .6 .6 .6 .04 .12\n\n",
           "void metal ball_mat\n0\n0\n5 .8 .8 .75 .7 .1\n\n"]
    out.append(_poly("floor_mat", "floor", [(0, 0, 0), (X, 0, 0), (X, Y, 0), (0, Y, 0)]))
    out.append(_poly("wall_mat", "ceiling", [(0, 0, Z), (0, Y, Z), (X, Y, Z), (X, 0, Z)]))
    out.append(_poly("wall_mat", "north", [(0, Y, 0), (X, Y, 0), (X, Y, Z), (0, Y, Z)]))
    out.append(_poly("wall_mat", "west", [(0, 0, 0), (0, Y, 0), (0, Y, Z), (0, 0, Z)]))
    out.append(_poly("wall_mat", "east", [(X, 0, 0), (X, 0, Z), (X, Y, Z), (X, Y, 0)]))
    out.append(_poly("wall_mat", "south", [(0, 0, 0), (0, 0, Z), (X, 0, Z), (X, 0, 0)]))
    sizes = rng.uniform(0.3, 1.2, size=(nboxes, 3))
    pos = rng.uniform(0.0, 1.0, size=(nboxes, 2))
    rho = rng.uniform(0.3, 0.8, size=nboxes)
    lift = rng.uniform(0.002, 0.02, size=nboxes)
    for i in range(nboxes):
        s = sizes[i]
        r = rho[i]
        kind = i % 4
        if kind == 0:
            out.append(f"void plastic box_mat{i}\n0\n0\n5 {r:.9g} {r:.9g} {r:.9g} .06 .2\n\n")
        elif kind == 1:
            out.append(f"void metal box_mat{i}\n0\n0\n5 {r:.9g} {r * .9:.9g} {r * .8:.9g} .8 .04\n\n")
        elif kind == 2:
            out.append(f"void metal box_mat{i}\n0\n0\n5 {r:.9g} {r:.9g} {r:.9g} .9 0\n\n")
        else:
            out.append(_mat_plastic(f"box_mat{i}", (r,) * 3))
        out.append(_box(f"box_mat{i}", f"box{i}", (pos[i, 0] * (X - s[0]), pos[i, 1] * (Y - s[1]), lift[i]), s))
    c = rng.uniform((1, 1, 0.4), (X - 1, Y - 1, Z - 0.8), size=(nspheres, 3))
    rad = rng.uniform(0.15, 0.4, size=nspheres)
    for i in range(nspheres):
        out.append(f"ball_mat sphere ball{i}\n0\n0\n4 {c[i, 0]:.9g} {c[i, 1]:.9g} {c[i, 2]:.9g} {rad[i]:.9g}\n\n")
    out.append("void light light_mat\n0\n0\n3 100 100 100\n\n")
    cx, cy = X / 2, Y / 2
    out.append(_poly("light_mat", "light", [(cx - .5, cy - .5, Z - 0.01), (cx - .5, cy + .5, Z - 0.01),
                                            (cx + .5, cy + .5, Z - 0.01), (cx + .5, cy - .5, Z - 0.01)]))
    return "".join(out)


def trans_room(seed: int = 0, nboxes: int = 30) -> str:
    """The room with translucent (``trans``) surfaces: a smooth diffuser
    sheet under the ceiling light (transmissivity 0.6, a fifth of it
    specular), a few rough frosted panels standing in the room, and
    plastic boxes; the ceiling light of ``daylight_room``."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    out = [_mat_plastic("room_mat", (0.5, 0.5, 0.5)), _room_shell("room_mat"),
           "void trans diffuser\n0\n0\n7 .8 .8 .8 0 0 .6 .2\n\n",
           "void trans frosted\n0\n0\n7 .7 .75 .8 .05 .1 .5 .4\n\n"]
    cx, cy = X / 2, Y / 2
    out.append(_poly("diffuser", "sheet", [(cx - 2, cy - 1.5, 2.2), (cx + 2, cy - 1.5, 2.2),
                                           (cx + 2, cy + 1.5, 2.2), (cx - 2, cy + 1.5, 2.2)]))
    for i in range(4):
        x0 = rng.uniform(1, X - 3)
        y0 = rng.uniform(1, Y - 1)
        ang = rng.uniform(0, np.pi)
        dx, dy = 1.5 * np.cos(ang), 1.5 * np.sin(ang)
        out.append(_poly("frosted", f"panel{i}", [(x0, y0, 0.1), (x0 + dx, y0 + dy, 0.1),
                                                  (x0 + dx, y0 + dy, 1.9), (x0, y0, 1.9)]))
    sizes = rng.uniform(0.2, 0.8, size=(nboxes, 3))
    pos = rng.uniform(0.0, 1.0, size=(nboxes, 2))
    rho = rng.uniform(0.2, 0.7, size=nboxes)
    for i in range(nboxes):
        sz = sizes[i]
        out.append(_mat_plastic(f"box_mat{i}", (rho[i],) * 3))
        out.append(_box(f"box_mat{i}", f"box{i}", (pos[i, 0] * (X - sz[0]), pos[i, 1] * (Y - sz[1]), 0.005), sz))
    out.append("void light light_mat\n0\n0\n3 100 100 100\n\n")
    out.append(_poly("light_mat", "light", [(cx - .5, cy - .5, Z - 0.01), (cx - .5, cy + .5, Z - 0.01),
                                            (cx + .5, cy + .5, Z - 0.01), (cx + .5, cy - .5, Z - 0.01)]))
    return "".join(out)


def lamp_room(seed: int = 0, nboxes: int = 60) -> str:
    """The room of ``daylight_room`` (fewer boxes) lit by a sphere light
    (radius 0.15 m) and a disk light (ring of radius 0.3 m facing down)
    instead of the polygon: the circular source shapes."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    out = [_mat_plastic("room_mat", (0.5, 0.5, 0.5)), _room_shell("room_mat")]
    sizes = rng.uniform(0.2, 1.2, size=(nboxes, 3))
    pos = rng.uniform(0.0, 1.0, size=(nboxes, 2))
    rho = rng.uniform(0.2, 0.7, size=nboxes)
    for i in range(nboxes):
        s = sizes[i]
        out.append(_mat_plastic(f"box_mat{i}", (rho[i],) * 3))
        out.append(_box(f"box_mat{i}", f"box{i}", (pos[i, 0] * (X - s[0]), pos[i, 1] * (Y - s[1]), 0.005), s))
    out.append("void light bulb_mat\n0\n0\n3 200 180 160\n\n")
    out.append(f"bulb_mat sphere bulb\n0\n0\n4 {X * 0.3:.9g} {Y * 0.5:.9g} {Z - 0.5:.9g} 0.15\n\n")
    out.append("void light disk_mat\n0\n0\n3 80 80 90\n\n")
    out.append(f"disk_mat ring disk\n0\n0\n8 {X * 0.7:.9g} {Y * 0.5:.9g} {Z - 0.01:.9g} 0 0 -1 0 0.3\n\n")
    return "".join(out)


def tube_room(seed: int = 0, nboxes: int = 60) -> str:
    """The boxes of ``lamp_room`` lit by two cylinder lights (fluorescent
    tubes of 1.2 m, radius 2 cm, one along x and one along y, 0.3 m under
    the ceiling)."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    out = [_mat_plastic("room_mat", (0.5, 0.5, 0.5)), _room_shell("room_mat")]
    sizes = rng.uniform(0.2, 1.2, size=(nboxes, 3))
    pos = rng.uniform(0.0, 1.0, size=(nboxes, 2))
    rho = rng.uniform(0.2, 0.7, size=nboxes)
    for i in range(nboxes):
        s = sizes[i]
        out.append(_mat_plastic(f"box_mat{i}", (rho[i],) * 3))
        out.append(_box(f"box_mat{i}", f"box{i}", (pos[i, 0] * (X - s[0]), pos[i, 1] * (Y - s[1]), 0.005), s))
    out.append("void light tube_mat\n0\n0\n3 300 300 280\n\n")
    z = Z - 0.3
    out.append(f"tube_mat cylinder tube_x\n0\n0\n7 {X * .3 - .6:.9g} {Y * .5:.9g} {z:.9g} {X * .3 + .6:.9g} "
               f"{Y * .5:.9g} {z:.9g} 0.02\n\n")
    out.append(f"tube_mat cylinder tube_y\n0\n0\n7 {X * .7:.9g} {Y * .5 - .6:.9g} {z:.9g} {X * .7:.9g} "
               f"{Y * .5 + .6:.9g} {z:.9g} 0.02\n\n")
    return "".join(out)


def spot_room(seed: int = 0, nboxes: int = 60) -> str:
    """The boxes of ``lamp_room`` lit by spotlights: a ceiling panel with a
    100 degree cone aimed down and tilted, and a sphere with a 140 degree
    cone aimed down towards +x."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    out = [_mat_plastic("room_mat", (0.5, 0.5, 0.5)), _room_shell("room_mat")]
    sizes = rng.uniform(0.2, 1.2, size=(nboxes, 3))
    pos = rng.uniform(0.0, 1.0, size=(nboxes, 2))
    rho = rng.uniform(0.2, 0.7, size=nboxes)
    for i in range(nboxes):
        s = sizes[i]
        out.append(_mat_plastic(f"box_mat{i}", (rho[i],) * 3))
        out.append(_box(f"box_mat{i}", f"box{i}", (pos[i, 0] * (X - s[0]), pos[i, 1] * (Y - s[1]), 0.005), s))
    out.append("void spotlight panel_mat\n0\n0\n7 150 150 140 100 0.3 0 -1\n\n")
    cx, cy = X * 0.35, Y / 2
    out.append(_poly("panel_mat", "panel", [(cx - .4, cy - .4, Z - 0.01), (cx - .4, cy + .4, Z - 0.01),
                                            (cx + .4, cy + .4, Z - 0.01), (cx + .4, cy - .4, Z - 0.01)]))
    out.append("void spotlight bulb_mat\n0\n0\n7 300 280 250 140 1 0 -1.2\n\n")
    out.append(f"bulb_mat sphere bulb\n0\n0\n4 {X * 0.7:.9g} {Y * 0.5:.9g} {Z - 0.6:.9g} 0.1\n\n")
    return "".join(out)


def mirror_room(seed: int = 0, nboxes: int = 60) -> str:
    """The boxes of ``lamp_room`` under the ceiling light of
    ``daylight_room``, with two wall mirrors (one tinted) and a mirror
    sphere."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    out = [_mat_plastic("room_mat", (0.5, 0.5, 0.5)), _room_shell("room_mat"),
           "void mirror silver\n0\n0\n3 .9 .9 .9\n\n", "void mirror bronze\n0\n0\n3 .8 .6 .4\n\n"]
    sizes = rng.uniform(0.2, 1.2, size=(nboxes, 3))
    pos = rng.uniform(0.0, 1.0, size=(nboxes, 2))
    rho = rng.uniform(0.2, 0.7, size=nboxes)
    for i in range(nboxes):
        s = sizes[i]
        out.append(_mat_plastic(f"box_mat{i}", (rho[i],) * 3))
        out.append(_box(f"box_mat{i}", f"box{i}", (pos[i, 0] * (X - s[0]), pos[i, 1] * (Y - s[1]), 0.005), s))
    out.append(_poly("silver", "mirror_w", [(0.01, 2, 0.5), (0.01, 2, 2.5), (0.01, 6, 2.5), (0.01, 6, 0.5)]))
    out.append(_poly("bronze", "mirror_n", [(3, Y - 0.01, 0.5), (7, Y - 0.01, 0.5), (7, Y - 0.01, 2.5),
                                            (3, Y - 0.01, 2.5)]))
    out.append(f"silver sphere ball\n0\n0\n4 {X * 0.6:.9g} {Y * 0.4:.9g} 1.8 0.3\n\n")
    out.append("void light light_mat\n0\n0\n3 100 100 100\n\n")
    cx, cy = X / 2, Y / 2
    out.append(_poly("light_mat", "light", [(cx - .5, cy - .5, Z - 0.01), (cx - .5, cy + .5, Z - 0.01),
                                            (cx + .5, cy + .5, Z - 0.01), (cx + .5, cy - .5, Z - 0.01)]))
    return "".join(out)


def furniture(seed: int = 0) -> str:
    """An object to instance, in its own coordinates around the origin: a
    table (top and four legs as boxes), a sphere and a cylinder on it, a
    cone beside it; plastic of three reflectances, one of them rough."""
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.3, 0.8, size=3)
    out = [_mat_plastic("wood", (rho[0], rho[0] * 0.8, rho[0] * 0.6)),
           f"void plastic paint\n0\n0\n5 {rho[1]:.9g} {rho[1]:.9g} {rho[1]:.9g} .04 .1\n\n",
           _mat_plastic("steel", (rho[2],) * 3)]
    out.append(_box("wood", "top", (-0.6, -0.4, 0.7), (1.2, 0.8, 0.05)))
    for k, (x, y) in enumerate(((-0.55, -0.35), (0.5, -0.35), (-0.55, 0.3), (0.5, 0.3))):
        out.append(_box("steel", f"leg{k}", (x, y, 0.0), (0.05, 0.05, 0.7)))
    out.append("paint sphere ball\n0\n0\n4 0.2 0.1 0.95 0.2\n\n")
    out.append("steel cylinder can\n0\n0\n7 -0.3 -0.1 0.75 -0.3 -0.1 1.05 0.08\n\n")
    out.append("paint cone lamp\n0\n0\n8 0.9 0.0 0.0 0.9 0.0 0.6 0.25 0.02\n\n")
    return "".join(out)


def instance_room(sub_octree: str, seed: int = 0, n: int = 12) -> str:
    """The room shell and ceiling light of ``daylight_room`` with ``n``
    instances of the octree file ``sub_octree`` on the floor: rotated about
    z, some scaled, one mirrored, every third one with its own material
    (the instance's modifier replaces the instanced surfaces' own)."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    out = [_mat_plastic("room_mat", (0.5, 0.5, 0.5)), _room_shell("room_mat"),
           _mat_plastic("override", (0.7, 0.3, 0.2))]
    for i in range(n):
        x, y = rng.uniform((1.2, 1.2), (X - 1.2, Y - 1.2))
        args = ["-rz", f"{rng.uniform(0, 360):.6g}"]
        if i % 4 == 1:
            args += ["-s", f"{rng.uniform(0.6, 1.4):.6g}"]
        if i == 2:
            args += ["-mx"]
        args += ["-t", f"{x:.6g}", f"{y:.6g}", "0.002"]
        mod = "override" if i % 3 == 0 else "override_metal" if metal and i % 3 == 1 else "void"
        out.append(f"{mod} instance inst{i}\n{1 + len(args)} {sub_octree} {' '.join(args)}\n0\n0\n\n")
    out.append("void light light_mat\n0\n0\n3 100 100 100\n\n")
    cx, cy = X / 2, Y / 2
    out.append(_poly("light_mat", "light", [(cx - .5, cy - .5, Z - 0.01), (cx - .5, cy + .5, Z - 0.01),
                                            (cx + .5, cy + .5, Z - 0.01), (cx + .5, cy - .5, Z - 0.01)]))
    return "".join(out)


def mesh_obj(nu: int = 24, nv: int = 12, nsheet: int = 16, seed: int = 0, normals: bool = False,
             uv: bool = False) -> str:
    """A Wavefront OBJ for obj2mesh, in its own coordinates around the
    origin: a UV sphere of radius 0.45 centred 0.45 above the origin
    (material ``mesh_red``) and a bumpy square sheet of side 1.2 at height
    0.9 .. 1.0 (``mesh_grey``), triangles only; with ``normals``, every
    vertex carries a normal (the sphere's radial direction, the sheet's
    height-field normal by central differences) and the faces name them;
    with ``uv``, every vertex carries texture coordinates as well (the
    sphere's longitude and latitude fractions, the sheet's position)."""
    rng = np.random.default_rng(seed)
    V, N, T, out = [], [], [], []
    for j in range(nv + 1):
        th = np.pi * j / nv
        for i in range(nu):
            ph = 2 * np.pi * i / nu
            V.append((0.45 * np.sin(th) * np.cos(ph), 0.45 * np.sin(th) * np.sin(ph), 0.45 + 0.45 * np.cos(th)))
            N.append((np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)))
            T.append((i / nu, j / nv))
    out.append("usemtl mesh_red")
    for j in range(nv):
        for i in range(nu):
            a, b = j * nu + i % nu + 1, j * nu + (i + 1) % nu + 1
            c, d = (j + 1) * nu + (i + 1) % nu + 1, (j + 1) * nu + i % nu + 1
            if j > 0:
                out.append(f"f {a} {c} {b}")
            if j < nv - 1:
                out.append(f"f {a} {d} {c}")
    base = len(V)
    h = rng.uniform(0.9, 1.0, size=(nsheet + 1, nsheet + 1))
    gy, gx = np.gradient(h, 1.2 / nsheet)
    for j in range(nsheet + 1):
        for i in range(nsheet + 1):
            V.append((-0.6 + 1.2 * i / nsheet, -0.6 + 1.2 * j / nsheet, h[j, i]))
            n = np.array([-gx[j, i], -gy[j, i], 1.0])
            N.append(tuple(n / np.linalg.norm(n)))
            T.append((i / nsheet, j / nsheet))
    out.append("usemtl mesh_grey")
    for j in range(nsheet):
        for i in range(nsheet):
            a = base + j * (nsheet + 1) + i + 1
            b, c, d = a + 1, a + nsheet + 2, a + nsheet + 1
            out += [f"f {a} {b} {c}", f"f {a} {c} {d}"]
    text = "".join(f"v {x:.7f} {y:.7f} {z:.7f}\n" for x, y, z in V)
    if normals:
        text += "".join(f"vn {x:.7f} {y:.7f} {z:.7f}\n" for x, y, z in N)
    if uv:
        text += "".join(f"vt {u:.7f} {v:.7f}\n" for u, v in T)
    if normals or uv:
        form = "{k}/{k}/{k}" if normals and uv else "{k}//{k}" if normals else "{k}/{k}"
        out = [" ".join([t[0]] + [form.format(k=k) for k in t[1:]]) if t[0] == "f" else " ".join(t)
               for t in (ln.split() for ln in out)]
    return text + "\n".join(out) + "\n"


def mesh_materials() -> str:
    """The materials ``mesh_obj``'s triangles name (obj2mesh -a)."""
    return (_mat_plastic("mesh_red", (0.7, 0.25, 0.2)) +
            "void plastic mesh_grey\n0\n0\n5 0.5 0.5 0.5 0.03 0.05\n\n")


def mesh_room(mesh_file: str, seed: int = 0, n: int = 10, metal: bool = False) -> str:
    """The room shell and ceiling light of ``instance_room`` with ``n``
    placements of the compiled mesh ``mesh_file`` on the floor: rotated
    about z, some scaled, one mirrored; every third one with its own
    material (which replaces the mesh's), the others with the mesh's; with
    ``metal``, the second of every three with a rough metal of its own."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    out = [_mat_plastic("room_mat", (0.5, 0.5, 0.5)), _room_shell("room_mat"),
           _mat_plastic("override", (0.3, 0.6, 0.3))]
    if metal:
        out.append("void metal override_metal\n0\n0\n5 0.7 0.6 0.4 0.6 0.08\n\n")
    for i in range(n):
        x, y = rng.uniform((1.2, 1.2), (X - 1.2, Y - 1.2))
        args = ["-rz", f"{rng.uniform(0, 360):.6g}"]
        if i % 4 == 1:
            args += ["-s", f"{rng.uniform(0.6, 1.4):.6g}"]
        if i == 2:
            args += ["-mx"]
        args += ["-t", f"{x:.6g}", f"{y:.6g}", "0.002"]
        mod = "override" if i % 3 == 0 else "override_metal" if metal and i % 3 == 1 else "void"
        out.append(f"{mod} mesh mesh{i}\n{1 + len(args)} {mesh_file} {' '.join(args)}\n0\n0\n\n")
    out.append("void light light_mat\n0\n0\n3 100 100 100\n\n")
    cx, cy = X / 2, Y / 2
    out.append(_poly("light_mat", "light", [(cx - .5, cy - .5, Z - 0.01), (cx - .5, cy + .5, Z - 0.01),
                                            (cx + .5, cy + .5, Z - 0.01), (cx + .5, cy - .5, Z - 0.01)]))
    return "".join(out)


def klems_bsdf_xml(seed: int = 0, basis: str = "full", front: bool = True, back: bool = True,
                   rows: bool = False, base: float = 0.002) -> str:
    """A WINDOW 6 style XML matrix BSDF of synthetic glazing in a Klems
    basis (defined in the file as WINDOW 6 writes it): "Visible"
    transmission with a straight-through peak (exiting patch opposite in
    azimuth, same ring), a smooth forward lobe, a floor ``base`` and seeded
    noise; "Transmission Front" and/or "Transmission Back" blocks, data
    ordered by columns (one line per exiting patch) or rows."""
    rng = np.random.default_rng(seed)
    rings = {"full": [(0, 5, 1), (5, 15, 8), (15, 25, 16), (25, 35, 20), (35, 45, 24), (45, 55, 24),
                      (55, 65, 24), (65, 75, 16), (75, 90, 12)],
             "half": [(0, 6.5, 1), (6.5, 19.5, 8), (19.5, 32.5, 12), (32.5, 45.5, 16), (45.5, 58.5, 20),
                      (58.5, 71.5, 12), (71.5, 90, 8)]}[basis]
    name = {"full": "LBNL/Klems Full", "half": "LBNL/Klems Half"}[basis]
    centres = []
    for lo, hi, nph in rings:
        for k in range(nph):
            centres.append((np.radians(0.5 * (lo + hi)), 2 * np.pi * k / nph, lo, hi, nph))
    n = len(centres)
    th = np.array([c[0] for c in centres])
    ph = np.array([c[1] for c in centres])
    d = np.array([[np.sin(t) * np.cos(p), np.sin(t) * np.sin(p), np.cos(t)] for t, p in zip(th, ph)])

    def matrix(scale):
        m = base + 0.3 * scale * np.maximum(0, d[:, None, 2] * d[None, :, 2]) ** 2
        m += 0.02 * rng.random((n, n))
        for i in range(n):                          # straight through: opposite azimuth, same ring
            j = int(np.argmin(np.linalg.norm(d - d[i] * np.array([-1, -1, 1]), axis=1)))
            m[j, i] += 12.0 * scale * np.cos(th[i])
        return m                                    # m[exiting, incident]

    def block(direction, m):
        data = m.T if rows else m
        body = "\n".join(" ".join(f"{v:.6e}" for v in row) for row in data)
        return (f"\t\t<WavelengthDataBlock>\n\t\t\t<WavelengthDataDirection>{direction}</WavelengthDataDirection>\n"
                f"\t\t\t<ColumnAngleBasis>{name}</ColumnAngleBasis>\n\t\t\t<RowAngleBasis>{name}</RowAngleBasis>\n"
                f"\t\t\t<ScatteringDataType>BTDF</ScatteringDataType>\n\t\t\t<ScatteringData>\n{body}\n"
                "\t\t\t</ScatteringData>\n\t\t</WavelengthDataBlock>\n")

    blocks = ("".join(f"\t\t\t<AngleBasisBlock>\n\t\t\t\t<Theta>{0.5 * (lo + hi) if lo else 0}</Theta>\n"
                      f"\t\t\t\t<nPhis>{nph}</nPhis>\n\t\t\t\t<ThetaBounds>\n\t\t\t\t\t<LowerTheta>{lo}</LowerTheta>\n"
                      f"\t\t\t\t\t<UpperTheta>{hi}</UpperTheta>\n\t\t\t\t</ThetaBounds>\n\t\t\t</AngleBasisBlock>\n"
                      for lo, hi, nph in rings))
    out = ['<?xml version="1.0" encoding="UTF-8"?>\n',
           '<WindowElement xmlns="http://windows.lbl.gov" xmlns:xsi="http://www.w3.org/2001/XMLSchema-instance">\n',
           "<WindowElementType>System</WindowElementType>\n<FileType>BSDF</FileType>\n<Optical>\n<Layer>\n",
           "\t<Material>\n\t\t<Name>synthetic glazing</Name>\n\t\t<DeviceType>Other</DeviceType>\n\t</Material>\n",
           f"\t<DataDefinition>\n\t\t<IncidentDataStructure>{'Rows' if rows else 'Columns'}</IncidentDataStructure>\n",
           f"\t\t<AngleBasis>\n\t\t\t<AngleBasisName>{name}</AngleBasisName>\n{blocks}\t\t</AngleBasis>\n",
           "\t</DataDefinition>\n\t<WavelengthData>\n\t\t<LayerNumber>System</LayerNumber>\n",
           '\t\t<Wavelength unit="Integral">Visible</Wavelength>\n']
    if back:
        out.append(block("Transmission Back", matrix(1.0)))
    if front:
        out.append(block("Transmission Front", matrix(0.8)))
    out.append("\t</WavelengthData>\n</Layer>\n</Optical>\n</WindowElement>\n")
    return "".join(out)


def shape_zoo(seed: int = 0, n: int = 40) -> str:
    """Room with every primitive type the intersectors handle: spheres,
    bubbles, cones, cups, cylinders, tubes, rings and polygons, gray plastic
    and metal, and the ceiling light of ``daylight_room``."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    out = [_mat_plastic("room_mat", (0.5, 0.5, 0.5)), _room_shell("room_mat")]
    out.append("void metal shiny\n0\n0\n5 .6 .6 .6 .8 0\n\n")
    for i in range(n):
        rho = rng.uniform(0.2, 0.7)
        out.append(_mat_plastic(f"zoo_mat{i}", (rho, rho * 0.9, rho * 0.8)))
        mod = "shiny" if i % 7 == 3 else f"zoo_mat{i}"
        c = rng.uniform((1, 1, 0.3), (X - 1, Y - 1, Z - 0.6))
        r = rng.uniform(0.1, 0.4)
        kind = i % 7
        if kind == 0:
            out.append(f"{mod} sphere sph{i}\n0\n0\n4 {c[0]:.9g} {c[1]:.9g} {c[2]:.9g} {r:.9g}\n\n")
        elif kind == 1:
            out.append(f"{mod} bubble bub{i}\n0\n0\n4 {c[0]:.9g} {c[1]:.9g} {c[2]:.9g} {r:.9g}\n\n")
        elif kind in (2, 3, 4, 5):
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            p1 = c + d * rng.uniform(0.2, 0.6)
            name = {2: "cone", 3: "cup", 4: "cylinder", 5: "tube"}[kind]
            if kind in (2, 3):
                r2 = rng.uniform(0.0, 0.3)
                args = f"8 {c[0]:.9g} {c[1]:.9g} {c[2]:.9g} {p1[0]:.9g} {p1[1]:.9g} {p1[2]:.9g} {r:.9g} {r2:.9g}"
            else:
                args = f"7 {c[0]:.9g} {c[1]:.9g} {c[2]:.9g} {p1[0]:.9g} {p1[1]:.9g} {p1[2]:.9g} {r:.9g}"
            out.append(f"{mod} {name} {name}{i}\n0\n0\n{args}\n\n")
        else:
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            out.append(f"{mod} ring ring{i}\n0\n0\n8 {c[0]:.9g} {c[1]:.9g} {c[2]:.9g} {d[0]:.9g} {d[1]:.9g} "
                       f"{d[2]:.9g} {r * 0.3:.9g} {r:.9g}\n\n")
    out.append("void light light_mat\n0\n0\n3 100 100 100\n\n")
    cx, cy = X / 2, Y / 2
    out.append(_poly("light_mat", "light", [(cx - .5, cy - .5, Z - 0.01), (cx - .5, cy + .5, Z - 0.01),
                                            (cx + .5, cy + .5, Z - 0.01), (cx + .5, cy - .5, Z - 0.01)]))
    return "".join(out)


def random_rays(n: int, seed: int = 1) -> np.ndarray:
    """(n, 6) rays from random interior points in uniformly random directions."""
    rng = np.random.default_rng(seed)
    X, Y, Z = ROOM
    o = rng.uniform((0.2, 0.2, 0.2), (X - 0.2, Y - 0.2, Z - 0.2), size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.hstack([o, d])


def sensor_grid(nx: int, ny: int, z: float = 0.8) -> np.ndarray:
    """(nx*ny, 6) float64 array of ``ox oy oz dx dy dz``, cell-centred over
    the room floor plan, facing +z, row-major in y then x."""
    X, Y, _ = ROOM
    xs = (np.arange(nx) + 0.5) * (X / nx)
    ys = (np.arange(ny) + 0.5) * (Y / ny)
    gx, gy = np.meshgrid(xs, ys)
    n = nx * ny
    out = np.zeros((n, 6))
    out[:, 0] = gx.ravel()
    out[:, 1] = gy.ravel()
    out[:, 2] = z
    out[:, 5] = 1.0
    return out


def rays_ascii(rays: np.ndarray) -> bytes:
    return "".join(" ".join(f"{v:.17g}" for v in r) + "\n" for r in rays).encode()


def dc_sky(M: int, K: int, N: int, seed: int = 0):
    """Daylight-coefficient matrix (M, K, 3) and sky matrix (K, N, 3), float32.

    DC: lognormal(mu=-6, sigma=2) with 30% of the (row, patch) entries exactly
    zero in all three channels.  Sky: for each hour column, a diffuse
    lognormal(mu=2, sigma=1) background plus a sun spike log-uniform in
    [1e4, 1e6] on one random patch; about half the columns (night) all zero.
    """
    rng = np.random.default_rng(seed)
    dc = rng.lognormal(-6.0, 2.0, size=(M, K, 3)).astype(np.float32)
    dc[rng.random((M, K)) < 0.3] = 0.0
    sky = rng.lognormal(2.0, 1.0, size=(K, N, 3)).astype(np.float32)
    sun = rng.integers(0, K, size=N)
    spike = np.exp(rng.uniform(np.log(1e4), np.log(1e6), size=N)).astype(np.float32)
    sky[sun, np.arange(N), :] += spike[:, None]
    night = rng.random(N) < 0.5
    sky[:, night, :] = 0.0
    return dc, sky


def polygons(rad_text: str) -> list:
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


def aimed_rays(polys: list, inset: float, seed: int = 9):
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
