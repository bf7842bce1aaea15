"""rfluxmtx on the GPU: flux transfer matrices between a sender and receivers.

Same call as ``pyradiance.rfluxmtx`` (src/pyradiance/util.py:833-869).  The
reference program (util/rfluxmtx.c) reads the receiver file for surfaces
tagged by ``#@rfluxmtx`` directives, turns each receiver modifier into
rcontrib bin arguments, and then either passes the caller's rays through to
rcontrib (sender ``-``) or samples rays leaving the sender surfaces bin by
bin.  Here the same arguments drive the in-process GPU rcontrib
(``Rcontrib.run_array``); the sender rays are drawn on the host.

Hemisphere bases: uniform (``h=u``), Klems full / half / quarter (``h=kf``,
``kh``, ``kq``; the bases of util/klems_full.cal, klems_half.cal and
klems_quarter.cal, built into the bin compiler), Reinhart (``h=r``,
``h=rN``), Shirley-Chiu (``h=scN``, util/disk2square.cal's scbin, built
in) and, for receivers, the CIE sky scanner (``h=cie``, util/cieskyscan.cal's
cbin, built in).  Bin jitter (``-bj``) is passed to the bin parameters
as ``JTR`` as rfluxmtx passes it (none of these bases reads it).
Receivers with ``o=`` write their columns to that file (``%s``: the
modifier; ``%d``: one file per bin).
"""
from __future__ import annotations

import math
from pathlib import Path
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import GbError, Scene

PARAMSTART = "@rfluxmtx"
_SURF_TYPES = {"polygon", "ring", "source"}
_FTINY = 1e-6


class _Surf:
    """One sender or receiver element (util/rfluxmtx.c:1035-1111 add_surface)."""

    def __init__(self, styp: str, name: str, fa: list[float]):
        self.styp, self.name, self.fa = styp, name, np.asarray(fa, dtype=np.float64)
        if styp == "ring":
            if len(fa) != 8:
                raise GbError(-1, f"bad argument count for surface element '{name}'")
            n = self.fa[3:6]
            ln = np.linalg.norm(n)
            if ln == 0:
                raise GbError(-1, f"bad orientation for surface element '{name}'")
            self.nrm = n / ln
            r0, r1 = sorted(self.fa[6:8])
            self.r0, self.r1 = r0, r1
            self.area = math.pi * (r1 * r1 - r0 * r0)
        elif styp == "polygon":
            if len(fa) < 9 or len(fa) % 3:
                raise GbError(-1, f"bad argument count for surface element '{name}'")
            v = self.fa.reshape(-1, 3)
            s = np.zeros(3)
            e1 = v[1] - v[0]
            for i in range(2, len(v)):          # finish_polygon (rfluxmtx.c:1013-1033)
                e2 = v[i] - v[0]
                s += np.cross(e1, e2)
                e1 = e2
            ln = np.linalg.norm(s)
            self.nrm = s / ln if ln > 0 else s
            self.area = 0.5 * ln
        else:                                   # distant source: reversed direction
            if len(fa) != 4:
                raise GbError(-1, f"bad argument count for surface element '{name}'")
            n = -self.fa[:3]
            ln = np.linalg.norm(n)
            if ln == 0:
                raise GbError(-1, f"bad orientation for surface element '{name}'")
            self.nrm = n / ln
            a = math.sin(math.pi / 180 / 2 * self.fa[3])
            self.area = math.pi * a * a


class _Params:
    """Directives of one sender or receiver group (rfluxmtx.c:336-411)."""

    def __init__(self):
        self.sign = "+"
        self.hemis = ""
        self.hsiz = 0
        self.vup = np.zeros(3)
        self.outfn = None
        self.surfs: list[_Surf] = []

    def parse(self, text: str):
        for tok in text.split():
            if tok.startswith("h=") and len(tok) > 2:
                h = tok[2:]
                self.sign = "+"
                if h[0] in "+-":
                    self.sign, h = h[0], h[1:]
                if not h:
                    raise GbError(-1, f"bad parameter string: {text}")
                self.hemis = h
                digits = "".join(ch for ch in h if ch.isdigit())
                self.hsiz = int(digits) if digits else 0
                self.hsiz += not self.hsiz
            elif tok.startswith("u=") and len(tok) > 2:
                self.vup = _direction(tok[2:], text)
            elif tok.startswith("o=") and len(tok) > 2:
                self.outfn = tok[2:].strip("\"'")
            else:
                raise GbError(-1, f"bad parameter string: {text}")

    def normal(self) -> np.ndarray:
        n = sum((s.nrm * s.area for s in self.surfs), np.zeros(3))
        ln = np.linalg.norm(n)
        if ln == 0:
            raise GbError(-1, "undefined normal for hemisphere sampling")
        return n / ln

    def up(self, nrm: np.ndarray) -> np.ndarray:
        if np.linalg.norm(self.vup) > 0:
            return self.vup / np.linalg.norm(self.vup)
        return np.array([0.0, 0.0, 1.0]) if abs(nrm[2]) < .7 else np.array([0.0, 1.0, 0.0])


def _direction(s: str, text: str) -> np.ndarray:
    """u= value: [+-]X/Y/Z or x,y,z (rfluxmtx.c:296-333 get_direction)."""
    sign = 1.0
    while s and s[0] in "+-":
        sign = -sign if s[0] == "-" else sign
        s = s[1:]
    if s.upper() in ("X", "Y", "Z"):
        v = np.zeros(3)
        v["XYZ".index(s.upper())] = sign
        return v
    try:
        v = np.array([float(x) for x in s.split(",")])
    except ValueError:
        v = np.zeros(0)
    if v.shape != (3,) or np.linalg.norm(v) == 0:
        raise GbError(-1, f"bad parameter string: {text}")
    v[0] *= sign
    return v / np.linalg.norm(v)


def _objects(path):
    """(directives, modifier, type, name, real arguments) of each object of a
    scene file, with the ``#@rfluxmtx`` lines that precede it
    (rfluxmtx.c:1198-1252 load_scene)."""
    text = Path(path).read_text()
    toks: list[tuple[str, str | None]] = []
    for line in text.splitlines():
        st = line.strip()
        if st.startswith("!"):
            raise GbError(-3, "command expansion ('!') in sender or receiver files is not supported")
        if st.startswith("#"):
            w = st[1:].split(None, 1)
            if w and w[0] == PARAMSTART and not st[1:2].isspace():
                toks.append(("", w[1] if len(w) > 1 else ""))
            continue
        toks.extend((t, None) for t in line.split())
    out, params, i = [], "", 0

    def word():
        nonlocal i, params
        while i < len(toks) and toks[i][1] is not None:
            params += " " + toks[i][1]
            i += 1
        if i >= len(toks):
            return None
        i += 1
        return toks[i - 1][0]

    while True:
        mod = word()
        if mod is None:
            break
        typ, name = word(), word()
        if name is None:
            raise GbError(-1, f"{path}: truncated object")
        if typ == "alias":
            word()
            continue
        try:
            ns = int(word())
            for _ in range(ns):
                word()
            ni = int(word())
            for _ in range(ni):
                word()
            nf = int(word())
            fa = [float(word()) for _ in range(nf)]
        except (TypeError, ValueError):
            raise GbError(-1, f"{path}: bad arguments for '{name}'") from None
        out.append((params, mod, typ, name, fa))
        params = ""
    return out


def _receivers(path, jitter: str | None = None) -> list[dict]:
    """Receiver modifiers as rcontrib modifier arguments (rfluxmtx.c:427-582
    finish_receiver, :1116-1151 add_recv_object)."""
    groups: list[tuple[str, _Params]] = []
    pending = ""
    for params, mod, typ, name, fa in _objects(path):
        pending += params
        if typ not in _SURF_TYPES:
            continue
        if not groups or groups[-1][0] != mod:
            p = _Params()
            if groups:                          # clear_params(.., 1) keeps the basis
                q = groups[-1][1]
                p.sign, p.hemis, p.hsiz = q.sign, q.hemis, q.hsiz
            if pending.strip():
                p.parse(pending)
            pending = ""
            groups.append((mod, p))
        s = _Surf(typ, name, fa)
        if s.area > _FTINY * _FTINY:
            groups[-1][1].surfs.append(s)
    if not groups:
        raise GbError(-1, "missing receiver surface!")
    specs, ospec = [], None
    for mod, p in groups:
        if p.outfn is not None:                 # rcontrib -o: this and the following modifiers
            ospec = p.outfn                     # (%s the modifier, %d one file per bin)
        if not p.hemis:
            raise GbError(-1, "missing hemisphere sampling type!")
        if not p.surfs:
            raise GbError(-1, f"receiver '{mod}' has no surface of non-zero area")
        nrm = p.normal()
        vup = p.up(nrm)
        h = p.hemis.lower()
        jtr = ",JTR=" + jitter if jitter is not None else ""   # rfluxmtx.c:413-424 addbinjitter
        spec = dict(modifier=mod, calfile=None, params=None, nbins=None, binv=None, expr=None, output=ospec)
        if h[0] in "u1":
            if p.surfs[-1].styp != "source":
                spec["binv"] = "if(-Dx*%g-Dy*%g-Dz*%g,0,-1)" % tuple(nrm)
            else:
                spec["binv"] = "0"
            spec["nbins"] = "1"
        elif h[:2] == "sc":
            if p.hsiz <= 1:
                raise GbError(-1, "missing size for Shirley-Chiu sampling!")
            spec["calfile"] = "disk2square.cal"
            spec["params"] = "SCdim=%d,rNx=%g,rNy=%g,rNz=%g,Ux=%g,Uy=%g,Uz=%g,RHS=%s1" % (
                p.hsiz, *nrm, *vup, p.sign) + jtr
            spec["binv"], spec["nbins"] = "scbin", "SCdim*SCdim"
        elif h[0] in "rt":
            spec["calfile"] = "reinhartb.cal"
            spec["params"] = "MF=%d,rNx=%g,rNy=%g,rNz=%g,Ux=%g,Uy=%g,Uz=%g,RHS=%s1" % (
                p.hsiz, *nrm, *vup, p.sign) + jtr
            spec["binv"], spec["nbins"] = "rbin", "Nrbins"
        elif h[0] == "k" and (len(h) == 1 or h[1] in "f1h2q4"):
            kind = "f" if len(h) == 1 or h[1] in "f1" else ("h" if h[1] in "h2" else "q")
            cal, fn, nb = {"f": ("klems_full.cal", "kbin", "Nkbins"), "h": ("klems_half.cal", "khbin", "Nkhbins"),
                           "q": ("klems_quarter.cal", "kqbin", "Nkqbins")}[kind]
            spec["calfile"], spec["nbins"] = cal, nb
            spec["params"] = "RHS=%s1" % p.sign + jtr
            spec["binv"] = "%s(%g,%g,%g,%g,%g,%g)" % (fn, *nrm, *vup)
        elif h == "cie":                               # util/rfluxmtx.c:523-533
            spec["calfile"] = "cieskyscan.cal"
            spec["params"] = "rNx=%g,rNy=%g,rNz=%g,Ux=%g,Uy=%g,Uz=%g,RHS=%s1" % (*nrm, *vup, p.sign) + jtr
            spec["binv"], spec["nbins"] = "cbin", "Ncbins"
        else:
            raise GbError(-3, f"hemisphere sampling h={p.hemis} is not supported")
        if not h[0] in "u1":
            for s in p.surfs:
                if s.styp == "source" and abs(s.area - math.pi) > 1e-3:
                    raise GbError(-1, f"source '{s.name}' must be 180-degrees")
        specs.append(spec)
    return specs


# ------------------------------------------------------------ sender sampling

_KLEMS = {"1": ((0, 5, 15, 25, 35, 45, 55, 65, 75, 90), (1, 8, 16, 20, 24, 24, 24, 16, 12)),
          "2": ((0, 6.5, 19.5, 32.5, 45.5, 58.5, 71.5, 90), (1, 8, 12, 16, 20, 12, 8)),
          "4": ((0, 9, 27, 45, 63, 90), (1, 8, 12, 12, 8))}
_TNAZ = (30, 30, 24, 24, 18, 12, 6)


def _perpendicular(n: np.ndarray) -> np.ndarray:
    a = np.zeros(3)
    a[int(np.argmin(np.abs(n)))] = 1.0
    u = np.cross(a, n)
    return u / np.linalg.norm(u)


def _triangulate(v2: np.ndarray) -> list[tuple[int, int, int]]:
    """Ear clipping of a simple polygon given in 2D (counter-clockwise made)."""
    idx = list(range(len(v2)))
    area = 0.5 * sum(v2[i, 0] * v2[(i + 1) % len(v2), 1] - v2[(i + 1) % len(v2), 0] * v2[i, 1]
                     for i in range(len(v2)))
    if area < 0:
        idx.reverse()
    tris = []

    def cross(o, a, b):
        return (a[0] - o[0]) * (b[1] - o[1]) - (a[1] - o[1]) * (b[0] - o[0])

    guard = 0
    while len(idx) > 3 and guard < 10000:
        guard += 1
        for k in range(len(idx)):
            a, b, c = idx[k - 1], idx[k], idx[(k + 1) % len(idx)]
            if cross(v2[a], v2[b], v2[c]) <= 0:
                continue
            if any(cross(v2[a], v2[b], v2[p]) >= 0 and cross(v2[b], v2[c], v2[p]) >= 0 and
                   cross(v2[c], v2[a], v2[p]) >= 0 for p in idx if p not in (a, b, c)):
                continue
            tris.append((a, b, c))
            idx.pop(k)
            break
        else:
            raise GbError(-1, "cannot triangulate sender polygon")
    tris.append(tuple(idx))
    return tris


def _origins(s: _Surf, x: np.ndarray, rng) -> np.ndarray:
    """Points on a sender element, uniform by area (rfluxmtx.c:609-722)."""
    if s.styp == "ring":
        u = _perpendicular(s.nrm)
        v = np.cross(s.nrm, u)
        r = np.sqrt(x * s.area / math.pi + s.r0 * s.r0)
        t = 2 * math.pi * rng.random(len(x))
        return s.fa[:3] + (r * np.cos(t))[:, None] * u + (r * np.sin(t))[:, None] * v
    if s.styp != "polygon":
        raise GbError(-1, f"illegal sender surface '{s.name}'")
    v = s.fa.reshape(-1, 3)
    u = _perpendicular(s.nrm)
    w = np.cross(s.nrm, u)
    v2 = np.stack([v @ u, v @ w], axis=1)
    tris = _triangulate(v2) if len(v) > 3 else [(0, 1, 2)]
    ta = np.array([abs((v2[b, 0] - v2[a, 0]) * (v2[c, 1] - v2[a, 1]) - (v2[b, 1] - v2[a, 1]) * (v2[c, 0] - v2[a, 0]))
                   * .5 for a, b, c in tris])
    cum = np.cumsum(ta / ta.sum())
    k = np.minimum(np.searchsorted(cum, x, side="left"), len(tris) - 1)
    t = np.array(tris)[k]
    s1 = np.sqrt(rng.random(len(x)))
    a = rng.random(len(x)) * s1
    b = 1.0 - s1
    v0, v1, v2_ = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    return v0 + a[:, None] * (v1 - v0) + b[:, None] * (v2_ - v0)


def _square2disk(x: np.ndarray, y: np.ndarray):
    """Shirley and Chiu's concentric map of the unit square onto the unit
    disk ("A Low Distortion Map Between Disk and Square", 1997), the square's
    four triangular regions about its centre each mapped to a quarter of the
    disk (common/disk2square.c)."""
    a, b = 2 * x - 1, 2 * y - 1
    r = np.empty_like(a)
    phi = np.zeros_like(a)
    q = math.pi / 4
    m1 = (a > -b) & (a > b)
    m2 = (a > -b) & ~(a > b)
    m3 = ~(a > -b) & (a < b)
    m4 = ~(a > -b) & ~(a < b)
    r[m1], phi[m1] = a[m1], q * (b[m1] / a[m1])
    r[m2], phi[m2] = b[m2], q * (2 - a[m2] / b[m2])
    r[m3], phi[m3] = -a[m3], q * (4 + b[m3] / a[m3])
    r[m4] = -b[m4]
    nz = m4 & (b != 0)
    phi[nz] = q * (6 - a[nz] / b[nz])
    return r * np.cos(phi), r * np.sin(phi)


def _sender_rays(p: _Params, sampcnt: int, rng) -> tuple[np.ndarray, int]:
    """Rays leaving the sender, sampcnt per bin of its basis, bin by bin
    (rfluxmtx.c:724-1010: sample_origin, sample_uniform, sample_reinhart,
    sample_klems, prepare_sampler)."""
    if not p.surfs:
        raise GbError(-1, "no sender surface!")
    if not p.hemis:
        raise GbError(-1, "missing sender sampling type!")
    nrm = p.normal()
    vup = p.up(nrm)
    udir = np.cross(vup, nrm)
    if np.linalg.norm(udir) == 0:
        raise GbError(-1, "up vector coincides with sender normal")
    udir /= np.linalg.norm(udir)
    vdir = np.cross(nrm, udir)
    if p.sign == "-":
        udir = -udir
    h = p.hemis.lower()
    n = sampcnt
    if h[0] in "u1":
        nb = 1
        r = np.sqrt(rng.random(n))
        ph = 2 * math.pi * rng.random(n)
        duvw = np.stack([r * np.cos(ph), r * np.sin(ph), np.sqrt(np.maximum(0, 1 - r * r))], axis=1)
        bins = [duvw]
    elif h[:2] == "sc":
        sc = p.hsiz
        if sc <= 1:
            raise GbError(-1, "missing size for Shirley-Chiu sampling!")
        nb = sc * sc
        bins = []
        for b in range(nb):
            dx, dy = _square2disk((b // sc + rng.random(n)) / sc, (b % sc + rng.random(n)) / sc)
            bins.append(np.stack([dx, dy, np.sqrt(np.maximum(0.0, 1 - dx * dx - dy * dy))], axis=1))
    elif h[0] in "rt":
        mf = p.hsiz
        rowmax = 7 * mf + 1
        rah = (.5 * math.pi) / (rowmax - .5)
        rnaz = [1 if r >= rowmax - 1 else mf * _TNAZ[r // mf] for r in range(rowmax)]
        nb = sum(rnaz)
        bins = []
        for row in range(rowmax):
            for col in range(rnaz[row]):
                s1, s2 = rng.random(n), rng.random(n)
                if row >= rowmax - 1:
                    s1 = s1 * s1
                alt = (row + s1) * rah
                azi = 2 * math.pi * (col + s2 - .5) / rnaz[row]
                bins.append(np.stack([np.sin(azi) * np.cos(alt), -np.cos(azi) * np.cos(alt), np.sin(alt)], axis=1))
    elif h[0] == "k" and (len(h) == 1 or h[1] in "f1h2q4"):
        key = "1" if len(h) == 1 or h[1] in "f1" else ("2" if h[1] in "h2" else "4")
        tmin, nphi = _KLEMS[key]
        nb = sum(nphi)
        bins = []
        for li, nph in enumerate(nphi):
            c0, c1 = math.cos(math.radians(tmin[li])) ** 2, math.cos(math.radians(tmin[li + 1])) ** 2
            for k in range(nph):
                r0, r1 = rng.random(n), rng.random(n)
                cz = np.sqrt((1 - r0) * c0 + r0 * c1)
                azi = 2 * math.pi * (k + r1 - .5) / nph
                sz = np.sqrt(1 - cz * cz)
                bins.append(np.stack([np.cos(azi) * sz, np.sin(azi) * sz, cz], axis=1))
    else:
        raise GbError(-3, f"sender sampling h={p.hemis} is not supported")
    duvw = np.concatenate(bins)
    dirs = -(duvw[:, :1] * udir + duvw[:, 1:2] * vdir + duvw[:, 2:3] * nrm)
    x = rng.random(len(dirs))
    if len(p.surfs) == 1:
        s = p.surfs[0]
        if (dirs @ s.nrm >= _FTINY).any():
            raise GbError(-1, f"internal - sample behind sender '{s.name}'")
        orig = _origins(s, x, rng)
    else:
        proj = np.stack([-(dirs @ s.nrm) * s.area for s in p.surfs], axis=1)
        proj = np.maximum(proj, 0.0)
        tot = proj.sum(axis=1)
        if (tot < _FTINY * _FTINY).any():
            raise GbError(-1, "internal - sample behind all sender elements!")
        cum = np.cumsum(proj, axis=1) / tot[:, None]
        which = np.minimum((x[:, None] > cum).sum(axis=1), len(p.surfs) - 1)
        orig = np.zeros_like(dirs)
        for j, s in enumerate(p.surfs):
            m = which == j
            if m.any():
                orig[m] = _origins(s, rng.random(int(m.sum())), rng)
    return np.concatenate([orig, dirs], axis=1), nb


def _sender(path) -> _Params:
    """Sender surfaces and directives (rfluxmtx.c:1154-1195 add_send_object)."""
    p = _Params()
    pending = ""
    for params, mod, typ, name, fa in _objects(path):
        pending += params
        if typ not in _SURF_TYPES:
            continue
        if typ == "source":
            raise GbError(-1, "cannot use source as a sender!")
        if pending.strip():
            p.parse(pending)
        pending = ""
        s = _Surf(typ, name, fa)
        if s.area > _FTINY * _FTINY:
            p.surfs.append(s)
    return p


# ------------------------------------------------------------------ driver

def _screen(params: Sequence[str]):
    """Split rfluxmtx's own options from those passed to rcontrib, with each
    option's argument count (rfluxmtx.c:1267-1420)."""
    jitter = None
    rc, fmt, xres, yres, sampcnt, iropt, ldopt = [], ["a", "a"], None, None, 0, None, None
    a = 0
    params = list(params)
    while a < len(params):
        o = params[a]
        if not o.startswith("-") or len(o) < 2:
            raise GbError(-1, f"unsupported option '{o}'")
        c = o[1]
        if c == "v":
            a += 1
            continue
        if c == "f" and len(o) > 2:
            if o[2] == "o" or o[2] not in "afdc":
                raise GbError(-1, f"unsupported option '{o}'")
            fmt = [o[2], o[3] if len(o) > 3 else o[2]]
            a += 1
            continue
        if c in "xy" and len(o) == 2:
            if c == "x":
                xres = params[a + 1]
            else:
                yres = params[a + 1]
            a += 2
            continue
        if o == "-c":
            sampcnt = int(params[a + 1])
            if sampcnt <= 0:
                raise GbError(-1, "bad sample count")
            a += 2
            continue
        if c in "Ii" and len(o) <= 3:
            iropt = o
            a += 1
            continue
        if o == "-bj":                          # rfluxmtx.c:1356-1360: passed to the bin parameters
            if a + 1 >= len(params):
                raise GbError(-1, "missing bin jitter value")
            jitter = params[a + 1]
            a += 2
            continue
        if o.startswith("-ld"):                # passed on in pass-through mode only
            ldopt = o
            a += 1
            continue
        if c in "wVuhr":
            na = 1
        elif c in "nstoe" or c == "l":
            na = 2
        elif c == "f":
            na = 2                             # -f calfile
        elif c == "c":
            na = {"s": 2, "w": 3}.get(o[2:3], 0)
        elif c == "b":
            if o[2:3] != "v":
                raise GbError(-1, f"unsupported option '{o}'")
            na = 1
        elif c == "d":
            na = 1 if o[2:3] == "v" else 2
        elif c == "a":
            na = 4 if o[2:3] == "v" else 2
        elif c == "m" and len(o) > 2:
            na = 4 if o[2] in "ea" else 2
        else:
            na = 0
        if na <= 0 or a + na > len(params):
            raise GbError(-1, f"unsupported option '{o}'")
        rc.extend(params[a:a + na])
        a += na
    return rc, fmt, xres, yres, sampcnt, iropt, ldopt, jitter


def rfluxmtx_array(receiver, surface=None, rays=None, params: Sequence[str] | None = None, octree=None,
                   scene=None, seed: int = 0):
    """(contributions (rows, bins, 3), rcontrib arguments, modifier specs,
    output format, yres) of an rfluxmtx run."""
    from . import Rcontrib, read_rays
    rc, fmt, xres, yres, sampcnt, iropt, ldopt, jitter = _screen(params or [])
    specs = _receivers(receiver, jitter)
    # oconv -f [-i octree] scene... receiver: the receiver goes last (rfluxmtx.c:139-178)
    files = ([str(octree)] if octree is not None else []) + [str(s) for s in (scene or [])] + [str(receiver)]
    sc = Scene(rad_files=files)
    if surface is None:                         # pass-through mode
        if iropt:
            rc.append(iropt)
        if xres:
            rc += ["-x", str(xres)]
        if yres:
            rc += ["-y", str(yres)]
        if ldopt:
            rc.append(ldopt)
        sampcnt = sampcnt or 1
        rc += [f"-f{fmt[0]}{fmt[1]}", "-c", str(sampcnt)]
        r = read_rays(rays or b"", fmt[0])
        nrows = int(yres) * (int(xres) if xres else 1) if yres else None
    else:
        if iropt:
            raise GbError(-1, "-i, -I supported for pass-through only")
        sampcnt = sampcnt or 10000
        p = _sender(surface)
        r, nsbins = _sender_rays(p, sampcnt, np.random.default_rng(seed))
        rc += [f"-fd{fmt[1]}", "-c", str(sampcnt), "-y", str(nsbins)]
        nrows = nsbins
    R = Rcontrib(b"", sc, params=rc)
    for s in specs:
        R.mods.append({k: v for k, v in s.items() if k != "output"})
    R.outputs = [s.get("output") for s in specs]
    out = R.run_array(r)
    return out, R, fmt[1], nrows


def _rfluxmtx(receiver, surface=None, rays: bytes | None = None, params: Sequence[str] | None = None,
              octree=None, scene=None) -> bytes:
    """rfluxmtx (same arguments as pyradiance.rfluxmtx): the flux transfer
    matrix as rcontrib writes it."""
    from . import _fmt_values, _header
    out, R, fout, nrows = rfluxmtx_array(receiver, surface, rays, params, octree, scene)
    args = R.args + [a for m in R.mods for a in ("-m", m["modifier"])]

    def write(arr) -> bytes:
        parts = []
        if R._opts.h:
            extra = [f"NROWS={nrows}"] if nrows else []
            extra.append(f"NCOLS={arr.shape[1]}")
            parts.append(_header("rcontrib", args, octree, fout, 3, extra))
        if fout == "a":
            flat = arr.reshape(arr.shape[0], -1)
            parts.append("".join("".join(f"{x:.6e}\t" for x in row) + "\n" for row in flat).encode())
        else:
            parts.append(_fmt_values(arr.reshape(-1, 3), fout))
        return b"".join(parts)

    if not any(R.outputs):
        return write(out)
    # receivers with o=: their columns go to files (a %s in the name is the
    # modifier), the others to the standard output (rt/rc2.c:131-250)
    files: dict[str | None, list[np.ndarray]] = {}
    col = 0
    for m, spec, nb in zip(R.mods, R.outputs, _nbins_each(R.mods)):
        name = None if spec is None else (spec.replace("%s", m["modifier"]) if "%s" in spec else spec)
        files.setdefault(name, []).append(out[:, col:col + nb])
        col += nb
    stdout = b""
    for name, cols in files.items():
        data = write(np.concatenate(cols, axis=1))
        if name is None:
            stdout = data
        else:
            Path(name).parent.mkdir(parents=True, exist_ok=True)
            Path(name).write_bytes(data)
    return stdout


def _nbins_each(mods: list[dict]) -> list[int]:
    out = []
    for m in mods:
        v = {k: (str(m[k]).encode() if m.get(k) is not None else None)
             for k in ("modifier", "binv", "nbins", "params", "calfile", "expr")}
        arr = (_lib.GbModspec * 1)(_lib.GbModspec(v["modifier"], v["binv"], v["nbins"], v["params"], v["calfile"],
                                                  v["expr"]))
        n = _lib.C.c_int(0)
        _lib.check(_lib.lib().gb_rcontrib_nbins(arr, 1, _lib.C.byref(n)))
        out.append(n.value)
    return out

