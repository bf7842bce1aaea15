"""Klems matrix BSDFs (WINDOW 6 XML) as dctimestep's transmission matrix.

Restates ``cm_loadBTDF`` (util/cmbsdf.c:146-181) over the matrix BSDF loader
of common/bsdf_m.c (SDloadMtx :663-727, load_bsdf_data :407-531,
extract_diffuse / subtract_min :595-661) for grayscale ("Visible") data in
the Klems bases or bases the file defines:

* "Transmission Front" data in the file is the BSDF's back transmission and
  "Transmission Back" its front one (bsdf_m.c:418-438: WINDOW 6's front and
  back are reversed); the matrix is the back transmission when the file has
  it, else the front one turned around by reciprocity (cmbsdf.c:64-131:
  incident patch i and exiting patch o of the result read the value of
  exiting patch i' and incident patch o', the patches 180 degrees round in
  azimuth, bsdf_m.c:137-299 fo_getvec, fo_getndx, fi_/bi_/bo_ variants).
* Each component's smallest value (over values shifted by a fixed
  position-dependent factor within 3e-4, bsdf_m.c:294-305 mBSDF_color) is
  taken out as a Lambertian part when above 0.01/pi and added back when the
  matrix is built, so values below it become it.
* Element (o, i) of the result is the BSDF value times the projected solid
  angle of the incident patch (bsdf_m.c:185-207 io_getohm), in single
  precision as the reference holds it; grey values give equal RGB.

A file without transmission data gives the zero matrix of the full Klems
basis, as the reference's Lambertian fallback does.  Spectral (CIE-X/Y/Z)
data, tensor-tree BSDFs and BRDFs are refused (the reference's
cm_loadBTDF refuses tensor trees too).
"""
from __future__ import annotations

import math
import re
import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np

from ._lib import GbError

# the built-in bases (bsdf_m.c:22-55): (name, [(lower theta of ring, phis)...], upper 90)
KLEMS = {
    "LBNL/Klems Full": [(0., 1), (5., 8), (15., 16), (25., 20), (35., 24), (45., 24), (55., 24), (65., 16),
                        (75., 12)],
    "LBNL/Klems Half": [(0., 1), (6.5, 8), (19.5, 12), (32.5, 16), (45.5, 20), (58.5, 12), (71.5, 8)],
    "LBNL/Klems Quarter": [(0., 1), (9., 8), (27., 12), (45., 12), (63., 8)],
}


class Basis:
    """Rings of patches: tmin[k] the lower polar bound of ring k (degrees),
    tmin[-1] = 90, nphis[k] its patches."""

    def __init__(self, name: str, rings, top: float = 90.0):
        self.name = name
        self.tmin = [float(t) for t, _ in rings] + [float(top)]
        self.nphis = [int(n) for _, n in rings]
        self.n = sum(self.nphis)
        self.first = np.cumsum([0] + self.nphis)

    def ring(self, ndx: int):
        li = int(np.searchsorted(self.first, ndx, side="right") - 1)
        return li, ndx - int(self.first[li])

    def ohm(self, ndx: int) -> float:
        """Projected solid angle of a patch (io_getohm)."""
        li, _ = self.ring(ndx)
        t0, t1 = math.radians(self.tmin[li]), math.radians(self.tmin[li + 1])
        return math.pi * (math.cos(t0) ** 2 - math.cos(t1) ** 2) / self.nphis[li]

    def centre(self, ndx: int):
        """Exiting-front direction through the middle of a patch (fo_getvec
        at ndx + 0.5: the middle of the ring's cos^2 range, the patch's
        azimuth centre)."""
        li, k = self.ring(ndx)
        d = 0.5 * math.cos(math.radians(self.tmin[li])) ** 2 + 0.5 * math.cos(math.radians(self.tmin[li + 1])) ** 2
        z = math.sqrt(d)
        azi = 2.0 * math.pi * k / self.nphis[li]
        s = math.sqrt(1.0 - z * z)
        return (math.cos(azi) * s, math.sin(azi) * s, z)

    def index(self, v) -> int:
        """Patch of an exiting-front direction (fo_getndx)."""
        if v[2] < 0 or v[2] > 1.00001:
            return -1
        pol = math.degrees(math.acos(max(-1.0, min(1.0, v[2]))))
        azi = math.degrees(math.atan2(v[1], v[0]))
        if azi < 0.0:
            azi += 360.0
        li = 1
        while self.tmin[li] <= pol:
            if li >= len(self.nphis):
                return -1
            li += 1
        li -= 1
        k = int(azi / 360.0 * self.nphis[li] + 0.5)
        if k >= self.nphis[li]:
            k = 0
        return int(self.first[li]) + k


def _local(tag: str) -> str:
    return tag.rsplit("}", 1)[-1]


def _child(el, name):
    for c in el:
        if _local(c.tag) == name:
            return c
    return None


def _children(el, name):
    return [c for c in el if _local(c.tag) == name]


def _text(el, *path) -> str:
    for p in path:
        el = _child(el, p) if el is not None else None
    return (el.text or "").strip() if el is not None else ""


def _read_layer(path):
    try:
        root = ET.parse(str(path)).getroot()
    except (ET.ParseError, OSError) as e:
        raise GbError(-1, f"cannot read BSDF '{path}': {e}")
    layer = _child(_child(root, "Optical"), "Layer") if _child(root, "Optical") is not None else None
    if layer is None:
        raise GbError(-1, f"BSDF '{path}': no Optical/Layer element")
    return layer


def _subtract_min(m: np.ndarray) -> float:
    """Take out the smallest value as a Lambertian part (subtract_min on a
    grey matrix m[o, i], in place); returns cieY / pi (0 if not taken)."""
    nout, ninc = m.shape
    i = np.arange(ninc, dtype=np.float64)[None, :]
    o = np.arange(nout, dtype=np.float64)[:, None]
    d = 2.0 * ninc / (i + .22545) + 4.0 * nout / (o + .70281)
    d -= np.floor(d)
    coef = (m.astype(np.float64) * (1.0 + 6e-4 * (d - .5))).astype(np.float32)
    ymin = np.float32(coef.min())
    if ymin <= .01 / math.pi:
        return 0.0
    m -= ymin
    return float(ymin)


def load_btdf(path) -> np.ndarray:
    """The transmission matrix of a Klems matrix BSDF file: (exiting
    patches, incident patches, 3) float32, each value times the incident
    patch's projected solid angle (cm_loadBTDF)."""
    layer = _read_layer(path)
    dd = _child(layer, "DataDefinition")
    structure = _text(dd, "IncidentDataStructure") if dd is not None else ""
    if structure.lower() == "rows":
        rows_in = True
    elif structure.lower() == "columns":
        rows_in = False
    else:
        raise GbError(-3, f"unsupported BSDF '{path}' (incident data structure '{structure}')")
    bases = {k: Basis(k, v) for k, v in KLEMS.items()}
    for ab in _children(dd, "AngleBasis"):                    # load_angle_basis
        name = _text(ab, "AngleBasisName")
        if not name or name in bases:
            continue
        rings, upper = [], 90.0
        for blk in _children(ab, "AngleBasisBlock"):  # ring k starts at ring k-1's upper bound
            rings.append((upper if rings else 0.0, int(_text(blk, "nPhis"))))
            upper = float(_text(blk, "ThetaBounds", "UpperTheta"))
        if not rings:
            raise GbError(-1, f"BSDF '{path}': empty angle basis '{name}'")
        bases[name] = Basis(name, rings, upper)
    tf = tb = None                       # (matrix[o, i], incident basis, exiting basis)
    for wd in _children(layer, "WavelengthData"):
        kind = _text(wd, "Wavelength")
        if kind.lower() in ("cie-x", "cie-z"):
            raise GbError(-3, f"spectral BSDF '{path}' is not supported")
        if kind.lower() != "visible":
            continue
        for blk in _children(wd, "WavelengthDataBlock"):
            direction = _text(blk, "WavelengthDataDirection").lower()
            if direction not in ("transmission front", "transmission back"):
                continue
            cb, rb = _text(blk, "ColumnAngleBasis"), _text(blk, "RowAngleBasis")
            if cb not in bases or rb not in bases:
                raise GbError(-1, f"BSDF '{path}': undefined angle basis '{cb if cb not in bases else rb}'")
            ib, ob = bases[cb], bases[rb]
            vals = np.array([float(x) for x in re.split(r"[\s,]+", _text(blk, "ScatteringData")) if x],
                            dtype=np.float64)
            if vals.size < ib.n * ob.n:
                raise GbError(-1, f"Bad/missing BSDF ScatteringData in '{path}'")
            vals = np.maximum(vals[: ib.n * ob.n], 0.0).astype(np.float32)
            m = vals.reshape(ib.n, ob.n).T.copy() if rows_in else vals.reshape(ob.n, ib.n).copy()
            if direction == "transmission front":
                tb = (m, ib, ob)
            else:
                tf = (m, ib, ob)
    if tf is None and tb is None:
        # no transmission matrix: its Lambertian part alone in the full Klems
        # basis (cm_bsdf_Lamb, util/cmbsdf.c:122-143), zero with no data to take
        # one from
        return np.zeros((145, 145, 3), dtype=np.float32)
    recip = tb is None
    m, ib, ob = tf if recip else tb
    diff = np.float32(_subtract_min(m))
    if recip:
        # cm_bsdf_recip: rows are incident patches, columns exiting ones; the
        # value of column c, row r is the front matrix's value for the exiting
        # patch opposite c's incident direction and the incident patch
        # opposite r's exiting direction (recip_out_from_in, recip_in_from_out)
        ro = [ob.index((-x, -y, z)) for x, y, z in (ib.centre(c) for c in range(ob.n))]
        ri = [ib.index((-x, -y, z)) for x, y, z in (ob.centre(r) for r in range(ib.n))]
        res = np.empty((ib.n, ob.n), dtype=np.float32)
        for c in range(ob.n):
            f = m[ro[c], ri]
            col = np.where(f <= 0, np.float32(0), f) + diff
            res[:, c] = (col.astype(np.float64) * ob.ohm(ro[c])).astype(np.float32)
    else:
        # cm_bsdf: rows are exiting patches, columns incident ones
        res = np.empty(m.shape, dtype=np.float32)
        for c in range(ib.n):
            f = m[:, c]
            col = np.where(f <= 0, np.float32(0), f) + diff
            res[:, c] = (col.astype(np.float64) * ib.ohm(c)).astype(np.float32)
    return np.repeat(res[:, :, None], 3, axis=2)

