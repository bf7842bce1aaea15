"""GB300 drop-in for pyradiance's ray-tracing hot path.

``rtrace``, ``Rcontrib`` and ``dctimestep`` keep the call signatures, option
semantics and byte formats of ``pyradiance.rtrace``
(src/pyradiance/rt.py:278-362), ``pyradiance.Rcontrib`` (rt.py:165-235) and
``pyradiance.dctimestep`` (src/pyradiance/util.py:140-192), but run in
process on the GPU through ``libgbrad.so`` instead of spawning the Radiance
programs.  Errors raise ``RuntimeError`` as the reference's
``handle_called_process_error`` does (src/pyradiance/anci.py:13-29).
"""
from __future__ import annotations

import os
import re
import ctypes as C
import time
from pathlib import Path
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import GbError, GbModspec, Scene, check, last_stats, lib, parse_opts, ptr

__all__ = ["rtrace", "Rcontrib", "dctimestep", "rfluxmtx", "rmtxop", "Rmtxop", "Scene", "load_scene", "read_rays", "GbError", "last_stats"]

_SCENES: dict = {}


def load_scene(octree) -> Scene:
    """Scene for an octree path (cached per path and modification time) or
    for a list of scene text files (octree built on the host)."""
    if isinstance(octree, Scene):
        return octree
    if isinstance(octree, (list, tuple)):
        return Scene(rad_files=octree)
    p = str(octree)
    key = (os.path.abspath(p), os.path.getmtime(p) if os.path.exists(p) else 0)
    sc = _SCENES.get(key)
    if sc is None:
        if p.endswith(".rad"):
            sc = Scene(rad_files=[p])
        else:
            sc = Scene(p)
        _SCENES[key] = sc
    return sc


def _wrap(fn):
    def inner(*a, **k):
        try:
            return fn(*a, **k)
        except GbError as e:
            raise RuntimeError(f"An error occurred with exit code {-e.code}: {e}") from None
    inner.__name__ = fn.__name__
    inner.__doc__ = fn.__doc__
    inner.__wrapped__ = fn
    return inner


# ---------------------------------------------------------------- formats

def read_rays(data: bytes, fmt: str) -> np.ndarray:
    """Ray records (n, 6) float64 from rtrace/rcontrib input bytes
    (rt/rtrace.c:505-548 getvec; rt/rc2.c:259-290)."""
    if fmt == "a":
        vals = np.array(data.split(), dtype=np.float64) if data.strip() else np.zeros(0)
        n = len(vals) // 6
        return vals[: 6 * n].reshape(n, 6)
    if fmt == "f":
        a = np.frombuffer(data, dtype=np.float32)
        n = len(a) // 6
        return a[: 6 * n].reshape(n, 6).astype(np.float64)
    if fmt == "d":
        a = np.frombuffer(data, dtype=np.float64)
        n = len(a) // 6
        return a[: 6 * n].reshape(n, 6).copy()
    raise RuntimeError(f"Illegal i/o format: {fmt}")


def _header(prog: str, args: list[str], octree, fmt: str, ncomp: int | None, extra: list[str] | None = None) -> bytes:
    lines = ["#?RADIANCE"]
    if octree is not None and not isinstance(octree, (Scene, list, tuple)):
        try:
            with open(octree, "rb") as f:
                head = f.read(4096)
            for ln in head.split(b"\n\n")[0].split(b"\n")[1:]:
                s = ln.decode(errors="replace")
                if s and not s.startswith("FORMAT="):
                    lines.append(s)
        except OSError:
            pass
    lines.append(" ".join([prog, *map(str, args)]))
    lines.append("SOFTWARE= " + lib().gb_version().decode())
    now = time.time()
    lines.append(time.strftime("CAPDATE= %Y:%m:%d %H:%M:%S", time.localtime(now)))
    lines.append(time.strftime("GMT= %Y:%m:%d %H:%M:%S", time.gmtime(now)))
    if ncomp:
        lines.append(f"NCOMP={ncomp}")
    lines.extend(extra or [])
    if fmt in ("f", "d"):
        lines.append("BigEndian=0")
    name = {"a": "ascii", "f": "float", "d": "double", "c": "32-bit_rle_rgbe"}[fmt]
    text = "\n".join(lines) + "\n" + "FORMAT=" + name
    align = {"f": 4, "d": 8}.get(fmt, 0)
    if align:                       # common/header.c:190-222 padding
        pos = (len(text.encode()) + 2) % align
        text += " " * ((align - pos) if pos else 0)
    return (text + "\n\n").encode()


def _ascii_rows(vals: np.ndarray, sep: str = "\t", end: str = "\t\n") -> list[str]:
    """Each row of a 2-D array as text: numbers in %e (six digits, as the
    reference's puta in rt/rtrace.c and rt/rc2.c) joined by sep, the row
    ended by end."""
    vals = np.asarray(vals, dtype=np.float64)
    if vals.ndim == 1:
        vals = vals[:, None]
    if vals.shape[1] == 0:
        return [end] * len(vals)
    row = sep.join(["%e"] * vals.shape[1]) + end
    return [row % tuple(r) for r in vals.tolist()]


def _ascii_block(vals: np.ndarray, sep: str = "\t", end: str = "\t\n") -> bytes:
    """The text of _ascii_rows, formatted by the library's host threads
    (gb_format_rows)."""
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    if vals.ndim == 1:
        vals = vals[:, None]
    nrows, ncols = vals.shape
    if nrows == 0:
        return b""
    cap = nrows * (ncols * (16 + len(sep)) + len(end)) + 1
    buf = C.create_string_buffer(cap)
    n = C.c_int64(0)
    check(lib().gb_format_rows(vals.ctypes.data, nrows, ncols, sep.encode(), end.encode(), buf, cap, C.byref(n)))
    return buf.raw[:n.value]


def _fmt_values(vals: np.ndarray, fmt: str) -> bytes:
    if fmt == "a":
        return _ascii_block(vals)
    if fmt == "f":
        return np.ascontiguousarray(vals, dtype=np.float32).tobytes()
    if fmt == "d":
        return np.ascontiguousarray(vals, dtype=np.float64).tobytes()
    raise RuntimeError("color (-fc) output is not supported")


# ------------------------------------------------------------------ rtrace

_CAST_ONLY = set("odLpNnsmMwWc~")


def _rtrace(rays: bytes, octree, header: bool = True, inform: str = "a", outform: str = "a",
            irradiance: bool = False, irradiance_lambertian: bool = False, outspec: str | None = None,
            trace_exclude: str = "", trace_include: str = "", trace_exclude_file=None,
            trace_include_file=None, uncorrelated: bool = False, xres: int | None = None,
            yres: int | None = None, nproc: int | None = None, params: Sequence[str] | None = None,
            report: bool = False, version: bool = False) -> bytes:
    """Run rtrace on the GPU (same signature as pyradiance.rtrace)."""
    if version:
        return (lib().gb_version().decode() + "\n").encode()
    if not isinstance(rays, bytes):
        raise TypeError("Rays must be bytes")
    args: list[str] = []
    if not header:
        args.append("-h")
    if irradiance:
        args.append("-I")
    elif irradiance_lambertian:
        args.append("-i")
    args.append(f"-f{inform}{outform}")
    if outspec:
        args.append(f"-o{outspec}")
    # the same single argument as src/pyradiance/rt.py:342-349, which the
    # option parser rejects as rt/rtmain.c:210-214 does (the list's name
    # must be a separate argument): a command line error either way
    if trace_exclude:
        args.append(f"-te{trace_exclude}")
    elif trace_include:
        args.append(f"-ti{trace_include}")
    elif trace_exclude_file:
        args.append(f"-tE{trace_exclude_file}")
    elif trace_include_file:
        args.append(f"-tI{trace_include_file}")
    if uncorrelated:
        args.append("-u+")
    if xres is not None:
        args += ["-x", str(xres)]
    if yres is not None:
        args += ["-y", str(yres)]
    if nproc:
        args += ["-n", str(nproc)]
    if params is not None:
        args += list(params)
    opts, used = parse_opts(args, _lib.GB_PROG_RTRACE)
    if used != len(args):
        raise GbError(-1, f"command line error at '{args[used]}'")
    spec = opts.outspec.decode() or "v"
    fin, fout = opts.fin.decode(), opts.fout.decode()
    sc = load_scene(octree)
    r = read_rays(rays, fin)
    n = len(r)
    dirlen = np.sqrt((r[:, 3:6] ** 2).sum(axis=1)) if n else np.zeros(0)
    need_val = any(ch not in _CAST_ONLY for ch in spec)
    vals = np.zeros((n, 3)) if need_val else None
    hit = np.full(n, -1, dtype=np.int32)
    hitt = np.zeros(n)
    good = dirlen > 0
    rr = np.ascontiguousarray(r[good]) if n else r
    ng = len(rr)
    gv = np.zeros((ng, 3)) if need_val else None
    gh = np.zeros(ng, dtype=np.int32)
    gt = np.zeros(ng)
    if ng:
        check(lib().gb_rtrace(sc.handle, opts, ptr(rr), ng, ptr(gv), ptr(gh), ptr(gt)))
    if need_val:
        vals[good] = gv
    hit[good] = gh
    hitt[good] = gt
    nrm_geo = nrm_shade = uvs = None
    if any(ch in "nNc" for ch in spec):          # first-hit normals and (u,v) (rt/rtrace.c:766-820)
        nrm_geo, nrm_shade, uvs = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 2))
        gN, gn, guv = np.zeros((ng, 3)), np.zeros((ng, 3)), np.zeros((ng, 2))
        gh2, gt2 = np.zeros(ng, dtype=np.int32), np.zeros(ng)
        if ng:
            check(lib().gb_rtrace_hits(sc.handle, opts, ptr(rr), ng, ptr(gh2), ptr(gt2), ptr(gN), ptr(gn),
                                       ptr(guv)))
        nrm_geo[good], nrm_shade[good], uvs[good] = gN, gn, guv
    out = []
    ncomp = 0                                    # rt/rtrace.c:244-370 setrtoutput
    for ch in spec:
        ncomp += {"v": 3, "V": 3, "W": 3, "o": 3, "d": 3, "p": 3, "N": 3, "n": 3, "L": 1, "l": 1, "w": 1,
                  "s": 1, "m": 1, "M": 1, "c": 2}.get(ch, 0)
    if opts.h:
        out.append(_header("rtrace", args, octree, fout, ncomp or None))
    unit = np.where(good[:, None], r[:, 3:6] / np.where(dirlen > 0, dirlen, 1)[:, None], 0.0) if n else r[:, 3:6]
    hitm = hit >= 0
    # the output columns in spec order: numeric blocks (n x k) or names (n)
    items = []
    for ch in spec:
        if ch in "vV":                              # a primary ray's contribution is its value
            items.append(vals)
        elif ch == "o":
            items.append(r[:, 0:3])
        elif ch == "d":
            items.append(unit)
        elif ch == "L":
            items.append(np.where(hitm, hitt, 1e10)[:, None])
        elif ch == "p":
            items.append(np.where(hitm[:, None], r[:, 0:3] + unit * np.where(hitm, hitt, 0.0)[:, None], 0.0))
        elif ch in "smM":
            get = {"s": sc.object_name, "m": sc.modifier_name, "M": sc.material_name}[ch]
            cache: dict[int, str] = {}
            names = []
            for h in hit.tolist():
                if h < 0:
                    names.append("*")
                else:
                    if h not in cache:
                        cache[h] = get(h)
                    names.append(cache[h])
            items.append(names)
        elif ch == "w":
            items.append(np.ones((n, 1)))
        elif ch == "W":                             # a primary ray's coefficient (rt/rtrace.c:847-860)
            items.append(np.ones((n, 3)))
        elif ch == "N":
            items.append(nrm_geo)
        elif ch == "n":
            items.append(nrm_shade)
        elif ch == "c":
            items.append(uvs)
        else:
            raise GbError(-3, f"output option -o{ch} is not supported")
    if fout == "a":
        # every value and name followed by a tab, a newline after each ray
        # (rt/rtrace.c:471-500 printvals, puta, oputs)
        cols = [_ascii_rows(it, end="\t") if isinstance(it, np.ndarray) else [nm + "\t" for nm in it]
                for it in items]
        if n:
            rows = ["".join(parts) + "\n" for parts in zip(*cols)] if cols else ["\n"] * n
            out.append("".join(rows).encode())
    else:
        if any(not isinstance(it, np.ndarray) for it in items):
            raise GbError(-1, "names need ascii output")
        if items and n:
            out.append(_fmt_values(np.concatenate([np.asarray(it, dtype=np.float64) for it in items], axis=1),
                                   fout))
    return b"".join(out)


rtrace = _wrap(_rtrace)


# ---------------------------------------------------------------- rcontrib

class Rcontrib:
    """rcontrib on the GPU (same constructor and methods as pyradiance.Rcontrib)."""

    def __init__(self, inp: bytes, octree, nproc: int = 1, yres: int | None = None, inform: str | None = None,
                 outform: str | None = None, report: int = 0, params: Sequence[str] | None = None):
        self.octree = octree
        self.inp = inp
        self.args: list[str] = ["-n", str(nproc)]
        if params is not None:
            self.args.extend(params)
        if None not in (inform, outform):
            self.args.append(f"-f{inform}{outform}")
        if yres is not None:
            self.args.extend(["-y", str(yres)])
        if report:
            self.args.extend(["-t", str(report)])
        self.mods: list[dict] = []
        self.mod_args: list[str] = []
        self._ospec: str | None = None
        self._xres: int | None = None
        self._yres: int | None = None
        self.seed = None
        self.replica = 0
        self.last_rays = 0

    def add_modifier(self, modifier: str | None = None, modifier_path: str | None = None,
                     calfile: str | None = None, expression: str | None = None, nbins: str | None = None,
                     binv: str | None = None, param: str | None = None, xres: int | None = None,
                     yres: int | None = None, output: str | None = None):
        # the arguments pyradiance passes for this modifier, in its order
        # (src/pyradiance/rt.py:190-228); -o, -x and -y stay in force for
        # the modifiers after it, as rcontrib reads them
        arglist: list[str] = []
        for flag, v in (("-f", calfile), ("-e", expression), ("-bn", nbins), ("-b", binv), ("-p", param),
                        ("-x", xres), ("-y", yres), ("-o", output)):
            if v is not None:
                arglist += [flag, str(v)]
        if modifier is not None:
            arglist += ["-m", modifier]
        elif modifier_path is not None:
            arglist += ["-M", str(modifier_path)]
        else:
            raise ValueError("Modifier or modifier path must be provided.")
        self.mod_args.extend(arglist)
        if output is not None:
            self._ospec = str(output)
        if xres is not None:
            self._xres = int(xres)
        if yres is not None:
            self._yres = int(yres)
        names = [modifier] if modifier is not None else [
            w for w in Path(modifier_path).read_text().split() if w]
        for nm in names:
            self.mods.append(dict(modifier=nm, calfile=calfile, expr=expression, nbins=nbins, binv=binv,
                                  params=param, output=self._ospec))
        return self

    def _specs(self):
        keep = []
        arr = (GbModspec * len(self.mods))()
        for i, m in enumerate(self.mods):
            vals = {k: (str(v).encode() if v is not None else None) for k, v in m.items() if k != "output"}
            keep.append(vals)
            arr[i] = GbModspec(vals["modifier"], vals["binv"], vals["nbins"], vals["params"], vals["calfile"],
                               vals["expr"])
        return arr, keep

    def run_array(self, rays: np.ndarray | None = None) -> np.ndarray:
        """Contributions as a (records, total bins, 3) float64 array."""
        opts, used = parse_opts(self.args, _lib.GB_PROG_RCONTRIB)
        if used != len(self.args):
            raise GbError(-1, f"command line error at '{self.args[used]}'")
        if self._xres is not None:
            opts.x = self._xres
        if self._yres is not None:
            opts.y = self._yres
        if self.seed is not None:
            opts.seed = int(self.seed)
        opts.replica = int(self.replica)
        if rays is None:
            r = _rc_rays(self.inp, opts.fin.decode())
        else:
            r = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 6)
        specs, keep = self._specs()
        nb = _lib.C.c_int(0)
        check(lib().gb_rcontrib_nbins(specs, len(self.mods), _lib.C.byref(nb)))
        accum = max(1, opts.c)
        nrec = len(r) // accum
        out = np.zeros((max(nrec, 0), nb.value, 3))
        if len(r):
            cnt = _lib.C.c_int64(0)
            sc = load_scene(self.octree)
            check(lib().gb_rcontrib(sc.handle, opts, specs, len(self.mods), ptr(r), len(r), ptr(out),
                                    _lib.C.byref(cnt)))
            self.last_rays = cnt.value
        self._opts = opts
        return out

    def run_batch(self, jobs) -> list[np.ndarray]:
        """Many sensor grids at once: jobs is a sequence of (octree or Scene,
        rays n x 6); each grid's contributions come back as run_array's.
        The grids of one scene are traced as one wavefront and different
        scenes concurrently (gb_rcontrib_batch)."""
        opts, used = parse_opts(self.args, _lib.GB_PROG_RCONTRIB)
        if used != len(self.args):
            raise GbError(-1, f"command line error at '{self.args[used]}'")
        if self.seed is not None:
            opts.seed = int(self.seed)
        opts.replica = int(self.replica)
        specs, keep = self._specs()
        nb = _lib.C.c_int(0)
        check(lib().gb_rcontrib_nbins(specs, len(self.mods), _lib.C.byref(nb)))
        accum = max(1, opts.c)
        scenes, rays, outs = [], [], []
        for scene, r in jobs:
            sc = scene if isinstance(scene, Scene) else load_scene(scene)
            r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 6)
            scenes.append(sc)
            rays.append(r)
            outs.append(np.zeros((len(r) // accum, nb.value, 3)))
        k = len(scenes)
        vp = _lib.C.c_void_p
        c_sc = (vp * max(1, k))(*[s.handle.value for s in scenes])
        c_in = (vp * max(1, k))(*[r.ctypes.data for r in rays])
        c_out = (vp * max(1, k))(*[o.ctypes.data for o in outs])
        c_n = (_lib.C.c_int64 * max(1, k))(*[len(r) for r in rays])
        cnt = _lib.C.c_int64(0)
        check(lib().gb_rcontrib_batch(k, c_sc, opts, specs, len(self.mods), c_in, c_n, c_out, _lib.C.byref(cnt)))
        self.last_rays = cnt.value
        return outs

    def _call(self) -> bytes:
        """rcontrib's output streams (rt/rc2.c:131-250 getostream): the
        modifiers without an output specification go to the returned bytes,
        the others to files named by their specification (%s: the
        modifier; %d and the like: one file per bin), each stream with its
        own header; an existing file is an error, as rcontrib does not
        overwrite without -fo."""
        from .rflux import _nbins_each
        nb = _nbins_each(self.mods)
        start = np.concatenate([[0], np.cumsum(nb)]).astype(int)
        # streams: (file name or None, [(modifier, bin or None)]); rt/rc2.c:41-97 ofname:
        # at most one %s (the modifier) and one %d-like (the bin) in a specification
        streams: list[tuple[str | None, list]] = []
        for i, m in enumerate(self.mods):
            spec = m.get("output")
            conv = re.findall(r"%[0-9]*([a-zA-Z%])", spec) if spec is not None else []
            conv = [c for c in conv if c != "%"]
            if any(c not in "sdioxX" for c in conv) or conv.count("s") > 1 or \
                    sum(c in "dioxX" for c in conv) > 1:
                raise GbError(-1, f"bad output format '{spec}'")
            per_bin = any(c in "dioxX" for c in conv)
            for b in (range(int(nb[i])) if per_bin else [None]):
                if spec is None:
                    name = None
                elif per_bin:
                    name = spec % ((m["modifier"], b) if "s" in conv and conv.index("s") == 0 else
                                   ((b, m["modifier"]) if "s" in conv else (b,)))
                else:
                    name = spec % (m["modifier"],) if "s" in conv else spec
                for nm, idx in streams:
                    if nm == name:
                        idx.append((i, b))
                        break
                else:
                    streams.append((name, [(i, b)]))
        for name, _ in streams:
            if name is not None and Path(name).exists():
                raise GbError(-2, f"cannot open '{name}' for writing")
        arr = self.run_array()
        opts = self._opts
        fout = opts.fout.decode()
        result = b""
        for name, idx in streams:
            cols = np.concatenate([arr[:, start[i]:start[i + 1]] if b is None else arr[:, start[i] + b:start[i] + b + 1]
                                   for i, b in idx], axis=1)
            parts = []
            i0, b0 = idx[0]
            spec = self.mods[i0].get("output")
            if opts.h:
                extra = []
                if name is not None and ((spec is not None and "%s" in spec) or cols.shape[1] == 1):
                    extra.append(f"MODIFIER={self.mods[i0]['modifier']}")
                if name is not None and b0 is not None:
                    extra.append(f"BIN={b0}")
                if opts.y > 0:
                    extra.append(f"NROWS={opts.y * max(opts.x, 1)}")
                if opts.x <= 0 or cols.shape[1] > 1:
                    extra.append(f"NCOLS={cols.shape[1]}")
                parts.append(_header("rcontrib", self.args + self.mod_args, self.octree, fout, 3, extra))
            if cols.shape[1] == 1 and opts.x > 0 and opts.y > 0:     # rt/rc2.c:129-134 printresolu
                parts.append(f"-Y {opts.y} +X {opts.x}\n".encode())
            if fout == "a":
                parts.append(_ascii_block(cols.reshape(cols.shape[0], -1), end="\t\n"))
            else:
                parts.append(_fmt_values(cols.reshape(-1, 3), fout))
            data = b"".join(parts)
            if name is None:
                result = data
            else:
                Path(name).parent.mkdir(parents=True, exist_ok=True)
                Path(name).write_bytes(data)
        return result

    def __call__(self) -> bytes:
        return _wrap(self._call)()


def _rc_rays(data: bytes, fmt: str) -> np.ndarray:
    r = read_rays(data, fmt)
    d = np.sqrt((r[:, 3:6] ** 2).sum(axis=1)) if len(r) else np.zeros(0)
    if len(r) and (d == 0).any():
        raise GbError(-3, "zero-direction (flush) records are not supported")
    return r


# -------------------------------------------------------------- dctimestep

def _read_matrix(src, fmt_hint: str | None = None):
    """Radiance matrix file or bytes -> (rows, cols, 3) float32 array
    (util/cmatrix.c:82-122 header, :191 cm_load)."""
    data = Path(src).read_bytes() if not isinstance(src, bytes) else src
    nrows = ncols = 0
    fmt = fmt_hint
    big = None
    body = data
    if data.startswith(b"#?"):
        end = data.find(b"\n\n")
        head, body = data[:end], data[end + 2:]
        for ln in head.split(b"\n"):
            s = ln.decode(errors="replace").strip()
            if s.startswith("NROWS="):
                nrows = int(s[6:])
            elif s.startswith("NCOLS="):
                ncols = int(s[6:])
            elif s.startswith("NCOMP=") and int(s[6:]) != 3:
                raise GbError(-1, "unexpected # components (must be 3)")
            elif s.startswith("FORMAT="):
                fmt = {"ascii": "a", "float": "f", "double": "d"}.get(s[7:].strip(), s[7:].strip())
            elif s.startswith("BigEndian="):
                big = s[10:] == "1"
    if fmt == "a" or fmt is None:
        vals = np.array(body.split(), dtype=np.float64)
    elif fmt == "f":
        vals = np.frombuffer(body, dtype=">f4" if big else "<f4").astype(np.float64)
    elif fmt == "d":
        vals = np.frombuffer(body, dtype=">f8" if big else "<f8")
    else:
        raise GbError(-3, f"matrix format '{fmt}' is not supported")
    if nrows <= 0 and ncols > 0:
        nrows = len(vals) // (3 * ncols)
    if ncols <= 0 and nrows > 0:
        ncols = len(vals) // (3 * nrows)
    if nrows <= 0 or ncols <= 0:
        raise GbError(-1, "missing matrix dimensions")
    return np.ascontiguousarray(vals[: nrows * ncols * 3].reshape(nrows, ncols, 3), dtype=np.float32)


DCT_MODES = {"fp32": _lib.GB_DCT_FP32, "bf16x3": _lib.GB_DCT_BF16X3, "fp64": _lib.GB_DCT_FP64,
             "fp16x3": _lib.GB_DCT_FP16X3, "fp16": _lib.GB_DCT_FP16}


def dctimestep_array(dc: np.ndarray, sky: np.ndarray, mode: str = "fp16x3") -> np.ndarray:
    """R = DC x sky per channel on the GPU; (M,K,3) x (K,N,3) -> (M,N,3) float32.
    The default, the pre-scaled FP16 split on the tensor cores, stays within
    1e-5 relative of an FP64 product; "fp32", "fp64" (CUDA cores), "bf16x3"
    and "fp16" (tensor cores, less accurate) are the other forms."""
    dc = np.ascontiguousarray(dc, dtype=np.float32)
    sky = np.ascontiguousarray(sky, dtype=np.float32)
    M, K, _ = dc.shape
    K2, N, _ = sky.shape
    if K != K2:
        raise GbError(-1, "matrix dimension mismatch")
    out = np.empty((M, N, 3), dtype=np.float32)
    m = DCT_MODES[mode]
    check(lib().gb_dctimestep(ptr(dc), ptr(sky), M, K, N, m, ptr(out)))
    return out


def _dctimestep(*mtx, nstep: int | None = None, header: bool = True, xres: int | None = None,
                yres: int | None = None, inform: str | None = None, outform: str | None = None,
                ospec: str | None = None) -> bytes | None:
    """dctimestep on the GPU (same signature as pyradiance.dctimestep): the
    two-matrix form DC x sky, and the four-matrix form V x T x D x sky of
    util/dctimestep.c:243-264 and :324-330, multiplied as the reference
    does, D x sky first, then T, then V, each product on the GPU's tensor
    cores (pre-scaled FP16 split, within 1e-5 of FP64) with FP32
    intermediates (the reference's matrices hold floats).  A transmission
    matrix given as a Klems matrix BSDF (an .xml file) is converted as
    cm_loadBTDF converts it (pyradiance_gb300/bsdf.py)."""
    if len(mtx) not in (2, 4):
        raise ValueError("mtx must be a list of 2 or 4 items")
    if ospec:
        raise GbError(-3, "output specification files are not supported")
    if len(mtx) == 4:
        tx = mtx[1]
        if isinstance(tx, (str, Path)) and not str(tx).startswith("!") and str(tx).lower().endswith(".xml"):
            from .bsdf import load_btdf
            T = load_btdf(tx)                        # util/dctimestep.c:250-254
        else:
            T = _read_matrix(tx)
        V, D = _read_matrix(mtx[0]), _read_matrix(mtx[2])
        sky = _read_matrix(mtx[3], inform)
        for a, b, what in ((D, sky, "daylight and sky"), (T, D, "transmission and daylight"),
                           (V, T, "view and transmission")):
            if a.shape[1] != b.shape[0]:
                raise GbError(-1, f"{what} matrices do not match ({a.shape[1]} columns, {b.shape[0]} rows)")
        R = dctimestep_array(V, dctimestep_array(T, dctimestep_array(D, sky)))
    else:
        dc = _read_matrix(mtx[0])
        sky = _read_matrix(mtx[1], inform)
        R = dctimestep_array(dc, sky)
    fout = outform or "a"
    parts = []
    if header:                                   # util/dctimestep.c: the command, the time, the shape
        cmd = ["dctimestep"]
        if nstep:
            cmd += ["-n", str(nstep)]
        for flag, v in (("-x", xres), ("-y", yres)):
            if v:
                cmd += [flag, str(v)]
        if inform:
            cmd.append(f"-i{inform}")
        if outform:
            cmd.append(f"-o{outform}")
        cmd += [str(m) for m in mtx if not isinstance(m, bytes)]
        now = time.time()
        lines = ["#?RADIANCE", " ".join(cmd), time.strftime("CAPDATE= %Y:%m:%d %H:%M:%S", time.localtime(now)),
                 time.strftime("GMT= %Y:%m:%d %H:%M:%S", time.gmtime(now)),
                 f"NROWS={R.shape[0]}", f"NCOLS={R.shape[1]}", "NCOMP=3"]
        if fout in ("f", "d"):
            lines.append("BigEndian=0")
        lines.append("FORMAT=" + {"a": "ascii", "f": "float", "d": "double"}[fout])
        parts.append(("\n".join(lines) + "\n\n").encode())
    if fout == "a":                              # a colour's three values by spaces, colours by tabs
        if R.shape[1]:
            row = "\t".join([" ".join(["%e"] * 3)] * R.shape[1]) + "\n"
            parts.append("".join(row % tuple(r) for r in R.reshape(R.shape[0], -1).tolist()).encode())
        else:
            parts.append(b"\n" * R.shape[0])
    else:
        parts.append(_fmt_values(R.reshape(-1, 3), fout))
    return b"".join(parts)


dctimestep = _wrap(_dctimestep)

from .rflux import _rfluxmtx  # noqa: E402

rfluxmtx = _wrap(_rfluxmtx)

from .rmtx import _rmtxop, Rmtxop  # noqa: E402

rmtxop = _wrap(_rmtxop)

from .simul import (RCcontrib, RcontribSimulManager, RcOutputOp, RTdoFIFO, RTimmIrrad, RTlimDist,  # noqa: E402
                    RTmask, RtraceSimulManager, RTtraceSources, get_default_ray_params, get_ray_params, loadfunc,
                    set_ray_params)
