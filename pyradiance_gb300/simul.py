"""In-process simulation managers with pyradiance's binding API.

pyradiance exposes Radiance's ``RtraceSimulManager`` and
``RcontribSimulManager`` through nanobind (src/binding/radiance_ext.cpp:
170-458) with global ray parameters (``get_ray_params`` /
``set_ray_params``, src/binding/params.cpp:182-345).  The classes here keep
those names, methods and flag values, and run each flushed bundle as one GPU
call (``gb_rtrace`` / ``gb_rcontrib``): the rays are traced as a wavefront
on the device, and the per-ray callbacks are made afterwards on the host, in
ray order (``RTdoFIFO`` is always honoured).

Differences that follow from the device running the rays: the trace callback
sees the bundle's primary rays only (their children never leave the
device), and a ray record carries its origin, direction, value, distance,
hit point, hit object and ray number; surface normals and material
colours are not returned.
"""
from __future__ import annotations

import copy
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import GbError, check, lib, parse_opts, ptr

# rt/RtraceSimulManager.h:86
RTdoFIFO, RTtraceSources, RTlimDist, RTimmIrrad, RTmask = 1, 2, 4, 8, 15
RCcontrib = RTmask + 1
PRIMARY = 1                                     # rt/ray.h ray type


@dataclass
class RayParams:
    """The ray parameters of src/binding/params.cpp:182-330 (rtrace's
    defaults, rt/raycalls.c:121-150)."""
    i: bool = False
    u: bool = True
    dj: float = 0.0
    dt: float = 0.03
    dc: float = 0.75
    dr: int = 2
    dp: int = 512
    dv: bool = True
    ds: float = 0.2
    mg: float = 0.0
    ms: float = 0.0
    st: float = 0.15
    ss: float = 1.0
    bv: bool = True
    lr: int = -10
    lw: float = 1e-4
    aw: int = 0
    aa: float = 0.1
    ar: int = 256
    ad: int = 1024
    as_: int = 512
    ab: int = 0
    av: list = field(default_factory=lambda: [0.0, 0.0, 0.0])

    def args(self) -> list[str]:
        """The parameters as rtrace options."""
        b = lambda v: "+" if v else "-"            # noqa: E731
        return [f"-i{b(self.i)}", f"-u{b(self.u)}", "-dj", str(self.dj), "-dt", str(self.dt), "-dc", str(self.dc),
                "-dr", str(self.dr), "-dp", str(self.dp), f"-dv{b(self.dv)}", "-ds", str(self.ds),
                "-st", str(self.st), "-ss", str(self.ss), f"-bv{b(self.bv)}", "-lr", str(self.lr),
                "-lw", str(self.lw), "-aa", str(self.aa), "-ar", str(self.ar), "-ad", str(self.ad),
                "-as", str(self.as_), "-ab", str(self.ab), "-av", *map(str, self.av)]


_PARAMS = RayParams()


_CALFILE: str | None = None


def loadfunc(calfile: str) -> None:
    """Function file for the modifiers' bin expressions (pyradiance's
    ``loadfunc``: the function context the managers' bins are compiled in)."""
    global _CALFILE
    _CALFILE = str(calfile)


def get_default_ray_params() -> RayParams:
    return RayParams()


def get_ray_params() -> RayParams:
    return copy.deepcopy(_PARAMS)


def set_ray_params(rp: RayParams | None = None) -> None:
    global _PARAMS
    _PARAMS = copy.deepcopy(rp) if rp is not None else RayParams()


@dataclass
class Ray:
    """What a callback receives for one ray (the fields of RAY bound in
    src/binding/radiance_ext.cpp:90-125 that the GPU returns)."""
    rorg: tuple
    rdir: tuple
    rmax: float
    rweight: float
    rno: int
    rtype: int
    rcol: tuple
    rot: float
    rop: tuple
    ro: int


def _bundle(orig_direc) -> np.ndarray:
    a = np.ascontiguousarray(orig_direc, dtype=np.float64)
    if a.ndim != 2 or a.shape[1] != 3 or a.shape[0] % 2:
        raise ValueError("orig_direc must be an array of origin, direction rows (2n x 3)")
    return a.reshape(-1, 6)


class RtraceSimulManager:
    """Radiance's RtraceSimulManager (rt/RtraceSimulManager.h) on the GPU."""

    def __init__(self):
        self.rt_flags = 0
        self._scene = None
        self._queue: list[tuple[np.ndarray, int]] = []
        self._cooked = None
        self._trace = None

    def load_octree(self, octn) -> int:
        from . import load_scene
        self._scene = load_scene(octn)
        return self._scene.nobjects()

    def set_thread_count(self, nt: int = 0) -> int:
        return 1                                # one device, one stream

    def ready(self) -> bool:
        return self._scene is not None

    def set_cooked_call(self, callback) -> None:
        self._cooked = callback

    def set_trace_call(self, callback) -> None:
        self._trace = callback

    def cleanup_callbacks(self) -> None:
        self._cooked = self._trace = None

    def enqueue_bundle(self, orig_direc, rID0: int = 0) -> int:
        """Queue rays (origin, direction row pairs); they are traced at the
        next flush.  Returns the number queued."""
        if not self.ready():
            raise RuntimeError("octree not loaded")
        r = _bundle(orig_direc)
        self._queue.append((r, int(rID0)))
        return len(r)

    def flush_queue(self) -> int:
        """Trace every queued ray as one device call and make the callbacks."""
        if not self._queue:
            return 0
        rays = np.concatenate([r for r, _ in self._queue])
        rno = np.concatenate([np.arange(len(r)) + (r0 if r0 else 1) for r, r0 in self._queue])
        self._queue = []
        args = _PARAMS.args()
        if self.rt_flags & RTimmIrrad:
            args.append("-I+")
        opts, used = parse_opts(args, _lib.GB_PROG_RTRACE)
        if used != len(args):
            raise GbError(-1, f"ray parameter error at '{args[used]}'")
        n = len(rays)
        vals = np.zeros((n, 3))
        hit = np.full(n, -1, dtype=np.int32)
        hitt = np.zeros(n)
        dlen = np.linalg.norm(rays[:, 3:6], axis=1)
        good = dlen > 0
        rr = np.ascontiguousarray(rays[good])
        if len(rr):
            gv, gh, gt = np.zeros((len(rr), 3)), np.zeros(len(rr), dtype=np.int32), np.zeros(len(rr))
            check(lib().gb_rtrace(self._scene.handle, opts, ptr(rr), len(rr), ptr(gv), ptr(gh), ptr(gt)))
            vals[good], hit[good], hitt[good] = gv, gh, gt
        unit = rays[:, 3:6] / np.where(dlen > 0, dlen, 1)[:, None]
        for i in range(n):
            hp = rays[i, :3] + unit[i] * hitt[i] if hit[i] >= 0 else np.zeros(3)
            ray = Ray(tuple(rays[i, :3]), tuple(unit[i]), 0.0, 1.0, int(rno[i]), PRIMARY, tuple(vals[i]),
                      float(hitt[i]) if hit[i] >= 0 else 1e10, tuple(hp), int(hit[i]))
            if self._trace is not None:
                self._trace(ray, None)
            if self._cooked is not None:
                self._cooked(ray, None)
        return n

    def cleanup(self, everything: bool = False) -> None:
        self._queue = []
        if everything:
            self._scene = None
            self.cleanup_callbacks()


class RcOutputOp:
    """Output file modes (rt/RcontribSimulManager.h RCOutputOp)."""
    NEW, FORCE, RECOVER = 0, 1, 2


class RcontribSimulManager:
    """Radiance's RcontribSimulManager (rt/RcontribSimulManager.h) on the
    GPU: modifiers with bin expressions, rays in bundles, results kept as an
    array and written to the modifiers' output files."""

    def __init__(self, octn=None):
        self.xres = 0
        self.yres = 0
        self.accum = 1
        self.out_op = RcOutputOp.NEW
        self._flags = 0
        self._scene = None
        if octn:
            self.load_octree(octn)
        self._mods: list[dict] = []
        self._rows: list[np.ndarray] = []
        self._prepped = False

    # flags and scene
    def has_flag(self, fl: int) -> bool:
        return bool(self._flags & fl)

    def set_flag(self, fl: int, val: bool = True) -> bool:
        self._flags = (self._flags | fl) if val else (self._flags & ~fl)
        return True

    def load_octree(self, octn) -> bool:
        from . import load_scene
        self._scene = load_scene(octn)
        return True

    def set_thread_count(self, nt: int = 0) -> int:
        return 1

    def n_threads(self) -> int:
        return 1

    def ready(self) -> bool:
        return self._scene is not None and bool(self._mods)

    # modifiers
    def add_modifier(self, modn: str, outspec: str | None = None, prms: str = "", binval: str = "",
                     bincnt: int = 1) -> bool:
        self._mods.append(dict(modifier=modn, output=outspec, params=prms or None, binv=binval or None,
                               nbins=str(int(bincnt)), calfile=None, expr=None))
        return True

    def add_mod_file(self, modfn: str, outspec: str | None = None, prms: str | None = None,
                     binval: str | None = None, bincnt: int = 1) -> bool:
        for nm in Path(modfn).read_text().split():
            self.add_modifier(nm, outspec, prms or "", binval or "", bincnt)
        return True

    def clear_modifiers(self) -> None:
        self._mods = []

    def prep_output(self) -> int:
        """Check the modifiers (their bin programs compile) and return the
        record length in values."""
        if self._scene is None:
            raise RuntimeError("octree not loaded")
        self._prepped = True
        return 3 * sum(self._nbins())

    def _specs(self):
        arr = (_lib.GbModspec * len(self._mods))()
        keep = []
        cal = _CALFILE
        for i, m in enumerate(self._mods):
            v = {k: (str(m[k]).encode() if m.get(k) is not None else None)
                 for k in ("modifier", "binv", "nbins", "params", "calfile", "expr")}
            if v["calfile"] is None and cal:
                v["calfile"] = str(cal).encode()
            keep.append(v)
            arr[i] = _lib.GbModspec(v["modifier"], v["binv"], v["nbins"], v["params"], v["calfile"], v["expr"])
        return arr, keep

    def _nbins(self) -> list[int]:
        from .rflux import _nbins_each
        cal = _CALFILE
        return _nbins_each([{**m, "calfile": m.get("calfile") or cal} for m in self._mods])

    def get_row_max(self) -> int:
        return self.yres * max(self.xres, 1) if self.yres > 0 else 0

    def get_row_count(self) -> int:
        return sum(len(r) for r in self._rows)

    def get_row_finished(self) -> int:
        return self.get_row_count()

    def rcontrib(self, rays) -> int:
        """Trace a bundle (origin, direction row pairs; accum rays a record)
        and append its records.  Returns the number of records."""
        if not self._prepped:
            self.prep_output()
        r = _bundle(rays)
        args = _PARAMS.args() + ["-c", str(max(1, int(self.accum)))]
        if self._flags & RTimmIrrad:
            args.append("-I+")
        opts, used = parse_opts(args, _lib.GB_PROG_RCONTRIB)
        if used != len(args):
            raise GbError(-1, f"ray parameter error at '{args[used]}'")
        specs, keep = self._specs()
        nb = sum(self._nbins())
        out = np.zeros((len(r) // max(1, opts.c), nb, 3))
        if len(r):
            cnt = _lib.C.c_int64(0)
            check(lib().gb_rcontrib(self._scene.handle, opts, specs, len(self._mods), ptr(r), len(r), ptr(out),
                                    _lib.C.byref(cnt)))
        self._rows.append(out)
        return len(out)

    def flush_queue(self) -> int:
        return 0                                # bundles are traced as they come

    def reset_row(self, r: int = 0) -> bool:
        self._rows = []
        return True

    def get_output_array(self) -> np.ndarray:
        """All records so far as (records, total bins x 3)."""
        if not self._rows:
            return np.zeros((0, 3 * sum(self._nbins())))
        a = np.concatenate(self._rows)
        return a.reshape(len(a), -1)

    def _write_outputs(self) -> None:
        from . import _fmt_values, _header
        if not self._rows or not any(m["output"] for m in self._mods):
            return
        a = np.concatenate(self._rows)
        files: dict[str, list[np.ndarray]] = {}
        col = 0
        for m, nb in zip(self._mods, self._nbins()):
            spec = m["output"]
            if spec:
                if "%d" in spec:
                    raise GbError(-3, f"per-bin output files ({spec}) are not supported")
                name = spec.replace("%s", m["modifier"]) if "%s" in spec else spec
                files.setdefault(name, []).append(a[:, col:col + nb])
            col += nb
        for name, cols in files.items():
            if Path(name).exists() and self.out_op == RcOutputOp.NEW:
                raise GbError(-1, f"output file '{name}' exists (use RcOutputOp.FORCE)")
            arr = np.concatenate(cols, axis=1)
            extra = [f"NROWS={len(arr)}", f"NCOLS={arr.shape[1]}"]
            Path(name).write_bytes(_header("rcontrib", [], None, "f", 3, extra) +
                                   _fmt_values(arr.reshape(-1, 3), "f"))

    def cleanup(self, everything: bool = False) -> None:
        self._write_outputs()
        self._rows = []
        self._prepped = False
        if everything:
            self._mods = []
            self._scene = None

    def __enter__(self):
        return self

    def __exit__(self, type=None, value=None, traceback=None):
        self.cleanup(True)
        return False
