"""ctypes front end of the CPU oracle (liboracle.so, built from radoracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg as the checker or the timed baseline, never by
the library.  Options use the same struct as the library's C ABI
(include/gbrad.h gb_opts); defaults per program are restated here from
rt/raycalls.c:121-150 (rtrace) and rt/rcontrib.c:24-58 (rcontrib).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"


class Opts(C.Structure):
    _fields_ = [
        ("prog", C.c_int), ("ab", C.c_int), ("ad", C.c_int), ("as_", C.c_int), ("ar", C.c_int),
        ("aw", C.c_int), ("aa", C.c_double), ("av", C.c_double * 3), ("lr", C.c_int),
        ("lw", C.c_double), ("dj", C.c_double), ("ds", C.c_double), ("dt", C.c_double),
        ("dc", C.c_double), ("dr", C.c_int), ("dp", C.c_int), ("dv", C.c_int),
        ("st", C.c_double), ("ss", C.c_double), ("bv", C.c_int), ("I", C.c_int), ("i", C.c_int),
        ("u", C.c_int), ("h", C.c_int), ("n", C.c_int), ("c", C.c_int), ("V", C.c_int),
        ("fin", C.c_char), ("fout", C.c_char), ("outspec", C.c_char * 32), ("x", C.c_int),
        ("y", C.c_int), ("ld", C.c_double), ("seed", C.c_uint64), ("replica", C.c_uint32),
    ]


class Modspec(C.Structure):
    _fields_ = [("modifier", C.c_char_p), ("binv", C.c_char_p), ("nbins", C.c_char_p),
                ("params", C.c_char_p), ("calfile", C.c_char_p), ("expr", C.c_char_p)]


def build() -> Path:
    """Compile liboracle.so with its Makefile (gcc/g++, OpenMP)."""
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        L.orc_scene_open.restype = C.c_void_p
        L.orc_scene_open.argtypes = [C.c_char_p, C.c_int]
        L.orc_scene_close.argtypes = [C.c_void_p]
        L.orc_scene_nobjects.restype = C.c_int64
        L.orc_scene_nobjects.argtypes = [C.c_void_p]
        L.orc_scene_object_name.restype = C.c_char_p
        L.orc_scene_object_name.argtypes = [C.c_void_p, C.c_int64]
        L.orc_last_error.restype = C.c_char_p
        L.orc_rtrace.argtypes = [C.c_void_p, C.POINTER(Opts), C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_int, C.POINTER(C.c_int64)]
        L.orc_rcontrib.argtypes = [C.c_void_p, C.POINTER(Opts), C.POINTER(Modspec), C.c_int, C.c_void_p,
                                   C.c_int64, C.c_void_p, C.c_int, C.POINTER(C.c_int64)]
        L.orc_nbins.argtypes = [C.POINTER(Modspec), C.c_int, C.c_char_p, C.c_int]
        L.orc_dctimestep.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_void_p,
                                     C.c_int]
        _lib = L
    return _lib


def default_opts(prog: str, **kw) -> Opts:
    o = Opts()
    o.prog = 1 if prog == "rcontrib" else 0
    o.fin = o.fout = b"a"
    o.h, o.n, o.u, o.bv, o.dv, o.lr, o.ar, o.dc, o.dp, o.ss, o.c = 1, 1, 1, 1, 1, -10, 256, .75, 512, 1.0, 1
    o.outspec = b"v"
    if prog == "rcontrib":
        o.dj, o.ds, o.dt, o.dr, o.st, o.lw, o.ab, o.aa, o.ad, o.as_ = .9, .2, 0., 3, .02, 2e-3, 1, 0., 350, 0
    else:
        o.dj, o.ds, o.dt, o.dr, o.st, o.lw, o.ab, o.aa, o.ad, o.as_ = 0., .2, .03, 2, .15, 1e-4, 0, .1, 1024, 512
    for k, v in kw.items():
        setattr(o, "as_" if k == "as" else k, v)
    return o


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Scene:
    def __init__(self, path, rad: bool | None = None):
        path = str(path)
        is_rad = path.endswith(".rad") if rad is None else rad
        self.h = lib().orc_scene_open(path.encode(), int(is_rad))
        if not self.h:
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())

    def nobjects(self) -> int:
        return lib().orc_scene_nobjects(self.h)

    def object_name(self, i: int) -> str:
        return lib().orc_scene_object_name(self.h, i).decode()

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_scene_close(self.h)
            self.h = None


def rtrace(scene: Scene, opts: Opts, rays: np.ndarray, values: bool = True, hits: bool = True,
           threads: int = 1):
    rays = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 6)
    n = len(rays)
    rgb = np.zeros((n, 3)) if values else None
    hid = np.zeros(n, dtype=np.int32) if hits else None
    ht = np.zeros(n) if hits else None
    cnt = C.c_int64(0)
    rc = lib().orc_rtrace(scene.h, C.byref(opts), _p(rays), n, _p(rgb), _p(hid), _p(ht), threads, C.byref(cnt))
    if rc != 0:
        raise RuntimeError("oracle: " + lib().orc_last_error().decode())
    return rgb, hid, ht, cnt.value


def rcontrib(scene: Scene, opts: Opts, mods: list[dict], rays: np.ndarray, threads: int = 1):
    """Returns (records, total bins, 3) float64 and the number of rays traced."""
    rays = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 6)
    arr = (Modspec * len(mods))()
    keep = []
    for i, m in enumerate(mods):
        vals = {k: (str(m[k]).encode() if m.get(k) is not None else None)
                for k in ("modifier", "binv", "nbins", "params", "calfile", "expr")}
        keep.append(vals)
        arr[i] = Modspec(vals["modifier"], vals["binv"], vals["nbins"], vals["params"], vals["calfile"],
                         vals["expr"])
    err = C.create_string_buffer(512)
    nbt = lib().orc_nbins(arr, len(mods), err, 512)
    if nbt < 0:
        raise RuntimeError("oracle: " + err.value.decode())
    accum = max(1, opts.c)
    out = np.zeros((len(rays) // accum, nbt, 3))
    cnt = C.c_int64(0)
    rc = lib().orc_rcontrib(scene.h, C.byref(opts), arr, len(mods), _p(rays), len(rays), _p(out), threads,
                            C.byref(cnt))
    if rc != 0:
        raise RuntimeError("oracle: " + lib().orc_last_error().decode())
    return out, cnt.value


def dctimestep(dc: np.ndarray, sky: np.ndarray, threads: int = 1) -> np.ndarray:
    dc = np.ascontiguousarray(dc, dtype=np.float32)
    sky = np.ascontiguousarray(sky, dtype=np.float32)
    M, K, _ = dc.shape
    N = sky.shape[1]
    out = np.zeros((M, N, 3), dtype=np.float32)
    lib().orc_dctimestep(_p(dc), _p(sky), M, K, N, _p(out), threads)
    return out


def octree_digest(path, rad: bool | None = None, objlim: int = 6, resolu: int = 16384):
    """(nodes, sets, hash) of an octree file or of the octree built from scene
    text (oconv's -n objlim and -r resolution)."""
    path = str(path)
    is_rad = path.endswith(".rad") if rad is None else rad
    L = lib()
    L.orc_octree_digest.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_uint64)]
    out = (C.c_uint64 * 3)()
    if L.orc_octree_digest(path.encode(), int(is_rad), objlim, resolu, out) != 0:
        raise RuntimeError("oracle: " + L.orc_last_error().decode())
    return [int(out[0]), int(out[1]), int(out[2])]
