"""ctypes binding of libgbrad.so (the C ABI declared in include/gbrad.h).

The library is loaded from this package directory; if it is missing it is
built first (nvcc is required).  There is no fallback: every entry point
runs on the GPU or raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIBPATH = _HERE / "libgbrad.so"
_lock = threading.Lock()
_lib = None

GB_PROG_RTRACE = 0
GB_PROG_RCONTRIB = 1
GB_DCT_FP32 = 0
GB_DCT_BF16X3 = 1
GB_DCT_FP64 = 2
GB_DCT_FP16X3 = 3
GB_DCT_FP16 = 4

ERRORS = {-1: "EINVAL", -2: "EIO", -3: "EUNSUPPORTED", -4: "ECUDA", -5: "ENOMEM", -6: "EOVERFLOW"}


class GbOpts(C.Structure):
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


class GbModspec(C.Structure):
    _fields_ = [("modifier", C.c_char_p), ("binv", C.c_char_p), ("nbins", C.c_char_p),
                ("params", C.c_char_p), ("calfile", C.c_char_p), ("expr", C.c_char_p)]


class GbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_SIGS = {
    "gb_scene_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "gb_scene_load_rad": (C.c_int, [C.POINTER(C.c_char_p), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "gb_scene_free": (None, [C.c_void_p]),
    "gb_probe_l2": (C.c_int, [C.c_int64, C.c_int, C.POINTER(C.c_double)]),
    "gb_format_rows": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_char_p, C.c_char_p, C.c_void_p, C.c_int64,
                                 C.POINTER(C.c_int64)]),
    "gb_scene_octree_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_uint64), C.POINTER(C.c_int)]),
    "gb_scene_nobjects": (C.c_int64, [C.c_void_p]),
    "gb_scene_object_name": (C.c_char_p, [C.c_void_p, C.c_int64]),
    "gb_scene_modifier_name": (C.c_char_p, [C.c_void_p, C.c_int64]),
    "gb_scene_material_name": (C.c_char_p, [C.c_void_p, C.c_int64]),
    "gb_opts_default": (C.c_int, [C.c_int, C.POINTER(GbOpts)]),
    "gb_opts_parse": (C.c_int, [C.c_int, C.POINTER(C.c_char_p), C.c_int, C.POINTER(GbOpts), C.POINTER(C.c_int)]),
    "gb_rtrace": (C.c_int, [C.c_void_p, C.POINTER(GbOpts), C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                            C.c_void_p]),
    "gb_rtrace_hits": (C.c_int, [C.c_void_p, C.POINTER(GbOpts), C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_void_p]),
    "gb_rtrace_device_noalloc": (C.c_int, [C.c_void_p, C.POINTER(GbOpts), C.c_void_p, C.c_int64, C.c_void_p,
                                            C.c_void_p]),
    "gb_rtrace_grad": (C.c_int, [C.c_void_p, C.POINTER(GbOpts), C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                 C.c_int64]),
    "gb_scene_material_slots": (C.c_int64, [C.c_void_p]),
    "gb_scene_material_slot": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int)]),
    "gb_scene_material_rgb": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "gb_rcontrib": (C.c_int, [C.c_void_p, C.POINTER(GbOpts), C.POINTER(GbModspec), C.c_int, C.c_void_p,
                              C.c_int64, C.c_void_p, C.POINTER(C.c_int64)]),
    "gb_rcontrib_nbins": (C.c_int, [C.POINTER(GbModspec), C.c_int, C.POINTER(C.c_int)]),
    "gb_rcontrib_batch": (C.c_int, [C.c_int, C.POINTER(C.c_void_p), C.POINTER(GbOpts), C.POINTER(GbModspec), C.c_int,
                                    C.POINTER(C.c_void_p), C.POINTER(C.c_int64), C.POINTER(C.c_void_p),
                                    C.POINTER(C.c_int64)]),
    "gb_dctimestep": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int, C.c_void_p]),
    "gb_dctimestep_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int,
                                       C.c_void_p, C.c_void_p]),
    "gb_last_stats": (C.c_int, [C.POINTER(C.c_int64)] * 4),
    "gb_last_profile": (C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                  C.c_int, C.POINTER(C.c_double)]),
    "gb_last_error": (C.c_char_p, []),
    "gb_version": (C.c_char_p, []),
}


def lib():
    """The loaded library (built on first use when absent)."""
    global _lib
    with _lock:
        if _lib is None:
            if not _LIBPATH.exists():
                from .build import build
                build()
            L = C.CDLL(str(_LIBPATH))
            for name, (res, args) in _SIGS.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != 0:
        raise GbError(rc, lib().gb_last_error().decode(errors="replace"))


def last_stats() -> dict:
    v = [C.c_int64() for _ in range(4)]
    lib().gb_last_stats(*[C.byref(x) for x in v])
    return {"rays": v[0].value, "steps": v[1].value, "contribs": v[2].value, "launches": v[3].value}


KERNELS = ["cast", "root", "expand", "primary", "trace", "shade"]
COUNTERS = ["rays", "steps", "contribs", "overflow", "badbin", "nodes", "tests", "spare"]


def last_profile() -> dict:
    """Per-kernel device time (ms), launches and counters of the last call."""
    out = {}
    region = C.c_double(0)
    for k, name in enumerate(KERNELS):
        ms = C.c_double(0)
        nl = C.c_int64(0)
        cnt = (C.c_int64 * 8)()
        lib().gb_last_profile(k, C.byref(ms), C.byref(nl), cnt, 8, C.byref(region))
        if nl.value:
            out[name] = {"ms": ms.value, "launches": nl.value, **{c: int(cnt[i]) for i, c in enumerate(COUNTERS)}}
    out["region_ms"] = region.value
    return out


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def parse_opts(args, prog: int) -> tuple[GbOpts, int]:
    o = GbOpts()
    check(lib().gb_opts_default(prog, C.byref(o)))
    enc = [str(a).encode() for a in args]
    arr = (C.c_char_p * max(1, len(enc)))(*enc)
    used = C.c_int(0)
    check(lib().gb_opts_parse(len(enc), arr, prog, C.byref(o), C.byref(used)))
    return o, used.value


class Scene:
    """A scene on the GPU: a Radiance octree, or scene files built into one."""

    def __init__(self, path=None, rad_files=None, objlim: int = 0, resolu: int = 0):
        self._h = C.c_void_p()
        L = lib()
        if rad_files is not None:
            files = [str(f).encode() for f in rad_files]
            arr = (C.c_char_p * len(files))(*files)
            check(L.gb_scene_load_rad(arr, len(files), objlim, resolu, C.byref(self._h)))
        else:
            check(L.gb_scene_load(str(path).encode(), C.byref(self._h)))

    @property
    def handle(self):
        return self._h

    def nobjects(self) -> int:
        return lib().gb_scene_nobjects(self._h)

    def object_name(self, i: int) -> str:
        return lib().gb_scene_object_name(self._h, i).decode()

    def modifier_name(self, i: int) -> str:
        return lib().gb_scene_modifier_name(self._h, i).decode()

    def material_name(self, i: int) -> str:
        return lib().gb_scene_material_name(self._h, i).decode()

    def material_slot(self, name: str) -> int:
        sl = C.c_int(-1)
        check(lib().gb_scene_material_slot(self._h, name.encode(), C.byref(sl)))
        return sl.value

    def material_rgb(self, slot: int, rgb=None) -> np.ndarray:
        """The colour of a material slot; replaced by rgb when given."""
        old = np.zeros(3)
        new = None if rgb is None else np.ascontiguousarray(rgb, dtype=np.float64)
        check(lib().gb_scene_material_rgb(self._h, slot, ptr(old), ptr(new)))
        return old

    def close(self) -> None:
        if self._h:
            lib().gb_scene_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
