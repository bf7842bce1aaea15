"""rmtxop's single-matrix operations with pyradiance's signature.

``pyradiance.rmtxop(inp, outform, transpose, scale, transform, reflectance)``
(src/pyradiance/util.py:873-910) runs util/rmtxop.c on one matrix: an
optional component transform (``-c``, with the scale folded into it), else a
scale (``-s``), then a transpose (``-t``), in the order of rmtxop.c:288-381
(loadop).  These are element-wise passes over a matrix in host memory; the
products of the daylight chain run on the GPU through ``dctimestep``.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from ._lib import GbError


def read_rmatrix(src) -> np.ndarray:
    """A Radiance matrix (file path or bytes) as a (rows, cols, components)
    float64 array (util/rmatrix.c header keys NROWS, NCOLS, NCOMP, FORMAT)."""
    data = Path(src).read_bytes() if not isinstance(src, bytes) else src
    nrows = ncols = 0
    ncomp = 3
    fmt, big, body = "a", False, data
    if data.startswith(b"#?"):
        end = data.find(b"\n\n")
        head, body = data[:end], data[end + 2:]
        for ln in head.split(b"\n"):
            s = ln.decode(errors="replace").strip()
            if s.startswith("NROWS="):
                nrows = int(s[6:])
            elif s.startswith("NCOLS="):
                ncols = int(s[6:])
            elif s.startswith("NCOMP="):
                ncomp = int(s[6:])
            elif s.startswith("FORMAT="):
                fmt = {"ascii": "a", "float": "f", "double": "d"}.get(s[7:].strip(), s[7:].strip())
            elif s.startswith("BigEndian="):
                big = s[10:] == "1"
    if fmt == "a":
        vals = np.array(body.split(), dtype=np.float64)
    elif fmt == "f":
        vals = np.frombuffer(body, dtype=">f4" if big else "<f4").astype(np.float64)
    elif fmt == "d":
        vals = np.frombuffer(body, dtype=">f8" if big else "<f8").astype(np.float64)
    else:
        raise GbError(-3, f"matrix format '{fmt}' is not supported")
    if nrows <= 0 or ncols <= 0:
        raise GbError(-1, "missing matrix dimensions")
    if len(vals) < nrows * ncols * ncomp:
        raise GbError(-1, "truncated matrix")
    return vals[: nrows * ncols * ncomp].reshape(nrows, ncols, ncomp).copy()


def write_rmatrix(m: np.ndarray, fmt: str, cmd: str) -> bytes:
    """Header and data of a matrix as rmtxop writes it."""
    lines = ["#?RADIANCE", cmd, f"NROWS={m.shape[0]}", f"NCOLS={m.shape[1]}", f"NCOMP={m.shape[2]}"]
    if fmt in ("f", "d"):
        lines.append("BigEndian=0")
    lines.append("FORMAT=" + {"a": "ascii", "f": "float", "d": "double"}[fmt])
    head = ("\n".join(lines) + "\n\n").encode()
    if fmt == "a":
        rows = ["\t".join(" ".join(f"{v:.7e}" for v in px) for px in row) for row in m]
        return head + ("\n".join(rows) + "\n").encode()
    return head + np.ascontiguousarray(m, dtype="<f4" if fmt == "f" else "<f8").tobytes()


def rmtxop_array(m: np.ndarray, transpose: bool = False, scale=None, transform=None) -> np.ndarray:
    """The operations on a (rows, cols, components) array; the matrix is held
    in single precision between operations, as util/rmatrix.c holds it."""
    f32 = lambda a: a.astype(np.float32).astype(np.float64)   # noqa: E731
    m = f32(m)
    n = m.shape[2]
    sca = None if scale is None else np.atleast_1d(np.asarray(scale, dtype=np.float64))
    if transform is not None:
        if isinstance(transform, str):
            raise GbError(-3, "symbolic component transforms are not supported")
        cm = np.asarray(transform, dtype=np.float64).ravel()
        if cm.size == 0 or cm.size % n:
            raise GbError(-1, f"-c must have N x {n} coefficients")
        cm = cm.reshape(-1, n)
        if sca is not None:                         # scale folded into the transform
            if sca.size == 1:
                cm = cm * sca[0]
            elif sca.size == cm.shape[0]:
                cm = cm * sca[:, None]
            else:
                raise GbError(-1, f"-s must have one or {cm.shape[0]} factors")
            sca = None
        m = f32(m @ cm.T)
    if sca is not None:
        if sca.size == 1:
            sca = np.repeat(sca, m.shape[2])
        elif sca.size != m.shape[2]:
            raise GbError(-1, f"-s must have one or {m.shape[2]} factors")
        m = f32(m * sca)
    if transpose:
        m = np.ascontiguousarray(m.transpose(1, 0, 2))
    return m


def _rmtxop(inp, outform: str = "a", transpose: bool = False, scale: float | None = None, transform=None,
            reflectance: str | None = None) -> bytes:
    """rmtxop on one matrix (same arguments as pyradiance.rmtxop)."""
    if reflectance is not None:
        raise GbError(-3, "BSDF reflectance matrices (-rf / -rb) are not supported")
    if outform not in ("a", "f", "d"):
        raise GbError(-3, f"output format '{outform}' is not supported")
    m = rmtxop_array(read_rmatrix(inp), transpose, scale, transform)
    return write_rmatrix(m, outform, "rmtxop")
