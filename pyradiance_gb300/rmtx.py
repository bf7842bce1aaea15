"""rmtxop with pyradiance's signatures.

``pyradiance.rmtxop(inp, outform, transpose, scale, transform, reflectance)``
(src/pyradiance/util.py:873-910) runs util/rmtxop.c on one matrix: an
optional component transform (``-c``, with the scale folded into it), else a
scale (``-s``), then a transpose (``-t``), in the order of rmtxop.c:288-381
(loadop).  ``pyradiance.Rmtxop`` (util.py:912-965) chains several matrices,
each with those operations, by matrix products and element-wise sums,
products and quotients (rmtxop.c:383-520 binaryop, op_left2right,
op_right2left).  The element-wise passes run over matrices in host memory,
held in single precision as util/rmatrix.c holds them; the matrix products
run on the GPU (the FP64 dctimestep kernel: double sums of single-precision
products, rounded to single precision, as rmx_multiply computes them).
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


def _product(a: np.ndarray, b: np.ndarray, name: str) -> np.ndarray:
    """rmx_multiply (util/rmatrix.c:806-838) on the GPU."""
    from . import dctimestep_array
    if a.shape[2] != b.shape[2]:
        raise GbError(-1, f"{name}: # components do not match")
    if a.shape[1] != b.shape[0]:
        raise GbError(-1, f"{name}: mismatched dimensions")
    n = a.shape[2]
    if n not in (1, 3):
        raise GbError(-3, f"{name}: products of {n}-component matrices are not supported")
    if n == 1:
        a, b = np.repeat(a, 3, axis=2), np.repeat(b, 3, axis=2)
    r = dctimestep_array(a, b, mode="fp64").astype(np.float64)
    return r[..., :1] if n == 1 else r


def _elementwise(a: np.ndarray, op: str, b: np.ndarray, name: str) -> np.ndarray:
    """rmx_sum and rmx_elemult (util/rmatrix.c:840-925) in single precision;
    a quotient by zero gives zero, as there."""
    if a.shape[:2] != b.shape[:2]:
        raise GbError(-1, f"{name}: mismatched dimensions")
    a32, b32 = a.astype(np.float32), b.astype(np.float32)
    if op == "+":
        if a.shape[2] != b.shape[2]:
            raise GbError(-1, f"{name}: matrix sum failed")
        return (a32 + b32).astype(np.float64)
    if b.shape[2] > 1 and b.shape[2] != a.shape[2]:
        raise GbError(-1, f"{name}: element-wise {'division' if op == '/' else 'multiplication'} failed")
    if op == "*":
        return (a32 * b32).astype(np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        if b.shape[2] == 1:                        # d = 1/d in double, stored as a float
            d = b[..., 0]
            inv = np.where(d == 0, 0.0, 1.0 / np.where(d == 0, 1.0, d)).astype(np.float32)
            r = a32 * inv[..., None]
            r[d == 0] = 0
        else:
            r = np.where(b32 == 0, np.float32(0), a32 / np.where(b32 == 0, np.float32(1), b32))
    return r.astype(np.float64)


class Rmtxop:
    """pyradiance.Rmtxop (src/pyradiance/util.py:912-965): matrices added
    with ``add_input`` (each with its own scale, component transform and
    transpose), joined by ``op`` to the one before: "." matrix product, "+"
    sum, "*" and "/" element-wise product and quotient; evaluated left to
    right, or, for a chain of products only whose rightmost matrix is
    narrower than the leftmost is tall, right to left (rmtxop.c:501-525
    prefer_right2left).  Calling the object returns the result in the
    output format ("a", "f" or "d") as rmtxop writes it."""

    def __init__(self, outform: str = "a", color: str | None = None):
        if color is not None:
            raise GbError(-3, "symbolic colour transforms (-C) are not supported")
        if outform not in ("a", "f", "d"):
            raise GbError(-3, f"output format '{outform}' is not supported")
        self.outform = outform
        self.parts = []
        self._stdin = False

    def add_input(self, input_data, op: str = ".", scale=None, transform=None, transpose: bool = False,
                  refl_side: str | None = None, color: str | None = None):
        if refl_side is not None:
            raise GbError(-3, "BSDF reflectance matrices (-rf / -rb) are not supported")
        if color is not None:
            raise GbError(-3, "symbolic colour transforms (-C) are not supported")
        if self.parts and op not in (".", "+", "*", "/"):
            raise GbError(-1, f"unknown operation '{op}'")
        if isinstance(input_data, bytes):
            if self._stdin:
                raise ValueError("stdin is already taken")
            self._stdin = True
        self.parts.append((input_data, op if self.parts else None, scale, transform, transpose))
        return self

    def _load(self, i: int) -> np.ndarray:
        src, _, scale, transform, transpose = self.parts[i]
        return rmtxop_array(read_rmatrix(src), transpose, scale, transform)

    def result(self) -> np.ndarray:
        """The combined matrix, (rows, cols, components) float64 holding
        single-precision values."""
        if not self.parts:
            raise GbError(-1, "no matrix to operate on")
        ops = [p[1] for p in self.parts[1:]]
        name = lambda i: str(self.parts[i][0])[:60] if not isinstance(self.parts[i][0], bytes) else "-"  # noqa: E731
        mats = [self._load(i) for i in range(len(self.parts))]
        if len(mats) > 2 and all(o == "." for o in ops):
            right, left = mats[-1], mats[0]
            r2l = right.shape[1] == 1 or (right.shape[1] < right.shape[0] and right.shape[1] < left.shape[0])
            if r2l:
                res = mats[-1]
                for i in range(len(mats) - 2, -1, -1):
                    res = _product(mats[i], res, name(i + 1))
                return res
        res = mats[0]
        for i, op in enumerate(ops, start=1):
            res = _product(res, mats[i], name(i)) if op == "." else _elementwise(res, op, mats[i], name(i))
        return res

    def __call__(self) -> bytes:
        return write_rmatrix(self.result(), self.outform, "rmtxop")
