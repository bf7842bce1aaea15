"""Sensor values as a differentiable function of material colours.

`sensor_values(scene, rays, materials, args)` returns what `gb_rtrace`
computes for the rays (with ``-I`` the irradiance at each sensor) as a
torch tensor whose gradient with respect to the given material colours
comes from `gb_rtrace_grad`: the paths of the forward call are replayed from
the same random streams and every contribution is differentiated through
the reflectances (plastic, metal: diffuse terms) and glass transmissivities
on its path.  Sampling decisions are held fixed, so the gradient is that of
the Monte Carlo estimate at a fixed seed; give ``-u-`` or a seed so that the
forward and the replay draw the same streams.

No counterpart in pyradiance; the forward is the rtrace call of
src/pyradiance/rt.py:278-362.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib


def _opts(args) -> _lib.GbOpts:
    o, used = _lib.parse_opts(list(args), _lib.GB_PROG_RTRACE)
    if used != len(args):
        raise _lib.GbError(-1, f"command line error at '{args[used]}'")
    if o.u != 0 and not o.seed:
        raise _lib.GbError(-1, "gradients need correlated sampling (-u-) or an explicit seed")
    return o


class _SensorValues(torch.autograd.Function):
    @staticmethod
    def forward(ctx, flat, scene, slots, widths, rays, opts):
        colours = _expand(flat.detach().cpu().double().numpy(), widths)
        for sl, rgb in zip(slots, colours):
            scene.material_rgb(sl, rgb)
        n = len(rays)
        out = np.zeros((n, 3))
        _lib.check(_lib.lib().gb_rtrace(scene.handle, opts, _lib.ptr(rays), n, _lib.ptr(out), None, None))
        ctx.scene, ctx.slots, ctx.widths, ctx.rays, ctx.opts = scene, slots, widths, rays, opts
        ctx.colours = colours
        return torch.from_numpy(out).to(flat.device)

    @staticmethod
    def backward(ctx, g_out):
        scene, slots, widths, rays, opts = ctx.scene, ctx.slots, ctx.widths, ctx.rays, ctx.opts
        for sl, rgb in zip(slots, ctx.colours):          # the forward's parameters
            scene.material_rgb(sl, rgb)
        dl = np.ascontiguousarray(g_out.detach().cpu().double().numpy())
        ns = int(_lib.lib().gb_scene_material_slots(scene.handle))
        grad = np.zeros((ns, 3))
        _lib.check(_lib.lib().gb_rtrace_grad(scene.handle, opts, _lib.ptr(rays), len(rays), _lib.ptr(dl),
                                             _lib.ptr(grad), ns))
        parts = []
        for sl, w in zip(slots, widths):
            parts.append(grad[sl] if w == 3 else np.array([grad[sl].sum()]))
        flat = torch.from_numpy(np.concatenate(parts)).to(g_out.device)
        return flat, None, None, None, None, None


def _expand(flat: np.ndarray, widths) -> list:
    out, k = [], 0
    for w in widths:
        v = flat[k:k + w]
        out.append(v if w == 3 else np.repeat(v, 3))
        k += w
    return out


def sensor_values(scene, rays, materials: dict, args=("-I+", "-ab", "2", "-aa", "0", "-u-")) -> torch.Tensor:
    """gb_rtrace values of `rays` (n x 6) in `scene` (a Scene) with the
    colours of the named materials set from `materials` (name -> tensor of
    3 values, or of 1 value used for all three channels), differentiable
    with respect to those tensors."""
    names = list(materials)
    slots = [scene.material_slot(nm) for nm in names]
    tens = [torch.as_tensor(materials[nm], dtype=torch.float64).reshape(-1) for nm in names]
    widths = [int(t.numel()) for t in tens]
    if any(w not in (1, 3) for w in widths):
        raise ValueError("each material colour has 1 or 3 values")
    flat = torch.cat(tens)
    rays = np.ascontiguousarray(rays, dtype=np.float64)
    return _SensorValues.apply(flat, scene, slots, widths, rays, _opts(args))
