"""gb_rtrace_device_noalloc against gb_rtrace (needs a GB300).

The entry point traces rays that are already in device memory and carves
all of its working memory from a static device array.  It runs the same
kernels as gb_rtrace, so the values agree up to the order of FP64 atomic
additions; each case calls it twice in a row, which also checks that the
counters in the static array are reset between calls.  The rays are
written on a torch side stream that the call is given, with no host
synchronisation in between, so the test also checks that the call is
ordered after the caller's writes.  The file name sorts
last so that the cases also run after every other GPU test in one process.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(scene_dir):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import _lib
    _lib.lib()
    torch.cuda.set_device(0)
    scenes = {k: gb.Scene(rad_files=[scene_dir / f"{k}.rad"]) for k in ("c1", "c2", "zoo")}
    return torch, _lib, scenes


def opts(_lib, **kw):
    o, _ = _lib.parse_opts([], _lib.GB_PROG_RTRACE)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def host_rtrace(_lib, sc, o, rays):
    rgb = np.zeros((len(rays), 3))
    _lib.check(_lib.lib().gb_rtrace(sc.handle, o, _lib.ptr(rays), len(rays), _lib.ptr(rgb), None, None))
    return rgb


def noalloc_rtrace(torch, _lib, sc, o, rays, side=True):
    """Rays copied in and the output cleared on a torch side stream, with no
    host synchronisation before the call: the call is enqueued on that
    stream, so it must see the rays (side=False: torch's default stream)."""
    stream = torch.cuda.Stream() if side else torch.cuda.default_stream()
    with torch.cuda.stream(stream):
        h_rays = torch.from_numpy(rays).pin_memory()
        d_rays = h_rays.to("cuda", non_blocking=True)
        d_rgb = torch.full((len(rays), 3), float("nan"), dtype=torch.float64, device="cuda")
        rc = _lib.lib().gb_rtrace_device_noalloc(sc.handle, o, C.c_void_p(d_rays.data_ptr()), len(rays),
                                                 C.c_void_p(d_rgb.data_ptr()), C.c_void_p(stream.cuda_stream))
        _lib.check(rc)
        return d_rgb.cpu().numpy()


CASES = {
    # deterministic direct irradiance at 2000 sensors of the daylight room
    "c1_direct": ("c1", dict(I=1, ab=0, dj=0, ds=0, dr=0, u=0), 0.0),
    # radiance with mirror and glass chains: later generations through the queues
    "zoo_chains": ("zoo", dict(ab=0, dj=0, ds=0, dr=0, dt=0, u=0), 0.0),
    # Monte Carlo irradiance with one ambient bounce (first hemisphere queue)
    "c2_ambient": ("c2", dict(I=1, ab=1, ad=64, lw=1e-4, aa=0, as_=0, u=0, seed=31, dj=0.9, ds=0.2, st=0.02,
                              dt=0), 1e-9),
}


@pytest.mark.parametrize("case", list(CASES))
def test_noalloc_matches_rtrace_twice(env, case):
    torch, _lib, scenes = env
    scene, kw, rtol = CASES[case]
    sc = scenes[scene]
    if scene == "c1":
        rays = np.ascontiguousarray(golden("c1_direct.npz")["rays"], dtype=np.float64)
    elif scene == "zoo":
        rays = np.ascontiguousarray(golden("zoo.npz")["rays"], dtype=np.float64)
    else:
        from pyradiance_gb300 import workloads as w
        rays = np.ascontiguousarray(w.sensor_grid(32, 32), dtype=np.float64)
    o = opts(_lib, **kw)
    ref = host_rtrace(_lib, sc, o, rays)
    assert np.isfinite(ref).all() and ref.max() > 0
    for side in (True, False):
        got = noalloc_rtrace(torch, _lib, sc, o, rays, side=side)
        np.testing.assert_allclose(got, ref, rtol=rtol, atol=1e-300)


def test_noalloc_rejects_oversized_calls(env):
    """-I -ab 1 -ad 1024 gives 32 x 32 hemisphere samples per sensor; 256
    sensors then need more queue space than the static scratch holds."""
    torch, _lib, scenes = env
    from pyradiance_gb300 import workloads as w
    rays = np.ascontiguousarray(w.sensor_grid(16, 16), dtype=np.float64)
    o = opts(_lib, I=1, ab=1, ad=1024, lw=1e-4, aa=0, as_=0, u=0, seed=5)
    with pytest.raises(_lib.GbError) as e:
        noalloc_rtrace(torch, _lib, scenes["c2"], o, rays)
    assert e.value.code == -1 and "scratch" in str(e.value)
    # super-sampling (-as, rtrace's default 512) needs allocation: refused
    o.as_ = 512
    with pytest.raises(_lib.GbError) as e:
        noalloc_rtrace(torch, _lib, scenes["c2"], o, rays[:4])
    assert e.value.code == -3 and "-as" in str(e.value)
    # a host pointer is refused before any launch
    d_rgb = torch.zeros((4, 3), dtype=torch.float64, device="cuda")
    host_rays = np.ascontiguousarray(rays[:4])
    rc = _lib.lib().gb_rtrace_device_noalloc(scenes["c2"].handle, opts(_lib, ab=0), _lib.ptr(host_rays), 4,
                                             C.c_void_p(d_rgb.data_ptr()), None)
    assert rc == -1
    # more rays than the scratch can hold at any options: refused before any
    # size arithmetic
    big = torch.zeros((1 << 20, 6), dtype=torch.float64, device="cuda")
    out = torch.zeros((1 << 20, 3), dtype=torch.float64, device="cuda")
    rc = _lib.lib().gb_rtrace_device_noalloc(scenes["c2"].handle, opts(_lib, ab=1, ad=0, aa=0),
                                             C.c_void_p(big.data_ptr()),
                                             1 << 20, C.c_void_p(out.data_ptr()), None)
    assert rc == -1 and "scratch" in _lib.lib().gb_last_error().decode()
