"""Benchmark of the GPU rcontrib path (the daylight-coefficient workload).

Workload: 4,096 sensors (64 x 64 grid at z = 0.8, facing up) in the 10 x 8 x 3 m
room with a 3 x 2 m glass window and 20,000 random triangles, glow sky and
ground binned into Reinhart MF:1 (145 patches) + ground = 146 bins, run as
rcontrib -I+ -ab 3 -ad 1024 -lw 1e-4 -c 1.  A step is one full pass over the
4,096 sensors.  The metric is rays traced per second (every octree walk:
ambient, transmitted, reflected and shadow rays), in Mrays/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

value   device throughput: rays / (CUDA-event time of the kernel region on the
        library's stream), inputs and outputs resident in HBM;
e2e     the same through the C ABI with host buffers (sensor upload and
        bin download inside the timed region), wall clock per call;
e2e_bytes  the same through the pyradiance byte surface, Rcontrib(...)():
        rays parsed from bytes, output formatted to bytes (ASCII, and
        double in / float out);
L2 is flushed (256 MB write) before every timed step.  Multi-GPU runs shard
independent sensor replicas across ranks (weak scaling, no data collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "rcontrib Mrays/s (1 GB300)"
PARAMS = ["-I+", "-ab", "3", "-ad", "1024", "-lw", "1e-4", "-c", "1", "-u-"]
MODS = [dict(modifier="groundglow"),
        dict(modifier="skyglow", calfile="reinhartb.cal", param="MF=1", binv="rbin", nbins="Nrbins")]
WORKLOAD = ("rcontrib daylight coefficients: 4096 sensors (64x64 grid, z=0.8, +z), -I+ -ab 3 -ad 1024 "
            "-lw 1e-4 -c 1; room 10x8x3 m + 2x3 m glass window (transmissivity 0.6) + 20,000 random "
            "triangles; glow sky + ground, Reinhart MF:1 + ground = 146 bins")
# algorithmic bytes per unit of traversal work: one child code per node descent,
# set offset + count per cube visit, object record + vertices per test
# the config of both arms' lines (the two must name the same workload)
CONFIG = {"workload": None, "sensors_per_gpu": 4096,
          "l2": "GPU arm: L2 flushed (256 MB write) before each step; CPU arm: no cache control"}
B_NODE, B_STEP, B_TEST = 4, 8, 60
B_RAYIO = 48 + 32          # the walk kernel reads origin, direction, origin object; writes a 32-byte result


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks(kind: str = "hbm"):
    """Roofline denominator: HBM copy GB/s, or dense bf16 TFLOP/s (burst)."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"] if kind == "hbm" else d["bf16_tflops"]), "measured"
    return (6800.0 if kind == "hbm" else 1900.0), "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = tempfile.NamedTemporaryFile(mode="w+", delete=False, suffix=".csv")

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.flush()
        rows = [ln.split(",") for ln in Path(self.out.name).read_text().splitlines() if ln.strip()]
        os.unlink(self.out.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() in ("active", "1"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def l2_ceilings():
    """The walk's ceilings, measured on this GPU (gb_probe_l2): random
    64-byte record reads from a 32 MB table (L2-resident), independent
    (gather) and each from the place the last record names (chase, the
    dependent chain the walk's descent and object records form), with the
    walk kernel's launch shape.  GB/s."""
    import ctypes as C
    from pyradiance_gb300 import _lib
    out = {}
    for name, chase in (("gather", 0), ("chase", 1)):
        v = C.c_double(0)
        _lib.check(_lib.lib().gb_probe_l2(32 << 20, chase, C.byref(v)))
        out[name] = v.value
    return out


def make_scene(tmp: Path):
    from pyradiance_gb300 import workloads as w
    rad = tmp / "window_room.rad"
    rad.write_text(w.window_room())
    return rad, w.sensor_grid(64, 64)


# ------------------------------------------------------------ CPU baseline

def port_sample(rad: Path, rays: np.ndarray, nsteps: int, per_step: int, threads: int):
    """The oracle (an FP64 port of the reference algorithm, OpenMP threads
    over sensors) on `nsteps` samples of `per_step` sensors each, drawn in
    turn from a fixed shuffle of the grid (wrapping around).  Returns (rays,
    seconds) of each step."""
    from oracle import pyoracle as po
    sc = po.Scene(rad)
    o = po.default_opts("rcontrib", I=1, ab=3, ad=1024, lw=1e-4, c=1, u=0, seed=1)
    mods = [dict(modifier="groundglow"),
            dict(modifier="skyglow", calfile="reinhartb.cal", params="MF=1", binv="rbin", nbins="Nrbins")]
    idx = np.arange(len(rays))
    np.random.default_rng(0).shuffle(idx)
    out, pos = [], 0
    for _ in range(nsteps):
        sel = rays[np.take(idx, np.arange(pos, pos + per_step), mode="wrap")]
        pos += per_step
        o.replica = pos
        t0 = time.perf_counter()
        _, nr = po.rcontrib(sc, o, mods, sel, threads=threads)
        out.append((nr, time.perf_counter() - t0))
    return out


def cpu_baseline(rad: Path, rays: np.ndarray, seconds: float = 15.0):
    """The oracle port on all host cores over a bounded sample of the grid's
    sensors (about `seconds` of work).  Returns (Mrays/s, threads, sample
    description)."""
    threads = os.cpu_count() or 1
    per = 2 * threads
    first = port_sample(rad, rays, 1, per, threads)[0]
    steps = max(1, int(seconds / max(first[1], 1e-3)))
    res = [first] + port_sample(rad, rays, steps, per, threads)
    nr, t = sum(r[0] for r in res), sum(r[1] for r in res)
    return nr / t / 1e6, threads, f"{per * len(res)} sensor paths of the grid in {len(res)} samples of {per}"


def reference_arm(args):
    """--impl reference: the reference's CPU implementation of the path on
    the host cores, one bounded sample of the workload's sensors per step:
    the reference rcontrib compiled from its sources where it is present
    (oracle/_ref), else the oracle port of it.  Rays are counted with the
    oracle's counters on the same sensors (the GPU's definition)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as td:
        rad, rays = make_scene(Path(td))
        ref_bin = ROOT / "oracle" / "_ref" / "bin"
        per = 4 * threads
        if (ref_bin / "rcontrib").exists() and (ref_bin / "oconv").exists():
            from oracle import pyoracle as po
            from pyradiance_gb300 import workloads as w
            env = dict(os.environ, RAYPATH=f".:{ROOT / 'oracle' / '_ref' / 'lib'}")
            octp = Path(td) / "scene.oct"
            octp.write_bytes(subprocess.run([str(ref_bin / "oconv"), str(rad)], capture_output=True,
                                            check=True, env=env).stdout)
            sc = po.Scene(rad)
            o = po.default_opts("rcontrib", I=1, ab=3, ad=1024, lw=1e-4, c=1, u=0, seed=3)
            mods = [dict(modifier="groundglow"),
                    dict(modifier="skyglow", calfile="reinhartb.cal", params="MF=1", binv="rbin",
                         nbins="Nrbins")]
            idx = np.arange(len(rays))
            np.random.default_rng(0).shuffle(idx)
            total_rays, total_t = 0, 0.0
            for step in range(args.warmup + args.steps):
                sel = rays[np.take(idx, np.arange(step * per, (step + 1) * per), mode="wrap")]
                t0 = time.perf_counter()
                subprocess.run([str(ref_bin / "rcontrib"), "-h", "-n", str(threads), "-I+", "-ab", "3", "-ad",
                                "1024", "-lw", "1e-4", "-c", "1", "-fad", "-m", "groundglow", "-f",
                                "reinhartb.cal", "-p", "MF=1", "-b", "rbin", "-bn", "Nrbins", "-m", "skyglow",
                                str(octp)], input=w.rays_ascii(sel), capture_output=True, check=True, env=env,
                               cwd=td)
                t = time.perf_counter() - t0
                if step >= args.warmup:
                    _, nr = po.rcontrib(sc, o, mods, sel, threads=threads)
                    total_rays += nr
                    total_t += t
            kind, sample = "reference", f"{args.steps} samples of {per} sensors of the grid, rcontrib -n {threads}"
        else:
            port_sample(rad, rays, args.warmup, per, threads)
            res = port_sample(rad, rays, args.steps, per, threads)
            total_rays, total_t = sum(r[0] for r in res), sum(r[1] for r in res)
            kind, sample = "port", f"{args.steps} samples of {per} sensors of the grid, {threads} threads"
    v = total_rays / total_t / 1e6
    line = {"metric": METRIC, "value": round(v, 4), "unit": "Mrays/s", "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_t * 1e3 / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded scene and sensor grid)", "config": dict(CONFIG, workload=WORKLOAD),
            "cpu_baseline": {"value": round(v, 4), "unit": "Mrays/s", "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": round(v, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm

def traffic_from_profiles(kernel: str):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary, if one exists."""
    p = ROOT / "profiles" / f"k_{kernel}_rcontrib_window_room_traffic.txt"
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.startswith("dram_bytes_per_launch_full_size="):
            return float(ln.split("=", 1)[1])
    return None


DCT_SHAPE = (16384, 2306, 8760)    # 16,384 sensors x 2,306 Reinhart MF:4 patches x 8,760 hours


def night_hours(N):
    """The night hours of an annual hourly sky (column n = hour n % 24 of
    day n // 24): day length 12 +- 4 h over the year (longest at day 172),
    centred on noon, so that half of the hours are night, in one run per
    night as in an annual sky of a mid-latitude site."""
    n = np.arange(N)
    day, hour = n // 24, n % 24 + 0.5
    length = 12 + 4 * np.cos(2 * np.pi * (day - 172) / 365)
    return np.abs(hour - 12) >= length / 2


def dct_operands(dev, M, K, N, seed=0):
    """Annual daylight-coefficient operands: DC lognormal(-6, 2) with 30%
    exact zeros; sky lognormal(2, 1) diffuse background plus, in each
    daylight hour, one sun patch of 1e4..1e6 (log-uniform); the night hours
    (half of them, one run per night) are all-zero columns."""
    import torch
    g = torch.Generator(device=dev).manual_seed(seed)
    dc = torch.exp(torch.randn(M, K, 3, device=dev, generator=g) * 2 - 6)
    dc[torch.rand(M, K, device=dev, generator=g) < 0.3] = 0
    sky = torch.exp(torch.randn(K, N, 3, device=dev, generator=g) + 2)
    sun = torch.randint(0, K, (N,), device=dev, generator=g)
    peak = torch.exp(torch.empty(N, device=dev).uniform_(np.log(1e4), np.log(1e6), generator=g))
    sky[sun, torch.arange(N, device=dev), :] = peak[:, None]
    sky[:, torch.as_tensor(night_hours(N), device=dev)] = 0
    return dc, sky


def dct_cpu_baseline(dc, sky):
    """The oracle's restatement of cm_multiply (FP64 accumulation, zero rows
    and columns skipped, OpenMP over rows) on all host cores for two row
    samples of the operands (r and 2r rows): the difference gives the cost
    per row, the rest the fixed cost (the zero-column scan), and the sum
    scales to all rows."""
    from oracle import pyoracle as po
    threads = os.cpu_count() or 1
    M = dc.shape[0]
    b = np.ascontiguousarray(sky.cpu().numpy())
    r = 2 * threads
    ts = []
    for n in (r, 2 * r):
        a = np.ascontiguousarray(dc[np.linspace(0, M - 1, n).astype(int)].cpu().numpy())
        t0 = time.perf_counter()
        po.dctimestep(a, b, threads=threads)
        ts.append(time.perf_counter() - t0)
    per_row = max(ts[1] - ts[0], 1e-9) / r
    fixed = max(ts[0] - per_row * r, 0.0)
    return {"value": round(fixed + per_row * M, 2), "unit": "s per product", "cores": threads, "kind": "port",
            "sample": f"{r} and {2 * r} of the {M} rows ({ts[0]:.2f} s, {ts[1]:.2f} s), scaled to all rows"}


def dct_measure(dev, steps: int, rows: int | None = None):
    """DC x sky (dctimestep) on the device at the annual workload's full
    size: the tensor-core forms (FP16X3, BF16X3, FP16) and the FP32 CUDA-core
    kernel on the same resident operands, each a whole gb_dctimestep_device
    call timed with CUDA events on the calling stream (best of `steps`), the
    error of each against the FP64 kernel's product of the same operands,
    cuBLAS FP32 (torch.matmul per channel on de-interleaved copies, TF32
    off) for comparison, and the CPU restatement on a row sample."""
    import ctypes as C
    import torch
    from pyradiance_gb300 import _lib
    L = _lib.lib()
    M, K, N = DCT_SHAPE
    if rows:
        M = rows
    dc, sky = dct_operands(dev, M, K, N)
    st = torch.cuda.current_stream(dev)

    def timed(fn, reps):
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            torch.cuda.synchronize(dev)
            ts.append(e0.elapsed_time(e1))
        return min(ts)

    out = torch.empty(M, N, 3, device=dev)

    def call(mode):
        _lib.check(L.gb_dctimestep_device(C.c_void_p(dc.data_ptr()), C.c_void_p(sky.data_ptr()), M, K, N,
                                          mode, C.c_void_p(out.data_ptr()), C.c_void_p(st.cuda_stream)))

    call(_lib.GB_DCT_FP64)
    ref = out.double()
    nz = ref != 0
    flops = 2.0 * M * K * N * 3
    day = int((sky.abs().amax(dim=(0, 2)) > 0).sum())
    rows = int((dc.abs().amax(dim=(1, 2)) > 0).sum())
    flops_nz = 2.0 * rows * K * day * 3
    res = {"shape": {"M": M, "K": K, "N": N}, "flops": flops, "nonzero_columns": day, "nonzero_rows": rows,
           "flops_nonzero": flops_nz, "l2": "operands and output larger than L2"}
    reps = max(3, steps)
    for mode, name in ((_lib.GB_DCT_FP16X3, "fp16x3"), (_lib.GB_DCT_BF16X3, "bf16x3"), (_lib.GB_DCT_FP16, "fp16"),
                       (_lib.GB_DCT_FP32, "fp32")):
        call(mode)
        ms = timed(lambda: call(mode), reps if name != "fp32" else 3)
        rel = (out.double() - ref).abs()[nz] / ref.abs()[nz]
        res[name] = {"ms": round(ms, 3), "tflops": round(flops / ms / 1e9, 1),
                     "err_vs_fp64": {"mean_rel": float(rel.mean()), "max_rel": float(rel.max())}}
        del rel
    del ref, nz
    # cuBLAS FP32 on de-interleaved copies (copies outside the timed region)
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    a = [dc[..., c].contiguous() for c in range(3)]
    b = [sky[..., c].contiguous() for c in range(3)]
    o = [torch.empty(M, N, device=dev) for _ in range(3)]

    def sgemm():
        for c in range(3):
            torch.matmul(a[c], b[c], out=o[c])
    sgemm()
    ms = timed(sgemm, 3)
    torch.backends.cuda.matmul.allow_tf32 = prev
    res["cublas_fp32"] = {"ms": round(ms, 3), "tflops": round(flops / ms / 1e9, 1),
                          "note": "torch.matmul per channel on planar copies, TF32 off"}
    del a, b, o
    res["speedup_fp16x3_vs_fp32"] = round(res["fp32"]["ms"] / res["fp16x3"]["ms"], 2)
    res["speedup_fp16x3_vs_cublas_fp32"] = round(res["cublas_fp32"]["ms"] / res["fp16x3"]["ms"], 2)
    res["speedup_bf16x3_vs_fp32"] = round(res["fp32"]["ms"] / res["bf16x3"]["ms"], 2)
    peak, kind = peaks("bf16")
    tc = 3 * flops_nz / res["fp16x3"]["ms"] / 1e9
    res["tensor_frac"] = {"achieved_tflops": round(tc, 1), "peak": peak, "frac": round(tc / peak, 4),
                          "peak_source": kind,
                          "note": "FP16X3: three fp16 products per useful product over the non-zero rows and "
                                  "columns; the time is the whole call (scans, split, zero fill, product)"}
    res["cpu_baseline"] = dct_cpu_baseline(dc, sky)
    del dc, sky, out
    torch.cuda.empty_cache()
    return res


GRAD_ARGS = ["-I+", "-ab", "2", "-ad", "1024", "-aa", "0", "-as", "0", "-lw", "1e-4", "-u-"]


def c1_measure(steps: int):
    """The deterministic direct-irradiance workload (rtrace -I -ab 0 -dj 0
    -ds 0 -dr 0 on the 100 x 100 sensor grid of the room of 200 boxes):
    whole gb_rtrace calls through the C ABI (host rays in, host values and
    first-hit ids out), best of `steps` after one warm-up, with CUDA events
    not needed (the call returns when its results are on the host); and
    the oracle port of rtrace on all host cores on the same sensors (the
    reference program is not on the GPU host)."""
    import torch
    from pyradiance_gb300 import workloads as w
    from pyradiance_gb300 import _lib
    from oracle import pyoracle as po
    L = _lib.lib()
    with tempfile.TemporaryDirectory() as td:
        rad = Path(td) / "c1.rad"
        rad.write_text(w.daylight_room())
        import pyradiance_gb300 as gb
        sc = gb.Scene(rad_files=[rad])
        rays = np.ascontiguousarray(w.sensor_grid(100, 100), dtype=np.float64)
        n = len(rays)
        o, _ = _lib.parse_opts(["-I+", "-ab", "0", "-dj", "0", "-ds", "0", "-dr", "0"], _lib.GB_PROG_RTRACE)
        rgb = np.zeros((n, 3))
        hid = np.zeros(n, dtype=np.int32)
        ht = np.zeros(n)

        def call():
            _lib.check(L.gb_rtrace(sc.handle, o, _lib.ptr(rays), n, _lib.ptr(rgb), _lib.ptr(hid), _lib.ptr(ht)))
        call()
        torch.cuda.synchronize()
        ts = []
        for _ in range(max(3, steps)):
            t0 = time.perf_counter()
            call()
            ts.append(time.perf_counter() - t0)
        gpu_s = min(ts)
        # the same values for rays already in HBM (gb_rtrace_device_noalloc), CUDA events on its stream
        dev = torch.device("cuda", 0)
        d_rays = torch.as_tensor(rays, device=dev)
        d_rgb = torch.zeros(n, 3, dtype=torch.float64, device=dev)
        st = torch.cuda.current_stream(dev)
        import ctypes as C
        dts = []
        for _ in range(max(3, steps) + 1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            _lib.check(L.gb_rtrace_device_noalloc(sc.handle, o, C.c_void_p(d_rays.data_ptr()), n,
                                                  C.c_void_p(d_rgb.data_ptr()), C.c_void_p(st.cuda_stream)))
            e1.record(st)
            torch.cuda.synchronize(dev)
            dts.append(e0.elapsed_time(e1))
        dev_ms = min(dts[1:])
        threads = os.cpu_count() or 1
        osc = po.Scene(rad)
        oo = po.default_opts("rtrace", I=1, ab=0, dj=0, ds=0, dr=0, u=0)
        t0 = time.perf_counter()
        po.rtrace(osc, oo, rays, threads=threads)
        cpu_s = time.perf_counter() - t0
    return {"workload": "rtrace -I -ab 0 -dj 0 -ds 0 -dr 0: 10,000 sensors (100x100 grid, z=0.8, +z) in a 10x8x3 m "
                        "room of 200 random boxes (1,200 quads) with a 1x1 m ceiling light; values and first-hit ids",
            "gpu_ms_per_call": round(gpu_s * 1e3, 3), "gpu_sensors_per_s": round(n / gpu_s),
            "timing": "whole gb_rtrace call with host buffers (host to device and back inside, values and "
                      f"first-hit ids), best of {len(ts)}",
            "gpu_device_ms": round(dev_ms, 3),
            "device_timing": "values of rays already in HBM (gb_rtrace_device_noalloc), CUDA events, best of "
                             f"{len(dts) - 1}",
            "cpu_baseline": {"value_ms": round(cpu_s * 1e3, 1), "cores": threads, "kind": "port",
                             "sample": "all 10,000 sensors"},
            "speedup_vs_cpu": round(cpu_s / gpu_s, 1), "speedup_device_vs_cpu": round(cpu_s * 1e3 / dev_ms, 1),
            "note": "a small workload (about 20,000 rays): the call's fixed costs (copies, launches, two "
                    "synchronisations: first hits in FP64, then values) dominate it"}


def bytes_measure(sc, rays, steps: int):
    """The headline workload through the pyradiance byte surface: rays as
    bytes in, the rcontrib output as bytes out (Rcontrib(...)() as a
    pyradiance user calls it), ASCII both ways (the default) and double in,
    float out (-fdf); whole calls timed on the host, best of `steps` after
    one warm-up, rays from the library's counters."""
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import _lib
    res = {}
    forms = {"ascii": (None, None, "".join(f"{a:.9g} {b:.9g} {c:.9g} {d:.9g} {e:.9g} {f:.9g}\n"
                                           for a, b, c, d, e, f in rays).encode()),
             "binary": ("d", "f", np.ascontiguousarray(rays, dtype="<f8").tobytes())}
    for name, (fi, fo, inp) in forms.items():
        rc = gb.Rcontrib(inp, sc, inform=fi, outform=fo, params=PARAMS)
        for m in MODS:
            rc.add_modifier(**m)
        rc.seed = 20261203
        out = rc()
        ts = []
        for _ in range(max(3, steps)):
            t0 = time.perf_counter()
            out = rc()
            ts.append(time.perf_counter() - t0)
        best = min(ts)
        nray = _lib.last_stats()["rays"]
        res[name] = {"mrays_s": round(nray / best / 1e6, 1), "s_per_call": round(best, 4),
                     "in_bytes": len(inp), "out_bytes": len(out)}
    res["note"] = ("Rcontrib(inp, scene, inform, outform, params)() with the headline modifiers: the input parsed, "
                   "the GPU run, the output formatted, per call; best of the calls after one warm-up")
    return res


def grad_measure(steps: int):
    """Gradient of the MSE between 4,096 sensor irradiances and a target
    map (made by a seed-fixed ground-truth parameter set) with respect to 64
    material RGB reflectances (initialised U[0.2, 0.8]) and the glazing
    transmissivity: the window room with its 20,000 triangles in 64
    materials, -ab 2, 1,024 hemisphere samples per sensor.  The forward call
    and the path-replay gradient call (d loss / d value = 2 (e - target) / N
    from the forward's values), each timed with CUDA events around its
    kernels (best of `steps`)."""
    from pyradiance_gb300 import _lib
    from pyradiance_gb300 import workloads as w
    L = _lib.lib()
    with tempfile.TemporaryDirectory() as td:
        rad = Path(td) / "room64.rad"
        rad.write_text(w.window_room(seed=0, ntri=20000, nmat=64))
        import pyradiance_gb300 as gb
        sc = gb.Scene(rad_files=[rad])
    rays = np.ascontiguousarray(w.sensor_grid(64, 64))
    rng = np.random.default_rng(2024)
    slots = [sc.material_slot(f"tri_mat{m}") for m in range(64)] + [sc.material_slot("window_glass")]
    truth = [rng.uniform(0.2, 0.8, 3) for _ in range(64)] + [np.full(3, 0.5)]
    init = [rng.uniform(0.2, 0.8, 3) for _ in range(64)] + [np.full(3, 0.6)]
    o, _ = _lib.parse_opts(GRAD_ARGS, _lib.GB_PROG_RTRACE)
    n = len(rays)
    e = np.zeros((n, 3))
    for sl, v in zip(slots, truth):
        sc.material_rgb(sl, v)
    _lib.check(L.gb_rtrace(sc.handle, o, _lib.ptr(rays), n, _lib.ptr(e), None, None))
    target = e.copy()
    for sl, v in zip(slots, init):
        sc.material_rgb(sl, v)
    ns = int(L.gb_scene_material_slots(sc.handle))
    g = np.zeros((ns, 3))
    fwd, bwd, rays_f, loss = [], [], 0, 0.0
    for _ in range(max(3, steps)):
        _lib.check(L.gb_rtrace(sc.handle, o, _lib.ptr(rays), n, _lib.ptr(e), None, None))
        fwd.append(_lib.last_profile()["region_ms"])
        rays_f = _lib.last_stats()["rays"]
        loss = float(((e - target) ** 2).mean())
        dl = np.ascontiguousarray(2.0 * (e - target) / e.size)
        _lib.check(L.gb_rtrace_grad(sc.handle, o, _lib.ptr(rays), n, _lib.ptr(dl), _lib.ptr(g), ns))
        bwd.append(_lib.last_profile()["region_ms"])
    f, b = min(fwd), min(bwd)
    return {"workload": "window room, 20,000 triangles in 64 plastic materials + glass window, 4096 sensors, "
                        "rtrace " + " ".join(GRAD_ARGS) + "; d(MSE to a target map)/d(64 x RGB reflectance, "
                        "glass transmissivity)",
            "loss": loss, "forward_ms": round(f, 3), "gradient_ms": round(b, 3), "rays_per_forward": int(rays_f),
            "cost_ratio_forward_plus_gradient_vs_forward": round((f + b) / f, 3),
            "note": "the gradient call replays the forward's paths; timed regions are the kernel regions "
                    "(CUDA events); agreement with central differences and with differenced reference runs is "
                    "checked in the GPU tests"}


BATCH_ARGS = ["-I+", "-ab", "2", "-ad", "512", "-lw", "1e-4", "-c", "1", "-u-"]


def _room_text(args):
    """Scene text of one batching room (run in a worker process)."""
    import sys as _s
    _s.path.insert(0, str(ROOT))
    from pyradiance_gb300 import workloads as w
    path, seed, ntri, nwin = args
    Path(path).write_text(w.window_room(seed=seed, ntri=ntri, nmat=64, nwin=nwin, tessellated=True))
    return path


def batch_measure(steps: int):
    """Batched grids: 256 sensor grids of lognormal sizes (median 1,024,
    clipped to 64..16,384) over 16 window rooms of log-uniform triangle
    counts in [5e4, 2e6] (finer tessellations of the same furniture: edges
    shrink as the count grows, so the area stays that of 20,000 triangles)
    with 1..8 windows, rcontrib -ab 2 -ad 512 into Reinhart MF:1 + ground,
    all in one gb_rcontrib_batch call (per scene: one wavefront over its
    grids, the generation loop captured in a CUDA graph, queue size and walk
    shape from the scene's tuner); against one 16,384-sensor grid on the
    median scene with the same options.  Wall-clock rays/s of whole calls
    (host buffers in and out), best of `steps`; scene text is written by
    worker processes and loaded (octrees built on the GPU) before timing."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import pyradiance_gb300 as gb
    rng = np.random.default_rng(2026)
    ntri = np.exp(rng.uniform(np.log(5e4), np.log(2e6), 16)).astype(int)
    nwin = rng.integers(1, 9, 16)
    sizes = np.clip(np.exp(rng.normal(np.log(1024), 1.0, 256)), 64, 16384).astype(int)
    owner = rng.integers(0, 16, 256)
    with tempfile.TemporaryDirectory() as td:
        jobs_txt = [(str(Path(td) / f"room{k}.rad"), 100 + k, int(ntri[k]), int(nwin[k])) for k in range(16)]
        t0 = time.perf_counter()
        with cf.ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1),
                                    mp_context=mp.get_context("spawn")) as ex:
            paths = list(ex.map(_room_text, jobs_txt))
        t_text = time.perf_counter() - t0
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
            scenes = list(ex.map(lambda p: gb.Scene(rad_files=[p]), paths))
        t_load = time.perf_counter() - t0
    on_dev = sum(_octree_on_device(s) for s in scenes)

    def sensors(n, seed):
        r = np.random.default_rng(seed)
        xy = r.uniform((0.3, 0.3), (9.7, 7.7), size=(n, 2))
        return np.column_stack([xy, np.full(n, 0.8), np.zeros(n), np.zeros(n), np.ones(n)])
    jobs = [(scenes[owner[j]], sensors(int(sizes[j]), j)) for j in range(256)]
    rc = gb.Rcontrib(b"", None, params=BATCH_ARGS)
    for m in MODS:
        rc.add_modifier(**m)
    rc.seed = 7
    median = int(np.argsort(ntri)[8])
    single = sensors(16384, 99)
    t0 = time.perf_counter()
    rc.run_batch(jobs)                                   # warm-up (and the scenes' tuners)
    t_first = time.perf_counter() - t0
    rc.octree = scenes[median]
    rc.run_array(single)
    tb, tsg, rays_b, rays_s = [], [], 0, 0
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        rc.run_batch(jobs)
        tb.append(time.perf_counter() - t0)
        rays_b = rc.last_rays
        t0 = time.perf_counter()
        rc.run_array(single)
        tsg.append(time.perf_counter() - t0)
        rays_s = rc.last_rays
    vb, vs = rays_b / min(tb) / 1e6, rays_s / min(tsg) / 1e6
    return {"workload": f"256 grids (sizes lognormal median 1024, 64..16384; {int(sizes.sum())} sensors) over 16 "
                        f"window rooms of {int(ntri.min())}..{int(ntri.max())} triangles "
                        f"({int(ntri.sum())} in all) with {int(nwin.min())}..{int(nwin.max())} windows, rcontrib "
                        + " ".join(BATCH_ARGS) + ", Reinhart MF:1 + ground",
            "batch_mrays_s": round(vb, 1), "single_grid_mrays_s": round(vs, 1),
            "batch_vs_single": round(vb / vs, 3), "batch_s": round(min(tb), 3), "rays_batch": int(rays_b),
            "single_grid": f"16384 sensors on the median scene ({int(ntri[median])} triangles)",
            "scene_text_s": round(t_text, 2), "scene_load_s": round(t_load, 2),
            "octrees_built_on_gpu": int(on_dev), "first_batch_s_with_tuners": round(t_first, 3),
            "graphs": os.environ.get("GB_GRAPHS", "1") != "0"}


def _octree_on_device(sc) -> int:
    import ctypes as C
    from pyradiance_gb300 import _lib
    d = C.c_int()
    _lib.check(_lib.lib().gb_scene_octree_info(sc.handle, None, None, None, C.byref(d)))
    return d.value


def combine_ranks(dev_s: float, wall_s: float, rays: float, world: int, device=None):
    """Whole-job figures of a multi-rank run: the slowest rank's device and
    wall seconds, and the rays of all ranks (the ranks trace independent
    samples, so there is no other exchange)."""
    if world <= 1:
        return dev_s, wall_s, rays
    import torch
    import torch.distributed as dist
    t = torch.tensor([dev_s, wall_s, rays], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    sm = t.clone()
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(mx[1]), float(sm[2])


def gpu_arm(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import _lib

    dev = torch.device("cuda", local)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)   # 256 MB > L2

    with tempfile.TemporaryDirectory() as td:
        rad, rays = make_scene(Path(td))
        if args.sensors:
            rays = rays[np.linspace(0, len(rays) - 1, args.sensors).astype(int)]
        sc = gb.Scene(rad_files=[rad])
        rc = gb.Rcontrib(b"", sc, params=PARAMS)
        for m in MODS:
            rc.add_modifier(**m)
        rc.replica = rank                        # independent samples per rank
        rc.seed = 20261203
        rays = np.ascontiguousarray(rays)

        def step():
            flush.fill_(float(np.random.rand()))
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            out = rc.run_array(rays)
            wall = time.perf_counter() - t0
            prof = _lib.last_profile()
            st = _lib.last_stats()
            return out, wall, prof, st

        for _ in range(max(3, args.warmup)):
            step()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize(dev)
        clocks = ClockSampler(local)
        clocks.start()
        walls, regions, rays_tot, launches, profs = [], [], 0, 0, []
        for _ in range(args.steps):
            out, wall, prof, st = step()
            walls.append(wall)
            regions.append(prof["region_ms"])
            rays_tot += st["rays"]
            launches += st["launches"]
            profs.append(prof)
        torch.cuda.synchronize(dev)
        ck = clocks.stop()
        dev_s = sum(regions) / 1e3
        wall_s = sum(walls)
        dev_s, wall_s, rays_all = combine_ranks(dev_s, wall_s, float(rays_tot), world, dev)
        if rank != 0:
            return
        # dominant kernel and its roofline
        agg = {}
        for p in profs:
            for k, v in p.items():
                if k == "region_ms":
                    continue
                a = agg.setdefault(k, {"ms": 0.0, "launches": 0, "rays": 0, "steps": 0, "nodes": 0, "tests": 0})
                for f in a:
                    a[f] += v[f]
        dom = max(agg, key=lambda k: agg[k]["ms"])
        d = agg[dom]
        io = B_RAYIO * d["rays"] if dom == "trace" else 0      # ray record in, walk result out
        bytes_per_launch = (d["nodes"] * B_NODE + d["steps"] * B_STEP + d["tests"] * B_TEST + io) / d["launches"]
        ms_per_launch = d["ms"] / d["launches"]
        achieved = bytes_per_launch / (ms_per_launch / 1e3) / 1e9
        peak, peak_kind = peaks()
        l2c = l2_ceilings()
        traffic = traffic_from_profiles(dom)
        cpu_v, cores, sample = cpu_baseline(rad, rays, seconds=12.0) if not args.no_cpu else (None, 0, "skipped")
        value = rays_all / dev_s / 1e6
        e2e = rays_all / wall_s / 1e6
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": round(dev_s * 1e3 / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene and sensor grid)",
            "config": dict(CONFIG, workload=WORKLOAD, sensors_per_gpu=int(len(rays))),
            "detail": {"rays_per_step_per_gpu": int(rays_tot / args.steps), "kernels": {k: {
                "ms_per_step": round(v["ms"] / args.steps, 3), "launches": v["launches"]}
                for k, v in agg.items()}},
            "e2e": {"value": round(e2e, 3), "unit": "Mrays/s", "h2d_bytes_per_step": int(rays.nbytes),
                    "d2h_bytes_per_step": int(len(rays) * 146 * 3 * 8)},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": "k_" + dom, "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": traffic, "peak_source": peak_kind,
                         "l2_gather_ceiling": round(l2c["gather"], 1),
                         "frac_of_l2_gather": round(achieved / l2c["gather"], 4),
                         "l2_chase_ceiling": round(l2c["chase"], 1),
                         "frac_of_l2_chase": round(achieved / l2c["chase"], 4),
                         "note": "algorithmic bytes = node descents*4 + cube visits*8 + object tests*60 (+ rays*80 for "
                                 "the walk kernel's ray record and result); the scene lives in L1/L2 (DRAM traffic is "
                                 "a few percent of the algorithmic bytes), so the binding ceilings are the measured "
                                 "rates of random 64-byte reads from L2: independent (gather) and dependent (chase), "
                                 "gb_probe_l2 with the walk's launch shape"},
            "cpu_baseline": {"value": None if cpu_v is None else round(cpu_v, 4), "unit": "Mrays/s",
                             "cores": cores, "kind": "port", "sample": sample},
            "clocks": ck,
        }
        if not (args.sensors or args.no_extras):
            line["e2e_bytes"] = bytes_measure(sc, rays, min(args.steps, 5))
            line["c1_rtrace"] = c1_measure(args.steps)
            line["dctimestep"] = dct_measure(dev, args.steps)
            line["gradient"] = grad_measure(args.steps)
            line["batching"] = batch_measure(min(args.steps, 3))
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 30; 5 for the reference arm, whose steps are CPU samples)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--sensors", type=int, default=0,
                    help="profile a smaller case: this many sensors of the grid, without the dctimestep, "
                         "gradient and batching legs")
    ap.add_argument("--dct-rows", type=int, default=0,
                    help="profile dctimestep alone at this many rows (2,306 x 8,760 otherwise as the annual "
                         "workload); prints its result")
    ap.add_argument("--no-extras", action="store_true",
                    help="the rcontrib workload only (no dctimestep, gradient and batching legs)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 5 if args.impl == "reference" else 30
    if args.impl == "reference":
        reference_arm(args)
    elif args.dct_rows:
        import torch
        print(json.dumps(dct_measure(torch.device("cuda", 0), args.steps, rows=args.dct_rows)), flush=True)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
