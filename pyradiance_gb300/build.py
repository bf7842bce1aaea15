"""Builds libgbrad.so (the CUDA library behind the C ABI in include/gbrad.h).

Plain nvcc/gcc invocations, compiled in parallel, for sm_103a only.  Host
code is compiled with -ffp-contract=off, so that it rounds alike on x86 and
on aarch64 (where GCC contracts multiply-adds by default):

    python -m pyradiance_gb300.build          # or build() from Python

The library is written next to this file (pyradiance_gb300/libgbrad.so).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OBJ = HERE / "_build"
LIB = HERE / "libgbrad.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["trace.cu", "host.cu", "dct.cu", "dct_tc.cu", "octbuild_gpu.cu", "cast64.cu"]
# per-file flags: the device octree builder's FP64 tests must round as the
# host builder's, and the FP64 first-hit casts as the reference's (no
# contracted multiply-adds)
CU_FLAGS = {"octbuild_gpu.cu": ["-fmad=false"], "cast64.cu": ["-fmad=false"]}
CXX_SOURCES = ["binexpr.cpp", "textio.cpp"]
C_SOURCES = ["scene.c", "octbuild.c"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(src: Path, obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def build(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    OBJ.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "gbrad.h"]
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src, obj = CSRC / s, OBJ / (s + ".o")
        objs.append(obj)
        if force or _stale(src, obj, headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         *CU_FLAGS.get(s, []),
                         "-Xptxas", "-v" if verbose else "-O3", "-c", str(src), "-o", str(obj)])
    for s in CXX_SOURCES:
        src, obj = CSRC / s, OBJ / (s + ".o")
        objs.append(obj)
        if force or _stale(src, obj, headers):
            jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-I", "/usr/local/cuda/include",
                         "-c", str(src), "-o", str(obj)])
    for s in C_SOURCES:
        src, obj = CSRC / s, OBJ / (s + ".o")
        objs.append(obj)
        if force or _stale(src, obj, headers):
            jobs.append(["gcc", "-O2", "-fPIC", "-std=gnu99", "-ffp-contract=off", "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or not LIB.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart", "-lm", "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
