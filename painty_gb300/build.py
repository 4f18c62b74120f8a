"""Builds the painty_gb300 CUDA library in-tree for sm_103a.

    python painty_gb300/build.py           # -> painty_gb300/_lib/libpainty_gb300.so

(Run it as a script: importing the package itself requires the built library.)

One nvcc job per translation unit, run in parallel, then one link. No CPU fallback is built:
the library is CUDA-only and every entry point launches its own kernels.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "_lib"
LIB = OUT_DIR / "libpainty_gb300.so"
# The bounds-checked build of the same library (PAINTY_BOUNDS_CHECK): the stamp kernels test
# every computed index against its buffer before the access and report instead of faulting.
LIB_CHECKED = OUT_DIR / "libpainty_gb300_checked.so"
CHECKED_SOURCES = {"stamp.cu"}
# The phase-timing build (PAINTY_PHASE_TIMERS): the stamp loop adds each warp's clock cycles per
# phase into device counters (painty_take_phase_cycles), for profiling.
LIB_PHASES = OUT_DIR / "libpainty_gb300_phases.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build painty_gb300")


def cuda_lib_dir() -> str:
    return str(Path(nvcc()).resolve().parent.parent / "lib64")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


# Host code is built without floating-point contraction so the footprint resample and the
# stroke expansion give the same bits on x86-64 and aarch64 (and as painty's double code).
# Translation units listed in NO_FMAD also keep device code free of fused multiply-adds: their
# double kernels repeat painty's arithmetic as written (the others use explicit intrinsics).
NO_FMAD = {"texture.cu", "canvas_gpu.cu"}


def _compile(src: Path, obj: Path, defines=()) -> None:
    cmd = [nvcc(), *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-Wall", "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "-I", str(ROOT / "include"),
           "-I", str(CSRC), *[f"-D{d}" for d in defines], "-c", str(src), "-o", str(obj)]
    if src.name in NO_FMAD:
        cmd.insert(1, "--fmad=false")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")


def _link(objs, lib: Path) -> None:
    libdir = cuda_lib_dir()
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs),
           "-Xlinker", f"-rpath={libdir}", "-L", libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)


def build(verbose: bool = False, checked: bool = True) -> Path:
    """Builds the library and, with `checked`, its bounds-checked and phase-timing twins (the
    translation units in CHECKED_SOURCES compiled again with PAINTY_BOUNDS_CHECK or
    PAINTY_PHASE_TIMERS, the rest shared)."""
    OUT_DIR.mkdir(exist_ok=True)
    objs, checked_objs, phase_objs, jobs = [], [], [], []
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs) + 1, os.cpu_count() or 4))) as ex:
        for src in srcs:
            obj = OUT_DIR / (src.stem + ".o")
            objs.append(obj)
            jobs.append(ex.submit(_compile, src, obj))
            if checked and src.name in CHECKED_SOURCES:
                cobj = OUT_DIR / (src.stem + "_checked.o")
                checked_objs.append(cobj)
                jobs.append(ex.submit(_compile, src, cobj, ("PAINTY_BOUNDS_CHECK=1",)))
                pobj = OUT_DIR / (src.stem + "_phases.o")
                phase_objs.append(pobj)
                jobs.append(ex.submit(_compile, src, pobj, ("PAINTY_PHASE_TIMERS=1",)))
            else:
                checked_objs.append(obj)
                phase_objs.append(obj)
        for j in jobs:
            j.result()
    _link(objs, LIB)
    if checked:
        _link(checked_objs, LIB_CHECKED)
        _link(phase_objs, LIB_PHASES)
    for o in set(objs) | set(checked_objs) | set(phase_objs):
        o.unlink(missing_ok=True)
    if verbose:
        print(f"built {LIB}" + (f", {LIB_CHECKED} and {LIB_PHASES}" if checked else ""))
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
