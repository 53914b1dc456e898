"""In-tree build of the CUDA library (libshapes_gpu.so) for sm_103a.

Flags that are part of the numerical contract:
  -fmad=false                 no fused multiply-add: every product is rounded,
                              as in the reference (GHC emits no FMA);
  -Xcompiler -ffp-contract=off  the same for host-side code;
  no --use_fast_math          IEEE division, square root and denormals.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libshapes_gpu.so"
PROBE_LIB = OUT_DIR / "libshapes_probe.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-O2,-pthread", "-shared", "-lpthread"]

SOURCES = [CSRC / "shapes_gpu.cu", CSRC / "mlp.cu"]
HEADERS = [CSRC / "step_kernels.cuh", CSRC / "large_world.cuh", CSRC / "lw_order.cuh", CSRC / "learned.cuh",
           CSRC / "fp64_ops.cuh", CSRC / "shapes_sincos.h", CSRC / "shapes_sincos_tables.h", CSRC / "mlp.h",
           CSRC / "tc05.cuh", HERE.parent / "include" / "shapes_gpu.h"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists() and not shutil.which(cand):
        raise RuntimeError("nvcc not found")
    return cand


def needs_build(lib: Path, sources) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    return any(p.stat().st_mtime > t for p in list(sources) + [Path(__file__)])


def _compile(lib: Path, sources, verbose: bool):
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc(), *NVCC_FLAGS, "-o", str(tmp), *map(str, sources)]
    if verbose:
        print(" ".join(cmd))
    return subprocess.Popen(cmd), tmp, lib


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles the step library and the FP64 probe (in parallel) if stale."""
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    jobs = []
    if force or needs_build(LIB, SOURCES + HEADERS):
        jobs.append(_compile(LIB, SOURCES, verbose))
    probe_src = [CSRC / "fp64_probe.cu"]
    if force or needs_build(PROBE_LIB, probe_src + [CSRC / "fp64_ops.cuh", CSRC / "tc05.cuh", CSRC / "lw_order.cuh"]):
        jobs.append(_compile(PROBE_LIB, probe_src, verbose))
    for proc, tmp, lib in jobs:
        if proc.wait() != 0:
            raise RuntimeError(f"nvcc failed building {lib.name}")
        os.replace(tmp, lib)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
