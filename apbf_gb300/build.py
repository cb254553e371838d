"""Builds the native library libapbf_gb300.so (sm_103a) in-tree.

Every .cu file under csrc/ is compiled to an object in parallel, then linked
with nvcc into apbf_gb300/_lib/libapbf_gb300.so.  glue.cu is compiled with
-fmad=false: its stages are defined by plain FP32 arithmetic and must round
every operation on its own.
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
OUT_DIR = HERE / "_lib"
LIB = OUT_DIR / "libapbf_gb300.so"
OBJ_DIR = HERE / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
# translation units whose FP32 arithmetic must not be contracted into FMAs
NO_FMAD = {"glue.cu", "adaptive.cu", "constraints.cu"}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build apbf_gb300")
    return cand


def _compile(src: Path) -> Path:
    obj = OBJ_DIR / (src.stem + ".o")
    deps = [src, CSRC / "apbf_internal.cuh", HERE.parent / "include" / "apbf_gb300.h"]
    deps += list(CSRC.glob("*.cuh"))
    if obj.exists() and all(obj.stat().st_mtime >= d.stat().st_mtime for d in deps if d.exists()):
        return obj
    flags = list(COMMON)
    if src.name in NO_FMAD:
        flags.append("-fmad=false")
    cmd = [nvcc(), *ARCH, *flags, "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    OBJ_DIR.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    with cf.ThreadPoolExecutor(max_workers=min(len(sources), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, sources))
    if LIB.exists() and all(LIB.stat().st_mtime >= o.stat().st_mtime for o in objs):
        return LIB
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
