"""Builds the in-tree CUDA library ``phasefield_gb300/lib/libppf_gb300.so`` for sm_103a.

Every ``csrc/*.cu`` translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into one shared
library exporting the C ABI declared in ``include/ppf_gb300.h``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
OBJDIR = PKG / "_build"
LIB = LIBDIR / "libppf_gb300.so"

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo", "-O3", "-std=c++17",
    "-Xcompiler", "-fPIC",
    "--expt-relaxed-constexpr",
    "-I" + str(ROOT / "include"),
]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build phasefield_gb300")
    return exe


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _needs_rebuild() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + list((ROOT / "include").rglob("*.h")) + list((ROOT / "include").rglob("*.cuh")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.is_file())


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    if not force and not _needs_rebuild():
        return LIB
    OBJDIR.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    exe = nvcc()
    srcs = _sources()

    def compile_one(src: Path) -> Path:
        obj = OBJDIR / (src.stem + ".o")
        cmd = [exe, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [exe, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *map(str, objs), "-o", str(tmp),
           "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
