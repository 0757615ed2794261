"""Builds a PRISMS-PF application (``main.cc`` + ``custom_pde.h``) against the drop-in headers.

  python -m phasefield_gb300.app_build <application dir> [-o <executable>]

The application's sources are compiled unchanged with nvcc as CUDA C++ for sm_103a: the
drop-in ``prismspf/core/problem.h`` instantiates the matrix-free cell kernel for the
application's ``CustomPDE`` in its own translation unit, and the executable links the engine
library (``libppf_gb300.so``, built on demand) with an rpath to it.
"""
from __future__ import annotations

import argparse
import shutil
import subprocess
import sys
from pathlib import Path

from . import build as _build

ROOT = Path(__file__).resolve().parents[1]
INCLUDE = ROOT / "include"

APP_FLAGS = ["-std=c++20", "-x", "cu", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
             "-O3", "-lineinfo"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found")
    return exe


def compile_app(app_dir, output=None, extra_flags=(), link: bool = True) -> Path:
    """Compiles ``app_dir/main.cc``; returns the executable (or object when link=False)."""
    app_dir = Path(app_dir).resolve()
    main = app_dir / "main.cc"
    if not main.exists():
        raise FileNotFoundError(main)
    out = Path(output) if output else app_dir / ("main" if link else "main.o")
    cmd = [nvcc(), *APP_FLAGS, "-I" + str(INCLUDE), "-I" + str(app_dir), *extra_flags, str(main)]
    if link:
        lib = _build.build()
        cmd += ["-L" + str(lib.parent), "-lppf_gb300", "-Xlinker", "-rpath", "-Xlinker", str(lib.parent)]
    else:
        cmd += ["-c"]
    cmd += ["-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {main}:\n{r.stdout}\n{r.stderr}")
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("app_dir")
    ap.add_argument("-o", "--output", default=None)
    args = ap.parse_args(argv)
    exe = compile_app(args.app_dir, args.output)
    print(exe)
    return 0


if __name__ == "__main__":
    sys.exit(main())
