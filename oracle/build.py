"""TEST INFRASTRUCTURE — builds the CPU oracle (liboracle.so) into oracle/_build/.

The oracle is the checker for the CUDA path, never the product.  Flags pin IEEE-754
single-precision evaluation as written: no contraction into fused multiply-adds
(-ffp-contract=off, which matters on aarch64 where GCC contracts by default) and no fast
math.  OpenMP parallelises pixels and rays.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SOURCES = [HERE / "oracle.cpp"]
HEADERS = sorted(HERE.glob("*.h"))
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
         "-fno-math-errno", "-Wall", "-Wno-unused-variable"]


def build(force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    deps = SOURCES + HEADERS + [Path(__file__)]
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    cxx = shutil.which("g++") or "g++"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cxx, *FLAGS, *map(str, SOURCES), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
