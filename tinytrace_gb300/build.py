"""Builds libtinytrace_cuda.so in-tree for sm_103a (GB300).

Translation units are compiled in parallel with nvcc and linked into one shared library
under tinytrace_gb300/_build/.  Flags: -gencode arch=compute_103a,code=sm_103a, -O3,
-lineinfo, -fmad=false (no implicit contraction: the kernels' float results are specified
operation by operation and must match the CPU oracle bit for bit; fused multiply-adds are
written explicitly where wanted).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libtinytrace_cuda.so"
SOURCES = ["api.cu", "bvh_build.cu", "integrate.cu", "wavefront.cu", "primary.cu", "server.cu", "restir.cu", "cache.cu",
           "ingest.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-fmad=false",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off",
    "-Xptxas",
    "-warn-spills",
]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(path).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtinytrace_cuda.so")
    return path


def _run(cmd: list[str]) -> str:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return res.stdout + res.stderr


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compiles the CUDA sources (if changed) and returns the path of the shared library."""
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "tinytrace_cuda.h"]
    flags = NVCC_FLAGS + (extra_flags or [])
    exe = nvcc()

    def compile_one(src: str) -> tuple[Path, str]:
        s = CSRC / src
        o = BUILD / (Path(src).stem + ".o")
        if force or _stale(o, [s, *headers, Path(__file__)]):
            out = _run([exe, *flags, "-c", str(s), "-o", str(o)])
            return o, out
        return o, ""

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, out in results:
            if out:
                print(out)
    if force or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force=True))
