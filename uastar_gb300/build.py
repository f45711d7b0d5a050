"""Build the engine's shared library in-tree: uastar_gb300/libuastar_gb300.so.

The CUDA translation units are compiled for sm_103a only (one -gencode, in
parallel), the host utilities with g++, and everything is linked with nvcc.
Run as ``python -m uastar_gb300.build`` or through ``__graft_entry__.build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_build"
LIB = PKG / "libuastar_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["engine.cu", "pdb.cu", "batch.cu", "noalloc.cu"]
HOST_SOURCES = ["host_utils.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    OUT_DIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [PKG.parent / "include" / "uastar_gpu.h"]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        obj = OUT_DIR / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                         "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills", "-c", str(CSRC / src),
                         "-o", str(obj)])
    for src in HOST_SOURCES:
        obj = OUT_DIR / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-c", str(CSRC / src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lpthread"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
