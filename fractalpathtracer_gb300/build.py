"""Builds libfpt_cuda.so in-tree for sm_103a (nvcc only, no cmake).

Translation units compile in parallel: one object per scene kind for the
path-tracing kernels (they dominate the build), plus the voxel, MLP, bridge
and host I/O units.  The library links the CUDA runtime statically so it
loads on any box with the same driver.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libfpt_cuda.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "-I", os.path.join(HERE, "..", "include")]
KINDS = 6


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfpt_cuda.so")


def _units():
    """(source, object, extra flags) for every translation unit."""
    # Render kernels: approximate division/sqrt in the hot loops; the few
    # values that seed hashes use explicitly rounded intrinsics.
    fast = ["-prec-div=false", "-prec-sqrt=false"]
    units = []
    for k in range(KINDS):   # each kind in three parts (path tracer, primary/samples/diagnostics, surrogate)
        for part in range(3):
            units.append(("render_kind.cu", f"render_kind{k}_{part}.o", fast + [f"-DFPT_KIND={k}", f"-DFPT_PART={part}"]))
    units.append(("render_common.cu", "render_common.o", fast))
    # Voxel build and DDA: IEEE operations in source order (no contraction),
    # so brick tables and cell sequences are bit-identical to the CPU path.
    units.append(("voxel.cu", "voxel.o", ["-fmad=false"]))
    units.append(("mlp.cu", "mlp.o", []))
    units.append(("batch.cu", "batch.o", fast))
    units.append(("bridge.cu", "bridge.o", []))
    units.append(("image_io.cpp", "image_io.o", []))
    missing = sorted({u[0] for u in units if not os.path.exists(os.path.join(CSRC, u[0]))})
    if missing:
        raise RuntimeError(f"listed sources are missing from {CSRC}: {', '.join(missing)}")
    return units


def _compile(nvcc: str, unit, verbose: bool):
    src, obj, extra = unit
    out = os.path.join(BUILD_DIR, obj)
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    cmd = [nvcc, *ARCH, *COMMON, *extra, *lang, "-c", os.path.join(CSRC, src), "-o", out]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
    return out


def _stale(lib: str) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    for root in (CSRC, os.path.join(HERE, "..", "include")):
        for name in os.listdir(root):
            if os.path.getmtime(os.path.join(root, name)) > t:
                return True
    return os.path.getmtime(os.path.abspath(__file__)) > t


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    """Compiles every CUDA/C++ unit and links lib/libfpt_cuda.so; returns its path."""
    lib = os.path.join(OUT_DIR, LIB_NAME)
    if not force and not _stale(lib):
        return lib
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    units = _units()
    jobs = jobs or min(len(units), max(os.cpu_count() or 4, 4))
    with ThreadPoolExecutor(max_workers=jobs) as pool:
        objs = list(pool.map(lambda u: _compile(nvcc, u, verbose), units))
    tmp = lib + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", tmp, *objs, "-cudart", "static", "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
