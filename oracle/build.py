"""Build recipe of the CPU oracle (test infrastructure).

Compiles oracle/fpt_oracle.cpp into oracle/_ref/liboracle.so with g++ and
OpenMP.  -ffp-contract=off keeps every float operation separately rounded
(no fused multiply-add on either x86 or Arm), which the bit-exact voxel
and DDA comparisons rely on.  No -march=native: the same flags build on
the x86 development host and on the Arm GPU host.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "liboracle.so")
SOURCES = ["fpt_oracle.cpp"]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith((".cpp", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "fpt_cuda.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", tmp] + [os.path.join(HERE, s) for s in SOURCES]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
