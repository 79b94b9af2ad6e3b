"""The C header itself: a C translation unit compiled with gcc against
include/fpt_cuda.h sees the reference's pinned struct sizes (src/ffi.rs:494-507)
and the same member offsets as the ctypes mirror the tests and the host code
use.  Runs on the CPU; needs only gcc."""
import ctypes
import os
import shutil
import subprocess
import tempfile

import pytest

from fractalpathtracer_gb300 import ffi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = ["FptSdfInstruction", "FptPrimitiveInstance", "FptAffineTransform", "FptIndexedPrimitive",
           "FptTypedSoAProgram", "FptRenderConfig", "FptSdfProfileStats", "FptStitchPipelineStats",
           "FptStitchValidationStats", "FptBoundGridStats", "FptAsyncJitStats", "FptDiagnosticConfig",
           "FptMandelbulberFieldSample", "FptCudaSceneExt", "FptCudaPrimaryHit"]


def _c_layout():
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc is not available")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fpt_cuda.h"', "int main(void) {"]
    for name in STRUCTS:
        lines.append(f'  printf("S {name} %zu\\n", sizeof(struct {name}));')
        for field, *_ in getattr(ffi, name)._fields_:
            lines.append(f'  printf("O {name} {field} %zu\\n", offsetof(struct {name}, {field}));')
    lines += ["  return 0;", "}"]
    with tempfile.TemporaryDirectory() as tmp:
        src, exe = os.path.join(tmp, "layout.c"), os.path.join(tmp, "layout")
        with open(src, "w") as f:
            f.write("\n".join(lines) + "\n")
        subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o", exe],
                       check=True, capture_output=True, text=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    sizes, offsets = {}, {}
    for line in out.splitlines():
        parts = line.split()
        if parts[0] == "S":
            sizes[parts[1]] = int(parts[2])
        else:
            offsets[(parts[1], parts[2])] = int(parts[3])
    return sizes, offsets


def test_c_header_sizes_match_reference_pins():
    sizes, _ = _c_layout()
    for name, size in ffi.REFERENCE_SIZES.items():
        assert sizes[name] == size, (name, sizes[name], size)
    # the five sizes the reference's Rust tests pin (src/ffi.rs:494-507)
    assert sizes["FptSdfInstruction"] == 32 and sizes["FptRenderConfig"] == 30448
    assert sizes["FptSdfProfileStats"] == 288 and sizes["FptDiagnosticConfig"] == 24
    assert sizes["FptMandelbulberFieldSample"] == 16


def test_c_header_offsets_match_ctypes_mirror():
    sizes, offsets = _c_layout()
    for name in STRUCTS:
        cls = getattr(ffi, name)
        assert sizes[name] == ctypes.sizeof(cls), name
        for field, *_ in cls._fields_:
            assert offsets[(name, field)] == getattr(cls, field).offset, (name, field)
