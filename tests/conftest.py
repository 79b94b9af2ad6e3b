"""Test configuration: the `gpu` marker and shared fixtures.

GPU tests call the CUDA library through its C ABI and compare with the CPU
oracle; CPU tests cover the oracle against the reference's known answers,
the host-side logic, and the library's exported symbols.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    from oracle import build
    build.build()
    return oracle


@pytest.fixture(scope="session")
def native():
    """The CUDA library, built if needed; GPU tests fail loudly when it cannot load."""
    from fractalpathtracer_gb300 import build, native as nat
    build.build()
    nat.lib()
    return nat


def _read_png(path):
    """RGBA8 PNG (as the library writes it) -> (H, W, 4) uint8, top row first."""
    import struct
    import zlib

    import numpy as np
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", None
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 6
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    out = np.zeros((h, w * 4), np.int32)
    prev = np.zeros(w * 4, np.int32)
    for y in range(h):
        f, row = raw[y, 0], raw[y, 1:].astype(np.int32)
        if f == 0:
            cur = row
        elif f == 2:
            cur = (row + prev) & 255
        else:
            cur = row.copy()
            for x in range(w * 4):
                a = cur[x - 4] if x >= 4 else 0
                b = prev[x]
                c = prev[x - 4] if x >= 4 else 0
                if f == 1:
                    cur[x] = (row[x] + a) & 255
                elif f == 3:
                    cur[x] = (row[x] + (a + b) // 2) & 255
                else:
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    cur[x] = (row[x] + (a if pa <= pb and pa <= pc else (b if pb <= pc else c))) & 255
        out[y] = cur
        prev = cur
    return out.reshape(h, w, 4).astype(np.uint8)


@pytest.fixture(scope="session")
def read_png():
    return _read_png
