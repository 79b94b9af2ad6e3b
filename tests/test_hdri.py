"""Radiance HDRI hydration, on the CPU: the library's reader and 32x16 FP16
LUT (the host code every world-mode-2 render runs, restating
src/metal_bridge.mm:2163-2300) against the oracle's restatement, bit for
bit, on files written here with run-length and literal scanline packets,
both orientation flags, sizes that do not divide the LUT, and broken
headers."""
import os

import numpy as np
import pytest

import oracle
from fractalpathtracer_gb300 import scenes


def _write(path, rgbe, y_flag="-Y", x_flag="+X"):
    scenes.write_rgbe_file(path, rgbe)
    if (y_flag, x_flag) != ("-Y", "+X"):
        h, w = rgbe.shape[:2]
        data = open(path, "rb").read()
        data = data.replace(f"-Y {h} +X {w}\n".encode(), f"{y_flag} {h} {x_flag} {w}\n".encode(), 1)
        open(path, "wb").write(data)


def _sky(w, h, seed):
    rng = np.random.default_rng(seed)
    img = scenes.sky_equirect(w, h, (0.3, 0.8, 0.5), seed)
    img = img * rng.uniform(0.5, 2.0, img.shape).astype(np.float32)   # literal packets, not only runs
    img[: h // 4, : w // 3] = 0.25                                      # long runs
    return scenes.rgbe_encode(img.astype(np.float32))


@pytest.mark.parametrize("size,flags", [((512, 256), ("-Y", "+X")), ((100, 37), ("+Y", "-X")), ((33, 9), ("-Y", "-X"))])
def test_lut_bits_match_oracle(oracle_lib, native, tmp_path, size, flags):
    path = str(tmp_path / "sky.hdr")
    _write(path, _sky(size[0], size[1], 3), *flags)
    got = native.hdri_lut(path)
    ref = oracle.hdri_lut(path)
    assert got.shape == ref.shape == (32 * 16 * 3,)
    assert np.array_equal(got, ref)
    assert np.count_nonzero(got) > 100


def test_orientation_flags_change_the_lut(oracle_lib, native, tmp_path):
    a, b = str(tmp_path / "a.hdr"), str(tmp_path / "b.hdr")
    rgbe = _sky(64, 32, 5)
    _write(a, rgbe, "-Y", "+X")
    _write(b, rgbe, "+Y", "+X")
    la, lb = native.hdri_lut(a).reshape(16, 32, 3), native.hdri_lut(b).reshape(16, 32, 3)
    assert np.array_equal(la, lb[::-1])


def test_broken_files_fail_cleanly(native, tmp_path):
    from fractalpathtracer_gb300.native import NativeError
    p = str(tmp_path / "bad.hdr")
    with open(p, "wb") as f:
        f.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 40000 +X 64\n")
    with pytest.raises(NativeError, match="height"):
        native.hdri_lut(p)
    _write(p, _sky(64, 32, 1))
    data = open(p, "rb").read()
    open(p, "wb").write(data[: len(data) // 2])
    with pytest.raises(NativeError, match="HDRI"):
        native.hdri_lut(p)
    with pytest.raises(NativeError):
        native.hdri_lut(str(tmp_path / "missing.hdr"))
    assert not os.path.exists(str(tmp_path / "missing.hdr"))
