"""Diagnostic images (fpt_metal_diagnostic_render, the reference's sdf_diagnostic_kernel modes).

Depth, hit mask and normal images of a Mandelbulber scene use marchMandelbulber, the
same march as the primary-ray tracer, so they are pinned to the FP64 oracle's
primary rays: hit masks agree on >= 99% of pixels, the 8-bit depth code within 2 and
the normal code within 3 on >= 99% of common hits.  The final-colour mode equals the
path-traced render through postProcess when chromatic aberration and highlights are
off.  The path-cost modes count at least one march step per pixel.
"""
import numpy as np
import pytest

import oracle
from fractalpathtracer_gb300 import ffi, scenes

pytestmark = pytest.mark.gpu


def _diag(native, read_png, tmp_path, cfg, mode, max_distance=0.0):
    path = str(tmp_path / f"diag{mode}.png")
    native.diagnostic_render(cfg, mode, path, max_distance)
    return read_png(path)


def test_depth_hit_normal_match_fp64_primary_rays(native, read_png, tmp_path):
    cfg, ext = scenes.mandelbulb_primary(160, 120)
    ref = oracle.trace_primary(cfg, None, fp64=True)[::-1]   # rows top-first like the image
    hit_r = ref[..., 5] > 0
    hit = _diag(native, read_png, tmp_path, cfg, 3)[..., 0] > 127
    assert hit_r.mean() > 0.1
    assert (hit == hit_r).mean() >= 0.99
    depth = _diag(native, read_png, tmp_path, cfg, 0).astype(np.int32)[..., 0]
    both = hit & hit_r
    code = np.floor(np.clip(1.0 - ref[..., 0] / cfg.render[4], 0.0, 1.0) * 255.0).astype(np.int32)
    assert np.percentile(np.abs(depth[both] - code[both]), 99) <= 2
    normal = _diag(native, read_png, tmp_path, cfg, 1).astype(np.int32)[..., :3]
    ncode = np.floor(np.clip(ref[..., 1:4] * 0.5 + 0.5, 0.0, 1.0) * 255.0).astype(np.int32)
    err = np.abs(normal - ncode).max(-1)[both]
    assert np.percentile(err, 99) <= 3
    assert (normal[~hit] == 0).all()


def test_reference_scene_modes(native, read_png, tmp_path):
    cfg = ffi.default_config()
    cfg.width, cfg.height = 128, 96
    for mode in (0, 2, 3, 4, 5, 6, 8, 9):
        img = _diag(native, read_png, tmp_path, cfg, mode)
        assert img.shape == (96, 128, 4) and (img[..., 3] == 255).all()
    hit = _diag(native, read_png, tmp_path, cfg, 3)[..., 0] > 127
    assert hit.mean() > 0.5                      # the Cornell box fills most of the frame
    diffuse = _diag(native, read_png, tmp_path, cfg, 8)[..., 0]
    assert diffuse[hit].min() >= int(0.12 * 255) - 1
    assert (_diag(native, read_png, tmp_path, cfg, 9)[..., :3] == 0).all()   # no generated material


def test_final_colour_equals_render(native, read_png, tmp_path):
    cfg = ffi.default_config()
    cfg.width, cfg.height, cfg.samples = 96, 72, 16
    cfg.post[5] = 0.0
    cfg.post[6] = 0.0
    img = _diag(native, read_png, tmp_path, cfg, 7)
    _, rgba, _ = native.cuda_render(cfg, None, linear=False)
    assert np.array_equal(img, rgba)


def test_path_cost_modes(native, read_png, tmp_path):
    cfg = ffi.default_config()
    cfg.width, cfg.height, cfg.samples = 64, 48, 2
    steps = _diag(native, read_png, tmp_path, cfg, 11)[..., 0]
    assert (steps > 0).all() or steps.mean() > 0
    bounces = _diag(native, read_png, tmp_path, cfg, 14)[..., 0]
    assert bounces.max() <= 255 and bounces.mean() > 0
    with pytest.raises(native.NativeError, match="not supported"):
        _diag(native, read_png, tmp_path, cfg, 15)
