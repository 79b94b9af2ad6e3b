"""Primary-ray march on the GPU vs the FP64 oracle: power-8 Mandelbulb,
320x240, hit distance / analytic normal / step count per pixel.

Tolerances (FP32 GPU vs FP64 CPU): hit/miss agreement >= 99.5% of pixels;
on pixels both call hits, hit distance |dt| <= 5e-5 * (1 + t) for 99% of
them (the reference's field-parity gate, src/main.rs:3297) and the normal
angle <= 1 degree for 99%.
"""
import numpy as np
import pytest

import oracle
from fractalpathtracer_gb300 import scenes

pytestmark = pytest.mark.gpu


def _compare(gpu, ref):
    hit_g = gpu["hit"] > 0
    hit_r = ref[..., 5] > 0
    agree = (hit_g == hit_r).mean()
    both = hit_g & hit_r
    t_g = gpu["distance"][both]
    t_r = ref[..., 0][both]
    derr = np.abs(t_g - t_r) / (1 + t_r)
    n_g = gpu["normal"][both]
    n_r = ref[..., 1:4][both]
    ang = np.degrees(np.arccos(np.clip((n_g * n_r).sum(-1), -1, 1)))
    return agree, derr, ang, both


def test_mandelbulb_primary_matches_fp64(native):
    cfg, ext = scenes.mandelbulb_primary(320, 240)
    gpu, ms = native.trace_primary(cfg, ext)
    ref = oracle.trace_primary(cfg, ext, fp64=True)
    agree, derr, ang, both = _compare(gpu, ref)
    assert both.sum() > 10000
    assert agree >= 0.995, agree
    assert np.percentile(derr, 99) <= 5e-5, np.percentile(derr, 99)
    assert np.percentile(ang, 99) <= 1.0, np.percentile(ang, 99)
    steps_g = gpu["steps"][both].astype(np.float64)
    steps_r = ref[..., 4][both]
    assert abs(steps_g.mean() - steps_r.mean()) / steps_r.mean() < 0.05


def test_mandelbulb_normals_are_unit_and_face_camera(native):
    cfg, ext = scenes.mandelbulb_primary(160, 120)
    gpu, _ = native.trace_primary(cfg, ext)
    hit = gpu["hit"] > 0
    n = gpu["normal"][hit]
    assert np.allclose(np.linalg.norm(n, axis=-1), 1.0, atol=1e-4)
    # camera looks along +z from (0,0,-3): visible normals point back toward it
    assert (n[:, 2] < 0.2).mean() > 0.95


def test_reference_scene_primary_matches_oracle(native):
    """A reference built-in scene (sdf_id Mandelbox fractal, FPT march rule)."""
    from fractalpathtracer_gb300 import ffi
    cfg = ffi.default_config()
    cfg.width, cfg.height = 96, 72
    cfg.sdf_id = ffi.SDF_MANDELBOX_FRACTAL
    cfg.camera_position[:] = [0.5, 0.4, -4.5]
    cfg.set_values[2] = -1.0
    gpu, _ = native.trace_primary(cfg, None)
    ref = oracle.trace_primary(cfg, None, fp64=True)
    agree, derr, ang, both = _compare(gpu, ref)
    assert agree >= 0.98
    assert both.sum() > 100
    assert np.percentile(derr, 95) <= 1e-3
