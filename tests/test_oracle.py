"""The CPU oracle pinned against the reference's known answers (no GPU).

Fixtures in tests/golden come from the reference's own tests
(src/mandelbulber/orbit.rs:1866-1960; shaders/Shaders.metal:5164-5211).
"""
import json
import math
import os

import numpy as np
import pytest

from fractalpathtracer_gb300 import ffi, scenes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _orbit_ext(case):
    e = ffi.FptCudaSceneExt()
    if case["formula"] == "mandelbulb":
        e.formula = ffi.FORMULA_MANDELBULB
        e.power = case["power"]
    elif case["formula"] == "mandelbulb_power2":
        e.formula = ffi.FORMULA_MANDELBULB_POWER2
    else:
        e.formula = ffi.FORMULA_MANDELBOX
        e.box_scale = case["scale"]
        e.box_fold_limit = case["folding_limit"]
        e.box_fold_value = case["folding_value"]
        e.box_fixed_radius = case["fixed_radius"]
        e.box_min_radius = case["minimum_radius"]
    return e


def test_orbit_known_answers(oracle_lib):
    data = json.load(open(os.path.join(GOLDEN, "orbit_known_answers.json")))
    for case in data["cases"]:
        out = oracle_lib.orbit_step(_orbit_ext(case), case["point"], iterations=1, bailout=1e300, add_c=False)
        z, dr = out[:4], out[4]
        tol = case["tolerance"]
        exp = case["expect"]
        assert abs(dr - exp["derivative"]) < tol, case["name"]
        if "length" in exp:
            assert abs(math.sqrt((z ** 2).sum()) - exp["length"]) < tol, case["name"]
        if "z" in exp:
            assert np.allclose(z, exp["z"], atol=tol, rtol=0), case["name"]
        if "color" in exp:
            assert abs(out[9] - exp["color"]) < tol, case["name"]


def test_logarithmic_finalizer_edges(oracle_lib):
    # orbit.rs:648-660: r <= 1 gives 0; the point is inside the bulb at the origin.
    cfg, ext = scenes.mandelbulb_primary(8, 8)
    out = oracle_lib.sample_distance(cfg, ext, np.array([[0, 0, 0, 0]], np.float32))
    assert out[0, 0] == 0.0
    far = oracle_lib.sample_distance(cfg, ext, np.array([[0, 0, -3, 0]], np.float32))
    assert far[0, 0] > 1.0 and np.isfinite(far[0, 0])


def test_menger_fold_sign(oracle_lib):
    b = scenes.menger_plane(16, 16, 1)
    ext = b.ext
    ext.ground_plane = 0
    pts = np.array([[0, 0, 0, 0], [0.95, 0.95, 0.95, 0], [3, 0, 0, 0]], np.float32)
    d = oracle_lib.sample_distance(b.cfg, ext, pts)[:, 0]
    assert d[0] > 0      # central tunnel is empty
    assert d[1] < 0      # corner cube is solid
    assert 0.5 < d[2] < 2.5


def hash_points(n, seed=7, lo=-2.0, hi=2.0):
    rng = np.random.default_rng(seed)
    p = rng.uniform(lo, hi, (n, 4)).astype(np.float32)
    p[:, 3] = 0
    return p


@pytest.mark.parametrize("which", ["bulb", "box"])
def test_fp32_port_tracks_fp64(oracle_lib, which):
    """FP32 restatement vs FP64 within the reference's field-parity gate
    (5e-5 * (1 + |d|), src/main.rs:3297)."""
    if which == "bulb":
        cfg, ext = scenes.mandelbulb_primary(8, 8)
        pts = hash_points(4000, lo=-1.5, hi=1.5)
    else:
        b = scenes.mandelbox_path(8, 8, 1)
        cfg, ext = b.cfg, b.ext
        pts = hash_points(4000, lo=-4, hi=4)
    d64 = oracle_lib.sample_distance(cfg, ext, pts, fp64=True)[:, 0]
    d32 = oracle_lib.sample_distance(cfg, ext, pts, fp64=False)[:, 0]
    err = np.abs(d64 - d32) / (1 + np.abs(d64))
    assert np.percentile(err, 99) <= 5e-5
    assert np.mean(err > 5e-5) <= 2e-3


def test_primary_trace_fp32_vs_fp64(oracle_lib):
    cfg, ext = scenes.mandelbulb_primary(64, 48)
    r64 = oracle_lib.trace_primary(cfg, ext, fp64=True)
    r32 = oracle_lib.trace_primary(cfg, ext, fp64=False)
    agree = (r64[..., 5] == r32[..., 5]).mean()
    assert agree > 0.99
    both = (r64[..., 5] > 0) & (r32[..., 5] > 0)
    assert both.sum() > 200
    err = np.abs(r64[..., 0] - r32[..., 0])[both]
    assert np.percentile(err, 99) < 5e-5


def test_image_metrics_identity_and_shift(oracle_lib):
    rng = np.random.default_rng(0)
    a = rng.integers(0, 256, (64, 80, 4), dtype=np.uint8)
    a[..., 3] = 255
    m = oracle_lib.image_metrics(a, a)
    assert m["mae"] == 0 and m["ssim"] == pytest.approx(1.0) and m["lf_ssim"] == pytest.approx(1.0)
    b = a.copy()
    b[..., :3] = np.clip(b[..., :3].astype(int) + 3, 0, 255).astype(np.uint8)
    m2 = oracle_lib.image_metrics(a, b)
    assert 2.5 < m2["mae"] <= 3.0 and m2["max_abs"] == 3


def test_present_flips_rows(oracle_lib):
    cfg = ffi.default_config()
    cfg.width, cfg.height = 4, 3
    acc = np.zeros((3, 4, 4), np.float32)
    acc[0, :, :3] = 1.0  # bottom row white in accumulation order
    img = oracle_lib.present(cfg, acc)
    assert (img[2, :, :3] >= 254).all() and (img[0, :, :3] == 0).all()
