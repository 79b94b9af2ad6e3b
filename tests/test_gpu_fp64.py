"""FP64 hit-point continuation for deep-zoom cameras.

A camera 1e-3 off the power-8 Mandelbulb with a 0.05-degree field of view
puts the hit threshold (~1e-10) far below the FP32 resolution of the hit
position (~1e-7), so the FP32 march stops where its steps no longer move
the position.  With fp64_bisection the ray continues in FP64; hit distances
then match the FP64 oracle to 1e-9 (p99, absolute), at least 10x closer
than the FP32 march alone.
"""
import numpy as np
import pytest

import oracle
from fractalpathtracer_gb300 import scenes

pytestmark = pytest.mark.gpu


def _deep_zoom_camera():
    """Eye 1e-3 in front of the surface along a fixed off-axis ray from (0, 0, -3), found by an FP64 march with
    the oracle's distance estimator."""
    cfg, ext = scenes.mandelbulb_primary(8, 8)
    d = np.array([0.21, 0.13, 1.0])
    d /= np.linalg.norm(d)
    o = np.array([0.0, 0.0, -3.0])
    t = 0.0
    for _ in range(1000):
        de = oracle.sample_distance(cfg, ext, np.array([[*(o + d * t), 0.0]], np.float32), fp64=True)[0, 0]
        if de < max(t * 1e-7, 1e-9):
            break
        t += 0.99 * de
    eye = o + d * (t - 1e-3)
    return tuple(eye), tuple(eye + d)


def test_fp64_continuation_matches_fp64_oracle(native):
    eye, target = _deep_zoom_camera()
    cfg, ext64 = scenes.mandelbulb_deep_zoom(eye, target, 48, 36, fp64=True)
    _, ext32 = scenes.mandelbulb_deep_zoom(eye, target, 48, 36, fp64=False)
    ref = oracle.trace_primary(cfg, ext64, fp64=True)
    g64, _ = native.trace_primary(cfg, ext64)
    g32, _ = native.trace_primary(cfg, ext32)
    hit_r = ref[..., 5] > 0
    assert hit_r.mean() > 0.9
    both = hit_r & (g64["hit"] > 0)
    assert both.mean() > 0.9 * hit_r.mean()
    err64 = np.abs(g64["distance"][both].astype(np.float64) - ref[..., 0][both])
    b32 = hit_r & (g32["hit"] > 0)
    err32 = np.abs(g32["distance"][b32].astype(np.float64) - ref[..., 0][b32]) if b32.any() else np.array([np.inf])
    p64, p32 = np.percentile(err64, 99), np.percentile(err32, 99)
    print(f"deep zoom: t ~ {ref[..., 0][hit_r].mean():.3e}, FP32 hits {b32.mean():.3f} p99 err {p32:.3e}; "
          f"FP64 hits {both.mean():.3f} p99 err {p64:.3e}")
    assert p64 <= 1e-9
    assert p32 >= 10 * p64
