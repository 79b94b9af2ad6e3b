"""Batch distance samples on the GPU vs the FP64 oracle.

Gate of the reference's mandel-parity command (src/main.rs:3297,
3356-3361): |d_gpu - d_fp64| <= 5e-5 * (1 + |d_fp64|), p99 within the
gate, outlier fraction <= 2e-4 (here 1e-3 for the FP32 algebraic form of
the power-8 step against the FP64 trigonometric form).
"""
import numpy as np
import pytest

import oracle
from fractalpathtracer_gb300 import ffi, scenes

pytestmark = pytest.mark.gpu


def pts(n, lo, hi, seed=11):
    p = np.random.default_rng(seed).uniform(lo, hi, (n, 4)).astype(np.float32)
    p[:, 3] = 0
    return p


def _gate(d_gpu, d_ref, outliers=1e-3):
    err = np.abs(d_gpu - d_ref) / (1 + np.abs(d_ref))
    assert np.percentile(err, 99) <= 5e-5, np.percentile(err, 99)
    assert np.mean(err > 5e-5) <= outliers, np.mean(err > 5e-5)


def test_mandelbulb_field(native):
    cfg, ext = scenes.mandelbulb_primary(8, 8)
    p = pts(1 << 16, -1.5, 1.5)
    g = native.sample_distance(cfg, ext, p)
    r = oracle.sample_distance(cfg, ext, p, fp64=True)
    _gate(g[:, 0], r[:, 0])
    assert np.mean(g[:, 3] == r[:, 3]) > 0.999   # iteration counts


def test_mandelbox_field(native):
    b = scenes.mandelbox_path(8, 8, 1)
    p = pts(1 << 16, -4, 4)
    g = native.sample_distance(b.cfg, b.ext, p)
    r = oracle.sample_distance(b.cfg, b.ext, p, fp64=True)
    _gate(g[:, 0], r[:, 0])


def test_reference_ifs_field_sample(native):
    """fpt_mandelbulber_sample_field with the built-in Kaleidoscopic IFS (shaders/Shaders.metal:901-954)."""
    cfg = ffi.default_config()
    cfg.sdf_id = ffi.SDF_MANDELBULBER
    s = cfg.set_values
    s[0], s[1], s[2], s[3] = 1.0, 12.0, 10.0, 2.0
    s[4], s[5] = 7.0, 7.0                      # abs xyz, three fold planes
    s[6], s[7], s[8] = 1.0, 1.0, 1.0
    dirs = [(1, -1, 0), (0, 1, -1), (1, 0, -1)]
    for k, d in enumerate(dirs):
        n = np.array(d, float) / np.linalg.norm(d)
        s[12 + 3 * k:15 + 3 * k] = list(n)
    p = pts(1 << 15, -2, 2)
    g = native.sample_field(cfg, p)
    r = oracle.field_sample(cfg, None, p, fp64=True)
    _gate(g[:, 0], r[:, 0])
    assert np.mean(g[:, 3] == r[:, 3]) > 0.999


def test_analytic_gradient_matches_fp64(native):
    cfg, ext = scenes.mandelbulb_primary(8, 8)
    p = pts(4096, -1.3, 1.3)
    _, gg = native.sample_distance(cfg, ext, p, gradients=True)
    _, gr = oracle.sample_distance(cfg, ext, p, fp64=True, gradients=True)
    ng = np.linalg.norm(gg, axis=1)
    nr = np.linalg.norm(gr, axis=1)
    ok = (nr > 1e-6) & np.isfinite(ng)
    cosang = (gg[ok] * gr[ok]).sum(1) / (ng[ok] * nr[ok])
    assert np.percentile(np.degrees(np.arccos(np.clip(cosang, -1, 1))), 99) < 0.5


# Mandelbulbs of power 2.29, 10.6, 2.89, 5.24, 7.93; Mandelboxes; hybrids of 5, 12 and 16 iterations.
@pytest.mark.parametrize("k", [11, 14, 21, 27, 30, 1, 9, 12, 0, 3, 4])
def test_batch_scene_fields(native, k):
    """The formulas of the batched workload against the FP64 oracle: Mandelbulbs of non-integer power (the
    trigonometric step of orbit.rs:766-778), Mandelboxes of other scales, the bulb / Menger hybrid, with
    4-16 iterations (scene k of scenes.batch_scene)."""
    b = scenes.batch_scene(k)
    p = pts(1 << 15, -1.6 if b.ext.formula != ffi.FORMULA_MANDELBOX else -4.0,
            1.6 if b.ext.formula != ffi.FORMULA_MANDELBOX else 4.0, seed=20 + k)
    g = native.sample_distance(b.cfg, b.ext, p)
    r = oracle.sample_distance(b.cfg, b.ext, p, fp64=True)
    print(k, b.ext.formula, b.ext.power, b.ext.iterations,
          np.percentile(np.abs(g[:, 0] - r[:, 0]) / (1 + np.abs(r[:, 0])), 99))
    _gate(g[:, 0], r[:, 0], outliers=5e-3)
    assert np.mean(g[:, 3] == r[:, 3]) > 0.99   # iteration counts


def test_mandelbulb_power2_triplex_field(native):
    """Mandelbulber formula 3, the quadratic triplex of orbit.rs:752-764 (known answer pinned on the CPU at
    orbit.rs:1866-1874), marched as a scene: GPU field and analytic gradient against the FP64 oracle."""
    cfg, ext = scenes.mandelbulb_primary(8, 8)
    ext.formula = ffi.FORMULA_MANDELBULB_POWER2
    ext.iterations = 10
    ext.bailout = 4.0
    p = pts(1 << 16, -1.6, 1.6, seed=5)
    g, gg = native.sample_distance(cfg, ext, p, gradients=True)
    r, gr = oracle.sample_distance(cfg, ext, p, fp64=True, gradients=True)
    _gate(g[:, 0], r[:, 0])
    assert np.mean(g[:, 3] == r[:, 3]) > 0.999
    ng, nr = np.linalg.norm(gg, axis=1), np.linalg.norm(gr, axis=1)
    ok = (nr > 1e-6) & np.isfinite(ng) & (np.abs(r[:, 0]) > 1e-3)
    cosang = (gg[ok] * gr[ok]).sum(1) / (ng[ok] * nr[ok])
    assert np.percentile(np.degrees(np.arccos(np.clip(cosang, -1, 1))), 99) < 0.5
