"""Why the surrogate's box clip starts camera rays at the plain march's first step (CPU, FP64 oracle DE).

The Mandelbox's distance estimate is not a lower bound of the distance everywhere: seen from its camera,
DE(camera) exceeds the distance to surface points along many rays, so the reference march's first step
(the Mandelbulber rule of shaders/Shaders.metal:3700-3751: step d - th/2, threshold growing with the distance
to the camera) passes over that layer.  A march started at the box entry finds the layer instead (a different
hit); a march started at the plain march's first step visits the plain march's positions and finds the same
hits.  The GPU side of the rule is checked in tests/test_gpu_mlp.py::test_mandelbox_skip.
"""
import numpy as np

import oracle
from fractalpathtracer_gb300 import scenes


def _march(cfg, ext, cam, dirs, t0, k=1e-4 / 7.0, max_steps=256, max_dist=12.0):
    """Vectorised march of the Mandelbulber rule with the FP64 oracle DE; returns (t, hit)."""
    n = len(dirs)
    t = t0.astype(np.float64).copy()
    hit = np.zeros(n, bool)
    act = np.ones(n, bool)
    for _ in range(max_steps):
        idx = np.nonzero(act)[0]
        if not len(idx):
            break
        p = np.zeros((len(idx), 4), np.float32)
        p[:, :3] = cam + dirs[idx] * t[idx, None]
        d = oracle.sample_distance(cfg, ext, p, fp64=True)[:, 0]
        th = np.clip(t[idx] * k, 1e-7, 1.0)
        h = d < th
        hit[idx[h]] = True
        act[idx[h]] = False
        mv = idx[~h]
        t[mv] += np.minimum(np.maximum(d[~h] - 0.5 * th[~h], 0.0), 10.0)
        act &= t <= max_dist
    return t, hit


def test_box_entry_start_changes_hits_first_step_start_does_not():
    b = scenes.mandelbox_path(8, 8, 1, 1)
    cam = np.array([0.0, 1.5, -7.0])
    rng = np.random.default_rng(1)
    dirs = rng.uniform(-2.0, 2.0, (1500, 3)) - cam
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    lo, hi = scenes.SURROGATE_BOXES["mandelbox"]
    t0 = (np.array(lo) - cam) / dirs
    t1 = (np.array(hi) - cam) / dirs
    tn = np.maximum(np.minimum(t0, t1).max(axis=1), 0.0)
    assert (tn <= np.maximum(t0, t1).min(axis=1)).all()   # every ray meets the box
    q = np.zeros((1, 4), np.float32)
    q[0, :3] = cam
    d_cam = oracle.sample_distance(b.cfg, b.ext, q, fp64=True)[0, 0]
    s1 = max(d_cam - 0.5 * 1e-7, 0.0)   # the plain march's first step (threshold at the camera: the clamp minimum)
    t_plain, h_plain = _march(b.cfg, b.ext, cam, dirs, np.zeros(len(dirs)))
    t_entry, h_entry = _march(b.cfg, b.ext, cam, dirs, tn)
    t_first, h_first = _march(b.cfg, b.ext, cam, dirs, np.full(len(dirs), s1))
    both = h_plain & h_entry
    nearer = both & ((t_entry - t_plain) / (1 + t_plain) < -1e-3)
    print(f"DE(camera) {d_cam:.4f}; entry start finds a nearer surface on {nearer.mean():.3f} of rays")
    assert d_cam > 5.0 and nearer.mean() > 0.05          # the plain march's first step passes over surface
    assert (h_first == h_plain).all() and np.array_equal(t_first[h_plain], t_plain[h_plain])
