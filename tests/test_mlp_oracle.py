"""CPU checks of the surrogate network's FP64 restatement (the gradient oracle).

The oracle's analytic gradients are pinned against central finite
differences of its own loss (FP64, no BF16 rounding); the boxes used by the
skip march are checked to hold each scene's surface.
"""
import numpy as np

import oracle
from fractalpathtracer_gb300 import scenes

BOX = scenes.SURROGATE_BOXES["mandelbulb"]


def _points(n, seed=3):
    rng = np.random.default_rng(seed)
    p = np.zeros((n, 4), np.float32)
    p[:, :3] = rng.uniform(-1.2, 1.2, (n, 3))
    p[:, 3] = rng.uniform(-0.05, 0.6, n)
    return p


def test_oracle_gradients_match_finite_differences():
    params = scenes.random_mlp_params(1)
    pts = _points(12)
    g, loss = oracle.mlp_gradients(params, *BOX, pts, overestimate_weight=10.0, emulate_bf16=False)
    assert np.isfinite(g).all() and loss > 0
    rng = np.random.default_rng(7)
    # indices in every block: W0 (live columns), b0, W1, b1, W2, b2, W3, b3, W4, b4
    blocks = [(0, 7168), (7168, 7232), (7232, 11328), (11328, 11392), (11392, 15488), (15488, 15552), (15552, 19648),
              (19648, 19712), (19712, 19776), (19776, 19777)]
    idx = []
    for a, b in blocks:
        cand = np.arange(a, b)
        if a == 0:
            cand = cand[(cand % 112) < 99]
        idx += list(rng.choice(cand, size=min(4, len(cand)), replace=False))
    for i in idx:
        h = max(1e-3 * abs(float(params[i])), 1e-3)
        pp, pm = params.copy(), params.copy()
        pp[i] += np.float32(h)
        pm[i] -= np.float32(h)
        lp = oracle.mlp_gradients(pp, *BOX, pts, 10.0, emulate_bf16=False)[1]
        lm = oracle.mlp_gradients(pm, *BOX, pts, 10.0, emulate_bf16=False)[1]
        fd = (lp - lm) / (float(pp[i]) - float(pm[i]))
        assert abs(fd - g[i]) <= 2e-5 * max(1.0, abs(g[i])) + 1e-4 * abs(g[i]), (i, fd, g[i])


def test_oracle_forward_loss_consistent():
    params = scenes.random_mlp_params(2)
    pts = _points(64)
    out = oracle.mlp_forward(params, *BOX, pts, emulate_bf16=False)
    scale = 1.25
    y = pts[:, 3].astype(np.float64) / scale
    e = out / scale - y
    w = np.where(e > 0, 10.0, 1.0)
    _, loss = oracle.mlp_gradients(params, *BOX, pts, 10.0, emulate_bf16=False)
    assert abs(loss - (w * e * e).mean()) <= 1e-5 * loss + 1e-7
    # BF16 storage moves the output only slightly
    out_bf = oracle.mlp_forward(params, *BOX, pts, emulate_bf16=True)
    assert np.abs(out_bf - out).max() <= 0.03 * (np.abs(out).max() + 0.1)


def test_surrogate_boxes_hold_the_surfaces():
    for name, bundle in (("mandelbulb", scenes.mandelbulb_primary(8, 8)), ("mandelbox", tuple(scenes.mandelbox_path(8, 8, 1, 1)))):
        cfg, ext = bundle
        lo, hi = scenes.SURROGATE_BOXES[name]
        g = np.linspace(lo[0], hi[0], 41, dtype=np.float32)
        faces = []
        for ax in range(3):
            for s in (lo[ax], hi[ax]):
                a, b = np.meshgrid(g, g)
                p = np.zeros((a.size, 4), np.float32)
                rest = [i for i in range(3) if i != ax]
                p[:, ax] = s
                p[:, rest[0]], p[:, rest[1]] = a.ravel(), b.ravel()
                faces.append(p)
        d = oracle.sample_distance(cfg, ext, np.concatenate(faces), fp64=True)[:, 0]
        assert d.min() > 0.05, (name, d.min())
