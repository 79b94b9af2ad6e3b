"""Batched scenes: many scenes of uneven size and iteration count in one
render (persistent passes over all scenes, one CUDA graph per spp pass).

Batching changes no path: each scene's accumulation buffer equals, bit for
bit, a batch holding that scene alone.  Against its own fpt_cuda_render
(checked against the CPU oracle in test_gpu_render.py) a scene agrees on
>= 70% of pixels bit for bit (measured 82-84% at 4 spp), with MAE <= 2 and
LF-SSIM >= 0.99 on the 8-bit image: the two renders run different
instantiations of the same code (runtime formula dispatch vs one formula per
kernel), FMA contraction follows the inlining context, and a path whose
throughput or direction rounds differently leaves its pixel's sample noise
changed.  Mandelbox scenes come out bit-identical; the differences are in
the Mandelbulb / Menger hybrids.  The 64-scene workload (scene k seeded by k) runs with the
autotuner's launch shape.
"""
import numpy as np
import pytest

from fractalpathtracer_gb300 import native_ext as nx
from fractalpathtracer_gb300 import scenes

pytestmark = pytest.mark.gpu


def _close_to_single(native, b, lin_k, img_k):
    import oracle
    single, rgba, _ = native.cuda_render(b.cfg, b.ext, linear=True)
    same = np.all(lin_k == single, axis=-1).mean()
    return same, oracle.image_metrics(img_k, rgba)


def test_batch_equals_scene_alone(native):
    bundles = [scenes.batch_scene(k) for k in range(6)]
    lin, img, st = nx.render_batch(bundles, linear=True, rgba=True)
    assert st["scenes"] == 6 and st["passes"] == 4 and st["graph_launches"] == 4
    for k in (0, 3, 5):
        alone, alone_img, _ = nx.render_batch([bundles[k]], linear=True, rgba=True)
        assert np.array_equal(lin[k], alone[0]), k
        assert np.array_equal(img[k], alone_img[0]), k
    for k, b in enumerate(bundles):
        same, m = _close_to_single(native, b, lin[k], img[k])
        print(f"scene {k}: identical pixels {same:.4f}, {m}")
        assert same >= 0.7 and m["mae"] <= 2.0 and m["lf_ssim"] >= 0.99, (k, same, m)


def test_batch_mixed_bounces_and_sizes(native):
    bundles = [scenes.batch_scene(k, spp=2, bounces=1 + k % 3) for k in (3, 17, 40)]
    lin, img, st = nx.render_batch(bundles, rgba=True)
    for k, b in enumerate(bundles):
        same, m = _close_to_single(native, b, lin[k], img[k])
        print(f"scene {k}: identical pixels {same:.4f}, {m}")
        assert same >= 0.7 and m["mae"] <= 2.0 and m["lf_ssim"] >= 0.95, (k, same, m)   # 2 spp: noisier


def test_batch_rejects_mixed_sample_counts(native):
    a, b = scenes.batch_scene(0, spp=2), scenes.batch_scene(1, spp=4)
    with pytest.raises(native.NativeError, match="same sample count"):
        nx.render_batch([a, b])


def test_batch_64_scenes_autotuned(native):
    bundles = scenes.batch_scenes(64)
    tune = nx.autotune_batch(bundles, rounds=2)
    print("autotune:", tune)
    assert len(tune["tried"]) >= 4 and 0 <= tune["chosen"] < len(tune["tried"])
    _, _, st = nx.render_batch(bundles, linear=False)
    print("batch:", st, "Mpaths/s", st["paths"] / st["elapsed_ms"] / 1e3)
    assert st["tuned"] == 1 and st["workload_key"] == tune["workload_key"]
    assert st["paths"] == sum(b.cfg.width * b.cfg.height * 4 for b in bundles)
    assert st["elapsed_ms"] > 0
