"""Accumulated images on the GPU vs the CPU oracle at the same seed.

Image gates follow the reference's comparison metrics
(src/metal_bridge.mm:2383-2495, 6078-6104): MAE and RMSE on 8-bit output,
8x8 luminance SSIM and 64x64 low-frequency SSIM.  Per-path random numbers
are bit-identical (hash13 seeds or PCG counters), so remaining differences
come from FP32 rounding in marching (paths that diverge at silhouettes).
"""
import numpy as np
import pytest

import oracle
from fractalpathtracer_gb300 import ffi, scenes

pytestmark = pytest.mark.gpu


def _small(cfg, w, h, spp):
    cfg.width, cfg.height, cfg.samples = w, h, spp
    return cfg


def _check(native, cfg, ext, mae=2.0, rmse=8.0, ssim=0.95, lf=0.99):
    lin, rgba, _ = native.cuda_render(cfg, ext)
    acc, _ = oracle.render(cfg, ext)
    ref = oracle.present(cfg, acc)
    # both images are presented (top row first): the library's rgba output and the oracle's present
    m = oracle.image_metrics(rgba, ref)
    assert m["mae"] <= mae, m
    assert m["rmse"] <= rmse, m
    assert m["ssim"] >= ssim, m
    assert m["lf_ssim"] >= lf, m
    return lin, acc, m


def test_cornell_default(native):
    cfg = _small(ffi.default_config(), 96, 96, 4)
    _check(native, cfg, None)


def test_glass_ball(native):
    cfg = _small(ffi.default_config(), 80, 64, 4)
    cfg.sdf_id = ffi.SDF_GLASS_BALL
    cfg.camera_position[:] = [0.0, 0.1, -3.0]
    _check(native, cfg, None, mae=3.0, rmse=12.0, ssim=0.9, lf=0.98)


@pytest.mark.parametrize("sdf", [ffi.SDF_TOWER_FRACTAL, ffi.SDF_CAGE_FRACTAL, ffi.SDF_MENGER_SPONGE])
def test_reference_fractals(native, sdf):
    cfg = _small(ffi.default_config(), 80, 60, 2)
    cfg.sdf_id = sdf
    cfg.camera_position[:] = [0.2, 0.3, -4.0]
    if sdf == ffi.SDF_MENGER_SPONGE:
        cfg.set_values[0], cfg.set_values[1] = 1.0, 3.0
    cfg.sun[0] = 1.0
    _check(native, cfg, None, mae=4.0, rmse=16.0, ssim=0.85, lf=0.97)


def test_typed_program_scene(native):
    cfg = _small(ffi.default_config(), 80, 60, 2)
    cfg.sdf_id = ffi.SDF_PROGRAM
    prog = [(ffi.OP_TRANSLATE, 0, (0.0, 0.0, 0.5, 0)), (ffi.OP_BOX, 0, (0.6, 0.4, 0.5, 0)),
            (ffi.OP_SPHERE, 2, (0.7, 0, 0, 0)), (ffi.OP_PLANE, 0, (0, 1, 0, 1.0))]
    for i, (op, flags, d) in enumerate(prog):
        cfg.sdf_program[i].opcode = op
        cfg.sdf_program[i].flags = flags
        cfg.sdf_program[i].data[:] = list(d)
    cfg.sdf_program_count = len(prog)
    cfg.camera_position[:] = [0.5, 0.8, -3.0]
    cfg.sun[0] = 1.0
    _check(native, cfg, None)


def test_menger_plane_ggx_pcg(native):
    b = scenes.menger_plane(96, 54, 4, sky_size=(64, 32))
    _check(native, b.cfg, b.ext, mae=3.0, rmse=12.0, ssim=0.9, lf=0.98)


def test_mandelbulb_path(native):
    b = scenes.mandelbulb_path(96, 54, 2)
    _check(native, b.cfg, b.ext, mae=3.0, rmse=12.0, ssim=0.9, lf=0.98)


def test_accumulation_modes_identical(native):
    """batch == chunked == per-sample (the reference's capability test runs batch vs chunked with --strict)."""
    outs = []
    for mode in (ffi.ACCUMULATION_BATCH, ffi.ACCUMULATION_CHUNKED, ffi.ACCUMULATION_PER_SAMPLE):
        cfg = _small(ffi.default_config(), 64, 48, 5)
        cfg.sdf_accumulation_mode = mode
        cfg.sdf_chunk_samples = 2
        lin, _, _ = native.cuda_render(cfg, None)
        outs.append(lin)
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


def test_one_spp_differs_from_sixteen(native):
    a = native.cuda_render(_small(ffi.default_config(), 64, 48, 1), None)[0]
    b = native.cuda_render(_small(ffi.default_config(), 64, 48, 16), None)[0]
    assert not np.array_equal(a, b)


def test_metal_render_writes_png_and_compare(native, tmp_path):
    cfg = _small(ffi.default_config(), 64, 48, 2)
    out = str(tmp_path / "a.png")
    res = native.metal_render(cfg, out)
    assert res["linear"].shape == (48, 64, 4)
    rep = native.compare_images(out, out, str(tmp_path / "r.json"))
    assert rep["mean_absolute_error"] == 0 and rep["luminance_ssim"] == 1.0


def test_invalid_size_rejected(native):
    cfg = _small(ffi.default_config(), 0, 48, 1)
    with pytest.raises(native.NativeError, match="invalid render size"):
        native.cuda_render(cfg, None)


@pytest.mark.parametrize("w,h", [(1, 1), (37, 23), (9, 5)])
def test_ragged_sizes_match_oracle(native, w, h):
    """Image sizes that do not fill the 8x4 tiles of the wavefront (and a single pixel)."""
    b = scenes.mandelbulb_path(w, h, 2, 2)
    lin, _, _ = native.cuda_render(b.cfg, b.ext, linear=True)
    ref, _ = oracle.render(b.cfg, b.ext)
    assert lin.shape == (h, w, 4)
    assert (lin[..., 3] == 1.0).all() and np.isfinite(lin).all()
    close = np.isclose(lin[..., :3], ref[..., :3], rtol=1e-3, atol=1e-4).all(-1)
    # paths that round differently on the two sides diverge; most pixels agree to FP32 rounding
    assert close.mean() >= (0.0 if w * h == 1 else 0.8), close.mean()
    assert np.abs(lin[..., :3] - ref[..., :3]).max() <= 8.0


def test_zero_bounces_is_background(native):
    """render[0] = 0: no march; every pixel takes the camera ray's background term."""
    b = scenes.mandelbulb_path(32, 24, 2, 0)
    lin, _, _ = native.cuda_render(b.cfg, b.ext, linear=True)
    ref, _ = oracle.render(b.cfg, b.ext)
    assert np.abs(lin - ref).max() <= 1e-5


def test_profile_stats(native):
    """FptSdfProfileStats of a profiled render (the counters the reference's render metadata reports,
    src/main.rs:1491-1520): per-phase march steps and orbit iterations (the normal phase included), refinement
    steps, the longest march, the most march steps of one path, and the render time apportioned by counted work
    units (src/metal_bridge.mm:5712-5733)."""
    b = scenes.mandelbulb_path(96, 64, 2, 4)
    _, _, ms, prof = native.cuda_render(b.cfg, b.ext, linear=False, profile=True)
    p = {f: getattr(prof, f) for f, _ in type(prof)._fields_}
    print({k: (list(v) if hasattr(v, "__len__") else v) for k, v in p.items()})
    assert p["primary_steps"] > 0 and p["secondary_steps"] > 0 and p["shadow_steps"] > 0
    assert 0 < p["bounces"] <= p["normal_evals"] == p["material_evals"]
    assert p["distance_evals"] == p["primary_steps"] + p["secondary_steps"] + p["shadow_steps"]
    orbit = list(prof.orbit_iterations_by_phase)
    assert p["march_orbit_iterations"] == orbit[0] + orbit[1] + orbit[2] + orbit[3] > 0
    # one analytic (dual-number) normal per hit: 1..8 orbit iterations each
    assert p["normal_evals"] <= orbit[3] <= 8 * p["normal_evals"]
    assert prof.formula_slot_iterations[0] == p["march_orbit_iterations"]
    # every evaluation runs 1..8 iterations of the power-8 Mandelbulb
    for k, steps in enumerate(("primary_steps", "secondary_steps", "shadow_steps")):
        assert p[steps] <= orbit[k] <= 8 * p[steps]
    assert 0 < p["refinement_steps"] == p["refinement_distance_evals"]
    assert 0 < p["max_ray_steps"] <= 256 + 30
    # a path's steps over all its rays (camera, bounces, shadow rays): at least its longest ray, at most 9 rays' worth
    assert p["max_ray_steps"] <= p["max_pixel_steps"] <= 9 * (256 + 30)
    est = p["primary_ms_estimate"] + p["secondary_ms_estimate"] + p["shadow_ms_estimate"] + p["normal_ms_estimate"] + \
        p["bounce_ms_estimate"]
    assert abs(est - ms) <= 1e-6 * ms + 1e-9


def test_kernel_timing_without_profile(native):
    """fpt_cuda_set_kernel_timing: per-kernel event spans in a render without profile counters (the bench's timed
    renders); without it only profile renders record them.  The image does not change."""
    from fractalpathtracer_gb300 import native_ext as nx
    b = scenes.mandelbulb_path(160, 90, 2)
    _, plain, _ = native.cuda_render(b.cfg, b.ext, linear=False)
    assert nx.render_stats()["march_ms"] == 0.0
    nx.set_kernel_timing(True)
    try:
        _, timed, _ = native.cuda_render(b.cfg, b.ext, linear=False)
        rs = nx.render_stats()
    finally:
        nx.set_kernel_timing(False)
    assert rs["march_launches"] == b.cfg.render[0] + 1 and rs["march_ms"] > 0.0 and rs["shade_ms"] > 0.0
    assert rs["march_evals"] == 0   # counts need profile statistics
    assert np.array_equal(plain, timed)


def test_loop_time_limit(native):
    """A persistent loop that reaches its time limit stops and the render reports it (no fault); with the default
    limit back, the next render is the same as before."""
    from fractalpathtracer_gb300 import native_ext as nx
    b = scenes.mandelbulb_path(960, 540, 16, 4)   # enough rays per lane for the 1024-trip check interval
    _, before, _ = native.cuda_render(b.cfg, b.ext, linear=False)
    nx.set_loop_limit(2000)   # 2 us: the loops stop at their first check after 1024 trips
    try:
        with pytest.raises(native.NativeError, match="time limit"):
            native.cuda_render(b.cfg, b.ext, linear=False)
    finally:
        nx.set_loop_limit(0)
    _, after, _ = native.cuda_render(b.cfg, b.ext, linear=False)
    assert np.array_equal(before, after)
