"""GPU renders at the workloads' own sizes against the CPU oracle.

The oracle is too slow for whole 1080p frames at 16 spp, so each full-size GPU
frame is compared on bands of rows the oracle renders at the same seed
(identical per-path random numbers): the band of the GPU's accumulation and
the oracle's band are presented the same way and compared with the
reference's image metrics (src/metal_bridge.mm:2383-2495: MAE and RMSE on
8-bit output, 8x8 luminance SSIM, 64x64 low-frequency SSIM).

On fractal surfaces a path amplifies rounding: a hit point that moves by an
ulp changes the normal, the bounce direction and the rest of the path.  The
oracle's own FP32 and FP64 renders of a 1080p Mandelbulb band at 16 spp
differ by MAE 1.52 (SSIM 0.979), of the Mandelbox by MAE 1.88.  So the fractal
scenes are gated relative to that: per band, the GPU's distance from the FP32
oracle may exceed the oracle's own FP32-vs-FP64 distance r by at most 25%
(MAE <= 1.25 r + 0.25, RMSE <= 1.25 r + 1, 1 - SSIM <= 1.5 (1 - SSIM_r) + 0.005,
1 - LF-SSIM <= 1.5 (1 - LF-SSIM_r) + 0.002).  The surrogate modes move primary hit points by
ulps (their positions come from other step sequences), which is a second,
independent rounding perturbation of every path: against the FP32 oracle they
get twice the room (MAE <= 1.75 r + 0.25, 1 - SSIM <= 2 (1 - SSIM_r) + 0.005),
and against the GPU's plain render the single one.  Scenes whose
paths do not amplify rounding (the Menger fold with its plane, the voxel path,
the HDRI world) meet absolute gates close to zero.  The voxel DDA at 1024^3
and 1920x1080 is compared bit for bit on bands of rows.
"""
import ctypes

import numpy as np
import pytest

import oracle
from fractalpathtracer_gb300 import ffi, native_ext as nx, scenes

pytestmark = pytest.mark.gpu

GATE = {"mae": 1.5, "rmse": 8.0, "ssim": 0.95, "lf_ssim": 0.99}


def _copy(s):
    out = type(s)()
    ctypes.memmove(ctypes.byref(out), ctypes.byref(s), ctypes.sizeof(s))
    return out


def band_metrics(cfg, lin, acc, y0, y1):
    """Metrics of rows [y0, y1) (accumulation order, row 0 at the bottom) of two accumulations."""
    band = _copy(cfg)
    band.height = y1 - y0
    a = oracle.present(band, np.ascontiguousarray(lin[y0:y1]))
    b = oracle.present(band, np.ascontiguousarray(acc[y0:y1]))
    return oracle.image_metrics(a, b)


def check_bands(cfg, lin, acc, bands, gate=GATE, label=""):
    worst = {}
    for y0, y1 in bands:
        m = band_metrics(cfg, lin, acc, y0, y1)
        print(label, (y0, y1), {k: round(v, 4) for k, v in m.items()})
        assert m["mae"] <= gate["mae"], (label, y0, m)
        assert m["rmse"] <= gate["rmse"], (label, y0, m)
        assert m["ssim"] >= gate["ssim"], (label, y0, m)
        assert m["lf_ssim"] >= gate["lf_ssim"], (label, y0, m)
        for k, v in m.items():
            worst[k] = max(worst.get(k, v), v) if k in ("mae", "rmse", "max_abs") else min(worst.get(k, v), v)
    return worst


def oracle_bands(cfg, ext, bands, fp64=False):
    acc = np.zeros((cfg.height, cfg.width, 4), np.float32)
    for y0, y1 in bands:
        a, _ = oracle.render(cfg, ext, rows=(y0, y1), fp64=fp64)
        acc[y0:y1] = a[y0:y1]
    return acc


def check_bands_relative(cfg, lin, acc32, acc64, bands, label="", factor=1.25, ssim_factor=1.5):
    """Per band: the distance of `lin` from `acc32` within `factor` times the oracle's own FP32-vs-FP64
    distance (acc32 vs acc64)."""
    for y0, y1 in bands:
        m = band_metrics(cfg, lin, acc32, y0, y1)
        r = band_metrics(cfg, acc32, acc64, y0, y1)
        print(label, (y0, y1), "gpu", {k: round(v, 4) for k, v in m.items()},
              "fp32-vs-fp64", {k: round(v, 4) for k, v in r.items()})
        assert m["mae"] <= factor * r["mae"] + 0.25, (label, y0, m, r)
        assert m["rmse"] <= factor * r["rmse"] + 1.0, (label, y0, m, r)
        assert 1.0 - m["ssim"] <= ssim_factor * (1.0 - r["ssim"]) + 0.005, (label, y0, m, r)
        assert 1.0 - m["lf_ssim"] <= ssim_factor * (1.0 - r["lf_ssim"]) + 0.002, (label, y0, m, r)


C2_BANDS = [(120, 136), (352, 368), (568, 584)]
C5_BANDS = [(300, 316), (532, 548), (780, 796)]


def test_c2_menger_plane_1280x720_16spp(native):
    """Menger fold (5 iterations, scale 3) with the ground plane, 1280x720 16 spp 4 bounces, RR after 2,
    Lambert 0.7 + GGX 0.3, the seeded 512x256 RGBE sky, PCG seed 1 (measured: MAE <= 0.011, SSIM >= 0.9999)."""
    b = scenes.menger_plane(1280, 720, 16)
    lin, _, _ = native.cuda_render(b.cfg, b.ext)
    acc = oracle_bands(b.cfg, b.ext, C2_BANDS)
    check_bands(b.cfg, lin, acc, C2_BANDS, gate={"mae": 0.1, "rmse": 1.5, "ssim": 0.999, "lf_ssim": 0.9999}, label="C2")


@pytest.fixture(scope="module")
def bulb_1080p():
    b = scenes.mandelbulb_path(1920, 1080, 16)
    return b, oracle_bands(b.cfg, b.ext, C5_BANDS), oracle_bands(b.cfg, b.ext, C5_BANDS, fp64=True)


@pytest.fixture(scope="module")
def bulb_model(native):
    b = scenes.mandelbulb_path(64, 64, 1)
    lo, hi = scenes.SURROGATE_BOXES["mandelbulb"]
    model, _ = nx.mlp_create(b.cfg, b.ext, nx.mlp_config(lo, hi, points=1 << 20, steps=800, batch=8192, seed=1))
    yield model
    nx.mlp_destroy(model)


def test_c5_mandelbulb_plain_1080p_16spp(native, bulb_1080p):
    b, acc, acc64 = bulb_1080p
    lin, _, _ = native.cuda_render(b.cfg, b.ext)
    check_bands_relative(b.cfg, lin, acc, acc64, C5_BANDS, label="C5 plain")


@pytest.mark.parametrize("mode", [1, 2])
def test_c5_mandelbulb_surrogate_1080p_16spp(native, bulb_1080p, bulb_model, mode):
    """The surrogate-skip march (mode 1) and the box clip alone (mode 2) render the plain march's image."""
    b, acc, acc64 = bulb_1080p
    plain, _, _ = native.cuda_render(b.cfg, b.ext)
    e = _copy(b.ext)
    e.surrogate, e.surrogate_model = mode, bulb_model
    lin, _, _ = native.cuda_render(b.cfg, e)
    check_bands_relative(b.cfg, lin, acc, acc64, C5_BANDS, label=f"C5 surrogate {mode} vs oracle", factor=1.75,
                         ssim_factor=2.0)
    # against the GPU's plain render: one rounding perturbation (the reference distance is still FP32 vs FP64)
    for y0, y1 in C5_BANDS:
        m = band_metrics(b.cfg, lin, plain, y0, y1)
        r = band_metrics(b.cfg, acc, acc64, y0, y1)
        print(f"C5 surrogate {mode} vs plain", (y0, y1), {k: round(v, 4) for k, v in m.items()})
        assert m["mae"] <= 1.25 * r["mae"] + 0.25 and 1.0 - m["ssim"] <= 1.5 * (1.0 - r["ssim"]) + 0.005, (m, r)


def test_c5_mandelbox_plain_and_skip_1080p_16spp(native):
    b = scenes.mandelbox_path(1920, 1080, 16)
    acc = oracle_bands(b.cfg, b.ext, C5_BANDS)
    acc64 = oracle_bands(b.cfg, b.ext, C5_BANDS, fp64=True)
    lin, _, _ = native.cuda_render(b.cfg, b.ext)
    check_bands_relative(b.cfg, lin, acc, acc64, C5_BANDS, label="C5 box plain")
    lo, hi = scenes.SURROGATE_BOXES["mandelbox"]
    model, _ = nx.mlp_create(b.cfg, b.ext, nx.mlp_config(lo, hi, points=1 << 20, steps=800, batch=8192, seed=1))
    try:
        e = _copy(b.ext)
        e.surrogate, e.surrogate_model = 1, model
        lin_s, _, _ = native.cuda_render(b.cfg, e)
    finally:
        nx.mlp_destroy(model)
    check_bands_relative(b.cfg, lin_s, acc, acc64, C5_BANDS, label="C5 box skip vs oracle", factor=1.75, ssim_factor=2.0)
    for y0, y1 in C5_BANDS:
        m = band_metrics(b.cfg, lin_s, lin, y0, y1)
        r = band_metrics(b.cfg, acc, acc64, y0, y1)
        print("C5 box skip vs plain", (y0, y1), {k: round(v, 4) for k, v in m.items()})
        assert m["mae"] <= 1.25 * r["mae"] + 0.25 and 1.0 - m["ssim"] <= 1.5 * (1.0 - r["ssim"]) + 0.005, (m, r)


def test_c3_every_batched_scene(native):
    """All 64 scenes of the batched workload (one persistent launch per sample, CUDA graph replay) against
    the oracle's render of each scene alone: a 16-row band through the middle of every scene."""
    bundles = scenes.batch_scenes(64)
    lins, _, st = nx.render_batch(bundles)
    assert st["scenes"] == 64
    for k, b in enumerate(bundles):
        h = b.cfg.height
        band = [(h // 2 - 8, h // 2 + 8)]
        acc = oracle_bands(b.cfg, b.ext, band)
        acc64 = oracle_bands(b.cfg, b.ext, band, fp64=True)
        check_bands_relative(b.cfg, lins[k], acc, acc64, band, label=f"C3 scene {k}")


def test_c4_voxel_1024_1080p_primary_shadow_bit_exact(native):
    """1024^3 Mandelbox occupancy bricks, 1920x1080 primary + shadow rays: hit distance, cell, lit flag and the
    step counts of both rays equal the oracle's DDA through the same grid on five bands of rows."""
    cfg, ext = scenes.voxel_mandelbox(1024, 1920, 1080)
    info = nx.voxel_build(cfg, ext, 8)
    t, o, _, _ = nx.voxel_read(info, distance=False)
    hits, _, _ = nx.voxel_render(cfg, ext, image=False)
    for y0 in (0, 270, 536, 800, 1072):
        rows = (y0, y0 + 8)
        ref = oracle.voxel_primary(cfg, ext, t, o, rows=rows)[y0:y0 + 8]
        got = hits[y0:y0 + 8]
        assert np.array_equal(got["t"], ref[..., 0].astype(np.float32)), y0
        hit = got["t"] >= 0
        assert np.array_equal(got["cell"][hit].astype(np.float64), ref[..., 1][hit]), y0
        assert np.array_equal(got["lit"].astype(np.float64), ref[..., 2]), y0
        assert np.array_equal(got["steps"].astype(np.float64), ref[..., 3]), y0
        assert np.array_equal(got["shadow_steps"].astype(np.float64), ref[..., 4]), y0
    assert (hits["t"] >= 0).mean() > 0.05


def _voxel_scene(kind, offset_mode):
    if kind == "sphere":
        from tests.test_voxel_cpu import sphere_program
        cfg = sphere_program(48)
        cfg.width, cfg.height, cfg.samples = 96, 72, 4
        cfg.camera_position[:] = [0.0, 0.5, -4.0]
    else:
        cfg = ffi.default_config()
        cfg.sdf_id = ffi.SDF_MANDELBOX_FRACTAL
        cfg.voxel_resolution = 128
        cfg.voxel_bounds_min[:] = [-4.0, -4.0, -4.0]
        cfg.voxel_bounds_max[:] = [4.0, 4.0, 4.0]
        cfg.voxel_surface_band = 1.0
        cfg.width, cfg.height, cfg.samples = 160, 120, 4
        scenes.look_at(cfg, (5.5, 4.0, -9.0), (0.0, 0.0, 0.0))
    cfg.renderer_backend = ffi.RENDERER_VOXEL
    cfg.voxel_storage = ffi.VOXEL_STORAGE_SPARSE_BRICKS
    cfg.voxel_offset_mode = offset_mode
    cfg.sun[0] = 1.0
    return cfg


@pytest.mark.parametrize("kind", ["sphere", "mandelbox"])
@pytest.mark.parametrize("offset_mode", [0, 1])
def test_voxel_path_render_matches_oracle(native, tmp_path, kind, offset_mode):
    """The drop-in voxel renderer (fpt_metal_render, voxel backend: build + renderVoxelPath) against the
    oracle's restatement of renderVoxelPath (shaders/Shaders.metal:6526-6621) over the oracle's own build of
    the same cells, legacy and precision ray-origin offsets."""
    cfg = _voxel_scene(kind, offset_mode)
    res = native.metal_render(cfg, str(tmp_path / "v.png"))
    table, _, _, cells, _ = oracle.voxel_build(cfg, None, 4)
    acc = oracle.voxel_render(cfg, None, table, cells, 4)
    m = band_metrics(cfg, res["linear"], acc, 0, cfg.height)
    print(kind, offset_mode, m)
    # measured: identical images, or one pixel in 20,000 off by a few levels
    assert m["mae"] <= 0.05 and m["rmse"] <= 1.0 and m["ssim"] >= 0.9999 and m["lf_ssim"] >= 0.99999, m
    assert res["voxel_active_cells"] > 0


def test_voxel_unsupported_modes_fail_loudly(native, tmp_path):
    from fractalpathtracer_gb300.native import NativeError
    for field, value, msg in (("voxel_normal_mode", 2, "normal mode"), ("voxel_material_mode", 1, "material mode"),
                              ("voxel_leaf_refinement", 1, "leaf refinement"), ("voxel_coverage_mode", 1, "coverage")):
        cfg = _voxel_scene("sphere", 0)
        setattr(cfg, field, value)
        with pytest.raises(NativeError, match=msg):
            native.metal_render(cfg, str(tmp_path / "x.png"))


def test_hdri_world_mode_2_render(native, tmp_path):
    """World mode 2: the bridge hydrates the 32x16 LUT from a Radiance file written here and the kernels
    sample it (shaders/Shaders.metal:5795-5821); the oracle renders the same scene from its own LUT."""
    path = str(tmp_path / "sky.hdr")
    sky = scenes.sky_equirect(256, 128, (0.3, 0.8, 0.5), 7)
    scenes.write_rgbe_file(path, scenes.rgbe_encode(sky))
    cfg = ffi.default_config()
    cfg.sdf_id = ffi.SDF_GLASS_BALL
    cfg.width, cfg.height, cfg.samples = 96, 72, 8
    cfg.camera_position[:] = [0.0, 0.1, -3.0]
    cfg.world[0] = 2.0
    cfg.hdri_enabled = 1
    p = path.encode()
    ctypes.memmove(ctypes.addressof(cfg) + type(cfg).hdri_path.offset, p + b"\0", len(p) + 1)
    res = native.metal_render(cfg, str(tmp_path / "h.png"))
    ref_cfg = _copy(cfg)
    lut = oracle.hdri_lut(path)
    assert np.array_equal(lut, native.hdri_lut(path))
    ctypes.memmove(ctypes.addressof(ref_cfg) + type(ref_cfg).hdri_lut.offset, lut.ctypes.data, lut.nbytes)
    ref_cfg.hdri_width, ref_cfg.hdri_height = 32, 16
    acc, _ = oracle.render(ref_cfg, None)
    m = band_metrics(cfg, res["linear"], acc, 0, cfg.height)
    print("hdri", m)
    # measured: MAE 0.003, SSIM 0.99996
    assert m["mae"] <= 0.1 and m["rmse"] <= 1.5 and m["ssim"] >= 0.999 and m["lf_ssim"] >= 0.9999, m
    # the environment is really the file's: a world-mode-1 render of the same scene differs
    cfg.world[0] = 1.0
    res1 = native.metal_render(cfg, str(tmp_path / "s.png"))
    assert not np.allclose(res1["linear"], res["linear"])
