"""Voxel build and exact DDA on the GPU vs the CPU oracle -- bit-exact.

Brick tables, per-cell occupancy and fp16 distances, reference cells,
DDA cell sequences and primary/shadow hits must match exactly: the GPU
voxel unit and the oracle both round every float operation separately in
the same order (no fused multiply-add)."""
import numpy as np
import pytest

import oracle
from fractalpathtracer_gb300 import ffi, native_ext, scenes
from tests.test_voxel_cpu import sphere_program

pytestmark = pytest.mark.gpu


def test_reference_contract_and_brick_vs_dense(native):
    native.test_voxel_dda()     # fpt_test_voxel_dda: contract mask 0 and dense == bricks at 32^3


def test_occupancy_bricks_bit_exact_128(native):
    cfg, ext = scenes.voxel_mandelbox(128, 64, 64)
    info = native_ext.voxel_build(cfg, ext, 8)
    t, o, d, _ = native_ext.voxel_read(info)
    rt, ro, rd, _, rcells = oracle.voxel_build(cfg, ext, 8)
    assert info["active_bricks"] == int((rt > 0).sum())
    assert info["active_cells"] == rcells
    assert np.array_equal(t, rt)
    assert np.array_equal(o, ro)
    assert np.array_equal(d, rd)


def test_reference_cells_bit_exact(native):
    cfg = sphere_program(64)
    info = native_ext.voxel_build(cfg, None, 4)
    t, _, _, c = native_ext.voxel_read(info, occupancy=False, distance=False, cells=True)
    rt, _, _, rc, _ = oracle.voxel_build(cfg, None, 4)
    assert np.array_equal(t, rt)
    assert np.array_equal(c, rc)


def random_rays(n, seed=5):
    rng = np.random.default_rng(seed)
    o = rng.uniform(-6, 6, (n, 3))
    tgt = rng.uniform(-3, 3, (n, 3))
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # edge cases: axis-aligned directions, origins on the grid boundary, zero components
    d[:64] = np.eye(3)[np.arange(64) % 3] * np.where(np.arange(64) % 2, 1, -1)[:, None]
    o[64:96] = np.round(o[64:96])
    d[96:128, 1] = 0.0
    d[96:128] /= np.linalg.norm(d[96:128], axis=1, keepdims=True)
    return np.concatenate([o, d], 1).astype(np.float32)


def test_dda_sequences_bit_exact(native):
    cfg, ext = scenes.voxel_mandelbox(128, 64, 64)
    info = native_ext.voxel_build(cfg, ext, 8)
    t, o, _, _ = native_ext.voxel_read(info, distance=False)
    rays = random_rays(4096)
    cap = 3 * 128 + 3
    gh, gs, gl = native_ext.dda_sequence(rays, cap)
    rh, rs, rl = oracle.dda(cfg, 8, t, o, None, rays, cap)
    assert np.array_equal(gl, rl)
    assert np.array_equal(gs, rs)
    assert np.array_equal(gh["t"].astype(np.float64), rh[:, 0].astype(np.float32).astype(np.float64))
    assert (gh["lit"] == rh[:, 3]).all()
    assert (rh[:, 3] > 0).sum() > 100   # many rays do hit


def test_primary_and_shadow_bit_exact(native):
    cfg, ext = scenes.voxel_mandelbox(256, 320, 180)
    info = native_ext.voxel_build(cfg, ext, 8)
    t, o, _, _ = native_ext.voxel_read(info, distance=False)
    hits, rgba, _ = native_ext.voxel_render(cfg, ext)
    ref = oracle.voxel_primary(cfg, ext, t, o)
    assert (hits["t"] >= 0).sum() > 1000
    assert np.array_equal(hits["t"], ref[..., 0].astype(np.float32))
    hit = hits["t"] >= 0
    assert np.array_equal(hits["cell"][hit].astype(np.float64), ref[..., 1][hit])
    assert np.array_equal(hits["lit"].astype(np.float64), ref[..., 2])
    assert np.array_equal(hits["steps"].astype(np.float64), ref[..., 3])


def test_full_size_1024_spot_checks(native):
    """1024^3 Mandelbox: brick table raster order, occupancy totals, and 128 bricks recomputed on the CPU."""
    cfg, ext = scenes.voxel_mandelbox(1024, 64, 64)
    info = native_ext.voxel_build(cfg, ext, 8)
    assert info["brick_grid"] == 128
    t, o, d, _ = native_ext.voxel_read(info)
    nz = t[t > 0]
    assert np.array_equal(nz, np.arange(1, len(nz) + 1))
    assert int(o.sum()) == info["active_cells"]
    rng = np.random.default_rng(9)
    occupied = np.flatnonzero(t)
    picks = np.concatenate([rng.choice(occupied, 96, replace=False), rng.integers(0, len(t), 32)])
    for b in picks:
        bx, by, bz = b % 128, (b // 128) % 128, b // (128 * 128)
        ro, rd = oracle.voxel_brick(cfg, ext, 8, int(bx), int(by), int(bz))
        if t[b] == 0:
            assert ro.sum() == 0
            continue
        s = (int(t[b]) - 1) * 512
        assert np.array_equal(o[s:s + 512], ro), b
        assert np.array_equal(d[s:s + 512], rd), b


def test_voxel_path_render_through_drop_in(native, tmp_path):
    cfg = sphere_program(48)
    cfg.width, cfg.height, cfg.samples = 96, 72, 2
    cfg.renderer_backend = ffi.RENDERER_VOXEL
    cfg.camera_position[:] = [0.0, 0.5, -4.0]
    cfg.sun[0] = 1.0
    res = native.metal_render(cfg, str(tmp_path / "v.png"))
    assert res["voxel_active_cells"] > 0 and res["voxel_active_bricks"] > 0
    dense = sphere_program(48)
    ffi_fields = [f for f, _ in ffi.FptRenderConfig._fields_]
    for f in ffi_fields:
        setattr(dense, f, getattr(cfg, f))
    dense.voxel_storage = ffi.VOXEL_STORAGE_DENSE
    res_dense = native.metal_render(dense, str(tmp_path / "d.png"))
    assert np.array_equal(res["linear"], res_dense["linear"])
