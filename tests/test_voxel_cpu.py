"""Voxel oracle checks without a GPU: the reference's DDA contract cases,
IEEE fp16 rounding of stored distances, and raster-order brick tables."""
import json
import os
import struct

import numpy as np

import oracle
from fractalpathtracer_gb300 import ffi

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_dda_contract_cases_hold(oracle_lib):
    # shaders/Shaders.metal:5164-5211 restated; fixture tests/golden/dda_contract.json
    assert oracle.dda_contract() == 0
    data = json.load(open(os.path.join(GOLDEN, "dda_contract.json")))
    nf = data["advance"][1]["expect"][0]["entry_t"]
    assert struct.unpack("<I", struct.pack("<f", nf))[0] == struct.unpack("<I", struct.pack("<f", 1.0))[0] + 1


def test_fp16_distance_rounding_is_ieee_rne(oracle_lib):
    rng = np.random.default_rng(3)
    v = np.concatenate([rng.standard_normal(20000) * 50, rng.random(5000) * 1e-5,
                        [0.0, -0.0, 65504.0, 65519.0, 1e-8, 5.960464e-08]]).astype(np.float32)
    assert np.array_equal(oracle.float_to_half(v), v.astype(np.float16).view(np.uint16))


def sphere_program(res=32):
    cfg = ffi.default_config()
    cfg.sdf_id = ffi.SDF_PROGRAM
    cfg.sdf_program_count = 1
    cfg.sdf_program[0].opcode = ffi.OP_SPHERE
    cfg.sdf_program[0].data[0] = 1.0
    cfg.voxel_resolution = res
    cfg.voxel_surface_band = 0.5
    cfg.voxel_bounds_min[:] = [-2, -2, -2]
    cfg.voxel_bounds_max[:] = [2, 2, 2]
    return cfg


def test_brick_table_is_raster_ordered(oracle_lib):
    cfg = sphere_program(32)
    table, occ, dist, _, cells = oracle.voxel_build(cfg, None, 8)
    nz = table[table > 0]
    assert np.array_equal(nz, np.arange(1, len(nz) + 1))      # ids assigned in raster order
    assert int(occ.sum()) == cells
    # a surface band of cells around the unit sphere
    assert 0 < cells < 32 ** 3 // 4
