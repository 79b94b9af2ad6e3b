"""Typed SoA direct evaluator (fpt_test_typed_soa and the lowered render path).

The validation hook compares the lowered program (sdf_typed_soa) with the
interpreter on 2^20 hash-seeded points with the reference's tolerances:
distance 2e-5 * (1 + |d|), gradient 1e-4 (shaders/Shaders.metal:5106-5154),
and returns 1 on any failure, as the reference does.  Distances must agree at
every point.  The interpreter subtracts the accumulated translations one at a
time, the lowered form subtracts each centre once.  Where two primitives, or
two faces of a box, are within that rounding of a tie, the winner can differ
and with it the gradient.  These random overlapping scenes see about one such
point per million (bounded here at 8 of 2^20).  A render of the lowered
program matches the interpreted render.
"""
import numpy as np
import pytest

import oracle
from fractalpathtracer_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_typed_soa_validation(native, seed):
    cfg = scenes.flat_union_program(seed)
    st = native.test_typed_soa(cfg, strict=False)
    print(f"seed {seed}: distance failures {st.distance_failures}, gradient failures {st.gradient_failures}, "
          f"max errors {st.max_distance_error:.2e} / {st.max_gradient_error:.2e}")
    assert st.sample_count == 1 << 20
    assert st.distance_failures == 0 and st.max_distance_error <= 1e-4
    assert st.gradient_failures <= 8


def test_typed_soa_requires_lowering(native):
    cfg = scenes.flat_union_program(0)
    cfg.sdf_typed_soa.sphere_count = cfg.sdf_typed_soa.box_count = cfg.sdf_typed_soa.plane_count = 0
    with pytest.raises(native.NativeError, match="lowered typed program"):
        native.test_typed_soa(cfg)


def test_lowered_render_matches_interpreter(native):
    cfg = scenes.flat_union_program(1, width=128, height=96)
    cfg.samples = 4
    cfg.sun[0] = 1.0
    _, lowered, ms_l = native.cuda_render(cfg, None, linear=False)
    interp = scenes.flat_union_program(1, width=128, height=96)
    interp.samples = 4
    interp.sun[0] = 1.0
    interp.sdf_typed_soa.sphere_count = interp.sdf_typed_soa.box_count = interp.sdf_typed_soa.plane_count = 0
    _, ref, ms_i = native.cuda_render(interp, None, linear=False)
    m = oracle.image_metrics(lowered, ref)
    print("lowered vs interpreted:", m, f"{ms_l:.3f} ms vs {ms_i:.3f} ms")
    assert m["mae"] <= 0.5 and m["lf_ssim"] >= 0.995
