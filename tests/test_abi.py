"""C ABI: struct layouts match the reference's pinned sizes and the library
exports every entry point include/fpt_cuda.h declares (no GPU needed)."""
import ctypes
import os
import re

from fractalpathtracer_gb300 import ffi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_layout_sizes_match_reference():
    # src/ffi.rs:494-507
    assert ffi.layout_sizes() == ffi.REFERENCE_SIZES


def test_field_offsets_match_reference_order():
    c = ffi.FptRenderConfig
    assert c.width.offset == 0 and c.sdf_chunk_samples.offset == 44
    assert c.camera_position.offset == 60
    # the typed SoA block closes the struct
    assert c.sdf_typed_soa.offset + ctypes.sizeof(ffi.FptTypedSoAProgram) == 30448


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "fpt_cuda.h")).read()
    return sorted(set(re.findall(r"^int\s+(fpt_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(native):
    lib = native.lib()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert set(native.EXPORTED) <= set(declared_symbols())


def test_unsupported_entries_fail_cleanly_without_gpu(native):
    import ctypes as C
    lib = native.lib()
    err = C.create_string_buffer(256)
    assert lib.fpt_metal_preview(b"", b"", None, None, 0, None, None, 0, 0, err, len(err)) == 1
    assert b"unsupported" in err.value
    stats = ffi.FptAsyncJitStats()
    assert lib.fpt_test_async_stitch_context(b"", b"", b"", None, C.byref(stats), err, len(err)) == 1


def test_batch_scene_generator_is_seeded():
    from fractalpathtracer_gb300 import ffi, scenes
    a = scenes.batch_scenes(64)
    b = scenes.batch_scenes(64)
    kinds = set()
    for x, y in zip(a, b):
        assert bytes(x.cfg) == bytes(y.cfg) and bytes(x.ext) == bytes(y.ext)
        assert 64 <= x.cfg.width <= 512 and x.cfg.width == x.cfg.height
        assert 4 <= x.ext.iterations <= 16 and x.cfg.samples == 4 and x.cfg.render[0] == 3.0
        kinds.add(x.ext.formula)
        if x.ext.formula == ffi.FORMULA_MANDELBULB:
            assert 2.0 <= x.ext.power <= 12.0
        if x.ext.formula == ffi.FORMULA_MANDELBOX:
            assert -2.5 <= x.ext.box_scale <= -1.5
    assert kinds == {ffi.FORMULA_MANDELBULB, ffi.FORMULA_MANDELBOX, ffi.FORMULA_BULB_MENGER_HYBRID}


def test_flat_union_lowering_matches_program():
    """The typed-SoA arrays of scenes.flat_union_program give the program's distance (numpy restatement of both)."""
    import numpy as np
    from fractalpathtracer_gb300 import ffi, scenes
    cfg = scenes.flat_union_program(3)
    pts = np.random.default_rng(0).uniform(-2, 2, (2000, 3))
    # interpreter semantics: accumulated translations, union of primitives
    d_prog = np.full(len(pts), np.inf)
    p = pts.copy()
    for i in range(cfg.sdf_program_count):
        op = cfg.sdf_program[i]
        d = np.array(op.data[:])
        if op.opcode == ffi.OP_TRANSLATE:
            p = p - d[:3]
        elif op.opcode == ffi.OP_SPHERE:
            d_prog = np.minimum(d_prog, np.linalg.norm(p, axis=1) - d[0])
        elif op.opcode == ffi.OP_BOX:
            q = np.abs(p) - np.abs(d[:3])
            d_prog = np.minimum(d_prog, np.minimum(q.max(1), 0) + np.linalg.norm(np.maximum(q, 0), axis=1))
        elif op.opcode == ffi.OP_PLANE:
            n = d[:3] / np.linalg.norm(d[:3])
            d_prog = np.minimum(d_prog, p @ n + d[3])
    t = cfg.sdf_typed_soa
    d_soa = np.full(len(pts), np.inf)
    for i in range(t.sphere_count):
        d_soa = np.minimum(d_soa, np.linalg.norm(pts - [t.sphere_x[i], t.sphere_y[i], t.sphere_z[i]], axis=1) - t.sphere_radius[i])
    for i in range(t.box_count):
        q = np.abs(pts - [t.box_x[i], t.box_y[i], t.box_z[i]]) - [t.box_half_x[i], t.box_half_y[i], t.box_half_z[i]]
        d_soa = np.minimum(d_soa, np.minimum(q.max(1), 0) + np.linalg.norm(np.maximum(q, 0), axis=1))
    for i in range(t.plane_count):
        n = np.array([t.plane_x[i], t.plane_y[i], t.plane_z[i]])
        n /= np.linalg.norm(n)
        c = np.array([t.plane_center_x[i], t.plane_center_y[i], t.plane_center_z[i]])
        d_soa = np.minimum(d_soa, (pts - c) @ n + t.plane_offset[i])
    assert t.sphere_count + t.box_count + t.plane_count == 12
    assert np.abs(d_prog - d_soa).max() < 1e-5


def test_settings_validate_arguments_without_gpu(native):
    """Host-side settings reject out-of-range values before any CUDA call (runs without a GPU)."""
    import pytest
    from fractalpathtracer_gb300 import native_ext as nx
    with pytest.raises(ValueError):
        nx.set_network_engine(7)
    with pytest.raises(ValueError):
        nx.set_march_schedule(1, 0)
    with pytest.raises(ValueError):
        nx.set_march_schedule(0, 33)
    with pytest.raises(ValueError):
        nx.set_kernel_timing(2)
    nx.set_kernel_timing(False)
    nx.set_network_engine(nx.NET_MMA_SYNC)
    nx.set_network_engine(nx.NET_TCGEN05)
    nx.set_march_schedule(0, 0)
    nx.set_loop_limit(0)


def test_generated_mandelbulber_source_is_rejected_without_gpu(native):
    """A shader source generated from a Mandelbulber formula (the generator defines
    FPT_MANDEL_GENERATED_FIELD, src/mandelbulber/compiler.rs:1510) is refused with
    a message instead of rendering the built-in formula; the stock source is not."""
    import ctypes as C
    lib = native.lib()
    cfg = ffi.default_config()
    cfg.width, cfg.height = 4, 4
    src = b"#include <metal_stdlib>\n#define FPT_MANDEL_GENERATED_FIELD 1\nstatic float4 f();\n"
    err = C.create_string_buffer(512)
    rc = lib.fpt_metal_render(b"", b"", b"", b"/nonexistent/out.png", src, len(src), C.byref(cfg), None, None, None, None,
                              None, None, None, None, None, None, None, None, 0, err, len(err))
    assert rc == 1 and b"generated Mandelbulber formulas are not supported" in err.value
    d = ffi.FptDiagnosticConfig()
    err = C.create_string_buffer(512)
    rc = lib.fpt_metal_diagnostic_render(b"", b"/nonexistent/d.png", src, len(src), C.byref(cfg), C.byref(d), None, err,
                                         len(err))
    assert rc == 1 and b"generated Mandelbulber formulas are not supported" in err.value
    cfg.sdf_id = ffi.SDF_MANDELBULBER
    pts = (C.c_float * 4)(0.0, 0.0, 0.0, 1.0)
    out = ffi.FptMandelbulberFieldSample()
    err = C.create_string_buffer(512)
    rc = lib.fpt_mandelbulber_sample_field(b"", src, len(src), C.byref(cfg), pts, 1, C.byref(out), err, len(err))
    assert rc == 1 and b"generated Mandelbulber formulas are not supported" in err.value
    # the stock source (what the reference's src/main.rs passes on every other call) passes the check
    # and fails later, for the missing output path, before touching a GPU
    stock = b"#include <metal_stdlib>\nkernel void sdf_kernel();\n"
    err = C.create_string_buffer(512)
    rc = lib.fpt_metal_render(b"", b"", b"", None, stock, len(stock), C.byref(cfg), None, None, None, None,
                              None, None, None, None, None, None, None, None, 0, err, len(err))
    assert rc == 1 and b"missing output path" in err.value
