"""Loader and thin Python bindings of libfpt_cuda.so (the C ABI of include/fpt_cuda.h).

The library is the product: every call here goes through its exported C
entry points.  Missing or stale builds raise ``NativeError`` -- there is no
Python or CPU fallback for any of these functions.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import ffi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libfpt_cuda.so")

# Every symbol include/fpt_cuda.h declares.
EXPORTED = [
    "fpt_metal_render", "fpt_metal_diagnostic_render", "fpt_mandelbulber_sample_field", "fpt_compare_images",
    "fpt_metal_device_name", "fpt_test_voxel_dda", "fpt_test_async_stitch_context", "fpt_test_typed_soa",
    "fpt_metal_preview", "fpt_cuda_trace_primary", "fpt_cuda_render", "fpt_cuda_sample_distance",
    "fpt_cuda_voxel_build", "fpt_cuda_voxel_read", "fpt_cuda_dda_sequence", "fpt_cuda_voxel_render",
    "fpt_cuda_voxel_build_static", "fpt_cuda_mlp_create", "fpt_cuda_mlp_destroy", "fpt_cuda_mlp_predict",
    "fpt_cuda_mlp_get_params", "fpt_cuda_mlp_set_params", "fpt_cuda_mlp_gradients", "fpt_cuda_skip_stats",
    "fpt_cuda_render_stats", "fpt_cuda_render_batch", "fpt_cuda_autotune_batch", "fpt_cuda_set_launch_shape",
    "fpt_cuda_set_march_schedule",
    "fpt_cuda_set_network_engine",
    "fpt_cuda_set_kernel_timing",
    "fpt_test_bounded_waits",
    "fpt_cuda_set_loop_limit",
    "fpt_cuda_set_device", "fpt_cuda_get_device", "fpt_cuda_hdri_lut",
    "fpt_cuda_measure_fp32_peak", "fpt_cuda_certified_steps",
]


class NativeError(RuntimeError):
    """A C entry point returned 1 (its message is the exception text), or the library is missing."""


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NativeError(f"{LIB_PATH} is missing: build it with fractalpathtracer_gb300.build.build()")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L: C.CDLL) -> None:
    P = C.POINTER
    cfg = P(ffi.FptRenderConfig)
    ext = P(ffi.FptCudaSceneExt)
    err = [C.c_char_p, C.c_size_t]
    L.fpt_metal_render.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_size_t, cfg,
                                   P(C.c_double), P(C.c_double), P(C.c_uint64), P(C.c_uint32), P(C.c_uint64),
                                   P(C.c_uint32), P(ffi.FptBoundGridStats), P(C.c_uint32),
                                   P(ffi.FptStitchValidationStats), P(ffi.FptStitchPipelineStats),
                                   P(ffi.FptSdfProfileStats), P(C.c_float), C.c_size_t] + err
    L.fpt_metal_diagnostic_render.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_size_t, cfg,
                                              P(ffi.FptDiagnosticConfig), P(C.c_double)] + err
    L.fpt_mandelbulber_sample_field.argtypes = [C.c_char_p, C.c_char_p, C.c_size_t, cfg, P(C.c_float), C.c_size_t,
                                                P(ffi.FptMandelbulberFieldSample)] + err
    L.fpt_compare_images.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p] + err
    L.fpt_metal_device_name.argtypes = [C.c_char_p, C.c_size_t]
    L.fpt_test_voxel_dda.argtypes = [C.c_char_p] + err
    L.fpt_test_async_stitch_context.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, cfg, P(ffi.FptAsyncJitStats)] + err
    L.fpt_test_typed_soa.argtypes = [C.c_char_p, cfg, P(ffi.FptStitchValidationStats)] + err
    L.fpt_metal_preview.argtypes = [C.c_char_p, C.c_char_p, P(C.c_char_p), C.c_char_p, C.c_size_t, cfg, cfg,
                                    C.c_uint32, C.c_uint32] + err
    L.fpt_cuda_trace_primary.argtypes = [cfg, ext, P(ffi.FptCudaPrimaryHit), C.c_size_t, P(C.c_double)] + err
    L.fpt_cuda_render.argtypes = [cfg, ext, C.c_char_p, P(C.c_float), C.c_size_t, P(C.c_uint8), C.c_size_t,
                                  P(C.c_double), P(ffi.FptSdfProfileStats)] + err
    L.fpt_cuda_sample_distance.argtypes = [cfg, ext, P(C.c_float), C.c_size_t, P(C.c_float), P(C.c_float)] + err
    L.fpt_cuda_set_device.argtypes = [C.c_int32]
    L.fpt_cuda_hdri_lut.argtypes = [C.c_char_p, P(C.c_uint16), C.c_size_t] + err
    L.fpt_cuda_measure_fp32_peak.argtypes = [P(C.c_double), P(C.c_double)] + err
    L.fpt_cuda_certified_steps.argtypes = [cfg, ext, C.c_uint32, C.c_float, P(C.c_float), P(C.c_uint32), C.c_size_t] + err
    L.fpt_cuda_get_device.argtypes = [P(C.c_int32)]
    for name in EXPORTED:
        getattr(L, name).restype = C.c_int
    _declare_extra(L)


def _declare_extra(L: C.CDLL) -> None:
    """Side entry points added after the first set (voxel, MLP, batch); declared when present."""
    from . import native_ext
    native_ext.declare(L)


def _err():
    return C.create_string_buffer(1024)


def _raise(buf) -> None:
    raise NativeError(buf.value.decode("utf-8", "replace") or "unknown native error")


def _b(s):
    return s.encode() if isinstance(s, str) else s


def _ptr(arr: np.ndarray, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype))


def metal_render(config: ffi.FptRenderConfig, output_path: str, linear_output: bool = True, profile: bool = False) -> dict:
    """The reference's render call (src/main.rs:912-963 -> fpt_metal_render): renders and writes a PNG."""
    L = lib()
    build_ms, elapsed = C.c_double(), C.c_double()
    vmem, vbricks, vcells, vrej, scs = C.c_uint64(), C.c_uint32(), C.c_uint64(), C.c_uint32(), C.c_uint32()
    bgs, svs, sps, prof = ffi.FptBoundGridStats(), ffi.FptStitchValidationStats(), ffi.FptStitchPipelineStats(), ffi.FptSdfProfileStats()
    n = config.width * config.height * 4
    lin = np.zeros(n, np.float32) if linear_output else None
    e = _err()
    rc = L.fpt_metal_render(b"", b"", b"", _b(output_path), None, 0, C.byref(config), C.byref(build_ms), C.byref(elapsed),
                            C.byref(vmem), C.byref(vbricks), C.byref(vcells), C.byref(vrej), C.byref(bgs), C.byref(scs),
                            C.byref(svs), C.byref(sps), C.byref(prof) if profile else None,
                            _ptr(lin, C.c_float) if lin is not None else None, n if lin is not None else 0, e, len(e))
    if rc != 0:
        _raise(e)
    out = {"elapsed_ms": elapsed.value, "build_ms": build_ms.value, "voxel_memory_bytes": vmem.value,
           "voxel_active_bricks": vbricks.value, "voxel_active_cells": vcells.value}
    if lin is not None:
        out["linear"] = lin.reshape(config.height, config.width, 4)
    if profile:
        out["profile"] = prof
    return out


def cuda_render(config: ffi.FptRenderConfig, ext: ffi.FptCudaSceneExt | None = None, output_path: str | None = None,
                linear: bool = True, profile: bool = False, out_linear: np.ndarray | None = None,
                out_rgba: np.ndarray | None = None):
    """fpt_cuda_render: returns (linear HxWx4 float32 accumulation or None, rgba HxWx4 uint8 top row first, elapsed ms[, profile]).
    out_linear / out_rgba: caller-owned contiguous arrays (W*H*4 float32 / uint8, e.g. pinned host memory) to
    receive the results instead of new arrays."""
    L = lib()
    n = config.width * config.height * 4
    for a, dt in ((out_linear, np.float32), (out_rgba, np.uint8)):
        if a is not None and (a.dtype != dt or a.size != n or not a.flags["C_CONTIGUOUS"]):
            raise ValueError(f"output array must be a contiguous {np.dtype(dt).name} array of {n} elements")
    lin = (out_linear.reshape(-1) if out_linear is not None else np.zeros(n, np.float32)) if linear else None
    rgba = out_rgba.reshape(-1) if out_rgba is not None else np.zeros(n, np.uint8)
    elapsed = C.c_double()
    prof = ffi.FptSdfProfileStats()
    e = _err()
    rc = L.fpt_cuda_render(C.byref(config), C.byref(ext) if ext is not None else None,
                           _b(output_path) if output_path else None,
                           _ptr(lin, C.c_float) if lin is not None else None, n if lin is not None else 0,
                           _ptr(rgba, C.c_uint8), n, C.byref(elapsed), C.byref(prof) if profile else None, e, len(e))
    if rc != 0:
        _raise(e)
    res = (lin.reshape(config.height, config.width, 4) if lin is not None else None,
           rgba.reshape(config.height, config.width, 4), elapsed.value)
    return res + (prof,) if profile else res


HIT_DTYPE = np.dtype([("distance", np.float32), ("normal", np.float32, 3), ("steps", np.uint32), ("hit", np.uint32)])


def trace_primary(config: ffi.FptRenderConfig, ext: ffi.FptCudaSceneExt | None = None):
    """fpt_cuda_trace_primary: (H, W) structured array (row 0 = bottom) and elapsed ms."""
    L = lib()
    n = config.width * config.height
    hits = np.zeros(n, HIT_DTYPE)
    elapsed = C.c_double()
    e = _err()
    rc = L.fpt_cuda_trace_primary(C.byref(config), C.byref(ext) if ext is not None else None,
                                  hits.ctypes.data_as(C.POINTER(ffi.FptCudaPrimaryHit)), n, C.byref(elapsed), e, len(e))
    if rc != 0:
        _raise(e)
    return hits.reshape(config.height, config.width), elapsed.value


def sample_field(config: ffi.FptRenderConfig, points: np.ndarray) -> np.ndarray:
    """fpt_mandelbulber_sample_field: (n, 4) {distance, radius, derivative, iterations}."""
    L = lib()
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    out = np.zeros((len(pts), 4), np.float32)
    e = _err()
    rc = L.fpt_mandelbulber_sample_field(b"", None, 0, C.byref(config), _ptr(pts, C.c_float), len(pts),
                                         out.ctypes.data_as(C.POINTER(ffi.FptMandelbulberFieldSample)), e, len(e))
    if rc != 0:
        _raise(e)
    return out


def sample_distance(config: ffi.FptRenderConfig, ext: ffi.FptCudaSceneExt | None, points: np.ndarray, gradients: bool = False):
    """fpt_cuda_sample_distance: (n, 4) {distance, orbit, derivative, iterations} [and (n, 3) gradients]."""
    L = lib()
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    out = np.zeros((len(pts), 4), np.float32)
    g = np.zeros((len(pts), 3), np.float32) if gradients else None
    e = _err()
    rc = L.fpt_cuda_sample_distance(C.byref(config), C.byref(ext) if ext is not None else None, _ptr(pts, C.c_float),
                                    len(pts), _ptr(out, C.c_float), _ptr(g, C.c_float) if g is not None else None, e, len(e))
    if rc != 0:
        _raise(e)
    return (out, g) if gradients else out


def compare_images(baseline: str, candidate: str, report: str) -> dict:
    """fpt_compare_images: writes the JSON report and returns it parsed."""
    import json
    L = lib()
    e = _err()
    if L.fpt_compare_images(_b(baseline), _b(candidate), _b(report), e, len(e)) != 0:
        _raise(e)
    with open(report) as f:
        return json.load(f)


def certified_steps(config, ext, sun_direction, stride: int = 4, margin: float = 0.1) -> np.ndarray:
    """fpt_cuda_certified_steps: (samples, 6) plain / certified evaluations of camera, shadow and bounce rays."""
    samples = ((config.width + stride - 1) // stride) * ((config.height + stride - 1) // stride)
    out = np.zeros(samples * 6, np.uint32)
    sun = np.ascontiguousarray(sun_direction, np.float32)
    e = _err()
    if lib().fpt_cuda_certified_steps(C.byref(config), C.byref(ext) if ext is not None else None, stride, float(margin),
                                      _ptr(sun, C.c_float), _ptr(out, C.c_uint32), out.size, e, len(e)) != 0:
        _raise(e)
    return out.reshape(samples, 6)


def measure_fp32_peak() -> dict:
    """FP32 FMA throughput of the library's device (TFLOP/s) and the best launch time (ms)."""
    t, ms = C.c_double(), C.c_double()
    e = _err()
    if lib().fpt_cuda_measure_fp32_peak(C.byref(t), C.byref(ms), e, len(e)) != 0:
        _raise(e)
    return {"tflops": t.value, "launch_ms": ms.value}


def hdri_lut(path: str) -> np.ndarray:
    """The 32x16x3 FP16 LUT (bits) a world-mode-2 render builds from the .hdr at `path` (host code)."""
    lut = np.zeros(32 * 16 * 3, np.uint16)
    e = _err()
    if lib().fpt_cuda_hdri_lut(_b(path), _ptr(lut, C.c_uint16), lut.size, e, len(e)) != 0:
        _raise(e)
    return lut


def set_device(ordinal: int) -> None:
    """Binds the library's context to a CUDA device (before its first GPU call)."""
    if lib().fpt_cuda_set_device(int(ordinal)) != 0:
        raise NativeError(f"cannot bind CUDA device {ordinal} (not visible, or another device is already bound)")


def get_device() -> int | None:
    """Ordinal of the device the library's context is bound to (None without a GPU)."""
    v = C.c_int32(-1)
    return v.value if lib().fpt_cuda_get_device(C.byref(v)) == 0 else None


def device_name() -> str | None:
    buf = C.create_string_buffer(256)
    return buf.value.decode() if lib().fpt_metal_device_name(buf, len(buf)) == 0 else None


def diagnostic_render(config: ffi.FptRenderConfig, mode: int, output_path: str, max_distance: float = 0.0) -> float:
    L = lib()
    d = ffi.FptDiagnosticConfig()
    d.mode = mode
    d.max_distance = max_distance
    elapsed = C.c_double()
    e = _err()
    if L.fpt_metal_diagnostic_render(b"", _b(output_path), None, 0, C.byref(config), C.byref(d), C.byref(elapsed), e, len(e)) != 0:
        _raise(e)
    return elapsed.value


def test_voxel_dda() -> None:
    e = _err()
    if lib().fpt_test_voxel_dda(b"", e, len(e)) != 0:
        _raise(e)


def test_typed_soa(config: ffi.FptRenderConfig, strict: bool = True) -> ffi.FptStitchValidationStats:
    """fpt_test_typed_soa: validation statistics; strict=False returns them even when the hook reports failures."""
    st = ffi.FptStitchValidationStats()
    e = _err()
    if lib().fpt_test_typed_soa(b"", C.byref(config), C.byref(st), e, len(e)) != 0 and (strict or st.sample_count == 0):
        _raise(e)
    return st
