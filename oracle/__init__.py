"""ctypes bindings of the CPU oracle (test infrastructure only).

The oracle (oracle/fpt_oracle.cpp) restates FPT Metal's sphere-tracing path
on the CPU.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg use this module, and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            path = _build.build()
        L = C.CDLL(path)
        P = C.POINTER
        vp = C.c_void_p
        L.oracle_sample_distance.argtypes = [vp, vp, P(C.c_float), C.c_size_t, C.c_int, P(C.c_double), P(C.c_double)]
        L.oracle_field_sample.argtypes = [vp, vp, P(C.c_float), C.c_size_t, C.c_int, P(C.c_double)]
        L.oracle_orbit_step.argtypes = [vp, P(C.c_double), C.c_int, C.c_double, C.c_int, P(C.c_double)]
        L.oracle_trace_primary.argtypes = [vp, vp, C.c_int, C.c_uint32, C.c_uint32, P(C.c_double)]
        L.oracle_focus_distance.argtypes = [vp, vp, C.c_int]
        L.oracle_focus_distance.restype = C.c_double
        L.oracle_render.argtypes = [vp, vp, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_float), P(C.c_double)]
        L.oracle_render_path.argtypes = [vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, P(C.c_float)]
        L.oracle_present.argtypes = [vp, P(C.c_float), P(C.c_uint8)]
        L.oracle_image_metrics.argtypes = [P(C.c_uint8), P(C.c_uint8), C.c_uint32, C.c_uint32, P(C.c_double)]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _ref(x):
    return C.cast(C.pointer(x), C.c_void_p) if x is not None else None


def set_threads(n: int) -> None:
    lib().oracle_set_threads(n)


def max_threads() -> int:
    return lib().oracle_max_threads()


def sample_distance(cfg, ext, points, fp64=True, gradients=False):
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    out = np.zeros((len(pts), 4), np.float64)
    g = np.zeros((len(pts), 3), np.float64) if gradients else None
    lib().oracle_sample_distance(_ref(cfg), _ref(ext), pts.ctypes.data_as(C.POINTER(C.c_float)), len(pts), int(fp64),
                                 out.ctypes.data_as(C.POINTER(C.c_double)),
                                 g.ctypes.data_as(C.POINTER(C.c_double)) if g is not None else None)
    return (out, g) if gradients else out


def field_sample(cfg, ext, points, fp64=True):
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    out = np.zeros((len(pts), 4), np.float64)
    lib().oracle_field_sample(_ref(cfg), _ref(ext), pts.ctypes.data_as(C.POINTER(C.c_float)), len(pts), int(fp64),
                              out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def orbit_step(ext, point4, iterations=1, bailout=1e300, add_c=False):
    out = np.zeros(9, np.float64)
    p = np.ascontiguousarray(point4, np.float64)
    lib().oracle_orbit_step(_ref(ext), p.ctypes.data_as(C.POINTER(C.c_double)), iterations, bailout, int(add_c),
                            out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def trace_primary(cfg, ext, fp64=True, rows=None):
    """(H, W, 6) {distance, nx, ny, nz, steps, hit}; rows=(y0, y1) limits the traced rows."""
    y0, y1 = rows if rows is not None else (0, cfg.height)
    out = np.zeros((cfg.height, cfg.width, 6), np.float64)
    lib().oracle_trace_primary(_ref(cfg), _ref(ext), int(fp64), y0, y1, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def focus_distance(cfg, ext, fp64=False):
    return lib().oracle_focus_distance(_ref(cfg), _ref(ext), int(fp64))


def render(cfg, ext, rows=None, x_stride=1, fp64=False):
    """Batch accumulation of rows [y0, y1) (every x_stride-th pixel): (H, W, 4) float32 and evaluation count."""
    y0, y1 = rows if rows is not None else (0, cfg.height)
    acc = np.zeros((cfg.height, cfg.width, 4), np.float32)
    stats = np.zeros(4, np.float64)
    lib().oracle_render(_ref(cfg), _ref(ext), int(fp64), y0, y1, x_stride, acc.ctypes.data_as(C.POINTER(C.c_float)),
                        stats.ctypes.data_as(C.POINTER(C.c_double)))
    return acc, stats[0]


def present(cfg, accum):
    acc = np.ascontiguousarray(accum, np.float32)
    rgba = np.zeros((cfg.height, cfg.width, 4), np.uint8)
    lib().oracle_present(_ref(cfg), acc.ctypes.data_as(C.POINTER(C.c_float)), rgba.ctypes.data_as(C.POINTER(C.c_uint8)))
    return rgba


def image_metrics(a, b):
    a = np.ascontiguousarray(a, np.uint8)
    b = np.ascontiguousarray(b, np.uint8)
    out = np.zeros(6, np.float64)
    lib().oracle_image_metrics(a.ctypes.data_as(C.POINTER(C.c_uint8)), b.ctypes.data_as(C.POINTER(C.c_uint8)),
                               a.shape[1], a.shape[0], out.ctypes.data_as(C.POINTER(C.c_double)))
    return dict(zip(["mae", "rmse", "max_abs", "changed_pct", "ssim", "lf_ssim"], out.tolist()))
