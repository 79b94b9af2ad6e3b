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
        L.oracle_render_grid.argtypes = [vp, vp, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_float), P(C.c_double)]
        L.oracle_render_path.argtypes = [vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, P(C.c_float)]
        L.oracle_present.argtypes = [vp, P(C.c_float), P(C.c_uint8)]
        L.oracle_image_metrics.argtypes = [P(C.c_uint8), P(C.c_uint8), C.c_uint32, C.c_uint32, P(C.c_double)]
        L.oracle_voxel_build.argtypes = [vp, vp, C.c_uint32, P(C.c_uint32), P(C.c_uint8), P(C.c_uint16), P(C.c_uint32),
                                         C.c_size_t, P(C.c_ulonglong)]
        L.oracle_voxel_build.restype = C.c_longlong
        L.oracle_voxel_brick.argtypes = [vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_uint8), P(C.c_uint16)]
        L.oracle_dda.argtypes = [vp, C.c_uint32, P(C.c_uint32), P(C.c_uint8), P(C.c_uint32), P(C.c_float), C.c_size_t,
                                 C.c_uint32, P(C.c_uint32), P(C.c_uint32), P(C.c_double)]
        L.oracle_voxel_primary.argtypes = [vp, vp, P(C.c_uint32), P(C.c_uint8), C.c_uint32, C.c_uint32, P(C.c_double)]
        L.oracle_voxel_render.argtypes = [vp, vp, C.c_uint32, P(C.c_uint32), P(C.c_uint32), C.c_uint32, C.c_uint32,
                                          P(C.c_float)]
        L.oracle_dda_contract.restype = C.c_uint32
        L.oracle_hdri_lut.argtypes = [C.c_char_p, P(C.c_uint16), C.c_char_p, C.c_size_t]
        L.oracle_hdri_lut.restype = C.c_int
        L.oracle_float_to_half.argtypes = [C.c_float]
        L.oracle_float_to_half.restype = C.c_uint16
        fp = P(C.c_float)
        L.oracle_mlp_forward.argtypes = [fp, fp, fp, C.c_float, fp, C.c_size_t, C.c_int, P(C.c_double)]
        L.oracle_mlp_gradients.argtypes = [fp, fp, fp, C.c_float, fp, C.c_size_t, C.c_float, C.c_int, P(C.c_double),
                                           P(C.c_double)]
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
    """{x, y, z, w, dr, r, iterations, escaped, distance, colour} after `iterations` formula steps."""
    out = np.zeros(10, np.float64)
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


def render_grid(cfg, ext, y_stride, x_stride, fp64=False):
    """Batch accumulation of every y_stride-th row and x_stride-th column (a sample spread evenly over the
    frame): (H, W, 4) float32 with only those pixels filled, and the evaluation count."""
    acc = np.zeros((cfg.height, cfg.width, 4), np.float32)
    stats = np.zeros(4, np.float64)
    lib().oracle_render_grid(_ref(cfg), _ref(ext), int(fp64), 0, cfg.height, y_stride, x_stride,
                             acc.ctypes.data_as(C.POINTER(C.c_float)), stats.ctypes.data_as(C.POINTER(C.c_double)))
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


def _p(a, ty):
    return a.ctypes.data_as(C.POINTER(ty)) if a is not None else None


def voxel_build(cfg, ext, brick_size=8, max_cells=None):
    """CPU build: (table, occupancy, distance-as-fp16-bits or None, cells or None, active_cells)."""
    res = cfg.voxel_resolution
    bg = (res + brick_size - 1) // brick_size
    table = np.zeros(bg ** 3, np.uint32)
    cap = max_cells if max_cells is not None else bg ** 3 * brick_size ** 3
    occ = np.zeros(cap, np.uint8) if brick_size == 8 else None
    dist = np.zeros(cap, np.uint16) if brick_size == 8 else None
    cells = np.zeros((cap, 3), np.uint32) if brick_size != 8 else None
    active_cells = C.c_ulonglong()
    n = lib().oracle_voxel_build(_ref(cfg), _ref(ext), brick_size, _p(table, C.c_uint32), _p(occ, C.c_uint8), _p(dist, C.c_uint16),
                                 _p(cells, C.c_uint32), cap, C.byref(active_cells))
    if n < 0:
        raise ValueError("cell capacity too small")
    m = int(n) * brick_size ** 3
    return (table, occ[:m] if occ is not None else None, dist[:m] if dist is not None else None,
            cells[:m] if cells is not None else None, active_cells.value)


def voxel_brick(cfg, ext, brick_size, bx, by, bz):
    occ = np.zeros(brick_size ** 3, np.uint8)
    dist = np.zeros(brick_size ** 3, np.uint16)
    lib().oracle_voxel_brick(_ref(cfg), _ref(ext), brick_size, bx, by, bz, _p(occ, C.c_uint8), _p(dist, C.c_uint16))
    return occ, dist


def dda(cfg, brick_size, table, occ, cells, rays, capacity=0):
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    n = len(r)
    seq = np.zeros((n, capacity), np.uint32) if capacity else None
    seq_len = np.zeros(n, np.uint32) if capacity else None
    hits = np.zeros((n, 4), np.float64)
    lib().oracle_dda(_ref(cfg), brick_size, _p(table, C.c_uint32), _p(occ, C.c_uint8),
                     _p(np.ascontiguousarray(cells, np.uint32) if cells is not None else None, C.c_uint32),
                     _p(r, C.c_float), n, capacity, _p(seq, C.c_uint32), _p(seq_len, C.c_uint32), _p(hits, C.c_double))
    return hits, seq, seq_len


def voxel_primary(cfg, ext, table, occ, rows=None):
    y0, y1 = rows if rows is not None else (0, cfg.height)
    out = np.zeros((cfg.height, cfg.width, 5), np.float64)
    lib().oracle_voxel_primary(_ref(cfg), _ref(ext), _p(table, C.c_uint32), _p(occ, C.c_uint8), y0, y1, _p(out, C.c_double))
    return out


def voxel_render(cfg, ext, table, cells, brick_size=4, rows=None):
    """renderVoxelPath accumulated over the config's samples for rows [y0, y1) through reference cells
    (brick_size 4 with a page table, 0 dense): (H, W, 4) float32, row 0 at the bottom."""
    y0, y1 = rows if rows is not None else (0, cfg.height)
    acc = np.zeros((cfg.height, cfg.width, 4), np.float32)
    t = np.ascontiguousarray(table, np.uint32) if table is not None else None
    c = np.ascontiguousarray(cells, np.uint32)
    lib().oracle_voxel_render(_ref(cfg), _ref(ext), brick_size, _p(t, C.c_uint32), _p(c, C.c_uint32), y0, y1,
                              _p(acc, C.c_float))
    return acc


def hdri_lut(path):
    """The reference's 32x16x3 FP16 LUT (bits) of a Radiance .hdr file."""
    lut = np.zeros(32 * 16 * 3, np.uint16)
    err = C.create_string_buffer(256)
    if lib().oracle_hdri_lut(path.encode(), _p(lut, C.c_uint16), err, len(err)) != 0:
        raise ValueError(err.value.decode())
    return lut


def dda_contract():
    return int(lib().oracle_dda_contract())


def float_to_half(values):
    return np.array([lib().oracle_float_to_half(float(v)) for v in np.asarray(values, np.float32)], np.uint16)


def _mlp_frame(bounds_min, bounds_max):
    lo = np.asarray(bounds_min, np.float32)
    hi = np.asarray(bounds_max, np.float32)
    center = (np.float32(0.5) * (lo + hi)).astype(np.float32)
    half = (np.float32(0.5) * (hi - lo)).astype(np.float32)
    inv_half = (np.float32(1.0) / half).astype(np.float32)
    return center, inv_half, np.float32(half.max())


def mlp_forward(params, bounds_min, bounds_max, points, emulate_bf16=True):
    """FP64 network output (distance units) at xyzw points; the frame follows the CUDA model's box."""
    center, inv_half, scale = _mlp_frame(bounds_min, bounds_max)
    p = np.ascontiguousarray(params, np.float32)
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    out = np.zeros(len(pts), np.float64)
    lib().oracle_mlp_forward(_p(p, C.c_float), _p(center, C.c_float), _p(inv_half, C.c_float), float(scale),
                             _p(pts, C.c_float), len(pts), int(emulate_bf16), _p(out, C.c_double))
    return out


def mlp_gradients(params, bounds_min, bounds_max, points, overestimate_weight=10.0, emulate_bf16=True):
    """FP64 gradients (19777) and mean loss of the asymmetric loss over labelled xyzw points."""
    center, inv_half, scale = _mlp_frame(bounds_min, bounds_max)
    p = np.ascontiguousarray(params, np.float32)
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    g = np.zeros(len(p), np.float64)
    loss = np.zeros(1, np.float64)
    lib().oracle_mlp_gradients(_p(p, C.c_float), _p(center, C.c_float), _p(inv_half, C.c_float), float(scale),
                               _p(pts, C.c_float), len(pts), float(overestimate_weight), int(emulate_bf16),
                               _p(g, C.c_double), _p(loss, C.c_double))
    return g, float(loss[0])
