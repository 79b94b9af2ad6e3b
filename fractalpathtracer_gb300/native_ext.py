"""ctypes declarations and wrappers of the side entry points (voxel, MLP, batch)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import ffi


class FptCudaVoxelInfo(C.Structure):
    _fields_ = [("resolution", C.c_uint32), ("brick_size", C.c_uint32), ("brick_grid", C.c_uint32),
                ("active_bricks", C.c_uint32), ("active_cells", C.c_uint64), ("memory_bytes", C.c_uint64),
                ("build_ms", C.c_double)]


class FptCudaVoxelHit(C.Structure):
    _fields_ = [("t", C.c_float), ("cell", C.c_uint32), ("normal_axis", C.c_uint32), ("steps", C.c_uint32),
                ("shadow_steps", C.c_uint32), ("lit", C.c_uint32)]


class FptCudaMlpConfig(C.Structure):
    _fields_ = [("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3), ("points", C.c_uint32),
                ("near_fraction", C.c_float), ("near_band", C.c_float), ("batch", C.c_uint32), ("steps", C.c_uint32),
                ("lr", C.c_float), ("overestimate_weight", C.c_float), ("seed", C.c_uint32), ("_reserved", C.c_uint32 * 4)]


class FptCudaMlpStats(C.Structure):
    _fields_ = [("loss_first", C.c_float), ("loss_last", C.c_float), ("data_ms", C.c_double), ("train_ms", C.c_double),
                ("params", C.c_uint32), ("steps", C.c_uint32), ("label_scale", C.c_float), ("near_points", C.c_uint32)]


class FptCudaSkipStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("rows", "forwards", "exact_evals", "accepted", "rejected", "escaped",
                                          "handed_over", "reserved")]


class FptCudaRenderStats(C.Structure):
    _fields_ = [("kernel_launches", C.c_uint64), ("march_launches", C.c_uint64), ("shade_launches", C.c_uint64),
                ("skip_launches", C.c_uint64), ("march_evals", C.c_uint64), ("shade_evals", C.c_uint64),
                ("march_ms", C.c_double), ("shade_ms", C.c_double), ("skip_ms", C.c_double), ("total_ms", C.c_double),
                ("march_grid", C.c_uint32), ("skip_grid", C.c_uint32)]


class FptCudaBatchStats(C.Structure):
    _fields_ = [("elapsed_ms", C.c_double), ("build_ms", C.c_double), ("paths", C.c_uint64), ("scenes", C.c_uint32),
                ("passes", C.c_uint32), ("graph_launches", C.c_uint32), ("kernel_launches_per_pass", C.c_uint32),
                ("block_size", C.c_uint32), ("registers", C.c_uint32), ("wave_paths", C.c_uint32), ("tuned", C.c_uint32),
                ("workload_key", C.c_uint64), ("refill", C.c_uint32), ("_pad", C.c_uint32)]


class FptCudaTuneCandidate(C.Structure):
    _fields_ = [("block_size", C.c_uint32), ("registers", C.c_uint32), ("wave_paths", C.c_uint32), ("refill", C.c_uint32),
                ("median_ms", C.c_double)]


class FptCudaTuneResult(C.Structure):
    _fields_ = [("candidates", C.c_uint32), ("chosen", C.c_uint32), ("rounds", C.c_uint32), ("_pad", C.c_uint32),
                ("workload_key", C.c_uint64), ("tried", FptCudaTuneCandidate * 16)]


MLP_PARAMS = 19777

VOXEL_HIT_DTYPE = np.dtype([("t", np.float32), ("cell", np.uint32), ("normal_axis", np.uint32), ("steps", np.uint32),
                            ("shadow_steps", np.uint32), ("lit", np.uint32)])


def declare(L: C.CDLL) -> None:
    P = C.POINTER
    cfg, ext = P(ffi.FptRenderConfig), P(ffi.FptCudaSceneExt)
    err = [C.c_char_p, C.c_size_t]
    L.fpt_cuda_voxel_build.argtypes = [cfg, ext, C.c_uint32, P(FptCudaVoxelInfo)] + err
    L.fpt_cuda_voxel_read.argtypes = [P(C.c_uint32), C.c_size_t, P(C.c_uint8), P(C.c_uint16), P(C.c_uint32), C.c_size_t] + err
    L.fpt_cuda_dda_sequence.argtypes = [P(C.c_float), C.c_size_t, C.c_uint32, P(C.c_uint32), P(C.c_uint32),
                                        P(FptCudaVoxelHit)] + err
    L.fpt_cuda_voxel_render.argtypes = [cfg, ext, P(FptCudaVoxelHit), C.c_size_t, P(C.c_uint8), C.c_size_t,
                                        P(C.c_double)] + err
    L.fpt_cuda_voxel_build_static.argtypes = [cfg, ext, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
                                              C.c_size_t, P(FptCudaVoxelInfo)] + err
    fp = P(C.c_float)
    L.fpt_cuda_mlp_create.argtypes = [cfg, ext, P(FptCudaMlpConfig), P(C.c_uint64), P(FptCudaMlpStats)] + err
    L.fpt_cuda_mlp_destroy.argtypes = [C.c_uint64]
    L.fpt_cuda_mlp_predict.argtypes = [C.c_uint64, fp, C.c_size_t, fp] + err
    L.fpt_cuda_mlp_get_params.argtypes = [C.c_uint64, fp, C.c_size_t] + err
    L.fpt_cuda_mlp_set_params.argtypes = [C.c_uint64, fp, C.c_size_t] + err
    L.fpt_cuda_mlp_gradients.argtypes = [C.c_uint64, fp, C.c_size_t, C.c_float, fp, C.c_size_t, fp] + err
    L.fpt_cuda_skip_stats.argtypes = [P(FptCudaSkipStats)]
    L.fpt_cuda_render_stats.argtypes = [P(FptCudaRenderStats)]
    L.fpt_cuda_set_launch_shape.argtypes = [C.c_uint32, C.c_int32]
    L.fpt_cuda_set_march_schedule.argtypes = [C.c_uint32, C.c_uint32]
    L.fpt_cuda_set_network_engine.argtypes = [C.c_uint32]
    L.fpt_cuda_set_kernel_timing.argtypes = [C.c_uint32]
    L.fpt_test_bounded_waits.argtypes = [P(C.c_uint32), C.c_size_t] + err
    L.fpt_cuda_set_loop_limit.argtypes = [C.c_uint64]
    L.fpt_cuda_render_batch.argtypes = [cfg, ext, C.c_size_t, P(C.c_float), C.c_size_t, P(C.c_uint8), C.c_size_t,
                                        P(FptCudaBatchStats)] + err
    L.fpt_cuda_autotune_batch.argtypes = [cfg, ext, C.c_size_t, C.c_uint32, P(FptCudaTuneResult)] + err
    for name in ("fpt_cuda_voxel_build", "fpt_cuda_voxel_read", "fpt_cuda_dda_sequence", "fpt_cuda_voxel_render",
                 "fpt_cuda_voxel_build_static", "fpt_cuda_mlp_create", "fpt_cuda_mlp_destroy", "fpt_cuda_mlp_predict",
                 "fpt_cuda_mlp_get_params", "fpt_cuda_mlp_set_params", "fpt_cuda_mlp_gradients", "fpt_cuda_skip_stats",
                 "fpt_cuda_render_stats", "fpt_cuda_render_batch", "fpt_cuda_autotune_batch", "fpt_cuda_set_launch_shape",
                 "fpt_cuda_set_march_schedule", "fpt_cuda_set_network_engine", "fpt_cuda_set_kernel_timing",
                 "fpt_test_bounded_waits", "fpt_cuda_set_loop_limit"):
        getattr(L, name).restype = C.c_int


def _err():
    return C.create_string_buffer(1024)


def _check(rc, e):
    from .native import NativeError
    if rc != 0:
        raise NativeError(e.value.decode("utf-8", "replace"))


def voxel_build(cfg, ext, brick_size: int = 8) -> dict:
    from .native import lib
    info = FptCudaVoxelInfo()
    e = _err()
    _check(lib().fpt_cuda_voxel_build(C.byref(cfg), C.byref(ext) if ext is not None else None, brick_size, C.byref(info), e,
                                      len(e)), e)
    return {k: getattr(info, k) for k, _ in FptCudaVoxelInfo._fields_}


def voxel_read(info: dict, table=True, occupancy=True, distance=True, cells=False):
    from .native import lib
    nb = info["brick_grid"] ** 3
    bvol = info["brick_size"] ** 3 if info["brick_size"] else 1
    ncell = info["active_bricks"] * bvol if info["brick_size"] else info["resolution"] ** 3
    t = np.zeros(max(nb, 1), np.uint32) if table else None
    o = np.zeros(max(ncell, 1), np.uint8) if occupancy else None
    d = np.zeros(max(ncell, 1), np.uint16) if distance else None
    c = np.zeros((max(ncell, 1), 3), np.uint32) if cells else None
    e = _err()
    p = lambda a, ty: a.ctypes.data_as(C.POINTER(ty)) if a is not None else None
    _check(lib().fpt_cuda_voxel_read(p(t, C.c_uint32), nb, p(o, C.c_uint8), p(d, C.c_uint16), p(c, C.c_uint32), ncell, e, len(e)), e)
    return t, o, d, c


def dda_sequence(rays: np.ndarray, capacity: int = 0):
    from .native import lib
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    n = len(r)
    hits = np.zeros(n, VOXEL_HIT_DTYPE)
    seq = np.zeros((n, capacity), np.uint32) if capacity else None
    seq_len = np.zeros(n, np.uint32) if capacity else None
    e = _err()
    _check(lib().fpt_cuda_dda_sequence(r.ctypes.data_as(C.POINTER(C.c_float)), n, capacity,
                                       seq.ctypes.data_as(C.POINTER(C.c_uint32)) if seq is not None else None,
                                       seq_len.ctypes.data_as(C.POINTER(C.c_uint32)) if seq_len is not None else None,
                                       hits.ctypes.data_as(C.POINTER(FptCudaVoxelHit)), e, len(e)), e)
    return hits, seq, seq_len


def voxel_render(cfg, ext=None, image=True):
    from .native import lib
    n = cfg.width * cfg.height
    hits = np.zeros(n, VOXEL_HIT_DTYPE)
    rgba = np.zeros((cfg.height, cfg.width, 4), np.uint8) if image else None
    ms = C.c_double()
    e = _err()
    _check(lib().fpt_cuda_voxel_render(C.byref(cfg), C.byref(ext) if ext is not None else None,
                                       hits.ctypes.data_as(C.POINTER(FptCudaVoxelHit)), n,
                                       rgba.ctypes.data_as(C.POINTER(C.c_uint8)) if rgba is not None else None,
                                       rgba.size if rgba is not None else 0, C.byref(ms), e, len(e)), e)
    return hits.reshape(cfg.height, cfg.width), rgba, ms.value


def voxel_build_static(cfg, ext, device_table: int, table_len: int, device_occupancy: int, device_distance: int,
                       cell_capacity: int, stream: int | None = None) -> dict:
    """fpt_cuda_voxel_build_static: builds into caller-owned device buffers without allocating."""
    from .native import lib
    info = FptCudaVoxelInfo()
    e = _err()
    _check(lib().fpt_cuda_voxel_build_static(C.byref(cfg), C.byref(ext) if ext is not None else None, stream, device_table,
                                             table_len, device_occupancy, device_distance, cell_capacity, C.byref(info),
                                             e, len(e)), e)
    return {k: getattr(info, k) for k, _ in FptCudaVoxelInfo._fields_}


# ---------------------------------------------------------------- learned surrogate
def mlp_config(bounds_min, bounds_max, points=1 << 24, near_fraction=0.5, near_band=0.05, batch=16384, steps=2000,
               lr=2e-3, overestimate_weight=10.0, seed=1) -> FptCudaMlpConfig:
    mc = FptCudaMlpConfig()
    for k in range(3):
        mc.bounds_min[k] = float(bounds_min[k])
        mc.bounds_max[k] = float(bounds_max[k])
    mc.points, mc.near_fraction, mc.near_band = int(points), float(near_fraction), float(near_band)
    mc.batch, mc.steps, mc.lr = int(batch), int(steps), float(lr)
    mc.overestimate_weight, mc.seed = float(overestimate_weight), int(seed)
    return mc


def mlp_create(cfg, ext, mc: FptCudaMlpConfig):
    """Trains a surrogate on the GPU; returns (handle, stats dict)."""
    from .native import lib
    h = C.c_uint64()
    st = FptCudaMlpStats()
    e = _err()
    _check(lib().fpt_cuda_mlp_create(C.byref(cfg), C.byref(ext) if ext is not None else None, C.byref(mc), C.byref(h),
                                     C.byref(st), e, len(e)), e)
    return h.value, {k: getattr(st, k) for k, _ in FptCudaMlpStats._fields_}


def mlp_destroy(handle: int) -> None:
    from .native import lib
    lib().fpt_cuda_mlp_destroy(handle)


def _f32(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def mlp_predict(handle: int, points) -> np.ndarray:
    from .native import lib
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    out = np.zeros(len(pts), np.float32)
    e = _err()
    _check(lib().fpt_cuda_mlp_predict(handle, _f32(pts), len(pts), _f32(out), e, len(e)), e)
    return out


def mlp_get_params(handle: int) -> np.ndarray:
    from .native import lib
    out = np.zeros(MLP_PARAMS, np.float32)
    e = _err()
    _check(lib().fpt_cuda_mlp_get_params(handle, _f32(out), len(out), e, len(e)), e)
    return out


def mlp_set_params(handle: int, params) -> None:
    from .native import lib
    p = np.ascontiguousarray(params, np.float32)
    e = _err()
    _check(lib().fpt_cuda_mlp_set_params(handle, _f32(p), len(p), e, len(e)), e)


def mlp_gradients(handle: int, points, overestimate_weight=10.0):
    """(gradients[19777], mean loss) of the asymmetric loss over labelled xyzw points."""
    from .native import lib
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    g = np.zeros(MLP_PARAMS, np.float32)
    loss = C.c_float()
    e = _err()
    _check(lib().fpt_cuda_mlp_gradients(handle, _f32(pts), len(pts), overestimate_weight, _f32(g), len(g), C.byref(loss), e,
                                        len(e)), e)
    return g, loss.value


def skip_stats() -> dict:
    from .native import lib
    st = FptCudaSkipStats()
    lib().fpt_cuda_skip_stats(C.byref(st))
    return {k: getattr(st, k) for k, _ in FptCudaSkipStats._fields_ if k != "reserved"}


def render_stats() -> dict:
    """Launch count and per-kernel device times of the last render (times only for profile renders)."""
    from .native import lib
    st = FptCudaRenderStats()
    lib().fpt_cuda_render_stats(C.byref(st))
    return {k: getattr(st, k) for k, _ in FptCudaRenderStats._fields_}


# ---------------------------------------------------------------- batched scenes
def _batch_arrays(bundles):
    n = len(bundles)
    cfgs = (ffi.FptRenderConfig * n)()
    exts = (ffi.FptCudaSceneExt * n)()
    for k, b in enumerate(bundles):
        C.memmove(C.byref(cfgs[k]), C.byref(b.cfg), C.sizeof(ffi.FptRenderConfig))
        C.memmove(C.byref(exts[k]), C.byref(b.ext), C.sizeof(ffi.FptCudaSceneExt))
    return cfgs, exts


def render_batch(bundles, linear=True, rgba=False):
    """fpt_cuda_render_batch: per scene (H, W, 4) float32 accumulation (and uint8 images), plus stats."""
    from .native import lib
    cfgs, exts = _batch_arrays(bundles)
    sizes = [(b.cfg.height, b.cfg.width) for b in bundles]
    total = sum(h * w for h, w in sizes)
    lin = np.zeros(total * 4, np.float32) if linear else None
    img = np.zeros(total * 4, np.uint8) if rgba else None
    st = FptCudaBatchStats()
    e = _err()
    _check(lib().fpt_cuda_render_batch(cfgs, exts, len(bundles),
                                       lin.ctypes.data_as(C.POINTER(C.c_float)) if lin is not None else None,
                                       lin.size if lin is not None else 0,
                                       img.ctypes.data_as(C.POINTER(C.c_uint8)) if img is not None else None,
                                       img.size if img is not None else 0, C.byref(st), e, len(e)), e)
    out_lin, out_img, off = [], [], 0
    for h, w in sizes:
        if lin is not None:
            out_lin.append(lin[off * 4:(off + h * w) * 4].reshape(h, w, 4))
        if img is not None:
            out_img.append(img[off * 4:(off + h * w) * 4].reshape(h, w, 4))
        off += h * w
    return out_lin, out_img, {k: getattr(st, k) for k, _ in FptCudaBatchStats._fields_ if k != "_pad"}


def autotune_batch(bundles, rounds=3) -> dict:
    from .native import lib
    cfgs, exts = _batch_arrays(bundles)
    r = FptCudaTuneResult()
    e = _err()
    _check(lib().fpt_cuda_autotune_batch(cfgs, exts, len(bundles), rounds, C.byref(r), e, len(e)), e)
    tried = [{k: getattr(r.tried[i], k) for k, _ in FptCudaTuneCandidate._fields_ if k != "_pad"} for i in range(r.candidates)]
    return {"chosen": r.chosen, "rounds": r.rounds, "workload_key": r.workload_key, "tried": tried}


def set_launch_shape(wave_paths: int = 0, march_blocks: int = 0) -> None:
    from .native import lib
    lib().fpt_cuda_set_launch_shape(wave_paths, march_blocks)


NET_TCGEN05 = 0
NET_MMA_SYNC = 1


def set_loop_limit(limit_ns: int = 0) -> None:
    """Time limit of the persistent loops of later renders in ns (0: 10 s)."""
    from .native import lib
    lib().fpt_cuda_set_loop_limit(limit_ns)


def bounded_wait_check() -> dict:
    """fpt_test_bounded_waits: an mbarrier wait after an arrival and one with none (20 ms limit)."""
    from .native import lib
    r = (C.c_uint32 * 4)()
    e = _err()
    _check(lib().fpt_test_bounded_waits(r, 4, e, len(e)), e)
    return {"arrived": r[0], "not_arrived": r[1], "arrived_ns": r[2], "not_arrived_ns": r[3]}


def set_network_engine(engine: int = NET_TCGEN05) -> None:
    """Surrogate network engine of later skip passes and predictions: NET_TCGEN05 (default) or NET_MMA_SYNC."""
    from .native import lib
    if lib().fpt_cuda_set_network_engine(engine) != 0:
        raise ValueError("engine must be NET_TCGEN05 (0) or NET_MMA_SYNC (1)")


def set_kernel_timing(on: bool = True) -> None:
    """Per-kernel event spans (render_stats march/shade/skip ms) in every later render, not only profile renders."""
    from .native import lib
    if lib().fpt_cuda_set_kernel_timing(int(on)) != 0:
        raise ValueError("kernel timing is on (1) or off (0)")


def set_march_schedule(schedule: int = 0, batch: int = 0) -> None:
    """Lockstep march (schedule 0, the only one); `batch` finished lanes refill together (0: 8)."""
    from .native import lib
    if lib().fpt_cuda_set_march_schedule(schedule, batch) != 0:
        raise ValueError("schedule must be 0 and batch 0..32")


def certified_step_bound(cfg, ext, sun_direction, stride: int = 4, margin: float = 0.1) -> dict:
    """Perfect-proposal bound of the surrogate skip per ray type (fpt_cuda_certified_steps): plain-march and
    certified evaluations of camera, sun shadow and bounce rays of every `stride`-th pixel, and their ratio."""
    from . import native
    c = native.certified_steps(cfg, ext, sun_direction, stride, margin).astype(np.int64)
    out = {}
    for k, name in enumerate(("camera", "shadow", "bounce")):
        plain, cert = int(c[:, 2 * k].sum()), int(c[:, 2 * k + 1].sum())
        out[name] = {"rays": int((c[:, 2 * k] > 0).sum()), "plain_evals": plain, "certified_evals": cert,
                     "ratio": plain / max(cert, 1)}
    return out
