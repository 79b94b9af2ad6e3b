"""Scene builders for the seeded synthetic workloads.

Each builder returns an ``FptRenderConfig`` (the reference's config ABI,
starting from ``default_config``) and, where the scene needs features the
reference config cannot express, an ``FptCudaSceneExt``.

Workloads (the sizes of the benchmark and parity suite):
  * ``mandelbulb_primary``  power-8 Mandelbulb, 8 iterations, bailout 2,
    320x240 primary rays, camera (0,0,-3) looking at the origin with a 60
    degree vertical field of view, <= 256 march steps, hit threshold
    1e-4 * |p - camera| / 3 (1e-4 at the target distance, growing with
    distance like the pixel footprint), analytic-derivative normals.
  * ``menger_plane``        Menger fold (5 iterations, scale 3) unioned with a
    ground plane, 1280x720, 16 spp, 4 bounces, Russian roulette after bounce
    2, Lambert 0.7 + GGX alpha 0.3, procedural HDR sky (RGBE 512x256 from the
    seed, sun direction (0.3, 0.8, 0.5)), PCG seed 1, ACES tone map.
  * ``mandelbulb_path`` / ``mandelbox_path``  the surrogate workload scenes,
    1920x1080, 16 spp, 4 bounces.
  * ``voxel_mandelbox``     Mandelbox (scale -1.5, 12 iterations, minimum
    radius 0.5, fold limit 1) in a 1024^3 grid over [-4, 4]^3.
  * ``batch_scenes``        64 scenes drawn from seed k.
"""
from __future__ import annotations

import math
import os
import tempfile

import numpy as np

from . import ffi


def look_at(cfg: ffi.FptRenderConfig, eye, target) -> None:
    """Sets camera position and yaw/pitch so the camera looks at target (rotateCamera convention)."""
    d = np.asarray(target, np.float64) - np.asarray(eye, np.float64)
    horiz = math.hypot(d[0], d[2])
    cfg.camera_position[:] = [float(v) for v in eye]
    cfg.camera_yaw_pitch[:] = [math.atan2(d[0], d[2]), math.atan2(d[1], horiz)]
    cfg.camera_roll = 0.0


def fov_for_vertical(vertical_deg: float) -> float:
    """FPT camera_fov whose image-plane span [-0.5, 0.5] covers the given vertical field of view."""
    return math.degrees(2.0 * math.atan(2.0 * math.tan(math.radians(vertical_deg) * 0.5)))


def _mandelbulber_march(cfg: ffi.FptRenderConfig, threshold_per_unit: float, max_steps: int, max_dist: float) -> None:
    v = cfg.vset_values
    cfg.set_values[0] = 1.0           # world scale
    v[107] = 0.0                      # perspective projection
    v[108] = 0.0                      # no advanced step quality
    v[109] = 1e-6
    v[110] = 10.0                     # absolute maximum step
    v[113] = 1.0                      # DE factor
    v[114] = 1.0                      # normal epsilon = threshold
    v[115] = 1.0                      # distance-dependent threshold
    v[116] = threshold_per_unit
    v[117] = threshold_per_unit
    v[118] = 1e-7                     # threshold clamp
    v[119] = 1.0
    v[129] = 1.0                      # detail level (refinement band 0.999)
    cfg.render[1] = float(max_steps)
    cfg.render[4] = float(max_dist)
    cfg.render[5] = 0.0
    cfg.render[6] = 0.0
    cfg.render[7] = 0.0


def mandelbulb_ext(power: float = 8.0, iterations: int = 8, bailout: float = 2.0) -> ffi.FptCudaSceneExt:
    e = ffi.FptCudaSceneExt()
    e.formula = ffi.FORMULA_MANDELBULB
    e.power = power
    e.iterations = iterations
    e.bailout = bailout
    e.normal_mode = ffi.NORMAL_ANALYTIC
    return e


def mandelbox_ext(scale: float = -1.5, iterations: int = 12, min_radius: float = 0.5, fold_limit: float = 1.0,
                  bailout: float = 100.0) -> ffi.FptCudaSceneExt:
    e = ffi.FptCudaSceneExt()
    e.formula = ffi.FORMULA_MANDELBOX
    e.box_scale = scale
    e.iterations = iterations
    e.box_min_radius = min_radius
    e.box_fixed_radius = 1.0
    e.box_fold_limit = fold_limit
    e.box_fold_value = 2.0 * fold_limit
    e.bailout = bailout
    e.normal_mode = ffi.NORMAL_ANALYTIC
    return e


def mandelbulb_primary(width: int = 320, height: int = 240):
    """Primary-ray Mandelbulb workload (hit distance, analytic normal, step count per pixel)."""
    cfg = ffi.default_config()
    cfg.width, cfg.height, cfg.samples = width, height, 1
    cfg.sdf_id = ffi.SDF_MANDELBULBER
    cfg.camera_fov = fov_for_vertical(60.0)
    cfg.camera_dof = 0.0
    cfg.focus_distance = 3.0
    look_at(cfg, (0.0, 0.0, -3.0), (0.0, 0.0, 0.0))
    _mandelbulber_march(cfg, 1e-4 / 3.0, 256, 10.0)
    cfg.render[0] = 1.0
    cfg.set_values[1] = 8.0
    cfg.set_values[2] = 2.0
    return cfg, mandelbulb_ext()


def _shading(cfg: ffi.FptRenderConfig, ext: ffi.FptCudaSceneExt, seed: int) -> None:
    ext.rng = ffi.RNG_PCG
    ext.seed = seed
    ext.brdf = ffi.BRDF_LAMBERT_GGX
    ext.albedo = 0.7
    ext.ggx_alpha = 0.3
    ext.specular_f0 = 0.04
    ext.plane_albedo = 0.5
    cfg.sdf_russian_roulette = 1
    cfg.sdf_rr_start = 2.0
    cfg.sdf_rr_min_prob = 0.2
    cfg.post[0] = 3.0   # ACES
    cfg.sun[:] = [1.0, 0.0, 0.0, 3.0, 0.02]
    cfg.sun_color[:] = [1.0, 0.95, 0.88]


def sky_equirect(width: int, height: int, sun_dir, seed: int) -> np.ndarray:
    """Procedural HDR sky (float RGB, row 0 = +y pole) on the renderer's equirect convention:
    u = fract(atan2(z, x) / 2pi + 0.5), v = acos(y) / pi, texel centres.  Zenith-to-horizon gradient,
    a sun glow and seeded value-noise clouds."""
    s = np.asarray(sun_dir, np.float64)
    s = s / np.linalg.norm(s)
    u = (np.arange(width) + 0.5) / width
    v = (np.arange(height) + 0.5) / height
    phi = (u - 0.5) * 2.0 * np.pi
    theta = v * np.pi
    uu, tt = np.meshgrid(phi, theta)
    d = np.stack([np.cos(uu) * np.sin(tt), np.cos(tt), np.sin(uu) * np.sin(tt)], -1)
    up = np.clip(d[..., 1], -1.0, 1.0)
    zen = np.array([0.18, 0.32, 0.75])
    hor = np.array([0.85, 0.85, 0.92])
    gnd = np.array([0.22, 0.2, 0.18])
    t = np.clip(up, 0.0, 1.0)[..., None] ** 0.45
    col = np.where(up[..., None] >= 0.0, hor * (1 - t) + zen * t, gnd * np.clip(1.0 + up[..., None] * 2.0, 0.3, 1.0))
    cosang = np.clip(d @ s, -1.0, 1.0)
    col = col + np.array([1.0, 0.85, 0.6]) * (np.exp((cosang - 1.0) * 60.0) * 4.0)[..., None]
    col = col + np.array([30.0, 28.0, 25.0]) * (cosang > math.cos(math.radians(0.8)))[..., None]
    rng = np.random.default_rng(seed)
    grid = rng.random((17, 33))
    gy = np.clip(theta / np.pi * 16.0, 0, 16 - 1e-6)
    gx = (phi / (2 * np.pi) + 0.5) * 32.0
    gyy, gxx = np.meshgrid(gy, gx, indexing="ij")
    y0, x0 = np.floor(gyy).astype(int), np.floor(gxx).astype(int) % 32
    fy, fx = gyy - y0, gxx - np.floor(gxx)
    x1 = (x0 + 1) % 32
    n = (grid[y0, x0] * (1 - fx) + grid[y0, x1] * fx) * (1 - fy) + (grid[y0 + 1, x0] * (1 - fx) + grid[y0 + 1, x1] * fx) * fy
    cloud = np.clip((n - 0.45) * 2.5, 0.0, 1.0) * (up > 0.02)
    col = col * (1 - 0.6 * cloud[..., None]) + 0.9 * cloud[..., None]
    return np.ascontiguousarray(col.astype(np.float32))


def rgbe_encode(rgb: np.ndarray) -> np.ndarray:
    """Float RGB -> RGBE bytes (shared exponent of the largest channel, mantissa * 256 / 2^e)."""
    m = rgb.max(axis=-1)
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    ok = m > 1e-32
    frac, exp = np.frexp(m[ok])
    scale = frac * 256.0 / m[ok]
    out[ok, :3] = np.clip(rgb[ok] * scale[:, None], 0, 255).astype(np.uint8)
    out[ok, 3] = (exp + 128).astype(np.uint8)
    return out


def rgbe_decode(rgbe: np.ndarray) -> np.ndarray:
    """RGBE bytes -> float RGB exactly as the Radiance reader (src/metal_bridge.mm:2247-2254)."""
    e = rgbe[..., 3].astype(np.int32)
    scale = np.where(e == 0, 0.0, np.ldexp(1.0, e - (128 + 8))).astype(np.float32)
    return ((rgbe[..., :3].astype(np.float32) + 0.5) * scale[..., None]).astype(np.float32)


def write_rgbe_file(path: str, rgbe: np.ndarray) -> None:
    """Radiance .hdr with new-style run-length scanlines (the format the reference reader accepts)."""
    h, w = rgbe.shape[:2]
    with open(path, "wb") as f:
        f.write(f"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y {h} +X {w}\n".encode())
        for y in range(h):
            f.write(bytes([2, 2, w >> 8, w & 255]))
            for ch in range(4):
                row = rgbe[y, :, ch]
                x = 0
                out = bytearray()
                while x < w:
                    run = 1
                    while x + run < w and run < 127 and row[x + run] == row[x]:
                        run += 1
                    if run >= 3:
                        out += bytes([128 + run, int(row[x])])
                        x += run
                    else:
                        start = x
                        cnt = 0
                        while x < w and cnt < 128:
                            r = 1
                            while x + r < w and r < 3 and row[x + r] == row[x]:
                                r += 1
                            if r >= 3:
                                break
                            x += 1
                            cnt += 1
                        out += bytes([cnt]) + bytes(int(b) for b in row[start:start + cnt])
                f.write(out)


class SceneBundle:
    """Keeps host arrays referenced by an extension struct alive with it."""

    def __init__(self, cfg, ext, keep=()):
        self.cfg, self.ext, self.keep = cfg, ext, list(keep)

    def __iter__(self):
        return iter((self.cfg, self.ext))


def attach_sky(ext: ffi.FptCudaSceneExt, sky: np.ndarray):
    import ctypes as C
    sky = np.ascontiguousarray(sky, np.float32)
    ext.sky_height, ext.sky_width = sky.shape[:2]
    ext.sky_rgb = sky.ctypes.data_as(C.POINTER(C.c_float))
    return sky


def menger_plane(width: int = 1280, height: int = 720, spp: int = 16, seed: int = 1, sky_size=(512, 256)) -> SceneBundle:
    """Menger fold unioned with a ground plane, full path tracing with the seeded RGBE sky."""
    cfg = ffi.default_config()
    cfg.width, cfg.height, cfg.samples = width, height, spp
    cfg.sdf_id = ffi.SDF_MENGER_SPONGE
    cfg.camera_fov = fov_for_vertical(45.0)
    cfg.camera_dof = 0.0
    cfg.focus_distance = 4.0
    look_at(cfg, (2.6, 1.5, -3.4), (0.0, -0.15, 0.0))
    cfg.render[:] = [4.0, 256.0, 1e-4, 1e-4, 50.0, 0.0, 0.0, 0.0]
    cfg.world[:] = [1.0, 1.0, 0.0, 30.0, 1.0, 1.0, 0.0]
    ext = ffi.FptCudaSceneExt()
    ext.formula = ffi.FORMULA_MENGER_FOLD
    ext.menger_scale = 3.0
    ext.iterations = 5
    ext.bailout = 1.0e6
    ext.ground_plane = 1
    ext.plane_height = -1.0
    ext.normal_mode = ffi.NORMAL_ANALYTIC
    _shading(cfg, ext, seed)
    sun = (0.3, 0.8, 0.5)
    ext.sun_direction[:] = list(sun)
    ext.sun_intensity = 3.0
    sky = rgbe_decode(rgbe_encode(sky_equirect(sky_size[0], sky_size[1], sun, seed)))
    sky = attach_sky(ext, sky)
    return SceneBundle(cfg, ext, [sky])


def _fractal_path(ext: ffi.FptCudaSceneExt, width: int, height: int, spp: int, bounces: int, seed: int, eye, target,
                  threshold_per_unit: float) -> SceneBundle:
    cfg = ffi.default_config()
    cfg.width, cfg.height, cfg.samples = width, height, spp
    cfg.sdf_id = ffi.SDF_MANDELBULBER
    cfg.camera_fov = fov_for_vertical(60.0)
    cfg.camera_dof = 0.0
    cfg.focus_distance = 3.0
    look_at(cfg, eye, target)
    _mandelbulber_march(cfg, threshold_per_unit, 256, 12.0)
    cfg.render[0] = float(bounces)
    cfg.set_values[1] = float(ext.iterations)
    cfg.set_values[2] = float(ext.bailout)
    cfg.world[:] = [1.0, 1.0, 0.0, 30.0, 1.0, 1.0, 0.0]
    _shading(cfg, ext, seed)
    ext.sun_direction[:] = [0.3, 0.8, 0.5]
    ext.sun_intensity = 3.0
    return SceneBundle(cfg, ext)


def mandelbulb_path(width: int = 1920, height: int = 1080, spp: int = 16, bounces: int = 4, seed: int = 1) -> SceneBundle:
    return _fractal_path(mandelbulb_ext(), width, height, spp, bounces, seed, (0.0, 0.0, -3.0), (0.0, 0.0, 0.0), 1e-4 / 3.0)


def mandelbox_path(width: int = 1920, height: int = 1080, spp: int = 16, bounces: int = 4, seed: int = 1) -> SceneBundle:
    return _fractal_path(mandelbox_ext(), width, height, spp, bounces, seed, (0.0, 1.5, -7.0), (0.0, 0.0, 0.0), 1e-4 / 7.0)


def hybrid_ext(power: float = 8.0, iterations: int = 9, menger_scale: float = 3.0, period: int = 3,
               bailout: float = 4.0) -> ffi.FptCudaSceneExt:
    """Mandelbulb / Menger-fold hybrid: every period-th iteration is a Menger fold (2:1 for period 3)."""
    e = ffi.FptCudaSceneExt()
    e.formula = ffi.FORMULA_BULB_MENGER_HYBRID
    e.power = power
    e.iterations = iterations
    e.menger_scale = menger_scale
    e.hybrid_period = period
    e.bailout = bailout
    e.normal_mode = ffi.NORMAL_ANALYTIC
    return e


def mandelbulb_deep_zoom(eye, target, width: int = 64, height: int = 48, fov_deg: float = 0.05,
                         threshold_per_unit: float = 1e-7, fp64: bool = True):
    """Deep-zoom primary rays on the power-8 Mandelbulb: a camera a short way off the surface with a tiny field of
    view, so the hit threshold (pixel footprint) falls below the FP32 resolution of the hit position; `fp64` turns
    on the FP64 hit-point continuation."""
    cfg, ext = mandelbulb_primary(width, height)
    cfg.camera_fov = fov_for_vertical(fov_deg)
    look_at(cfg, eye, target)
    _mandelbulber_march(cfg, threshold_per_unit, 2000, 10.0)
    cfg.vset_values[118] = 1e-14      # threshold clamp below the zoom's footprint
    cfg.vset_values[109] = 1e-15
    cfg.set_values[1] = 8.0
    cfg.set_values[2] = 2.0
    ext.fp64_bisection = 1 if fp64 else 0
    return cfg, ext


def flat_union_program(seed: int = 0, spheres: int = 6, boxes: int = 5, planes: int = 1, width: int = 160,
                       height: int = 120) -> ffi.FptRenderConfig:
    """A typed program that is a flat union of translated spheres, boxes and planes, together with its typed-SoA
    lowering (sdf_typed_soa: each primitive's accumulated translation, sizes and source instruction), the form
    the reference's scene loader produces for such programs.  Voxel bounds frame the validation samples."""
    rng = np.random.default_rng(seed)
    cfg = ffi.default_config()
    cfg.width, cfg.height = width, height
    cfg.sdf_id = ffi.SDF_PROGRAM
    soa = cfg.sdf_typed_soa
    prog, acc = [], np.zeros(3)

    def move(to):
        nonlocal acc
        delta = np.asarray(to, np.float64) - acc
        prog.append((ffi.OP_TRANSLATE, 0, (*delta, 0.0)))
        acc = acc + delta
        return acc.astype(np.float32)

    kinds = ["s"] * spheres + ["b"] * boxes + ["p"] * planes
    rng.shuffle(kinds)
    for kind in kinds:
        if kind == "p":
            c = move((0.0, float(rng.uniform(-1.2, -0.8)), 0.0))
            normal = np.array([rng.uniform(-0.1, 0.1), 1.0, rng.uniform(-0.1, 0.1)], np.float32)
            offset = float(rng.uniform(-0.05, 0.05))
            src = len(prog)
            prog.append((ffi.OP_PLANE, 0, (*normal, offset)))
            i = soa.plane_count
            soa.plane_x[i], soa.plane_y[i], soa.plane_z[i] = (float(v) for v in normal)
            soa.plane_center_x[i], soa.plane_center_y[i], soa.plane_center_z[i] = (float(v) for v in c)
            soa.plane_offset[i], soa.plane_source[i] = offset, src
            soa.plane_count += 1
            continue
        c = move(rng.uniform(-1.5, 1.5, 3) * np.array([1.0, 0.6, 1.0]))
        src = len(prog)
        if kind == "s":
            r = float(rng.uniform(0.2, 0.5))
            prog.append((ffi.OP_SPHERE, 0, (r, 0.0, 0.0, 0.0)))
            i = soa.sphere_count
            soa.sphere_x[i], soa.sphere_y[i], soa.sphere_z[i] = (float(v) for v in c)
            soa.sphere_radius[i], soa.sphere_source[i] = r, src
            soa.sphere_count += 1
        else:
            h = rng.uniform(0.15, 0.45, 3).astype(np.float32)
            prog.append((ffi.OP_BOX, 0, (*h, 0.0)))
            i = soa.box_count
            soa.box_x[i], soa.box_y[i], soa.box_z[i] = (float(v) for v in c)
            soa.box_half_x[i], soa.box_half_y[i], soa.box_half_z[i] = (float(v) for v in h)
            soa.box_source[i] = src
            soa.box_count += 1
    for i, (op, flags, d) in enumerate(prog):
        cfg.sdf_program[i].opcode = op
        cfg.sdf_program[i].flags = flags
        cfg.sdf_program[i].data[:] = [float(v) for v in d]
    cfg.sdf_program_count = len(prog)
    cfg.voxel_bounds_min[:] = [-2.0, -2.0, -2.0]
    cfg.voxel_bounds_max[:] = [2.0, 2.0, 2.0]
    cfg.camera_position[:] = [0.0, 0.6, -5.0]
    return cfg


def batch_scene(k: int, spp: int = 4, bounces: int = 3) -> SceneBundle:
    """Scene k of the batched workload, drawn from a PCG64 stream seeded by k: a Mandelbulb (power
    U[2, 12]), a Mandelbox (scale U[-2.5, -1.5]) or a 2:1 Mandelbulb / Menger hybrid; iterations U{4..16};
    square image with a log-uniform side in [64, 512]; seeded camera azimuth."""
    rng = np.random.default_rng(k)
    kind = int(rng.integers(3))
    iters = int(rng.integers(4, 17))
    side = int(round(math.exp(rng.uniform(math.log(64.0), math.log(512.0)))))
    az = rng.uniform(0.0, 2.0 * math.pi)
    if kind == 0:
        ext = mandelbulb_ext(power=float(rng.uniform(2.0, 12.0)), iterations=iters, bailout=2.0)
        dist, thr = 3.0, 1e-4 / 3.0
    elif kind == 1:
        ext = mandelbox_ext(scale=float(rng.uniform(-2.5, -1.5)), iterations=iters)
        dist, thr = 7.0, 1e-4 / 7.0
    else:
        ext = hybrid_ext(iterations=iters)
        dist, thr = 3.5, 1e-4 / 3.5
    eye = (dist * math.sin(az), 0.25 * dist, -dist * math.cos(az))
    return _fractal_path(ext, side, side, spp, bounces, k + 1, eye, (0.0, 0.0, 0.0), thr)


def batch_scenes(count: int = 64, spp: int = 4, bounces: int = 3):
    """The batched workload: scenes 0..count-1 of batch_scene."""
    return [batch_scene(k, spp, bounces) for k in range(count)]


# Boxes holding all of each surrogate scene's surface (the power-8 Mandelbulb
# reaches |x| ~ 1.11, the scale -1.5 Mandelbox |x| ~ 2.01): the skip march
# treats rays leaving them as misses.
SURROGATE_BOXES = {
    "mandelbulb": ((-1.25, -1.25, -1.25), (1.25, 1.25, 1.25)),
    "mandelbox": ((-2.25, -2.25, -2.25), (2.25, 2.25, 2.25)),
}


def random_mlp_params(seed: int = 0, out_scale: float = 0.3) -> np.ndarray:
    """He-uniform parameters in the surrogate's layout (W0 padding columns zero), for parity tests."""
    rng = np.random.default_rng(seed)
    p = np.zeros(19777, np.float32)
    off = 0
    for layer in range(4):
        k, fan = (112, 99) if layer == 0 else (64, 64)
        w = rng.uniform(-1, 1, (64, k)) * np.sqrt(6.0 / fan)
        if layer == 0:
            w[:, 99:] = 0.0
        p[off:off + 64 * k] = w.ravel()
        off += 64 * k
        p[off:off + 64] = rng.uniform(-0.1, 0.1, 64)
        off += 64
    p[off:off + 64] = rng.uniform(-out_scale, out_scale, 64)
    p[off + 64] = 0.05
    return p


def voxel_mandelbox(resolution: int = 1024, width: int = 1920, height: int = 1080):
    """Mandelbox (scale -1.5, 12 iterations, min radius 0.5, fold limit 1) voxelized over [-4, 4]^3;
    primary + one shadow ray per pixel through the occupancy bricks."""
    cfg = ffi.default_config()
    cfg.width, cfg.height, cfg.samples = width, height, 1
    cfg.sdf_id = ffi.SDF_MANDELBOX_FRACTAL
    cfg.renderer_backend = ffi.RENDERER_VOXEL
    cfg.voxel_resolution = resolution
    cfg.voxel_bounds_min[:] = [-4.0, -4.0, -4.0]
    cfg.voxel_bounds_max[:] = [4.0, 4.0, 4.0]
    cfg.voxel_surface_band = 1.0
    cfg.camera_fov = fov_for_vertical(50.0)
    cfg.camera_dof = 0.0
    cfg.focus_distance = 8.0
    look_at(cfg, (5.5, 4.0, -9.0), (0.0, 0.0, 0.0))
    ext = mandelbox_ext()
    ext.sun_direction[:] = [0.3, 0.8, 0.5]
    ext.sun_intensity = 1.0
    return cfg, ext


def temp_path(name: str) -> str:
    return os.path.join(tempfile.gettempdir(), name)
