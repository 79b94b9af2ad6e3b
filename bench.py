"""Benchmark: Mpaths/s at 1920x1080, 16 spp, 4 bounces (power-8 Mandelbulb path tracing),
surrogate-skip march vs plain march.

One step = one full render of the frame (W*H*spp camera paths through all
their bounces) by libfpt_cuda.so.  `value` is the surrogate-skip march's
device throughput, measured with CUDA events on the library's stream (scene
and trained network resident in HBM); the plain march is measured the same
way beside it, and primary rays of both marches are compared for equal hit
distance.  `e2e` is the same metric through the public C ABI call with host
buffers (config upload and image readback inside the timed region).  The
working set (one 33 MB accumulation buffer) fits in L2, so L2 is flushed by
writing a 256 MB buffer between timed steps.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun (N > 1) every rank renders the full frame (replicas; weak
scaling) and rank 0 prints the line; value = all paths / max rank time.
"""
from __future__ import annotations

import argparse
import json

import numpy as np
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpaths/s at 1080p 16spp: surrogate-skip vs plain march at equal hit-dist error"
UNIT = "Mpaths/s"
W, H, SPP, BOUNCES = 1920, 1080, 16, 4


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 4 + i and r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def reduce_over_ranks(vals, world, device):
    """Element-wise maximum of per-rank timings over all ranks (the job time is the slowest replica's)."""
    if world <= 1:
        return list(vals)
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(vals), device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def job_throughput(paths_per_rank, steps, world, max_seconds):
    """Whole-job Mpaths/s: every rank renders `paths_per_rank` per step (replicas, weak scaling)."""
    return paths_per_rank * steps * world / max_seconds / 1e6


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


WORKLOAD = f"power-8 Mandelbulb path tracing {W}x{H} {SPP}spp {BOUNCES} bounces, RR after 2"


def run_reference(args, world, rank):
    """CPU arm: the oracle's FP32 restatement of the path, all host threads, bounded sample of the workload."""
    if rank != 0:
        return
    import oracle
    from fractalpathtracer_gb300 import scenes
    b = scenes.mandelbulb_path(W, H, SPP, BOUNCES)
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    ys, xs = CPU_GRID
    paths = ((H + ys - 1) // ys) * ((W + xs - 1) // xs) * SPP
    for _ in range(max(args.warmup, 0) and 1):
        small = ffi_copy_cfg(b.cfg)
        small.samples = 1
        oracle.render_grid(small, b.ext, ys * 8, xs * 8)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        oracle.render_grid(b.cfg, b.ext, ys, xs)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = paths * len(times) / total / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / len(times) * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD, "march": "plain (the reference has no surrogate)",
                   "parallelism": f"{cores} host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"every {ys}th row and {xs}th column of the {W}x{H} frame (a grid spread evenly "
                                   f"over the whole image), all {SPP} samples: {paths} paths per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# Algorithmic work of one power-8 Mandelbulb DE evaluation (8 iterations),
# counted on the reference's trigonometric form (src/mandelbulber/orbit.rs:
# 529-585): 25 FP32 ops per iteration (the fixed table frozen before
# measuring; its 7 transcendental calls per iteration are not counted as FP32
# work, and the algebraic power-8 step executes none).
DE_FP32_OPS = 200
MLP_FLOP = 2 * (99 * 64 + 3 * 64 * 64 + 64)              # one network row (37.3 kFLOP)
# CPU samples (reference arm and cpu_baseline): every 4th row and 4th column.
CPU_GRID = (4, 4)


def ffi_copy_cfg(cfg):
    import ctypes
    out = type(cfg)()
    ctypes.memmove(ctypes.byref(out), ctypes.byref(cfg), ctypes.sizeof(cfg))
    return out


def surrogate_config(scene: str = "mandelbulb"):
    """Training recipe of the learned skip: 16M points labelled by the exact DE (50% uniform in the
    box, 50% within 0.05 of the surface), asymmetric loss with 10x weight on overestimates."""
    from fractalpathtracer_gb300 import native_ext as nx, scenes
    lo, hi = scenes.SURROGATE_BOXES[scene]
    return nx.mlp_config(lo, hi, points=1 << 24, near_fraction=0.5, near_band=0.05, batch=16384, steps=4000,
                         lr=2e-3, overestimate_weight=10.0, seed=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-baseline", type=int, default=1)
    ap.add_argument("--only", default="", choices=["", "plain", "box", "skip", "voxel", "train", "predict"],
                    help="render only this march (profiling runs: no training unless skip, no JSON contract line)")
    ap.add_argument("--res", default=f"{W}x{H}", help="--only runs: image size WxH")
    ap.add_argument("--spp", type=int, default=SPP, help="--only runs: samples per pixel")
    ap.add_argument("--engine", default="tcgen05", choices=["tcgen05", "mma_sync"],
                    help="surrogate network engine of the skip arm")
    ap.add_argument("--voxel-res", type=int, default=1024, help="--only voxel: grid resolution")
    args = ap.parse_args()
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.only:
        run_only(args)
        return

    import ctypes
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from fractalpathtracer_gb300 import build, native, native_ext as nx, scenes
    build.build()
    native.lib()
    native.set_device(local)   # the library links its own CUDA runtime: bind it to this rank's GPU
    if native.get_device() != torch.cuda.current_device():
        raise RuntimeError(f"libfpt_cuda.so is bound to device {native.get_device()}, torch to {torch.cuda.current_device()}")
    engine = nx.NET_TCGEN05 if args.engine == "tcgen05" else nx.NET_MMA_SYNC
    nx.set_network_engine(engine)
    b = scenes.mandelbulb_path(W, H, SPP, BOUNCES)
    cfg, ext = b.cfg, b.ext
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    def series(e, steps, clocks=None):
        """Device-timed renders (library CUDA events) with L2 flushed before each.  The timed renders carry no
        profile counters (their atomics would add work to the kernels), only per-kernel event spans; the
        evaluation counts come from one profile render after them (the same frame, the same counts)."""
        out = {"ms": [], "march_ms": 0.0, "march_launches": 0, "march_evals": 0, "skip_ms": 0.0, "shade_ms": 0.0,
               "launches": 0, "phase_evals": None}
        nx.set_kernel_timing(True)
        try:
            for _ in range(steps):
                flush.zero_()
                torch.cuda.synchronize()
                _, _, ms = native.cuda_render(cfg, e, linear=False)
                rs = nx.render_stats()
                out["ms"].append(ms)
                out["march_ms"] += rs["march_ms"]
                out["march_launches"] += rs["march_launches"]
                out["skip_ms"] += rs["skip_ms"]
                out["shade_ms"] += rs["shade_ms"]
                out["launches"] += rs["kernel_launches"]
        finally:
            nx.set_kernel_timing(False)
        _, _, _, prof = native.cuda_render(cfg, e, linear=False, profile=True)
        out["march_evals"] = nx.render_stats()["march_evals"] * steps
        out["phase_evals"] = [int(prof.primary_steps), int(prof.secondary_steps), int(prof.shadow_steps)]
        return out

    # End-to-end through the public call: the results land in pinned host buffers (allocated once, reused).
    pinned_lin = torch.empty(W * H * 4, dtype=torch.float32, pin_memory=True).numpy()
    pinned_rgba = torch.empty(W * H * 4, dtype=torch.uint8, pin_memory=True).numpy()

    def e2e_series(e, steps):
        times = []
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            native.cuda_render(cfg, e, linear=True, out_linear=pinned_lin, out_rgba=pinned_rgba)
            times.append(time.perf_counter() - t)
        return times

    def reduce_max(vals):
        return reduce_over_ranks(vals, world, "cuda")

    paths = W * H * SPP
    fp32 = native.measure_fp32_peak()   # the FP32 roofline's denominator, measured on this GPU now
    # ---- plain march
    for _ in range(args.warmup):
        native.cuda_render(cfg, ext, linear=False)
    barrier()
    plain = series(ext, args.steps)
    barrier()
    plain_e2e = e2e_series(ext, args.steps)
    barrier()
    # ---- what a perfect proposal could save under the skip's certificate (per ray type, then weighted by the
    # plain frame's evaluations per phase)
    bound = nx.certified_step_bound(cfg, ext, list(ext.sun_direction), stride=4, margin=0.1)
    bound0 = nx.certified_step_bound(cfg, ext, list(ext.sun_direction), stride=4, margin=0.0)
    # ---- learned skip: train once (outside the timed region), then render
    model, train = nx.mlp_create(cfg, ext, surrogate_config())
    skip_ext = ffi_copy(ext)
    skip_ext.surrogate = 1
    skip_ext.surrogate_model = model
    for _ in range(args.warmup):
        native.cuda_render(cfg, skip_ext, linear=False)
    barrier()
    with ClockSampler(local) as clocks:
        skip = series(skip_ext, args.steps)
    barrier()
    skip_stats = nx.skip_stats()
    skip_e2e = e2e_series(skip_ext, args.steps)
    barrier()
    # ---- the same skip march with the network on the other engine (comparison only)
    other = nx.NET_MMA_SYNC if engine == nx.NET_TCGEN05 else nx.NET_TCGEN05
    nx.set_network_engine(other)
    for _ in range(args.warmup):
        native.cuda_render(cfg, skip_ext, linear=False)
    barrier()
    skip_other = series(skip_ext, args.steps)
    nx.set_network_engine(engine)
    barrier()
    # ---- the same march without the network (the model's box only)
    box_ext = ffi_copy(skip_ext)
    box_ext.surrogate = 2
    for _ in range(args.warmup):
        native.cuda_render(cfg, box_ext, linear=False)
    barrier()
    box = series(box_ext, args.steps)
    barrier()
    p_ms, p_e2e, s_ms, s_e2e, b_ms, o_ms = reduce_max([sum(plain["ms"]), sum(plain_e2e), sum(skip["ms"]), sum(skip_e2e),
                                                       sum(box["ms"]), sum(skip_other["ms"])])
    plain_value = job_throughput(paths, args.steps, world, p_ms / 1e3)
    plain_e2e_v = job_throughput(paths, args.steps, world, p_e2e)
    value = job_throughput(paths, args.steps, world, s_ms / 1e3)
    e2e = job_throughput(paths, args.steps, world, s_e2e)
    # ---- equal hit distance: primary rays of the same camera, plain vs skip march
    hp, _ = native.trace_primary(cfg, ext)
    hs, _ = native.trace_primary(cfg, skip_ext)
    both = (hp["hit"] > 0) & (hs["hit"] > 0)
    dt = np.abs(hp["distance"][both].astype(np.float64) - hs["distance"][both]) / (1.0 + hp["distance"][both])
    hit_agree = float(((hp["hit"] > 0) == (hs["hit"] > 0)).mean())
    nx.mlp_destroy(model)
    # ---- roofline of the dominant kernel (the march kernel), timed live over the timed region
    skip_kernel = "skip_march_tc_kernel" if engine == nx.NET_TCGEN05 else "skip_march_kernel"
    dom = "march_kernel" if skip["march_ms"] >= skip["skip_ms"] else skip_kernel
    march_launch_ms = skip["march_ms"] / max(skip["march_launches"], 1)
    evals_per_launch = skip["march_evals"] / max(skip["march_launches"], 1)
    achieved = evals_per_launch * DE_FP32_OPS / (march_launch_ms / 1e3) / 1e12
    plain_march_tflops = plain["march_evals"] * DE_FP32_OPS / (plain["march_ms"] / 1e3) / 1e12
    fp32_peak = fp32["tflops"]
    clk = clocks.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": s_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD,
                   "march": "surrogate-skip (value) vs plain", "l2": "flushed (256 MB write) between steps",
                   "parallelism": f"replicas x{world}",
                   "surrogate": "3->99 Fourier->4x64 SiLU->1 bf16, 16M points (50% near-surface), 4000 Adam steps"},
        "plain": {"value": plain_value, "e2e": plain_e2e_v, "ms_per_step": p_ms / args.steps,
                  "de_evals_per_s": plain["march_evals"] / (sum(plain["ms"]) / 1e3)},
        "skip_over_plain": value / plain_value,
        "network_engine": args.engine,
        "skip_other_engine": {"engine": "mma_sync" if engine == nx.NET_TCGEN05 else "tcgen05",
                              "value": job_throughput(paths, args.steps, world, o_ms / 1e3),
                              "ms_per_step": o_ms / args.steps, "skip_ms": skip_other["skip_ms"] / args.steps},
        "box_only": {"value": job_throughput(paths, args.steps, world, b_ms / 1e3), "ms_per_step": b_ms / args.steps,
                     "march_evals": box["march_evals"] // args.steps,
                     "note": "surrogate's box clip without the network (FPT_CUDA_SURROGATE_BOX)"},
        "hit_equality": {"primary_rays": W * H, "hit_agreement": hit_agree,
                         "p99_rel_dist_delta": float(np.percentile(dt, 99)) if dt.size else None,
                         "max_rel_dist_delta": float(dt.max()) if dt.size else None},
        "skip": {"exact_evals_in_skip": skip_stats["exact_evals"],
                 "march_evals": skip["march_evals"] // args.steps, "plain_march_evals": plain["march_evals"] // args.steps,
                 "network_rows": skip_stats["rows"], "accepted": skip_stats["accepted"],
                 "rejected": skip_stats["rejected"], "escaped": skip_stats["escaped"],
                 "skip_ms": skip["skip_ms"] / args.steps, "march_ms": skip["march_ms"] / args.steps,
                 "shade_ms": skip["shade_ms"] / args.steps, "train_ms": train["train_ms"], "data_ms": train["data_ms"],
                 "loss_first": train["loss_first"], "loss_last": train["loss_last"]},
        "perfect_proposal_bound": frame_bound(bound, bound0, plain["phase_evals"]),
        "e2e": {"value": e2e, "unit": UNIT, "host_buffers": "pinned, allocated once",
                "h2d_bytes_per_step": ctypes.sizeof(cfg) + ctypes.sizeof(ext),
                "d2h_bytes_per_step": W * H * 16 + W * H * 4},
        "gpu_launches": skip["launches"],
        "de_evals_per_s": (skip["march_evals"] + skip_stats["exact_evals"] * args.steps) / (sum(skip["ms"]) / 1e3),
        "roofline": {"bound": "fp32", "kernel": dom, "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": None,
                     "plain_march_frac": plain_march_tflops / fp32_peak,
                     "work": f"{DE_FP32_OPS} FP32 ops per DE evaluation x march-kernel evaluations",
                     "peak_source": f"measured in-process: FMA-chain kernel, 2048 threads/SM, best of 6 launches "
                                    f"({fp32['launch_ms']:.3f} ms each) on this GPU"},
        "clocks": {"sm_mhz": clk["sm_mhz"], "sm_max_mhz": clk["sm_max_mhz"], "reasons": clk["reasons"]},
    }
    if skip["skip_ms"] > 0:
        rows = skip_stats["rows"]   # live network rows per render (the statistics of the last render)
        tflops = rows * MLP_FLOP / (skip["skip_ms"] / args.steps / 1e3) / 1e12
        peaks = measured_peaks()
        line["roofline_skip_kernel"] = {"kernel": skip_kernel, "bound": "tensor", "achieved": tflops,
                                        "peak": peaks.get("bf16_tflops", 1900.0), "unit": "TFLOP/s",
                                        "frac": tflops / peaks.get("bf16_tflops", 1900.0),
                                        "peak_source": "MEASURED_PEAKS.json bf16 burst" if peaks else "fallback"}
    if rank == 0:
        line["other_configs"] = other_configs(native, nx, scenes, measured_peaks())
    if rank == 0 and args.cpu_baseline:
        try:
            import oracle
            cores = os.cpu_count() or 1
            oracle.set_threads(cores)
            ys, xs = CPU_GRID
            t = time.perf_counter()
            oracle.render_grid(cfg, ext, ys, xs)
            dt_cpu = time.perf_counter() - t
            n = ((H + ys - 1) // ys) * ((W + xs - 1) // xs) * SPP
            line["cpu_baseline"] = {"value": n / dt_cpu / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
                                    "sample": f"plain march, every {ys}th row and {xs}th column of the whole frame, "
                                              f"{SPP} spp ({n} paths, {dt_cpu:.1f} s)"}
        except Exception as exc:  # the baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                    "sample": f"failed: {exc}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def frame_bound(bound, bound0, phase_evals):
    """The most a perfect proposal could save on the frame: per ray type the ratio of plain to certified
    evaluations (camera / bounce / shadow rays of a pixel sample), applied to the plain frame's evaluations of
    primary / secondary / shadow rays; with the skip's hand-over margin 0.1 and with none."""
    out = {"per_ray_type_margin_0.1": bound, "per_ray_type_margin_0": bound0}
    if phase_evals:
        e = phase_evals
        for key, b in (("frame_bound_margin_0.1", bound), ("frame_bound_margin_0", bound0)):
            cert = e[0] / b["camera"]["ratio"] + e[1] / b["bounce"]["ratio"] + e[2] / b["shadow"]["ratio"]
            out[key] = sum(e) / cert
        out["plain_frame_evals_by_phase"] = e
    return out


def other_configs(native, nx, scenes, peaks):
    """Device-timed lines for the other workloads of the path (not the headline): 320x240 power-8 Mandelbulb
    primary rays; Menger fold + ground plane path tracing at 1280x720 16 spp; the 1024^3 Mandelbox occupancy-brick
    build and 1080p primary + shadow DDA (with its HBM roofline: 4 B brick-table read + 3 B occupancy / fp16
    distance per visited cell, 32 B output per pixel); 64 batched scenes; the learned skip on the Mandelbox."""
    med = lambda v: sorted(v)[len(v) // 2]
    out = {}
    cfg, ext = scenes.mandelbulb_primary(320, 240)
    for _ in range(3):
        native.trace_primary(cfg, ext)
    ms = med([native.trace_primary(cfg, ext)[1] for _ in range(7)])
    out["mandelbulb_primary_320x240"] = {"ms": ms, "Mrays_per_s": 320 * 240 / ms / 1e3}
    b = scenes.menger_plane(1280, 720, 16)
    for _ in range(2):
        native.cuda_render(b.cfg, b.ext, linear=False)
    ms = med([native.cuda_render(b.cfg, b.ext, linear=False)[2] for _ in range(3)])
    out["menger_plane_1280x720_16spp"] = {"ms": ms, "Mpaths_per_s": 1280 * 720 * 16 / ms / 1e3}
    cfg, ext = scenes.voxel_mandelbox(1024, 1920, 1080)
    info = nx.voxel_build(cfg, ext, 8)
    info = nx.voxel_build(cfg, ext, 8)
    for _ in range(2):
        nx.voxel_render(cfg, ext, image=False)
    runs = [nx.voxel_render(cfg, ext, image=False) for _ in range(5)]
    hits, _, ms = sorted(runs, key=lambda r: r[2])[2]
    cells = int(hits["steps"].astype(np.int64).sum() + hits["shadow_steps"].astype(np.int64).sum())
    nbytes = cells * 7 + hits.size * 32
    gbs = nbytes / (ms / 1e3) / 1e9
    hbm = peaks.get("hbm_gbs", 6800.0)
    out["mandelbox_voxel_1024"] = {
        "build_ms": info["build_ms"], "active_bricks": info["active_bricks"], "memory_bytes": info["memory_bytes"],
        "render_ms": ms, "Mrays_per_s": 2 * hits.size / ms / 1e3, "cells_visited": cells,
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                     "work": "7 B per visited cell + 32 B per pixel"}}
    # 64 batched scenes (seeded types, powers, iterations, 64^2..512^2, 4 spp, 3 bounces) in one persistent pass
    # per sample, each pass a CUDA graph; launch shape from the autotuner.
    bundles = scenes.batch_scenes(64)
    tune = nx.autotune_batch(bundles, rounds=2)
    nx.render_batch(bundles, linear=False)
    runs = [nx.render_batch(bundles, linear=False)[2] for _ in range(3)]
    st = sorted(runs, key=lambda r: r["elapsed_ms"])[1]
    out["batch_64_scenes_4spp"] = {"ms": st["elapsed_ms"], "Mpaths_per_s": st["paths"] / st["elapsed_ms"] / 1e3,
                                   "paths": st["paths"], "graph_launches": st["graph_launches"],
                                   "kernel_launches_per_pass": st["kernel_launches_per_pass"],
                                   "tuned_block": st["block_size"], "tuned_registers": st["registers"],
                                   "tuned_wave_paths": st["wave_paths"], "candidates": len(tune["tried"]),
                                   "candidate_median_ms": [round(c["median_ms"], 2) for c in tune["tried"]],
                                   "chosen": tune["chosen"]}
    # The learned skip on the Mandelbox (scale -1.5, 12 iterations): the same recipe, its own model.
    b = scenes.mandelbox_path(W, H, SPP, BOUNCES)
    model, train = nx.mlp_create(b.cfg, b.ext, surrogate_config("mandelbox"))
    arms = {}
    for name, mode in (("plain", 0), ("skip", 1), ("box_only", 2)):
        e = ffi_copy(b.ext)
        if mode:
            e.surrogate, e.surrogate_model = mode, model
        for _ in range(2):
            native.cuda_render(b.cfg, e, linear=False)
        ms = med([native.cuda_render(b.cfg, e, linear=False)[2] for _ in range(3)])
        arms[name] = {"ms": ms, "Mpaths_per_s": W * H * SPP / ms / 1e3}
        if mode == 1:
            arms[name]["skip_stats"] = nx.skip_stats()
            hp, _ = native.trace_primary(b.cfg, b.ext)
            hs, _ = native.trace_primary(b.cfg, e)
            both = (hp["hit"] > 0) & (hs["hit"] > 0)
            dt = np.abs(hp["distance"][both].astype(np.float64) - hs["distance"][both]) / (1.0 + hp["distance"][both])
            arms[name]["hit_agreement"] = float(((hp["hit"] > 0) == (hs["hit"] > 0)).mean())
            arms[name]["p99_rel_dist_delta"] = float(np.percentile(dt, 99)) if dt.size else None
    nx.mlp_destroy(model)
    arms["skip_over_plain"] = arms["skip"]["Mpaths_per_s"] / arms["plain"]["Mpaths_per_s"]
    arms["train_ms"] = train["train_ms"]
    arms["loss_last"] = train["loss_last"]
    out[f"mandelbox_skip_{W}x{H}_{SPP}spp"] = arms
    return out


def run_only(args):
    """One march variant at the bench workload, for profiler launch lists (small surrogate for skip/box)."""
    from fractalpathtracer_gb300 import build, native, native_ext as nx, scenes
    build.build()
    nx.set_network_engine(nx.NET_TCGEN05 if args.engine == "tcgen05" else nx.NET_MMA_SYNC)
    w, h = (int(v) for v in args.res.lower().split("x"))
    if args.only == "train":   # the surrogate's training recipe, `steps` x 10 Adam steps
        b = scenes.mandelbulb_path(64, 64, 1)
        mc = surrogate_config()
        mc.steps = args.steps * 10
        model, st = nx.mlp_create(b.cfg, b.ext, mc)
        nx.mlp_destroy(model)
        print(json.dumps({"only": "train", "steps": mc.steps, "train_ms": st["train_ms"], "loss_last": st["loss_last"]}), flush=True)
        return
    if args.only == "predict":   # the network alone: 8M-row predictions with seeded parameters (host copies included)
        b = scenes.mandelbulb_path(64, 64, 1)
        lo, hi = scenes.SURROGATE_BOXES["mandelbulb"]
        model, _ = nx.mlp_create(b.cfg, b.ext, nx.mlp_config(lo, hi, points=1 << 16, steps=1, batch=4096, seed=1))
        nx.mlp_set_params(model, scenes.random_mlp_params(11))
        rng = np.random.default_rng(5)
        pts = np.zeros((1 << 23, 4), np.float32)
        pts[:, :3] = rng.uniform(-1.25, 1.25, (1 << 23, 3))
        for _ in range(args.warmup):
            nx.mlp_predict(model, pts)
        ms = []
        for _ in range(args.steps):
            t = time.perf_counter()
            nx.mlp_predict(model, pts)
            ms.append((time.perf_counter() - t) * 1e3)
        nx.mlp_destroy(model)
        print(json.dumps({"only": "predict", "engine": args.engine, "rows": len(pts), "ms_with_copies": ms}), flush=True)
        return
    if args.only == "voxel":   # Mandelbox occupancy bricks (1024^3 by default), primary + shadow DDA
        cfg, ext = scenes.voxel_mandelbox(args.voxel_res, w, h)
        info = nx.voxel_build(cfg, ext, 8)
        for _ in range(args.warmup):
            nx.voxel_render(cfg, ext, image=False)
        ms = [nx.voxel_render(cfg, ext, image=False)[2] for _ in range(args.steps)]
        print(json.dumps({"only": "voxel", "build_ms": info["build_ms"], "ms": ms}), flush=True)
        return
    b = scenes.mandelbulb_path(w, h, args.spp, BOUNCES)
    cfg, ext = b.cfg, b.ext
    model = None
    if args.only != "plain":
        lo, hi = scenes.SURROGATE_BOXES["mandelbulb"]
        model, _ = nx.mlp_create(cfg, ext, nx.mlp_config(lo, hi, points=1 << 20, steps=400, batch=8192, seed=1))
        ext = ffi_copy(ext)
        ext.surrogate = 1 if args.only == "skip" else 2
        ext.surrogate_model = model
    for _ in range(args.warmup):
        native.cuda_render(cfg, ext, linear=False)
    ms = [native.cuda_render(cfg, ext, linear=False)[2] for _ in range(args.steps)]
    out = {"only": args.only, "engine": args.engine, "ms": ms, "stats": nx.render_stats()}
    if args.only == "skip":
        out["skip_stats"] = nx.skip_stats()
    print(json.dumps(out), flush=True)
    if model is not None:
        nx.mlp_destroy(model)


def ffi_copy(ext):
    import ctypes
    out = type(ext)()
    ctypes.memmove(ctypes.byref(out), ctypes.byref(ext), ctypes.sizeof(ext))
    return out


if __name__ == "__main__":
    main()
