"""Benchmark: Mpaths/s at 1920x1080, 16 spp, 4 bounces (power-8 Mandelbulb path tracing).

One step = one full render of the frame (W*H*spp camera paths through all
their bounces) by libfpt_cuda.so.  `value` is device throughput measured
with CUDA events on the library's stream (scene resident in HBM); `e2e` is
the same metric through the public C ABI call with host buffers (config
upload and image readback inside the timed region).  The working set (one
33 MB accumulation buffer) fits in L2, so L2 is flushed by writing a 256 MB
buffer between timed steps.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun (N > 1) every rank renders the full frame (replicas; weak
scaling) and rank 0 prints the line; value = all paths / max rank time.
"""
from __future__ import annotations

import argparse
import json
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


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def run_reference(args, world, rank):
    """CPU arm: the oracle's FP32 restatement of the path, all host threads, bounded sample of the workload."""
    if rank != 0:
        return
    import oracle
    from fractalpathtracer_gb300 import scenes
    b = scenes.mandelbulb_path(W, H, SPP, BOUNCES)
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    stride, rows = 16, (H // 2 - 8, H // 2 + 8)
    paths = ((rows[1] - rows[0]) * ((W + stride - 1) // stride)) * SPP
    for _ in range(max(args.warmup, 0) and 1):
        oracle.render(b.cfg, b.ext, rows=(rows[0], rows[0] + 1), x_stride=stride)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        oracle.render(b.cfg, b.ext, rows=rows, x_stride=stride)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = paths * len(times) / total / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / len(times) * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": f"power-8 Mandelbulb path tracing {W}x{H} {SPP}spp {BOUNCES} bounces", "march": "plain"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"rows {rows[0]}-{rows[1]} of {H}, every {stride}th column, all {SPP} samples"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-baseline", type=int, default=1)
    args = ap.parse_args()
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from fractalpathtracer_gb300 import build, native, scenes
    build.build()
    native.lib()
    b = scenes.mandelbulb_path(W, H, SPP, BOUNCES)
    cfg, ext = b.cfg, b.ext
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        native.cuda_render(cfg, ext, linear=False)
    # device-timed steps
    barrier()
    dev_ms = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            _, _, ms = native.cuda_render(cfg, ext, linear=False)
            dev_ms.append(ms)
    barrier()
    # end-to-end steps through the C ABI (config upload + linear and RGBA readback)
    e2e_s = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        native.cuda_render(cfg, ext, linear=True)
        e2e_s.append(time.perf_counter() - t)
    barrier()
    total_ms = sum(dev_ms)
    e2e_total = sum(e2e_s)
    if world > 1:
        t = torch.tensor([total_ms, e2e_total], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms, e2e_total = t.tolist()
    paths = W * H * SPP
    value = paths * args.steps * world / (total_ms / 1e3) / 1e6
    e2e = paths * args.steps * world / e2e_total / 1e6
    # one profiled render for the roofline's algorithmic work count
    _, _, prof_ms, prof = native.cuda_render(cfg, ext, linear=False, profile=True)
    evals = prof.distance_evals + prof.normal_evals
    flop_per_eval = 8 * 53 + 40    # algebraic power-8 step (53 FP32 ops / iteration) + finalize and march bookkeeping
    achieved_tflops = evals * flop_per_eval / (statistics.median(dev_ms) / 1e3) / 1e12
    fp32_peak = 152 * 128 * 2 * 2.070e9 / 1e12
    clk = clocks.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"power-8 Mandelbulb path tracing {W}x{H} {SPP}spp {BOUNCES} bounces, RR after 2",
                   "march": "plain", "l2": "flushed (256 MB write) between steps", "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 30448 + 176,
                "d2h_bytes_per_step": W * H * 16 + W * H * 4},
        "gpu_launches": 2 * args.steps,
        "de_evals_per_s": evals / (statistics.median(dev_ms) / 1e3),
        "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved_tflops / fp32_peak, "traffic": None,
                     "peak_source": "nominal 152 SM x 128 FP32 lanes x 2 x 2070 MHz (no measured FP32 peak)"},
        "clocks": {"sm_mhz": clk["sm_mhz"], "sm_max_mhz": clk["sm_max_mhz"], "reasons": clk["reasons"]},
    }
    if rank == 0 and args.cpu_baseline:
        try:
            import oracle
            cores = os.cpu_count() or 1
            oracle.set_threads(cores)
            stride, rows = 32, (H // 2 - 4, H // 2 + 4)
            t = time.perf_counter()
            oracle.render(cfg, ext, rows=rows, x_stride=stride)
            dt = time.perf_counter() - t
            n = (rows[1] - rows[0]) * ((W + stride - 1) // stride) * SPP
            line["cpu_baseline"] = {"value": n / dt / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
                                    "sample": f"rows {rows[0]}-{rows[1]}, every {stride}th column, {SPP} spp"}
        except Exception as exc:  # the baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                    "sample": f"failed: {exc}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
