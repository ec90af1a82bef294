"""Benchmark of the GB300 hierarchization transform (one JSON line).

python bench.py [--gpus N --steps K --warmup W] [--workload NAME]
                [--impl reference]

A step is one full forward (hierarchize) plus one full inverse
(dehierarchize) of the workload's grid(s), so the data stays bounded across
repetitions. ``value`` is grid points transformed per second by the
FP32-compensated path (2 * points per step), with the inputs resident in HBM;
the same workload in plain FP64 is timed beside it (``fp64``), and the FP32c
error against FP64 is reported. ``e2e`` repeats the FP32c step through the
public API with pinned host buffers, host<->device copies inside the timed
region. ``roofline`` is the per-axis lifting kernel: algorithmic bytes per
launch (one read and one write of the grid) over its CUDA-event duration.

``--impl reference`` times the reference's CPU algorithm (the oracle port in
oracle/; the reference itself needs DDC and Kokkos, which are absent) on all
host cores, for the same metric and workload.

For N > 1 (torchrun), each rank runs an independent replica of the workload
("replicas only": a single grid's transform does not shard without a ghost
exchange); value sums the ranks' points over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED_BASE = 20261203

WORKLOADS = {
    # 3D CDF (2,2) lifting at levels (9,9,9): 512^3 periodic points, sum of
    # 8 Gaussians (centres U[0,1]^3, widths U[0.02,0.2], amplitudes U[-1,1])
    # plus N(0, 1e-3) noise.
    "3d-biorthogonal-999": dict(level=(9, 9, 9), lmin=(0, 0, 0),
                                wavelet="biorthogonal", config_id=2),
    # 6D hat at levels (5,5,5,5,4,4): 32^4 * 16^2 points, product of
    # cos(k_i pi x_i), k_i in {1..4}, plus U[-1e-3, 1e-3].
    "6d-hat-555544": dict(level=(5, 5, 5, 5, 4, 4), lmin=(0,) * 6,
                          wavelet="hat", config_id=3),
}
DEFAULT_WORKLOAD = "3d-biorthogonal-999"


def make_input(spec, rng):
    """Seeded synthetic input in float64 (numpy, on the host)."""
    import numpy as np
    level = spec["level"]
    axes = [np.arange(1 << l) / float(1 << l) for l in level]
    cid = spec["config_id"]
    if cid == 2:
        out = np.zeros([1 << l for l in level])
        grids = np.meshgrid(*axes, indexing="ij", sparse=True)
        for _ in range(8):
            c = rng.uniform(0, 1, 3)
            w = rng.uniform(0.02, 0.2)
            a = rng.uniform(-1, 1)
            out += a * np.exp(-sum((g - ci) ** 2 for g, ci in zip(grids, c))
                              / (2 * w * w))
        out += rng.normal(0, 1e-3, out.shape)
        return out
    if cid == 3:
        ks = rng.integers(1, 5, len(level))
        f = None
        for d, (x, k) in enumerate(zip(axes, ks)):
            shape = [1] * len(level)
            shape[d] = len(x)
            v = np.cos(k * np.pi * x).reshape(shape)
            f = v if f is None else f * v
        return f + rng.uniform(-1e-3, 1e-3, [1 << l for l in level])
    raise ValueError(cid)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": mx, "samples": len(sm),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() and \
        dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, spec, world, rank):
    """CPU reference arm: the oracle port of paliwa's algorithm (packed-pole
    execution, the reference's fastest CPU mode) on all host cores."""
    if rank != 0:
        return
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cores = oracle.max_threads()
    rng = np.random.default_rng(SEED_BASE + spec["config_id"])
    x = make_input(spec, rng)
    level, lmin = spec["level"], spec["lmin"]
    npts = x.size

    def step():
        oracle.hierarchize(x, level, lmin, level, spec["wavelet"], mode=1)
        oracle.dehierarchize(x, level, lmin, level, spec["wavelet"], mode=1)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    value = 2 * npts * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "points/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": config_of(args, spec),
        "cpu_baseline": {"value": value, "unit": "points/s", "cores": cores,
                         "kind": "port",
                         "sample": f"full workload grid ({npts} points), "
                                   "forward + inverse per step, FP64, "
                                   "packed-pole mode, OpenMP"},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


METRIC = "points/s & % HBM roofline: batched FP32-comp vs plain FP64 at stated error"


def config_of(args, spec):
    return {"workload": args.workload, "level": list(spec["level"]),
            "lmin": list(spec["lmin"]), "wavelet": spec["wavelet"],
            "points": 1 << sum(spec["level"]),
            "step": "hierarchize + dehierarchize, all dimensions",
            "l2": "inputs larger than L2 (no flush needed)"}


def run_gpu(args, spec, world, rank, local):
    import numpy as np
    import torch

    import paliwa_gb300 as pg
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    level, lmin, wavelet = spec["level"], spec["lmin"], spec["wavelet"]
    ndim = len(level)
    rng = np.random.default_rng(SEED_BASE + spec["config_id"])
    x64 = make_input(spec, rng)
    npts = x64.size
    stream = torch.cuda.current_stream(dev)

    g64 = torch.from_numpy(x64).to(dev)
    g32 = torch.from_numpy(x64.astype(np.float32)).to(dev)

    # Accuracy of the compensated FP32 forward transform against FP64 (the
    # GPU FP64 path is bit-identical to the CPU oracle; see tests).
    pg.hierarchize(g64, level, lmin, level, wavelet)
    pg.hierarchize(g32, level, lmin, level, wavelet, compensated=True)
    diff = g32.double() - g64
    ref_max = float(g64.abs().max())
    err_max = float(diff.abs().max()) / ref_max
    err_rms = float(diff.pow(2).mean().sqrt() / g64.pow(2).mean().sqrt())
    del diff
    g64.copy_(torch.from_numpy(x64))
    g32.copy_(torch.from_numpy(x64.astype(np.float32)))

    def one_step(g, comp, evs=None):
        # per-axis calls so that each lift launch is bracketed by events
        for d in range(ndim):
            if evs is not None:
                evs.append(torch.cuda.Event(enable_timing=True))
                evs[-1].record(stream)
            pg.hierarchize_in(g, d, level, lmin, level, wavelet,
                              compensated=comp)
        for d in range(ndim):
            if evs is not None:
                evs.append(torch.cuda.Event(enable_timing=True))
                evs[-1].record(stream)
            pg.dehierarchize_in(g, d, level, lmin, level, wavelet,
                                compensated=comp)
        if evs is not None:
            evs.append(torch.cuda.Event(enable_timing=True))
            evs[-1].record(stream)

    def timed(g, comp):
        for _ in range(args.warmup):
            one_step(g, comp)
        barrier(world)
        torch.cuda.synchronize()
        evs = []
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(args.steps):
            one_step(g, comp, evs)
        end.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        total_ms = start.elapsed_time(end)
        launches = [evs[i].elapsed_time(evs[i + 1])
                    for i in range(len(evs) - 1) if (i + 1) % (2 * ndim + 1)]
        return total_ms, launches

    with ClockSampler(local) as clocks:
        ms32, launch32 = timed(g32, True)
    ms64, launch64 = timed(g64, False)

    ms32 = max_over_ranks(world, ms32)
    ms64 = max_over_ranks(world, ms64)
    pts_per_step = 2 * npts * world
    value = pts_per_step * args.steps / (ms32 / 1e3)
    value64 = pts_per_step * args.steps / (ms64 / 1e3)

    peak, peak_kind = peaks()
    bytes_launch32 = 2 * npts * 4
    avg32 = sum(launch32) / len(launch32)
    achieved = bytes_launch32 / (avg32 / 1e3) / 1e9
    bytes_launch64 = 2 * npts * 8
    avg64 = sum(launch64) / len(launch64)
    achieved64 = bytes_launch64 / (avg64 / 1e3) / 1e9

    # End to end through the public API: pinned host input, H2D, forward +
    # inverse, D2H of the result, every step.
    host_in = torch.from_numpy(x64.astype(np.float32)).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    ge = torch.empty(host_in.shape, dtype=torch.float32, device=dev)

    def e2e_step():
        ge.copy_(host_in, non_blocking=True)
        pg.hierarchize(ge, level, lmin, level, wavelet, compensated=True)
        pg.dehierarchize(ge, level, lmin, level, wavelet, compensated=True)
        host_out.copy_(ge, non_blocking=True)

    for _ in range(args.warmup):
        e2e_step()
    barrier(world)
    torch.cuda.synchronize()
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    e2e_ms = max_over_ranks(world, s.elapsed_time(e))
    e2e_value = pts_per_step * args.steps / (e2e_ms / 1e3)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(spec, x64)

    ksum = kernel_counts()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "points/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms32 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32c",
            "data": "synthetic", "config": config_of(args, spec),
            "fp64": {"value": value64, "unit": "points/s",
                     "ms_per_step": ms64 / args.steps,
                     "speedup_f32c_over_f64": value / value64,
                     "roofline_frac": achieved64 / peak},
            "error_f32c_vs_f64": {"max_rel": err_max, "rms_rel": err_rms,
                                  "norm": "max|e|/max|ref|, rms(e)/rms(ref)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "peak_kind": peak_kind,
                         "kernel": "lift_kernel (one axis, FP32c)",
                         "bytes_per_launch": bytes_launch32,
                         "avg_launch_ms": avg32},
            "clocks": clocks.summary(),
            "e2e": {"value": e2e_value, "unit": "points/s",
                    "h2d_bytes_per_step": npts * 4,
                    "d2h_bytes_per_step": npts * 4},
            "gpu_launches": args.steps * 2 * ndim * ksum,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)


def kernel_counts():
    """Lift launches per axis pass of the workloads here (all pencils fit one
    CTA: one launch per axis)."""
    return 1


def cpu_baseline(spec, x64):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle
    oracle.build()
    cores = oracle.max_threads()
    level, lmin = spec["level"], spec["lmin"]
    y = x64.copy()
    t0 = time.perf_counter()
    oracle.hierarchize(y, level, lmin, level, spec["wavelet"], mode=1)
    oracle.dehierarchize(y, level, lmin, level, spec["wavelet"], mode=1)
    dt = time.perf_counter() - t0
    return {"value": 2 * y.size / dt, "unit": "points/s", "cores": cores,
            "kind": "port",
            "sample": f"one forward + inverse of the full grid ({y.size} "
                      "points), FP64, packed-pole mode, OpenMP"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true",
                    help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    spec = WORKLOADS[args.workload]
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, spec, world, rank)
    else:
        run_gpu(args, spec, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
