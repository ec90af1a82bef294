"""Benchmark of the GB300 hierarchization transform (one JSON line).

python bench.py [--gpus N --steps K --warmup W] [--workload NAME]
                [--impl reference]

Workloads (seeded synthetic inputs; the reference publishes no dataset):
  4d-ct-20  (default) batched 4D combination technique: every level vector
            l >= 1 with |l|_1 = 20 - q, q = 0..3 (969 + 816 + 680 + 560 =
            3025 periodic component grids, 1,695,547,392 points), CDF (2,2)
            lifting ("biorthogonal", the wavelet of the reference's own CT
            driver), f(x) = prod_i 4 x_i (1 - x_i) exp(-a_i x_i), a_i ~ U[0,2].
  6d-ct-16  batched 6D CT, |l|_1 = 16 - q, q = 0..5 (7798 grids), sum of 4
            anisotropic Gaussians plus N(0, 1e-4) noise.
  3d-biorthogonal-999  one 512^3 grid, 8 Gaussians plus N(0, 1e-3) noise.
  6d-hat-555544        one 32^4 x 16^2 grid, product of cosines + noise.

A step is one full forward (hierarchize) plus one full inverse
(dehierarchize) of every grid of the workload, so the data stays bounded
across repetitions; inputs are far larger than the 129 MB L2. ``value`` is
grid points transformed per second (2 x points per step) by the
FP32-compensated path with the data resident in HBM; the plain FP64 path is
timed on the same workload (``fp64``), and the FP32c forward result is
compared with the FP64 one (normwise max / rms error, overall and per q).
``e2e`` repeats the FP32c step through the public API with pinned host
buffers and the host<->device copies inside the timed region, over at least
30 steps (``e2e.steps``; each step's time in ``e2e.step_ms_after_first``).
``roofline``
is the dominant lifting launch: algorithmic bytes (one read and one write of
each grid point it stores) over its CUDA-event duration, from an event-
bracketed pass over the same plan; ``roofline.step_frac`` is the whole
step's algorithmic traffic over the graph-timed step (with the batch's
groups running concurrently). ``--impl reference`` times the
reference's CPU algorithm (the oracle port in oracle/; the reference itself
needs DDC and Kokkos, which are absent) on all host cores.

For N > 1 (torchrun), each rank transforms an independent replica of the
workload ("replicas only"); value sums the ranks' points over the slowest
rank's time.

``--probe-axis LEVELS:DIM:MODE`` instead times one axis of one random grid,
``--probe-outputs LEVELS:DIM:MODE`` the restricted-output transform of one,
``--probe-batch LEVEL_SUM:MODE`` one direction of a smaller 4D batch launch
by launch (all three used for single-kernel captures).
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
METRIC = ("points/s & % HBM roofline: batched FP32-comp vs plain FP64 at "
          "stated error")

WORKLOADS = {
    "4d-ct-20": dict(kind="ct", ndim=4, level_sum=20, qmax=3, lmin=1,
                     wavelet="biorthogonal", config_id=4),
    "6d-ct-16": dict(kind="ct", ndim=6, level_sum=16, qmax=5, lmin=1,
                     wavelet="biorthogonal", config_id=5),
    # The 4D scheme at |l|_1 = 16 - q (1325 grids, 48 M points): the same
    # kernels on a few GB of device memory, for profiler captures.
    "4d-ct-16": dict(kind="ct", ndim=4, level_sum=16, qmax=3, lmin=1,
                     wavelet="biorthogonal", config_id=4),
    "3d-biorthogonal-999": dict(kind="grid", level=(9, 9, 9), lmin=(0, 0, 0),
                                wavelet="biorthogonal", config_id=2),
    "6d-hat-555544": dict(kind="grid", level=(5, 5, 5, 5, 4, 4),
                          lmin=(0,) * 6, wavelet="hat", config_id=3),
}
DEFAULT_WORKLOAD = "4d-ct-20"


# ---------------------------------------------------------------------------
# workload description and seeded inputs


class Workload:
    def __init__(self, name):
        spec = WORKLOADS[name]
        self.name, self.spec = name, spec
        self.wavelet = spec["wavelet"]
        if spec["kind"] == "ct":
            from paliwa_gb300 import ct as pct
            self.levels, self.coeffs = pct.combination_scheme(
                spec["ndim"], spec["level_sum"], spec["qmax"], spec["lmin"])
            d = spec["ndim"]
            self.lmin = (spec["lmin"],) * d
            top = spec["level_sum"] - (d - 1) * spec["lmin"]
            self.lmax = (top,) * d
            self.q = [spec["level_sum"] - sum(l) for l in self.levels]
        else:
            self.levels = [tuple(spec["level"])]
            self.coeffs = [1.0]
            self.lmin = tuple(spec["lmin"])
            self.lmax = tuple(spec["level"])
            self.q = [0]
        self.ndim = len(self.levels[0])
        self.points = sum(1 << sum(l) for l in self.levels)
        rng = __import__("numpy").random.default_rng(
            SEED_BASE + spec["config_id"])
        self._params(rng)

    def _params(self, rng):
        cid = self.spec["config_id"]
        d = self.ndim
        if cid == 4:
            self.a = rng.uniform(0, 2, d)
        elif cid == 5:
            self.gauss = [(rng.uniform(0, 1, d), rng.uniform(0.05, 0.3, d),
                           rng.uniform(-1, 1)) for _ in range(4)]
            self.noise_seed = int(rng.integers(1 << 31))
        elif cid == 2:
            self.gauss = [(rng.uniform(0, 1, 3), rng.uniform(0.02, 0.2),
                           rng.uniform(-1, 1)) for _ in range(8)]
            self.noise_seed = int(rng.integers(1 << 31))
        elif cid == 3:
            self.ks = rng.integers(1, 5, d)
            self.noise_seed = int(rng.integers(1 << 31))

    def grid_values(self, i):
        """float64 values of grid i on the host (numpy), x = k / 2^l."""
        import numpy as np
        lv = self.levels[i]
        xs = [np.arange(1 << l) / float(1 << l) for l in lv]
        shape = [1 << l for l in lv]
        cid = self.spec["config_id"]

        def outer(factors):
            f = factors[0]
            for g in factors[1:]:
                f = np.multiply.outer(f, g)
            return f

        if cid == 4:
            return outer([4 * x * (1 - x) * np.exp(-a * x)
                          for x, a in zip(xs, self.a)])
        if cid == 3:
            return outer([np.cos(k * np.pi * x) for x, k in zip(xs, self.ks)]
                         ) + np.random.default_rng(self.noise_seed).uniform(
                             -1e-3, 1e-3, shape)
        out = np.zeros(shape)
        for c, w, amp in self.gauss:
            w = np.broadcast_to(w, (len(lv),))
            out += amp * outer([np.exp(-(x - ci) ** 2 / (2 * wi * wi))
                                for x, ci, wi in zip(xs, c, w)])
        sigma = 1e-4 if cid == 5 else 1e-3
        seed = self.noise_seed + i
        return out + np.random.default_rng(seed).normal(0, sigma, shape)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.lines = index, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
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


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# multi-rank plumbing (replicas)


def dist_setup():
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
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def step_bytes(w, elem):
    """Algorithmic bytes of one step (forward + inverse): a read and a
    write of every grid point per axis that has levels to transform
    (level > minimum level)."""
    total = 0
    for lv in w.levels:
        n = 1 << sum(lv)
        total += sum(2 * n * elem for d in range(len(lv))
                     if lv[d] > w.lmin[d])
    return 2 * total


def config_of(w, args):
    c = {"workload": w.name, "grids": len(w.levels), "points": w.points,
         "ndim": w.ndim, "minimum_level": list(w.lmin),
         "maximum_level": list(w.lmax), "wavelet": w.wavelet,
         "step": "hierarchize + dehierarchize of every grid",
         "l2": "inputs larger than L2 (no flush needed)"}
    if w.spec["kind"] == "ct":
        c["level_sum"] = w.spec["level_sum"]
        c["q"] = list(range(w.spec["qmax"] + 1))
    else:
        c["level"] = list(w.levels[0])
    return c


# ---------------------------------------------------------------------------
# CPU: the oracle port of the reference algorithm


def cpu_transform_all(w, arrays, oracle):
    t0 = time.perf_counter()
    for x, lv in zip(arrays, w.levels):
        oracle.hierarchize(x, lv, w.lmin, w.lmax, w.wavelet, mode=1)
    for x, lv in zip(arrays, w.levels):
        oracle.dehierarchize(x, lv, w.lmin, w.lmax, w.wavelet, mode=1)
    return time.perf_counter() - t0


def run_reference(args, w, world, rank):
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cores = oracle.max_threads()
    arrays = [w.grid_values(i) for i in range(len(w.levels))]
    for _ in range(args.warmup):
        cpu_transform_all(w, arrays, oracle)
    dt = 0.0
    for _ in range(args.steps):
        dt += cpu_transform_all(w, arrays, oracle)
    value = 2 * w.points * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "points/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "config": config_of(w, args),
        "cpu_baseline": {
            "value": value, "unit": "points/s", "cores": cores,
            "kind": "port",
            "sample": "every grid of the workload, forward + inverse per "
                      "step, FP64, packed-pole mode, OpenMP"},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU


DRAM_RATIO_FILE = "profiles/dram_ratio_4d_ct_19.txt"
# Groups of grids whose host copies overlap each other's transforms in the
# end-to-end measurement.
E2E_GROUPS = 32
E2E_STEPS = 30
E2E_COPY_STREAMS = 1


def dram_ratio(kernel):
    """DRAM bytes per algorithmic byte of `kernel` (a name of
    paliwa_gb300.ct.kernel_name), measured by ncu on single-kernel captures
    of the 4D combination batch at |l|_1 = 19 - q (``--probe-batch 19:f32c``,
    2.8 GB on the device, three launches per kernel) and committed as
    'name = ratio' lines; None when not measured. The ratio of a launch's DRAM bytes to the bytes it must move does not
    depend on the number of grids, so it scales to the full workload."""
    path = os.path.join(ROOT, DRAM_RATIO_FILE)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if "=" in line and not line.startswith("#"):
                name, val = line.rsplit("=", 1)
                if name.strip() == kernel:
                    return float(val)
    return None


def upload_inputs(w, dev):
    """Packed device buffers (float64 and float32) of every grid, and a
    pristine float64 copy for accuracy checks."""
    import numpy as np
    import torch
    from paliwa_gb300 import ct as pct
    b64, v64 = pct.packed_grids(w.levels, torch.float64, dev)
    for i, v in enumerate(v64):
        v.copy_(torch.from_numpy(np.ascontiguousarray(
            w.grid_values(i)).reshape(-1)))
    b32, v32 = pct.packed_grids(w.levels, torch.float32, dev)
    b32.copy_(b64)
    return b64, v64, b32, v32


def time_steps(fwd, inv, steps, warmup, stream, world):
    import torch
    for _ in range(warmup):
        fwd()
        inv()
    barrier(world)
    torch.cuda.synchronize()
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for _ in range(steps):
        fwd()
        inv()
    e.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    return s.elapsed_time(e)


def bind_to_gpu_numa_node(index):
    """Restricts this process to the host cores of the NUMA node of CUDA
    device `index` (from its PCI address in sysfs). Returns the node, or
    None where the topology is not exposed (the affinity is then left as
    it is)."""
    import torch
    try:
        p = torch.cuda.get_device_properties(index)
        bus = "%04x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id,
                                    p.pci_device_id)
        with open(f"/sys/bus/pci/devices/{bus}/numa_node") as f:
            node = int(f.read())
        if node < 0:
            return None
        with open(f"/sys/devices/system/node/node{node}/cpulist") as f:
            spec = f.read().strip()
        cpus = set()
        for part in spec.split(","):
            a, _, b = part.partition("-")
            cpus.update(range(int(a), int(b or a) + 1))
        cpus &= os.sched_getaffinity(0)
        if not cpus:
            return None
        os.sched_setaffinity(0, cpus)
        return node
    except (AttributeError, OSError, ValueError):
        return None


def run_gpu(args, w, world, rank, local):
    import numpy as np
    import torch

    import paliwa_gb300 as pg
    from paliwa_gb300 import ct as pct

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)
    b64, v64, b32, v32 = upload_inputs(w, dev)
    pristine = b64.clone()
    # The uploads ran on the default stream; order the work stream after them.
    torch.cuda.synchronize()

    with torch.cuda.stream(stream):
        bt64 = pct.Batch(v64, w.levels, w.lmin, w.lmax, w.wavelet)
        bt32 = pct.Batch(v32, w.levels, w.lmin, w.lmax, w.wavelet,
                         compensated=True)
        tuning = None
        if not args.no_tune:
            # The library's autotuner picks a kernel per class of stages by
            # timing each direction; it leaves the grids' contents changed
            # by rounding, so the inputs are restored after it.
            t0 = time.time()
            changed32 = bt32.autotune(reps=2, stream=stream)
            changed64 = bt64.autotune(reps=2, stream=stream)
            tuning = {"classes_changed_f32c": changed32,
                      "classes_changed_f64": changed64,
                      "seconds": time.time() - t0}
            b64.copy_(pristine)
            b32.copy_(pristine)
            stream.synchronize()
        # Accuracy of the compensated FP32 forward transform against FP64:
        # against the FP64 transform of the FP64 inputs (the headline), and
        # against the FP64 transform of the same FP32-rounded inputs (the
        # arithmetic and the FP32 storage between axes). The FP64 transform
        # of the rounded inputs against that of the FP64 inputs is the floor
        # that rounding the inputs to FP32 alone sets; plain FP32
        # arithmetic is shown beside it.
        b64q = b32.double()
        b32p = b32.clone()

        def views(buf, like):
            esz = like[0].element_size()
            return [buf.narrow(0, (v.data_ptr() - like[0].data_ptr()) // esz,
                               v.numel()) for v in like]

        v64q = views(b64q, v64)
        v32p = views(b32p, v32)
        bt64q = pct.Batch(v64q, w.levels, w.lmin, w.lmax, w.wavelet)
        bt32p = pct.Batch(v32p, w.levels, w.lmin, w.lmax, w.wavelet)
        for bt in (bt64, bt32, bt64q, bt32p):
            bt.hierarchize(stream)
        stream.synchronize()
        bt64q.close()
        bt32p.close()
        qs = sorted(set(w.q))
        # grids are packed in q-major order: group contiguous ranges
        bounds = {}
        for i, (q, v) in enumerate(zip(w.q, v64)):
            start = (v.data_ptr() - v64[0].data_ptr()) // 8
            bounds.setdefault(q, [start, 0])
            bounds[q][1] = start + v.numel()

        def rel_errors(test, ref, with_q):
            out, per_q = {}, {}
            tot_max = tot_ref = tot_sq = tot_rsq = 0.0
            for q in qs:
                lo, hi = bounds[q]
                r = ref[lo:hi]
                e = test[lo:hi].double() - r
                emax, rmax = float(e.abs().max()), float(r.abs().max())
                esq, rsq = float(e.pow(2).sum()), float(r.pow(2).sum())
                per_q[str(q)] = {"max_rel": emax / rmax,
                                 "rms_rel": math.sqrt(esq / rsq)}
                tot_max, tot_ref = max(tot_max, emax), max(tot_ref, rmax)
                tot_sq, tot_rsq = tot_sq + esq, tot_rsq + rsq
                del e
            out["max_rel"] = tot_max / tot_ref
            out["rms_rel"] = math.sqrt(tot_sq / tot_rsq)
            if with_q and len(qs) > 1:
                out["per_q"] = per_q
            return out

        err = {"norm": "max|e|/max|ref| and rms(e)/rms(ref) over the grids"}
        err.update(rel_errors(b32, b64, True))
        err["same_fp32_inputs"] = rel_errors(b32, b64q, False)
        err["input_rounding_floor"] = rel_errors(b64q, b64, False)
        err["plain_fp32"] = rel_errors(b32p, b64, False)
        del b64q, b32p, v64q, v32p

        # Combine / restrict in FP64 (sparse grid of the kept subspaces).
        combine = None
        if w.spec["kind"] == "ct":
            ct = pct.CombinationTechnique(v32, w.levels, w.coeffs, w.lmax)
            sparse = ct.combine()
            ct.restrict(sparse)
            stream.synchronize()
            s0 = torch.cuda.Event(enable_timing=True)
            s1 = torch.cuda.Event(enable_timing=True)
            s2 = torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            ct.combine(sparse)
            s1.record(stream)
            ct.restrict(sparse)
            s2.record(stream)
            stream.synchronize()
            combine = {"sparse_points": ct.npoints,
                       "subspaces": ct.nsubspaces,
                       "combine_ms": s0.elapsed_time(s1),
                       "restrict_ms": s1.elapsed_time(s2),
                       "dtype": "f64 accumulation of f32 grids"}
            ct.close()
        b64.copy_(pristine)
        b32.copy_(pristine)
        stream.synchronize()
        del pristine

        with ClockSampler(local) as clocks:
            ms32 = time_steps(lambda: bt32.hierarchize(stream),
                              lambda: bt32.dehierarchize(stream),
                              args.steps, args.warmup, stream, world)
        ms64 = time_steps(lambda: bt64.hierarchize(stream),
                          lambda: bt64.dehierarchize(stream),
                          args.steps, args.warmup, stream, world)
        # Per-launch durations of the same plan, event-bracketed.
        prof = {}
        for name, bt in (("f32c", bt32), ("f64", bt64)):
            rows = []
            for fwd in (True, False):
                ms, by, kd = bt.profile(fwd, stream)
                rows += list(zip(ms, by, kd))
                if args.launch_table and rank == 0:
                    # The plan's launches in launch order (the order a
                    # profiler lists them in): kernel, algorithmic bytes.
                    for i, (m, b, k) in enumerate(zip(ms, by, kd)):
                        print(f"launch {name} {'fwd' if fwd else 'inv'} "
                              f"{i:3d} {pct.kernel_name(k):28s} {b:13d} B "
                              f"{m:8.3f} ms", file=sys.stderr)
            prof[name] = rows
        nlaunch = sum(bt32.launches())

    ms32 = max_over_ranks(world, ms32)
    ms64 = max_over_ranks(world, ms64)
    pts_step = 2 * w.points * world
    value = pts_step * args.steps / (ms32 / 1e3)
    value64 = pts_step * args.steps / (ms64 / 1e3)
    peak, peak_kind = peaks()

    def by_kernel(rows, peak):
        """Launches, time share, algorithmic bytes and HBM fraction of each
        kernel over one step."""
        out = {}
        tot = sum(r[0] for r in rows)
        for ms, by, code in rows:
            k = out.setdefault(pct.kernel_name(code), [0, 0.0, 0])
            k[0] += 1
            k[1] += ms
            k[2] += by
        return {name: {"launches": n, "share": ms / tot, "bytes": by,
                       "frac": by / (ms / 1e3) / 1e9 / peak}
                for name, (n, ms, by) in sorted(out.items())}

    def roof(rows):
        """The kernel with the largest share of a step's time: its name,
        launches, summed milliseconds and algorithmic bytes; and totals."""
        per = {}
        for ms, by, code in rows:
            k = per.setdefault(pct.kernel_name(code), [0, 0.0, 0])
            k[0] += 1
            k[1] += ms
            k[2] += by
        name = max(per, key=lambda n: per[n][1])
        tot_ms = sum(r[0] for r in rows)
        tot_b = sum(r[1] for r in rows)
        return (name, *per[name]), tot_ms, tot_b

    top32, tot32_ms, tot32_b = roof(prof["f32c"])
    top64, tot64_ms, tot64_b = roof(prof["f64"])
    top_name, top_n, top_ms, top_b = top32
    achieved = top_b / (top_ms / 1e3) / 1e9
    ratio = dram_ratio(top_name)
    traffic = None if ratio is None else ratio * top_b / top_n

    # End to end through the public API with pinned host buffers: every
    # step copies all grids in, transforms them forward and back, and copies
    # them out (paliwa_gb300.ct.HostBatch: copies of one group of grids
    # overlap the transform of another).
    bt32.close()
    bt64.close()
    del b64, v64
    hb = pct.HostBatch(w.levels, w.lmin, w.lmax, w.wavelet, torch.float32,
                       compensated=True, groups=E2E_GROUPS, device=dev,
                       batch_groups=1, copy_streams=E2E_COPY_STREAMS)
    # Pinned buffers in the host memory next to the GPU's host link: they
    # are allocated (and so placed) while this process runs on the cores of
    # the GPU's NUMA node; the full affinity is restored afterwards.
    saved = os.sched_getaffinity(0) if hasattr(os, "sched_getaffinity") \
        else None
    numa = bind_to_gpu_numa_node(local)
    host_in = torch.empty(hb.numel(), dtype=torch.float32).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    if saved is not None:
        os.sched_setaffinity(0, saved)
    host_in.copy_(b32)
    del b32, v32
    link = measure_link(host_in, host_out, hb.buf)

    # Events after every step, for the per-step times reported beside the
    # total (the total is what `value` uses).
    step_events = []

    def e2e_step():
        hb.run(host_in, host_out, stream=stream)
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(stream)
        step_events.append(ev)

    # At least E2E_STEPS timed steps: on the GB300 machines measured, copies
    # stall for 10-150 ms about every half second (steady steps otherwise),
    # so a mean over a few steps depends on where the stalls fall.
    k_e2e = max(args.steps, E2E_STEPS)
    with torch.cuda.stream(stream):
        e2e_ms = time_steps(e2e_step, lambda: None, k_e2e, args.warmup,
                            stream, world)
    timed_events = step_events[-(k_e2e + 1):]
    e2e_step_ms = [a.elapsed_time(b) for a, b in
                   zip(timed_events[:-1], timed_events[1:])]
    e2e_ms = max_over_ranks(world, e2e_ms)
    e2e_value = pts_step * k_e2e / (e2e_ms / 1e3)
    e2e_bytes = hb.numel() * 4
    # The host link in this run: each direction moves e2e_bytes per step,
    # both at once; the fraction compares that with the concurrent rate.
    e2e_each = e2e_bytes / (e2e_ms / 1e3 / k_e2e) / 1e9
    link["e2e_gbs_each_direction"] = e2e_each
    link["link_frac"] = e2e_each / link["concurrent_gbs_each"]
    hb.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        oracle.build()
        arrays = [w.grid_values(i) for i in range(len(w.levels))]
        dt = cpu_transform_all(w, arrays, oracle)
        cpu = {"value": 2 * w.points / dt, "unit": "points/s",
               "cores": oracle.max_threads(), "kind": "port",
               "sample": "every grid of the workload once, forward + "
                         "inverse, FP64, packed-pole mode, OpenMP"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "points/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms32 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32c",
            "data": "synthetic", "config": config_of(w, args),
            "fp64": {"value": value64, "unit": "points/s",
                     "ms_per_step": ms64 / args.steps,
                     "speedup_f32c_over_f64": value / value64,
                     "hbm_frac_all_launches":
                         tot64_b / (tot64_ms / 1e3) / 1e9 / peak},
            "error_f32c_vs_f64": err,
            "roofline": {
                "bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "traffic_source": None if ratio is None else
                    "DRAM bytes / algorithmic bytes of this kernel from "
                    "single-kernel ncu captures of the 4D batch at |l|_1 = "
                    "19 - q in "
                    + DRAM_RATIO_FILE + ", times this run's bytes per "
                    "launch",
                "peak_kind": peak_kind,
                "kernel": top_name + ", FP32c (largest share of the step)",
                "launches_per_step": top_n,
                "by_kernel": by_kernel(prof["f32c"], peak),
                "bytes_per_launch": top_b / top_n,
                "launch_ms": top_ms / top_n,
                "all_launches_frac":
                    tot32_b / (tot32_ms / 1e3) / 1e9 / peak,
                # The step itself: its algorithmic bytes (one read and one
                # write of every point per transformed axis and direction;
                # axes at the minimum level have no levels and move
                # nothing; the long pencils' halo passes are not counted)
                # over the graph-timed step (the groups' launches overlap
                # there; all_launches_frac times them one by one).
                "step_bytes": step_bytes(w, 4),
                "step_frac": step_bytes(w, 4) /
                    (ms32 / args.steps / 1e3) / 1e9 / peak,
                # The plan's own HBM traffic (a slab launch reads and
                # writes each point once for all of its axes): the sum of
                # the launches' bytes over the graph-timed step.
                "step_plan_bytes": tot32_b,
                "step_plan_frac": tot32_b /
                    (ms32 / args.steps / 1e3) / 1e9 / peak},
            "combine": combine,
            "autotune": tuning,
            "clocks": clocks.summary(),
            "e2e": {"value": e2e_value, "unit": "points/s",
                    "h2d_bytes_per_step": e2e_bytes,
                    "d2h_bytes_per_step": e2e_bytes,
                    "steps": k_e2e,
                    "groups": E2E_GROUPS, "host_numa_node": numa,
                    "link": link,
                    "step_ms_after_first": [round(x, 2) for x in e2e_step_ms]},
            "gpu_launches": args.steps * nlaunch,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    bt32.close()
    bt64.close()


def measure_link(host_in, host_out, dev_buf):
    """GB/s of the host link in this run: the whole pinned input copied to
    the device, the device buffer copied to the pinned output, and both at
    once on two streams (each direction's rate), best of two, CUDA events."""
    import torch
    nbytes = dev_buf.numel() * dev_buf.element_size()
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

    def once(h2d, d2h):
        torch.cuda.synchronize()
        ev[0].record(s_in)
        s_out.wait_event(ev[0])
        if h2d:
            with torch.cuda.stream(s_in):
                dev_buf.copy_(host_in, non_blocking=True)
        ev[1].record(s_in)
        ev[2].record(s_out)
        if d2h:
            with torch.cuda.stream(s_out):
                host_out.copy_(dev_buf, non_blocking=True)
        ev[3].record(s_out)
        torch.cuda.synchronize()
        if h2d and d2h:
            return max(ev[0].elapsed_time(ev[1]), ev[0].elapsed_time(ev[3]))
        return ev[0].elapsed_time(ev[1] if h2d else ev[3])

    out = {}
    for key, h2d, d2h in (("h2d_gbs", True, False), ("d2h_gbs", False, True),
                          ("concurrent_gbs_each", True, True)):
        ms = min(once(h2d, d2h) for _ in range(2))
        out[key] = nbytes / (ms / 1e3) / 1e9
    return out


def run_axis_probe(spec):
    """One axis of one grid, for kernel captures: ``LEVELS:DIM:MODE`` (e.g.
    ``12,7,7:0:f32c``; MODE f64, f32 or f32c) runs hierarchize_in along DIM
    of a random grid twice (CDF biorthogonal, lmin 0) and prints the second
    run's event-timed milliseconds and algorithmic GB/s."""
    import torch

    import paliwa_gb300 as pg
    lv, dim, mode = spec.split(":")
    level = tuple(int(x) for x in lv.split(","))
    dim = int(dim)
    dt = torch.float64 if mode == "f64" else torch.float32
    g = torch.rand([1 << l for l in level], dtype=dt, device="cuda")
    lmin = (0,) * len(level)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for r in range(2):
        if r == 1:
            ev[0].record()
        pg.hierarchize_in(g, dim, level, lmin, level, "biorthogonal",
                          compensated=(mode == "f32c"))
    ev[1].record()
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1])
    gbs = 2 * g.numel() * g.element_size() / ms / 1e6
    print(json.dumps({"probe": spec, "ms": ms, "GB/s": gbs}), flush=True)


def run_batch_probe(spec):
    """One direction of a smaller 4D combination batch, for kernel captures
    of a few GB: ``LEVEL_SUM:MODE[:noslabs][:tma]`` (MODE f64, f32 or f32c;
    e.g. ``19:f32c``, 709 M points, 2.8 GB) builds the 4D scheme at |l|_1 =
    LEVEL_SUM - q (q <= 3, lmin 1, CDF biorthogonal) on random values with
    the planner's default kernels (``tma``: every class of stages that the
    TMA wide kernel applies to set to it), runs the forward direction launch
    by launch (no graph, plan order, one stream) and prints one JSON line per
    launch: index, kernel, algorithmic bytes and event-timed milliseconds.
    The k-th launch of a kernel in that list is the k-th one a profiler
    filtered on the kernel's name sees."""
    import torch

    from paliwa_gb300 import ct as pct
    parts = spec.split(":")
    level_sum, mode = int(parts[0]), parts[1]
    slabs = "noslabs" not in parts[2:]
    tma_all = "tma" in parts[2:]
    levels, _ = pct.combination_scheme(4, level_sum, 3, 1)
    dt = torch.float64 if mode == "f64" else torch.float32
    buf, views = pct.packed_grids(levels, dt)
    buf.uniform_(-1, 1)
    top = level_sum - 3
    bt = pct.Batch(views, levels, (1,) * 4, (top,) * 4, "biorthogonal",
                   compensated=(mode == "f32c"), slabs=slabs)
    if tma_all:
        bt.set_tuning({c: "twide" for c, _, names, _ in bt.tuning(True)
                       if "twide" in names})
    ms, by, kd = bt.profile(forward=True)
    bt.status()
    for i, (m, b, k) in enumerate(zip(ms, by, kd)):
        print(json.dumps({"launch": i, "kernel": pct.kernel_name(k),
                          "bytes": b, "ms": m}), flush=True)
    bt.close()


def run_outputs_probe(spec):
    """The restricted-output transform on one grid, for kernel captures:
    ``LEVELS:DIM:MODE`` (MODE f64 or f32) hierarchizes along DIM (CDF
    biorthogonal, every level) with outputs = the first half of the axis,
    the whole grid as the window, twice, and prints the second run's
    event-timed milliseconds, the points written and the algorithmic GB/s
    of its lifting passes (three reads and one write per written point)."""
    import torch

    import paliwa_gb300 as pg
    lv, dim, mode = spec.split(":")
    level = tuple(int(x) for x in lv.split(","))
    dim = int(dim)
    dt = torch.float64 if mode == "f64" else torch.float32
    g = torch.rand([1 << l for l in level], dtype=dt, device="cuda")
    filters = pg.lifting_wavelet_filter_offsets_and_coefficients[
        "biorthogonal"]
    levels = list(range(level[dim], 0, -1))
    ext = [1 << l for l in level]
    ext[dim] //= 2
    outputs = ((0,) * len(level), ext, (1,) * len(level))
    bounds, writes = pg.transform_bounds(
        (0, (1 << level[dim]) // 2 - 1), level[dim], level[dim], levels,
        filters)
    per_col = 0
    for i, l in enumerate(levels):
        stride = 2 << (level[dim] - l)
        period = 1 << level[dim]
        for w in writes[i]:
            if w is not None:
                span = (w[1] - w[0]) % period
                per_col += span // stride + 1
    cols = g.numel() >> level[dim]
    written = per_col * cols
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for r in range(2):
        if r == 1:
            ev[0].record()
        pg.transform_outputs(g, dim, level, level, levels, filters, outputs)
    ev[1].record()
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1])
    gbs = 4 * written * g.element_size() / ms / 1e6
    print(json.dumps({"probe_outputs": spec, "ms": ms,
                      "points_written": written, "GB/s": gbs}), flush=True)


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
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuner (the planner's default "
                         "kernels)")
    ap.add_argument("--launch-table", action="store_true",
                    help="print the plan's launches (kernel, algorithmic "
                         "bytes, event-timed ms) to stderr")
    ap.add_argument("--probe-axis", metavar="LEVELS:DIM:MODE",
                    help="time one axis of one grid instead (for kernel "
                         "captures), e.g. 12,7,7:0:f32c")
    ap.add_argument("--probe-outputs", metavar="LEVELS:DIM:MODE",
                    help="time the restricted-output transform of one grid "
                         "(outputs: half the axis), e.g. 10,8,8:0:f64")
    ap.add_argument("--probe-batch", metavar="LEVEL_SUM:MODE[:noslabs][:tma]",
                    help="profile one direction of the 4D combination batch "
                         "at a smaller level sum launch by launch (for "
                         "kernel captures), e.g. 19:f32c")
    args = ap.parse_args()
    if args.probe_batch:
        run_batch_probe(args.probe_batch)
        return
    if args.probe_axis:
        run_axis_probe(args.probe_axis)
        return
    if args.probe_outputs:
        run_outputs_probe(args.probe_outputs)
        return
    args.warmup = max(3, args.warmup)
    world, rank, local = dist_setup()
    w = Workload(args.workload)
    if args.impl == "reference":
        run_reference(args, w, world, rank)
    else:
        run_gpu(args, w, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
