#!/usr/bin/env python3
"""Benchmark: FastNoise2 node-tree evaluation on GB300.

Default workload (the reference's configs[1]): FractalFBm over Perlin, 5 octaves,
gain 0.5, lacunarity 2, GenUniformGrid3D 256^3 from (-128,-128,-128), step 1,
seed 42.  A step is one pass over the 16,777,216-point grid.

  value  -- Mpoints/s of the device-resident path (fnGenUniformGrid3DDevice into
            HBM), CUDA-event timed per step on the launching stream, L2 flushed
            between steps (256 MiB write outside the timed events).
  e2e    -- the same metric through the reference-facing C-ABI call
            fnGenUniformGrid3D with a pinned host output buffer: launch, kernel,
            device->host copy of the 64 MiB result and the min/max read are all
            inside the timed region.

--impl reference times the CPU restatement of the reference's algorithm
(oracle/, "port"; the reference itself cannot be built here because its
FastSIMD dependency is not vendored) with every host thread on the same
workload, each step a bounded z-slab sample.

Multi-GPU: points are independent, so --gpus N runs N replicas (one process per
GPU under torchrun, no collective on the data path); value = all points / max
rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOADS = {
    # name: (tree factory name, kind, args, seed)
    "fbm-perlin-256": ("fbm_perlin_c1", "grid", ((-128.0, -128.0, -128.0), (256, 256, 256), (1.0, 1.0, 1.0)), 42),
    "simplex-64": ("simplex_c0", "grid", ((0.0, 0.0, 0.0), (64, 64, 64), (1.0, 1.0, 1.0)), 1337),
    "terrain-tileable-1024": ("terrain_c2", "tile", ((1024, 1024), (1.0, 1.0)), 7),
    "terrain-128": ("terrain_c2", "grid", ((0.0, 0.0, 0.0), (128, 128, 128), (1.0, 1.0, 1.0)), 7),
}
L2_FLUSH_BYTES = 256 << 20


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


def npoints(kind, args):
    if kind == "grid":
        return int(np.prod(args[1]))
    return int(args[0][0] * args[0][1])


def tree_for(name):
    from tests import trees
    return getattr(trees, WORKLOADS[name][0])()


def lane_ops_per_point(name):
    """FS-level operations per point, counted by the oracle's op counter."""
    from oracle.oracle import count_ops
    tname, kind, args, seed = WORKLOADS[name]
    dim = 4 if kind == "tile" else len(args[1])
    rng = np.random.default_rng(1)
    pts = rng.uniform(-200, 200, (32, dim))
    return count_ops(tree_for(name), pts, seed)


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks", suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [p.strip() for p in line.split(",")]
                    if len(parts) >= 9:
                        rows.append(parts)
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def read_traffic(name):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(name + " "):
            try:
                return float(line.split()[1])
            except (IndexError, ValueError):
                return None
    return None


def cpu_baseline(name, seconds=8.0, max_points=None):
    """Time the CPU restatement (all host threads) on a bounded sample of the workload."""
    from oracle.oracle import OracleTree
    tname, kind, args, seed = WORKLOADS[name]
    t = OracleTree(tree_for(name))
    threads = os.cpu_count()
    done = 0
    t0 = time.perf_counter()
    slab = 0
    if kind == "grid":
        off, cnt, st = args
        plane = int(np.prod(cnt[:-1]))
        zs = max(1, min(cnt[-1], 8))
        while time.perf_counter() - t0 < seconds:
            z0 = (slab * zs) % cnt[-1]
            z = min(zs, cnt[-1] - z0)
            o = list(off)
            o[-1] = float(np.float32(off[-1]) + np.float32(z0) * np.float32(st[-1]))
            t.grid(o, list(cnt[:-1]) + [z], st, seed, threads=threads)
            done += plane * z
            slab += 1
            if max_points and done >= max_points:
                break
        sample = f"{slab} z-slabs of {zs} planes ({done} points) of the {'x'.join(map(str, cnt))} grid"
    else:
        (xs, ys), (sx, sy) = args
        while time.perf_counter() - t0 < seconds:
            t.tileable(xs, ys, sx, sy, seed, threads=threads)
            done += xs * ys
            slab += 1
            if max_points and done >= max_points:
                break
        sample = f"{slab} full {xs}x{ys} tileable passes ({done} points)"
    dt = time.perf_counter() - t0
    return {"value": done / dt / 1e6, "unit": "Mpoints/s", "cores": threads, "kind": "port", "sample": sample}


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(a):
    rank, world, _ = dist_setup(a.gpus)
    if rank != 0:
        return
    name = a.workload
    kind, args = WORKLOADS[name][1], WORKLOADS[name][2]
    per_step = []
    for _ in range(a.warmup):
        cpu_baseline(name, seconds=0.5)
    for _ in range(a.steps):
        per_step.append(cpu_baseline(name, seconds=a.cpu_seconds / max(a.steps, 1)))
    v = statistics.median(s["value"] for s in per_step)
    line = {
        "impl": "reference", "metric": "Mpoints/s", "value": v, "unit": "Mpoints/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": npoints(kind, args) / (v * 1e6) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": name, "points_per_step": npoints(kind, args)},
        "cpu_baseline": {"value": v, "unit": "Mpoints/s", "cores": per_step[0]["cores"], "kind": "port",
                         "sample": per_step[0]["sample"] + " per step; CPU restatement of FastNoise2 (oracle/), "
                                   "the reference binary needs the unvendored FastSIMD"},
        "e2e": {"value": v, "unit": "Mpoints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_gpu(a):
    import torch
    rank, world, local = dist_setup(a.gpus)
    torch.cuda.set_device(local)
    import fastnoise2_gb300 as fn
    from tests.trees import to_product

    name = a.workload
    tname, kind, args, seed = WORKLOADS[name]
    pts = npoints(kind, args)
    root = tree_for(name)
    node = to_product(root)
    node.prepare(4 if kind == "tile" else len(args[1]))
    dev = torch.device("cuda", local)
    out = torch.empty(pts, dtype=torch.float32, device=dev)
    mm = torch.empty(2, dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def step():
        if kind == "grid":
            node.gen_uniform_grid_device(out.data_ptr(), *args, seed + rank, mm.data_ptr(), sptr)
        else:
            node.gen_tileable_2d_device(out.data_ptr(), args[0], args[1], seed + rank, mm.data_ptr(), sptr)

    for _ in range(max(a.warmup, 3)):
        step()
    torch.cuda.synchronize(dev)

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    sampler = ClockSampler(local)
    with sampler:
        barrier(world)
        torch.cuda.synchronize(dev)
        w0 = time.perf_counter()
        for i in range(a.steps):
            flush.zero_()                       # evict L2 between steps (outside the timed events)
            starts[i].record(stream)
            step()
            ends[i].record(stream)
        torch.cuda.synchronize(dev)
        barrier(world)
        wall = time.perf_counter() - w0
    clocks = sampler.summary()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = statistics.mean(step_ms)
    ms_max = allmax(ms, world)
    value = pts * world / (ms_max * 1e-3) / 1e6

    # end to end through the reference-facing C-ABI with pinned host memory
    e2e_med, e2e_value = None, None
    if a.e2e_steps > 0:
        host = torch.empty(pts, dtype=torch.float32, pin_memory=True).numpy()
        e2e_ms = []
        for i in range(max(a.warmup, 3) + a.e2e_steps):
            t0 = time.perf_counter()
            if kind == "grid":
                node.gen_uniform_grid(*args, seed + rank, out=host)
            else:
                node.gen_tileable_2d(args[0], args[1], seed + rank, out=host)
            if i >= max(a.warmup, 3):
                e2e_ms.append((time.perf_counter() - t0) * 1e3)
        e2e_med = allmax(statistics.median(e2e_ms), world)
        e2e_value = pts * world / (e2e_med * 1e-3) / 1e6

    if rank != 0:
        return
    peaks, peak_src = load_peaks()
    ops = lane_ops_per_point(name)
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    peak_lane = n_sm * 128 * sm_max * 1e6 / 1e12          # Tlane-op/s: FP32 lanes x max clock
    achieved = pts * ops / (ms * 1e-3) / 1e12
    hbm_bytes = pts * 4
    hbm_gbs = hbm_bytes / (ms * 1e-3) / 1e9
    traffic = read_traffic(name)
    cpu = cpu_baseline(name, seconds=a.cpu_seconds) if a.cpu_seconds > 0 else None
    line = {
        "metric": "Mpoints/s", "value": value, "unit": "Mpoints/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": name, "points_per_step": pts, "tree": tname, "seed": seed,
                   "l2": "flushed between steps (256 MiB write outside the timed events)",
                   "path": "interpreter kernel, device-resident output"},
        "wall_ms_per_step_incl_flush": wall * 1e3 / a.steps,
        "roofline": {"bound": "fp32-issue", "achieved": achieved, "peak": peak_lane, "unit": "Tlane-op/s",
                     "frac": achieved / peak_lane, "traffic": traffic,
                     "work_per_point": ops, "work_source": "FS-level ops per point counted by oracle/opcount.h",
                     "peak_source": f"{n_sm} SMs x 128 FP32 lanes x {sm_max:.0f} MHz ({peak_src} sm_max_mhz)",
                     "hbm": {"achieved_gbs": hbm_gbs, "peak_gbs": float(peaks.get("hbm_gbs", 6800.0)),
                             "frac": hbm_gbs / float(peaks.get("hbm_gbs", 6800.0)), "algorithmic_bytes_per_point": 4}},
        "e2e": {"value": e2e_value, "unit": "Mpoints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": pts * 4 + 8,
                "ms_per_step": e2e_med, "api": "fnGenUniformGrid3D / fnGenTileable2D into pinned host memory"},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": a.steps,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="fbm-perlin-256", choices=sorted(WORKLOADS))
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    a = ap.parse_args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_gpu(a)


if __name__ == "__main__":
    main()
