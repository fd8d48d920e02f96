#!/usr/bin/env python3
"""Benchmark: FastNoise2 node-tree evaluation on GB300.

Default workload "chunk-mix" (the metric's served-vs-per-call case): 4096
generation requests, sizes uniform over {16^3, 32^3, 64^3} 3D and {32^2,
128^2, 512^2} 2D grids, each with one of eight trees, random seeds and chunk
origins (tests/chunkmix.py; 395M points per step).  A step is one pass over
all 4096 requests.

  value      Mpoints/s of the batched path: all requests in one persistent
             launch (fnGenBatchDevice, captured CUDA graph, autotuned tiles),
             outputs resident in HBM, CUDA events on the launching stream.
  per_call   the same requests as 4096 plain launches (fnGenEachDevice).
  served     the request server (fnServer*): closed loop (all requests
             submitted at once) and open loop (Poisson arrivals), with
             p50/p99 submit-to-completion latency.
  e2e        the batched path through the public API with the device->host
             copy of every output into pinned host memory inside the timed region.

Other workloads (--workload): fbm-perlin-256 (FractalFBm(Perlin) 256^3, the
reference's configs[1]), simplex-64, terrain-tileable-1024, terrain-128.

--impl reference times the CPU restatement of the reference's algorithm
(oracle/, "port": the reference binary cannot be built here because its
FastSIMD dependency is not vendored): every step is one whole pass over the
same workload on a persistent pool of all host threads (whole requests per
thread for the chunk mix), plus a one-thread figure on a bounded sample.

Multi-GPU: requests are independent, so --gpus N runs N replicas (one process
per GPU, no collective on the data path); value = all points / max rank time.
"""
from __future__ import annotations

import argparse
import ctypes
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

GRID_WORKLOADS = {
    "fbm-perlin-256": ("fbm_perlin_c1", "grid", ((-128.0, -128.0, -128.0), (256, 256, 256), (1.0, 1.0, 1.0)), 42),
    "simplex-64": ("simplex_c0", "grid", ((0.0, 0.0, 0.0), (64, 64, 64), (1.0, 1.0, 1.0)), 1337),
    "terrain-tileable-1024": ("terrain_c2", "tile", ((1024, 1024), (1.0, 1.0)), 7),
    "terrain-128": ("terrain_c2", "grid", ((0.0, 0.0, 0.0), (128, 128, 128), (1.0, 1.0, 1.0)), 7),
}
WORKLOADS = ["chunk-mix", *GRID_WORKLOADS, "mesh-bloxel-128", "mesh-dmc-128"]
L2_FLUSH_BYTES = 256 << 20


# ---------------------------------------------------------------- helpers

def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


def tree_named(name):
    from tests import trees
    return getattr(trees, name)()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

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
        # nvidia-smi's start-up can take seconds on a fresh host and stalls GPU work while it
        # runs: wait for its first sample so that the start-up stays outside the timed region
        t0 = time.time()
        while self.proc and self.proc.poll() is None and time.time() - t0 < 30.0:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.05)
        time.sleep(0.2)
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
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
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


def parse_cpulist(text):
    cpus = set()
    for part in text.strip().split(","):
        if not part:
            continue
        if "-" in part:
            a, b = part.split("-")
            cpus.update(range(int(a), int(b) + 1))
        else:
            cpus.add(int(part))
    return cpus


def bind_near_gpu(local):
    """Keep this process (and the pinned host buffers it allocates later) on the CPUs the PCI
    topology lists next to GPU `local`, as numactl would: host<->device copies from a remote
    socket's memory run at a fraction of the local rate.  Returns what was found and done."""
    info = {"bound": False}
    try:
        rt = ctypes.CDLL("libcudart.so")
        buf = ctypes.create_string_buffer(64)
        if rt.cudaDeviceGetPCIBusId(buf, 64, int(local)) != 0:
            return info
        bus = buf.value.decode().lower()
        info["pci_bus_id"] = bus
        dev_dir = None
        for name in os.listdir("/sys/bus/pci/devices"):
            if name.lower().endswith(bus.split(":", 1)[1]) and int(name.split(":")[0], 16) == int(bus.split(":")[0], 16):
                dev_dir = os.path.join("/sys/bus/pci/devices", name)
                break
        if dev_dir is None:
            return info
        with open(os.path.join(dev_dir, "numa_node")) as f:
            info["gpu_numa_node"] = int(f.read().strip())
        with open(os.path.join(dev_dir, "local_cpulist")) as f:
            near = parse_cpulist(f.read())
        allowed = os.sched_getaffinity(0)
        both = near & allowed
        info["near_cpus_allowed"] = len(both)
        info["cpus_allowed"] = len(allowed)
        if both and both != allowed:
            os.sched_setaffinity(0, both)
            info["bound"] = True
    except (OSError, ValueError, AttributeError):
        pass
    return info


def dist_setup():
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


def ops_per_point(tree, dim, seed):
    """FS-level operations per point (oracle op counter, oracle/opcount.h)."""
    from oracle.oracle import count_ops
    rng = np.random.default_rng(1)
    return count_ops(tree, rng.uniform(-200, 200, (24, dim)), seed)


# ---------------------------------------------------------------- CPU side

class CpuWorkload:
    """One step of a workload on the CPU restatement (oracle/): the whole chunk mix as one
    batch on the oracle's persistent worker pool (whole requests per thread, largest first),
    or the whole grid / tileable image cut into contiguous slabs, one per thread."""

    def __init__(self, workload, rank=0):
        from oracle import oracle
        from tests import chunkmix, trees
        self.workload = workload
        self.oracle = oracle
        if workload == "chunk-mix":
            chunks = chunkmix.make_mix(4096)
            otrees = [oracle.OracleTree(m()) for m in trees.MIX_TREES]
            self.points = sum(c.points for c in chunks)
            self.out = np.empty(self.points, np.float32)
            self.mm = np.zeros((len(chunks), 2), np.float32)
            self.reqs, off = [], 0
            for k, c in enumerate(chunks):
                kind = oracle.KIND_GRID3D if len(c.count) == 3 else oracle.KIND_GRID2D
                self.reqs.append(oracle.request(otrees[c.tree], kind, self.out[off:off + c.points], self.mm[k],
                                                c.seed + rank, c.count, c.offset, (1.0,) * len(c.count)))
                off += c.points
            self.trees = otrees
            self.chunk_points = [c.points for c in chunks]
        else:
            tname, kind, args, seed = GRID_WORKLOADS[workload]
            self.tree = oracle.OracleTree(tree_named(tname))
            self.kind, self.args, self.seed = kind, args, seed + rank
            self.points = int(np.prod(args[1])) if kind == "grid" else int(args[0][0] * args[0][1])

    def step(self, threads):
        """One whole pass; returns seconds."""
        t0 = time.perf_counter()
        if self.workload == "chunk-mix":
            self.oracle.gen_requests(self.reqs, threads=threads)
        elif self.kind == "grid":
            self.tree.grid(*self.args, self.seed, threads=threads)
        else:
            (xs, ys), (sx, sy) = self.args
            self.tree.tileable(xs, ys, sx, sy, self.seed, threads=threads)
        return time.perf_counter() - t0

    def single_thread(self, seconds):
        """Mpoints/s of one thread on a bounded leading part of the workload: the first requests
        of the mix, or the first z-slabs / rows of the grid, about `seconds` of work."""
        t0 = time.perf_counter()
        done = 0
        if self.workload == "chunk-mix":
            n = 0
            while time.perf_counter() - t0 < seconds and n < len(self.reqs):
                self.oracle.gen_requests(self.reqs[n:n + 16], threads=1)
                done += sum(self.chunk_points[n:n + 16])
                n += 16
            what = f"first {min(n, len(self.reqs))} requests"
        elif self.kind == "grid":
            off, cnt, st = self.args
            plane = int(np.prod(cnt[:-1]))
            z0 = 0
            while time.perf_counter() - t0 < seconds and z0 < cnt[-1]:
                o = list(off)
                o[-1] = float(np.float32(off[-1]) + np.float32(z0) * np.float32(st[-1]))
                self.tree.grid(o, list(cnt[:-1]) + [1], st, self.seed, threads=1)
                done += plane
                z0 += 1
            what = f"first {z0} z-planes"
        else:
            (xs, ys), (sx, sy) = self.args
            reps = 0
            while time.perf_counter() - t0 < seconds:
                self.tree.tileable(xs, ys, sx, sy, self.seed, threads=1)
                done += xs * ys
                reps += 1
            what = f"{reps} whole images"
        return done / (time.perf_counter() - t0) / 1e6, f"{what} ({done} points)"


def cpu_baseline(workload, passes, single_seconds, rank=0):
    """The CPU restatement on the host cores: `passes` whole passes over the workload with every
    host thread (the median pass is reported), and one thread on a bounded sample."""
    from oracle import oracle
    w = CpuWorkload(workload, rank)
    threads = os.cpu_count()
    w.step(threads)                                      # warm: page in outputs, start the pool
    times = [w.step(threads) for _ in range(max(passes, 1))]
    t = statistics.median(times)
    one, one_sample = w.single_thread(single_seconds)
    return {"value": w.points / t / 1e6, "unit": "Mpoints/s", "cores": threads, "kind": "port",
            "sample": (f"{len(times)} whole passes over the workload ({w.points} points each, median {t * 1e3:.0f} ms); "
                       "CPU restatement of FastNoise2 (oracle/) on a persistent pool of all host threads, "
                       + ("whole requests per thread, largest first" if workload == "chunk-mix" else "one contiguous slab per thread")
                       + "; the reference binary needs the unvendored FastSIMD"),
            "single_thread": {"value": one, "unit": "Mpoints/s", "sample": one_sample},
            "host": oracle.cpu_description()}


def points_per_step(workload):
    if workload == "chunk-mix":
        from tests import chunkmix
        return sum(c.points for c in chunkmix.make_mix(4096))
    tname, kind, args, seed = GRID_WORKLOADS[workload]
    return int(np.prod(args[1])) if kind == "grid" else int(args[0][0] * args[0][1])


def run_reference(a):
    """The CPU restatement of the reference's path, every step one whole pass over the same
    workload (no sampling), on all host threads; rank 0 only."""
    rank, world, _ = dist_setup()
    if rank != 0:
        return
    from oracle import oracle
    w = CpuWorkload(a.workload)
    threads = os.cpu_count()
    for _ in range(a.warmup):
        w.step(threads)
    times = [w.step(threads) for _ in range(a.steps)]
    t = statistics.mean(times)
    v = w.points / t / 1e6
    one, one_sample = w.single_thread(3.0)
    line = {
        "impl": "reference", "metric": "Mpoints/s", "value": v, "unit": "Mpoints/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": a.workload, "points_per_step": w.points,
                   **({"requests": len(w.reqs), "rng": "numpy PCG64(20261203)"} if a.workload == "chunk-mix" else {})},
        "cpu_baseline": {"value": v, "unit": "Mpoints/s", "cores": threads, "kind": "port",
                         "sample": "every step one whole pass over the workload; CPU restatement of FastNoise2 "
                                   "(oracle/) on a persistent pool of all host threads, "
                                   + ("whole requests per thread, largest first" if a.workload == "chunk-mix"
                                      else "one contiguous slab per thread")
                                   + "; the reference binary needs the unvendored FastSIMD",
                         "single_thread": {"value": one, "unit": "Mpoints/s", "sample": one_sample},
                         "host": oracle.cpu_description(),
                         "ms_per_step_min": min(times) * 1e3, "ms_per_step_max": max(times) * 1e3},
        "e2e": {"value": v, "unit": "Mpoints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------- GPU: chunk mix

def run_chunkmix(a, rank, world, local):
    import torch
    import fastnoise2_gb300 as fn
    fn.set_auto_specialise(0)              # the kernel tier is chosen explicitly (--kernels)
    from tests import chunkmix, trees

    dev = torch.device("cuda", local)
    chunks = chunkmix.make_mix(4096)[:a.requests]
    nodes = [trees.to_product(m()) for m in trees.MIX_TREES]
    pts = sum(c.points for c in chunks)
    out = torch.empty(pts, dtype=torch.float32, device=dev)
    base = out.data_ptr()
    reqs, off = [], 0
    for c in chunks:
        kind = fn.KIND_GRID3D if len(c.count) == 3 else fn.KIND_GRID2D
        reqs.append(fn.make_request(nodes[c.tree], kind, base + 4 * off, c.seed + rank, c.count, c.offset, (1, 1, 1, 1)))
        off += c.points
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    fn.gen_each(reqs, sptr, sync=True)                 # compiles and uploads every program
    jit_s = None
    if a.kernels == "jit":
        t0 = time.perf_counter()
        fn.jit_compile([(n, d) for n in nodes for d in (2, 3, 4)])
        jit_s = time.perf_counter() - t0
    else:
        fn.set_jit_enabled(False)
    fn.autotune_batch(reqs, sptr)
    for _ in range(max(a.warmup, 3)):
        fn.gen_batch(reqs, sptr, sync=False)
        fn.gen_each(reqs, sptr, sync=False)
    torch.cuda.synchronize(dev)

    def timed(fnc, steps, label):
        # NVTX range per timed region, so a profiler can be limited to it
        # (ncu --nvtx --nvtx-include "<label>/")
        st = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        flush.zero_()
        fnc()                                       # one more untimed step: clocks back up after the idle wait
        for i in range(steps):
            flush.zero_()
            torch.cuda.nvtx.range_push(label)
            st[i].record(stream)
            fnc()
            en[i].record(stream)
            torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize(dev)
        ms = [s.elapsed_time(e) for s, e in zip(st, en)]
        spread[label] = {"min": min(ms), "median": statistics.median(ms), "max": max(ms)}
        return statistics.mean(ms)

    spread = {}
    sampler = ClockSampler(local)
    with sampler:
        barrier(world)
        torch.cuda.synchronize(dev)
        rarr = fn.request_array(reqs)                # descriptors built once, as a native caller would
        batch_ms = timed(lambda: fn.gen_batch(rarr, sptr, sync=False), a.steps, "batched")
        percall_ms = timed(lambda: fn.gen_each(rarr, sptr, sync=False), max(2, a.steps // 2), "per_call")
        barrier(world)
    # the same batch with every tree on its batch kernel's variant 0 (what runs without the
    # per-tree tuning), then the tuned table back
    variants_default_ms = None
    if a.kernels == "jit":
        with tempfile.TemporaryDirectory() as td:
            tuned = os.path.join(td, "tuned.txt")
            fn.autotune_save(tuned)
            lines = open(tuned).read().splitlines()
            trees_tuned = {ln.split()[1]: int(ln.split()[2]) for ln in lines if ln.startswith("tree ")}
            plain = os.path.join(td, "plain.txt")
            with open(plain, "w") as f:
                for ln in lines:
                    parts = ln.split()
                    f.write((" ".join(parts[:2] + ["0"] + parts[3:]) if ln.startswith("tree ") else ln) + "\n")
            fn.autotune_load(plain)
            fn.gen_batch(rarr, sptr, sync=True)
            variants_default_ms = timed(lambda: fn.gen_batch(rarr, sptr, sync=False), a.steps, "batched_variant0")
            fn.autotune_load(tuned)
            fn.gen_batch(rarr, sptr, sync=True)
    interp = None
    if a.kernels == "jit":                              # the same batch through the interpreter, for comparison
        fn.set_jit_enabled(False)
        fn.autotune_batch(reqs, sptr)
        fn.gen_batch(reqs, sptr, sync=True)
        interp_ms = timed(lambda: fn.gen_batch(reqs, sptr, sync=False), max(2, a.steps // 2), "interp_batched")
        interp_pc_ms = timed(lambda: fn.gen_each(reqs, sptr, sync=False), 2, "interp_per_call")
        fn.set_jit_enabled(True)
        interp = {"batched": pts / (interp_ms * 1e-3) / 1e6, "per_call": pts / (interp_pc_ms * 1e-3) / 1e6,
                  "unit": "Mpoints/s", "note": "same mix, interpreter kernels (fnSetJitEnabled(0))"}
    clocks = sampler.summary()
    fn.gen_batch(reqs, sptr, sync=True)
    binfo = fn.batch_info()                             # shape of the device batch
    batch_ms_max = allmax(batch_ms, world)
    value = pts * world / (batch_ms_max * 1e-3) / 1e6
    percall_value = pts * world / (allmax(percall_ms, world) * 1e-3) / 1e6

    # served: closed loop (everything submitted at once), then open loop (Poisson arrivals)
    del flush
    served = run_served(fn, chunks, nodes, rank, a, dev) if a.served else None

    # end to end: the same requests with host outputs (fnGenBatchHost: descriptors up, every
    # output and min/max down, slices copied while the next slice is generated)
    def host_batch_ms(base):
        hreqs, off = [], 0
        for c in chunks:
            kind = fn.KIND_GRID3D if len(c.count) == 3 else fn.KIND_GRID2D
            hreqs.append(fn.make_request(nodes[c.tree], kind, base + 4 * off, c.seed + rank, c.count, c.offset, (1, 1, 1, 1)))
            off += c.points
        harr = fn.request_array(hreqs)
        e2e = []
        for i in range(2 + a.e2e_steps):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            fn.gen_batch_host(harr)
            if i >= 2:
                e2e.append((time.perf_counter() - t0) * 1e3)
        return (allmax(statistics.median(e2e), world) if e2e else None), fn.batch_info()

    host = torch.empty(pts, dtype=torch.float32, pin_memory=True)
    e2e_ms, hinfo = host_batch_ms(host.data_ptr())
    pageable = np.zeros(pts, np.float32) + 0.0                 # an ordinary (written) array, as most callers pass
    pageable_ms, _ = host_batch_ms(pageable.ctypes.data)
    del pageable
    # the plain copy engine rate for the same bytes (device outputs -> the pinned host buffer)
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    host.copy_(out, non_blocking=True)
    c0.record(stream)
    host.copy_(out, non_blocking=True)
    c1.record(stream)
    torch.cuda.synchronize(dev)
    d2h_gbs = pts * 4 / (c0.elapsed_time(c1) * 1e-3) / 1e9

    if rank != 0:
        return
    peaks, peak_src = load_peaks()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    peak_lane = n_sm * 128 * sm_max * 1e6 / 1e12
    tree_ops = [ops_per_point(m(), 3, 1) for m in trees.MIX_TREES]
    tree_ops2 = [ops_per_point(m(), 2, 1) for m in trees.MIX_TREES]
    work = sum(c.points * (tree_ops[c.tree] if len(c.count) == 3 else tree_ops2[c.tree]) for c in chunks)
    achieved = work / (batch_ms * 1e-3) / 1e12
    hbm_gbs = pts * 4 / (batch_ms * 1e-3) / 1e9
    cpu = cpu_baseline("chunk-mix", a.cpu_passes, 3.0, rank) if a.cpu_passes > 0 else None
    if cpu is not None and served is not None and a.cpu_rates:
        served["cpu_open_loop"] = cpu_open_loop(chunks, a, rank)
    line = {
        "metric": "Mpoints/s", "value": value, "unit": "Mpoints/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": batch_ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "step_ms": spread.get("batched"),
        "config": {"workload": "chunk-mix", "requests": len(chunks), "points_per_step": pts,
                   "trees": [m.__name__ for m in trees.MIX_TREES], "rng": "numpy PCG64(20261203)",
                   "l2": "flushed between steps (256 MiB write outside the timed events)",
                   "path": "batched persistent launch (fnGenBatchDevice), CUDA graph, "
                           + ("specialised kernels (fnJitCompile)" if a.kernels == "jit" else "interpreter kernel"),
                   "jit_compile_s": jit_s, "host_placement": a.host_placement},
        "interpreter": interp,
        "per_call": {"value": percall_value, "unit": "Mpoints/s", "ms_per_step": percall_ms,
                     "api": "fnGenEachDevice: one launch per request"},
        "batched_vs_per_call": value / percall_value,
        "batch_kernel_variants": None if variants_default_ms is None else {
            "tuned_per_tree": {k: v for k, v in trees_tuned.items()},
            "variant0_everywhere": {"value": pts / (variants_default_ms * 1e-3) / 1e6, "unit": "Mpoints/s",
                                    "ms_per_step": variants_default_ms},
            "variants": "0: 256 threads, 64 regs; 1: 256, 80 regs; 2: 256, 128 regs; 3: 128, 64 regs; "
                        "4: 256, 128 regs, 2 points in flight"},
        "served": served,
        "roofline": {"bound": "fp32-issue", "achieved": achieved, "peak": peak_lane, "unit": "Tlane-op/s",
                     "frac": achieved / peak_lane, "traffic": read_traffic("chunk-mix"),
                     "work_per_point": work / pts, "work_source": "FS-level ops per point counted by oracle/opcount.h, per tree and dimensionality",
                     "peak_source": f"{n_sm} SMs x 128 FP32 lanes x {sm_max:.0f} MHz ({peak_src} sm_max_mhz)",
                     "hbm": {"achieved_gbs": hbm_gbs, "peak_gbs": float(peaks.get("hbm_gbs", 6800.0)),
                             "frac": hbm_gbs / float(peaks.get("hbm_gbs", 6800.0)), "algorithmic_bytes_per_point": 4}},
        "e2e": {"value": pts * world / (e2e_ms * 1e-3) / 1e6 if e2e_ms else None, "unit": "Mpoints/s",
                "h2d_bytes_per_step": hinfo["uploadBytes"], "d2h_bytes_per_step": pts * 4 + 8 * len(chunks),
                "ms_per_step": e2e_ms, "d2h_copy_gbs": d2h_gbs,
                "api": "fnGenBatchHost: host (pinned) outputs; request descriptors uploaded, every output and "
                       "min/max read back, slices of 2^25 points copied while the next slice is generated",
                "pageable": {"value": pts * world / (pageable_ms * 1e-3) / 1e6 if pageable_ms else None, "unit": "Mpoints/s",
                             "ms_per_step": pageable_ms,
                             "api": "the same call into an ordinary (pageable, written) array: on a Grace host the batch "
                                    "kernels store into it directly"}},
        "batch": binfo,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": a.steps * binfo["kernels"],          # one persistent kernel per tree and dimensionality
    }
    print(json.dumps(line))


def run_served(fn, chunks, nodes, rank, a, dev):
    """Closed-loop throughput and open-loop latency through the request server."""
    pool = int(a.pool_gb * (1 << 30))
    srv = fn.Server(pool_bytes=pool, streams=a.streams, max_batch_requests=a.max_batch_requests)
    reqs = []
    for c in chunks:
        kind = fn.KIND_GRID3D if len(c.count) == 3 else fn.KIND_GRID2D
        reqs.append(fn.make_request(nodes[c.tree], kind, 0, c.seed + rank, c.count, c.offset, (1, 1, 1, 1)))
    pts = sum(c.points for c in chunks)
    # warm: one full pass
    for t in [srv.submit(r) for r in reqs]:
        srv.wait(t)
        srv.release(t)
    srv.reset_stats()
    rarr = fn.request_array(reqs)               # descriptors built once, as a native caller would
    t0 = time.perf_counter()
    tickets = srv.submit_many(rarr, as_array=True)   # one frame's worth of chunk requests at once
    srv.wait_many(tickets)
    closed_s = time.perf_counter() - t0
    closed = srv.stats()
    for t in tickets:
        srv.release(t)
    result = {"closed_loop": {"value": pts / closed_s / 1e6, "unit": "Mpoints/s", "wall_ms": closed_s * 1e3,
                              "p50_ms": closed["p50Micros"] / 1e3, "p99_ms": closed["p99Micros"] / 1e3,
                              "batches": closed["batches"], "api": "fnServerSubmitMany + fnServerWaitMany"}}
    # open loop: the serving mix -- the chunk mix plus, every `extra_every` chunks, one
    # GenUniformGrid4D 32^4 and one GenPositionArray3D over 1M positions uniform in [-1e4, 1e4]^3
    import torch
    prng = np.random.default_rng(20261203)
    pos = [torch.from_numpy(prng.uniform(-1e4, 1e4, 1 << 20).astype(np.float32)).to(dev) for _ in range(3)]
    serve, serve_pts = [], []
    for k, (c, r) in enumerate(zip(chunks, reqs)):
        serve.append(r)
        serve_pts.append(c.points)
        if a.extra_every > 0 and k % a.extra_every == a.extra_every - 1:
            serve.append(fn.make_request(nodes[c.tree], fn.KIND_GRID4D, 0, c.seed + 1, (32, 32, 32, 32),
                                         tuple(c.offset) + (0.0,) * (4 - len(c.offset)), (1, 1, 1, 1)))
            serve_pts.append(32 ** 4)
            serve.append(fn.make_request(nodes[c.tree], fn.KIND_POSITIONS3D, 0, c.seed + 2, (1 << 20,), (0, 0, 0), (1, 1, 1),
                                         positions=[p.data_ptr() for p in pos]))
            serve_pts.append(1 << 20)
    for t in [srv.submit(r) for r in serve]:           # warm the extra kinds
        srv.wait(t)
        srv.release(t)
    # the per-call path needs outputs of its own: one device buffer holding every distinct request's output
    serve_total = int(sum(serve_pts))
    pc_out = torch.empty(serve_total, dtype=torch.float32, device=dev)
    pc_reqs, off = [], 0
    for r, n_pts in zip(serve, serve_pts):
        q = fn.GenRequest.from_buffer_copy(r)
        q._keep = r._keep
        q.out = pc_out.data_ptr() + 4 * off
        pc_reqs.append(q)
        off += n_pts
    stream = torch.cuda.current_stream(dev).cuda_stream
    fn.gen_each(pc_reqs, stream, sync=True)              # warm the per-call path
    open_loop, per_call_open = [], []
    rng = np.random.default_rng(5)
    for rate in a.rates:
        n = min(4 * len(serve), max(200, int(rate * a.open_seconds)))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n)) * 1e6      # microseconds after the start
        idx = [k % len(serve) for k in range(n)]
        served_pts = sum(serve_pts[k] for k in idx)
        # served: one native submitter follows the arrival schedule; latency counts from arrival
        srv.reset_stats()
        rarr = fn.request_array([serve[k] for k in idx])
        t_start = time.perf_counter()
        tickets = srv.submit_paced(rarr, arrivals)
        srv.wait_many(tickets, timeout_ms=120000)
        wall = time.perf_counter() - t_start
        st = srv.stats()
        for t in tickets:
            srv.release(t)
        open_loop.append({"rate_req_s": rate, "achieved_req_s": n / wall, "requests": n,
                          "p50_ms": st["p50Micros"] / 1e3, "p99_ms": st["p99Micros"] / 1e3,
                          "max_ms": st["maxMicros"] / 1e3, "Mpoints_s": served_pts / wall / 1e6, "batches": st["batches"],
                          "overlapped_batches": st["overlappedBatches"], "max_concurrent_batches": st["maxConcurrentBatches"]})
        # per-call: the same arrivals, one fnGen*Device launch per request on one stream
        parr = fn.request_array([pc_reqs[k] for k in idx])
        t_start = time.perf_counter()
        lat = fn.gen_each_paced(parr, arrivals, stream)
        wall = time.perf_counter() - t_start
        per_call_open.append({"rate_req_s": rate, "achieved_req_s": n / wall, "requests": n,
                              "p50_ms": float(np.percentile(lat, 50)) / 1e3, "p99_ms": float(np.percentile(lat, 99)) / 1e3,
                              "max_ms": float(lat.max()) / 1e3, "Mpoints_s": served_pts / wall / 1e6})
    del pc_out
    srv.close()
    result["open_loop"] = open_loop
    result["per_call_open_loop"] = per_call_open
    result["config"] = {"pool_gb": a.pool_gb, "streams": a.streams, "max_batch_requests": a.max_batch_requests,
                        "open_loop_mix": f"chunk mix + per {a.extra_every} chunks one GenUniformGrid4D 32^4 and one "
                                         "GenPositionArray3D 1M positions U[-1e4,1e4]^3; Poisson arrivals",
                        "open_loop_latency": "arrival -> min/max on the host; served: fnServerSubmitPaced + fnServerWaitMany; "
                                             "per_call_open_loop: fnGenEachPaced (one fnGen*Device launch per request on one "
                                             "stream, min/max copied back, completion seen by a second host thread)"}
    return result


def cpu_open_loop(chunks, a, rank=0):
    """The same open-loop serving mix on the host cores: the CPU restatement (oracle/) serves
    requests in arrival order on every host thread, whole requests per thread; latency counts
    from arrival to the request's output and min/max written."""
    from oracle import oracle
    from tests import trees
    otrees = [oracle.OracleTree(m()) for m in trees.MIX_TREES]
    prng = np.random.default_rng(20261203)
    pos = [prng.uniform(-1e4, 1e4, 1 << 20).astype(np.float32) for _ in range(3)]
    serve = []                                            # (tree, kind, count, offset, seed, positions, points)
    for k, c in enumerate(chunks):
        kind = oracle.KIND_GRID3D if len(c.count) == 3 else oracle.KIND_GRID2D
        serve.append((c.tree, kind, tuple(c.count), tuple(c.offset), c.seed + rank, (), c.points))
        if a.extra_every > 0 and k % a.extra_every == a.extra_every - 1:
            serve.append((c.tree, oracle.KIND_GRID4D, (32, 32, 32, 32), tuple(c.offset) + (0.0,) * (4 - len(c.offset)),
                          c.seed + 1, (), 32 ** 4))
            serve.append((c.tree, oracle.KIND_POSITIONS3D, (1 << 20,), (0, 0, 0), c.seed + 2, pos, 1 << 20))
    threads = os.cpu_count()
    rng = np.random.default_rng(5)
    result = []
    for rate in a.cpu_rates:
        n = min(len(serve), max(100, int(rate * a.cpu_open_seconds)))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n)) * 1e6
        outs, mms, reqs = [], [], []
        for k in range(n):
            tree, kind, cnt, off, seed, p, npts = serve[k]
            outs.append(np.empty(npts, np.float32))
            mms.append(np.zeros(2, np.float32))
            reqs.append(oracle.request(otrees[tree], kind, outs[-1], mms[-1], seed, cnt, off, (1.0,) * len(cnt), p))
        t0 = time.perf_counter()
        lat = oracle.serve_paced(reqs, arrivals, threads)
        wall = time.perf_counter() - t0
        npts = sum(serve[k][-1] for k in range(n))
        result.append({"rate_req_s": rate, "achieved_req_s": n / wall, "requests": n,
                       "p50_ms": float(np.percentile(lat, 50)) / 1e3, "p99_ms": float(np.percentile(lat, 99)) / 1e3,
                       "max_ms": float(lat.max()) / 1e3, "Mpoints_s": npts / wall / 1e6})
    return {"threads": threads, "rates": result, "host": oracle.cpu_description(),
            "api": "oracle on_serve_paced: Poisson arrivals (same mix and generator as the served open loop), "
                   "a FIFO served by every host thread, whole requests per thread"}


# ---------------------------------------------------------------- GPU: chunk meshing

def mesh_tree():
    """A terrain surface for the mesher: vertical gradient plus fractal noise."""
    from oracle.tree import N
    g = N("Gradient")
    g.set("Multiplier", 0.02, 1)
    return N("Add", LHS=N("FractalFBm", Source=N("Simplex", Feature_Scale=60.0), Octaves=4), RHS=g)


def run_mesh(a, rank, world, local):
    """fnBuildChunkMeshesBloxel (130^3 densities per chunk) or fnBuildChunkMeshesDmc (132^3) on
    the Node Editor's chunk size, 128^3 voxels: a row of 8 chunks across the surface per step, in
    one multi-chunk call; the same chunks one synchronous call each are reported beside it."""
    import torch
    import fastnoise2_gb300 as fn
    fn.set_auto_specialise(0)              # the kernel tier is chosen explicitly (--kernels)
    from tests.trees import to_product
    size, chunks = 128, 8
    dmc = a.workload == "mesh-dmc-128"
    build = fn.build_chunk_mesh_dmc if dmc else fn.build_chunk_mesh_bloxel
    api = "fnBuildChunkMeshesDmc" if dmc else "fnBuildChunkMeshesBloxel"
    apron = 4 if dmc else 2
    node = to_product(mesh_tree())
    if a.kernels == "jit":
        fn.jit_compile([(node, 3)])
    else:
        fn.set_jit_enabled(False)
    fn.set_mesh_density_form(fn.MESH_DENSITY_SPARSE if a.mesh_densities == "sparse" else fn.MESH_DENSITY_ARRAY)
    dev = torch.device("cuda", local)
    vcap, icap = 2 << 20, 4 << 20                       # per chunk: a 128^3 surface chunk needs ~0.5 M / 0.7 M
    bufs = [(torch.empty(vcap * 4, dtype=torch.float32, device=dev), torch.empty(icap, dtype=torch.int32, device=dev))
            for _ in range(chunks)]
    ptrs = [(v.data_ptr(), vcap, i.data_ptr(), icap) for v, i in bufs]
    stream = torch.cuda.current_stream(dev)
    positions = [(size * (k - chunks // 2), -size // 2, size * (rank % 4)) for k in range(chunks)]
    faces = []

    def step():
        res = fn.build_chunk_meshes("dmc" if dmc else "bloxel", node, size, positions, 1337 + rank, 0.0, False, ptrs,
                                    stream.cuda_stream)
        for r in res:
            if not r["fits"]:
                raise RuntimeError(f"{api}: mesh buffers too small ({r['vertexCount']} vertices)")
            faces.append(r["indexCount"] // 6)

    def step_single():
        for p, (vp, vc, ip, ic) in zip(positions, ptrs):
            build(node, size, p, 1337 + rank, 0.0, False, vp, vc, ip, ic, stream.cuda_stream)

    for _ in range(max(a.warmup, 3)):
        step()
    torch.cuda.synchronize(dev)
    faces.clear()
    sampler = ClockSampler(local)
    with sampler:
        barrier(world)
        step()                                      # one more untimed step: clocks back up after the idle wait
        torch.cuda.synchronize(dev)
        faces.clear()
        st = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
        for i in range(a.steps):
            torch.cuda.nvtx.range_push("timed")
            st[i].record(stream)
            step()
            en[i].record(stream)
            torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize(dev)
        barrier(world)
    clocks = sampler.summary()
    ms = statistics.mean(s_.elapsed_time(e_) for s_, e_ in zip(st, en))
    ms_max = allmax(ms, world)
    voxels = chunks * size ** 3
    value = voxels * world / (ms_max * 1e-3) / 1e6
    # the same chunks, one synchronous single-chunk call each (for comparison)
    step_single()
    torch.cuda.synchronize(dev)
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(a.steps):
        step_single()
    s1.record(stream)
    torch.cuda.synchronize(dev)
    single_ms = s0.elapsed_time(s1) / a.steps
    if rank != 0:
        return
    line = {
        "metric": "Mpoints/s", "value": value, "unit": "Mpoints/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": a.workload, "chunks_per_step": chunks, "chunk": [size] * 3,
                   "points_per_step": voxels, "densities_per_chunk": (size + apron) ** 3,
                   ("quads_per_chunk" if dmc else "faces_per_chunk"): statistics.mean(faces) if faces else 0,
                   "path": api + ": densities (" + ("specialised kernel" if a.kernels == "jit" else "interpreter")
                           + (") + cases/count/scan/vertex/quad mesher" if dmc else ") + count/scan/emit mesher")
                           + f", {chunks} chunks per call over 4 internal streams",
                   "density_form": a.mesh_densities,
                   "l2": (f"densities of a chunk ({(size + apron) ** 3 * 4 / 1e6:.1f} MB) stay in L2 between generation and meshing"
                          if a.mesh_densities == "array" else
                          "no density array: 2 classification bits per density, exact values only where the passes read them")},
        "e2e": {"value": value, "unit": "Mpoints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": (24 if dmc else 20) * chunks,
                "api": api + " (device mesh buffers; counts, heights and min/max read back per chunk)"},
        "single_chunk_calls": {"value": voxels / (single_ms * 1e-3) / 1e6, "unit": "Mpoints/s", "ms_per_step": single_ms,
                               "api": api.replace("Meshes", "Mesh") + ", one synchronous call per chunk"},
        "cpu_baseline": None,
        "clocks": clocks,
        # densities, then cases, count, 2 scan kernels, vertices, quads (dmc) or count, 3 scan kernels, emit (bloxel)
        "gpu_launches": a.steps * chunks * (7 if dmc else 6),
    }
    print(json.dumps(line))


# ---------------------------------------------------------------- GPU: single grids

def run_grid(a, rank, world, local):
    import torch
    from tests.trees import to_product
    tname, kind, args, seed = GRID_WORKLOADS[a.workload]
    pts = int(np.prod(args[1])) if kind == "grid" else int(args[0][0] * args[0][1])
    root = tree_named(tname)
    node = to_product(root)
    node.prepare(4 if kind == "tile" else len(args[1]))
    import fastnoise2_gb300 as fn
    fn.set_auto_specialise(0)              # the kernel tier is chosen explicitly (--kernels)
    if a.kernels == "jit":
        fn.jit_compile([(node, 4 if kind == "tile" else len(args[1]))])
    else:
        fn.set_jit_enabled(False)
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
        flush.zero_()
        step()                                      # one more untimed step: clocks back up after the idle wait
        torch.cuda.synchronize(dev)
        for i in range(a.steps):
            flush.zero_()
            torch.cuda.nvtx.range_push("timed")
            starts[i].record(stream)
            step()
            ends[i].record(stream)
            torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize(dev)
        barrier(world)
    clocks = sampler.summary()
    ms = statistics.mean(s.elapsed_time(e) for s, e in zip(starts, ends))
    ms_max = allmax(ms, world)
    value = pts * world / (ms_max * 1e-3) / 1e6

    def host_ms(host):
        samples = []
        for i in range(3 + a.e2e_steps):
            t0 = time.perf_counter()
            if kind == "grid":
                node.gen_uniform_grid(*args, seed + rank, out=host)
            else:
                node.gen_tileable_2d(args[0], args[1], seed + rank, out=host)
            if i >= 3:
                samples.append((time.perf_counter() - t0) * 1e3)
        return allmax(statistics.median(samples), world)

    e2e_ms = pageable_ms = None
    if a.e2e_steps > 0:
        e2e_ms = host_ms(torch.empty(pts, dtype=torch.float32, pin_memory=True).numpy())
        pageable_ms = host_ms(np.zeros(pts, np.float32) + 0.0)    # an ordinary (written) array, as a drop-in caller passes
    if rank != 0:
        return
    peaks, peak_src = load_peaks()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    peak_lane = n_sm * 128 * sm_max * 1e6 / 1e12
    ops = ops_per_point(root, 4 if kind == "tile" else len(args[1]), seed)
    achieved = pts * ops / (ms * 1e-3) / 1e12
    hbm_gbs = pts * 4 / (ms * 1e-3) / 1e9
    line = {
        "metric": "Mpoints/s", "value": value, "unit": "Mpoints/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": a.workload, "points_per_step": pts, "tree": tname, "seed": seed,
                   "l2": "flushed between steps (256 MiB write outside the timed events)",
                   "path": "per-call " + ("specialised kernel (fnJitCompile)" if a.kernels == "jit" else "interpreter kernel")
                           + ", device-resident output"},
        "roofline": {"bound": "fp32-issue", "achieved": achieved, "peak": peak_lane, "unit": "Tlane-op/s",
                     "frac": achieved / peak_lane, "traffic": read_traffic(a.workload), "work_per_point": ops,
                     "work_source": "FS-level ops per point counted by oracle/opcount.h",
                     "peak_source": f"{n_sm} SMs x 128 FP32 lanes x {sm_max:.0f} MHz ({peak_src} sm_max_mhz)",
                     "hbm": {"achieved_gbs": hbm_gbs, "peak_gbs": float(peaks.get("hbm_gbs", 6800.0)),
                             "frac": hbm_gbs / float(peaks.get("hbm_gbs", 6800.0)), "algorithmic_bytes_per_point": 4}},
        "e2e": {"value": pts * world / (e2e_ms * 1e-3) / 1e6 if e2e_ms else None, "unit": "Mpoints/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": pts * 4 + 8, "ms_per_step": e2e_ms,
                "api": "fnGenUniformGrid3D / fnGenTileable2D into pinned host memory",
                "pageable": {"value": pts * world / (pageable_ms * 1e-3) / 1e6 if pageable_ms else None,
                             "unit": "Mpoints/s", "ms_per_step": pageable_ms,
                             "api": "the same calls into an ordinary (pageable, written) numpy array"}},
        "cpu_baseline": cpu_baseline(a.workload, a.cpu_passes, 3.0, rank) if a.cpu_passes > 0 else None,
        "clocks": clocks,
        "gpu_launches": a.steps,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="chunk-mix", choices=WORKLOADS)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--kernels", default="jit", choices=["jit", "interp"],
                    help="specialised per-tree kernels (NVRTC) or the program interpreter")
    ap.add_argument("--cpu-passes", type=int, default=1,
                    help="cpu_baseline: whole passes of the CPU restatement over the workload (0 = leave it out)")
    ap.add_argument("--cpu-seconds", type=float, default=None, help=argparse.SUPPRESS)   # older spelling: 0 = no baseline
    ap.add_argument("--pool-gb", type=float, default=40.0)
    ap.add_argument("--streams", type=int, default=3)
    ap.add_argument("--max-batch-requests", type=int, default=512)
    ap.add_argument("--rates", type=float, nargs="*",
                    default=[1000.0, 5000.0, 10000.0, 20000.0, 50000.0, 100000.0, 200000.0, 400000.0])
    ap.add_argument("--cpu-rates", type=float, nargs="*", default=[100.0, 250.0, 500.0, 1000.0],
                    help="open-loop request rates for the CPU restatement's serving latency (none = leave it out)")
    ap.add_argument("--cpu-open-seconds", type=float, default=1.0,
                    help="seconds of Poisson arrivals per CPU open-loop rate")
    ap.add_argument("--extra-every", type=int, default=64,
                    help="serving mix: one GenUniformGrid4D 32^4 and one GenPositionArray3D 1M request per this many chunks")
    ap.add_argument("--open-seconds", type=float, default=0.5)
    ap.add_argument("--requests", type=int, default=4096,
                    help="chunk mix: use the first N requests of the 4096-request mix (smaller cases for profiling)")
    ap.add_argument("--mesh-densities", default="array", choices=["array", "sparse"],
                    help="mesh workloads: the chunk's density array, or the sparse form (fnSetMeshDensityForm)")
    ap.add_argument("--no-served", dest="served", action="store_false",
                    help="chunk mix: leave out the request-server measurements")
    a = ap.parse_args()
    if a.cpu_seconds is not None and a.cpu_seconds <= 0:
        a.cpu_passes = 0
    if a.impl == "reference":
        run_reference(a)
        return
    import torch
    rank, world, local = dist_setup()
    torch.cuda.set_device(local)
    a.host_placement = bind_near_gpu(local)
    if a.workload == "chunk-mix":
        run_chunkmix(a, rank, world, local)
    elif a.workload in ("mesh-bloxel-128", "mesh-dmc-128"):
        run_mesh(a, rank, world, local)
    else:
        run_grid(a, rank, world, local)


if __name__ == "__main__":
    main()
