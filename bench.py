"""Benchmark of gpugi's hot path on GB300.

Headline workload (the closest-hit query configuration): a displaced
icosphere of 65,536 triangles, bvhmake `sweep` SAH AABB hierarchy with
8-triangle leaf blocks, 2^20 rays per step (origins uniform in [-2,2]^3,
directions uniform on the sphere, tmax = inf). One step = one closest-hit
launch over one batch of 2^20 rays. Metric: Mrays/s closest-hit.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own
GPU (the path has no exchange step); value = all rays / max-over-ranks time.
`--impl reference` times the CPU restatement of the reference's shaders on
all host cores (the reference's GLSL path cannot run here).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s closest-hit"
UNIT = "Mrays/s"
N_RAYS = 1 << 20
N_BATCHES = 8  # rotating ray batches: 8 x 44 MB of rays+results > 129 MB L2
WORKLOAD = ("closest-hit queries: displaced icosphere 65,536 tris (level-6 icosphere truncated, radial "
            "U[-0.05,0.05], unit cube), bvhmake sweep SAH AABB BVH leaf 8, 2^20 rays/step, origins U[-2,2]^3, "
            "dirs uniform on S^2, tmax=inf")
FALLBACK_HBM_GBS = 6800.0
# Kernels of one step per trace mode (the roofline is taken over the whole step).
KERNELS = {0: "k_trace_closest<AABB>", 1: "k_trace_persistent<closest, AABB>",
           2: "k_trace_root_filter<closest, AABB> + k_trace_queue<closest, AABB>",
           3: "k_trace_root_filter<closest, AABB> + k_trace_group<closest, AABB, 8>",
           4: "k_trace_root_filter<closest, AABB> + k_trace_group<closest, AABB, 4>",
           5: "k_trace_root_filter<closest, AABB> + k_trace_group<closest, AABB, 16>"}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def link_bound(rays_block: np.ndarray, results_block: np.ndarray, dev) -> dict:
    """The host link's bound on the end-to-end rate: one step's rays copied
    in and its results copied out at the same time (one copy each way, on two
    streams), timed with CUDA events; the copies in both directions share
    the link, so this is below the sum of the one-way rates. The blocks are
    the page-locked (7, N) ray and (4, N) result arrays of one step."""
    import torch
    hin_t, hout_t = torch.from_numpy(rays_block), torch.from_numpy(results_block)
    din = torch.empty(hin_t.shape, dtype=torch.float32, device=dev)
    dout = torch.empty(hout_t.shape, dtype=torch.float32, device=dev)
    s_in, s_out = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
    cur = torch.cuda.current_stream(dev)

    def step():
        s_in.wait_stream(cur)
        s_out.wait_stream(cur)
        with torch.cuda.stream(s_in):
            din.copy_(hin_t, non_blocking=True)
        with torch.cuda.stream(s_out):
            hout_t.copy_(dout, non_blocking=True)
        cur.wait_stream(s_in)
        cur.wait_stream(s_out)

    for _ in range(3):
        step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 20
    e0.record(cur)
    for _ in range(reps):
        step()
    e1.record(cur)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / reps
    return {"value": N_RAYS / (ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": ms,
            "bytes_in": int(hin_t.numel() * 4), "bytes_out": int(hout_t.numel() * 4),
            "what": "one step's rays in and results out copied concurrently (one copy each way), CUDA events"}


def l2_read_gbs(ctx) -> float:
    """L2 read bandwidth (gpugi_measure_l2_bandwidth: one launch re-reads an
    L2-resident 32 MiB buffer 200 times). The driver's peaks file has no L2
    figure; this stands in for it as the second roofline."""
    import ctypes as C
    from gpugi_gb300 import cuda
    lib = cuda.lib()
    lib.gpugi_measure_l2_bandwidth.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.POINTER(C.c_double)]
    g = C.c_double()
    ctx.check(lib.gpugi_measure_l2_bandwidth(ctx.handle, 32 << 20, 200, C.byref(g)))
    return g.value


def profile_traffic():
    """DRAM bytes per launch of the traversal kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "trace_closest_icosphere65536.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return int(float(line.split(":", 1)[1].strip()))
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def bench_config(world: int) -> dict:
    """The `config` object of both arms' lines (the same workload)."""
    return {"workload": WORKLOAD,
            "l2": "inputs larger than L2: 8 rotating ray batches (8 x 44 MB rays+results)",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


def make_workload():
    from gpugi_gb300 import bvh, scenes
    sc = scenes.displaced_icosphere(65536, seed=1)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", leaf_size=8)
    batches = [scenes.random_rays(N_RAYS, seed=100 + k) for k in range(N_BATCHES)]
    return sc, b, batches


def cpu_tracer():
    """The reference's CPU implementation of the walk: its own shader text
    compiled as C++ (oracle/_ref, kind "reference") where it could be built,
    else the oracle's restatement of it (kind "port"). Returns (kind, trace)
    with trace(bvh, positions, rays, threads)."""
    import oracle
    try:
        from oracle import ref
        if ref.available():
            def trace(b, positions, rays, nthreads):
                os.environ["ORACLE_THREADS"] = str(nthreads)
                return ref.trace_closest(b, positions, rays)
            return "reference", trace
    except (ImportError, OSError, RuntimeError):
        pass
    return "port", lambda b, positions, rays, nthreads: oracle.trace_closest(b, positions, rays, num_threads=nthreads)


def cpu_baseline(b, positions, batches, seconds=10.0, threads=None):
    """The reference's walk on the host cores (cpu_tracer), over a bounded
    sample of the same workload: whole 2^20-ray batches until `seconds` of
    wall time have passed."""
    kind, trace = cpu_tracer()
    nthreads = threads or os.cpu_count() or 1
    trace(b, positions, batches[0], nthreads)  # warm-up, builds the library
    rays = 0
    t0 = time.perf_counter()
    k = 0
    while True:
        trace(b, positions, batches[k % len(batches)], nthreads)
        rays += N_RAYS
        k += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    what = ("the reference's traceray.glsl compiled as C++" if kind == "reference"
            else "the oracle's C++ restatement of traceray.glsl")
    return {"value": rays / el / 1e6, "unit": UNIT, "cores": nthreads, "kind": kind,
            "sample": f"{k} batches of 2^20 rays of this workload ({rays} rays, {el:.1f} s wall) on {nthreads} "
                      f"threads: {what}"}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def reduce_max(x: float, world: int, device) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, world, rank):
    if rank != 0:
        return
    sc, b, batches = make_workload()
    nthreads = os.cpu_count() or 1
    kind, trace = cpu_tracer()
    for k in range(args.warmup):
        trace(b, sc["positions"], batches[k % N_BATCHES], nthreads)
    t0 = time.perf_counter()
    for k in range(args.steps):
        trace(b, sc["positions"], batches[k % N_BATCHES], nthreads)
    el = time.perf_counter() - t0
    value = args.steps * N_RAYS / el / 1e6
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(args.gpus), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": kind,
                             "sample": f"{args.steps} steps x 2^20 rays on {nthreads} threads: " + (
                                 "the reference's traceray.glsl + intersectiontests.glsl compiled as C++ "
                                 "(its OpenGL path is unavailable on this box)" if kind == "reference" else
                                 "the oracle's C++ restatement of the reference's shaders (its OpenGL path is "
                                 "unavailable on this box and its shader text could not be compiled here)")},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch
    from gpugi_gb300 import cuda

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    sc, b, host_batches = make_workload()
    ctx = cuda.Context(local)
    ctx.set_trace_config(mode=args.trace_mode)
    ctx.set_host_pipeline(args.host_parts, args.zero_copy)
    ctx.set_scene_layout(args.shared_nodes, 0)
    ds = ctx.upload_scene(b, sc["positions"])
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    batches = [{k: torch.from_numpy(rb[k]).to(dev) for k in cuda.RAY_KEYS} for rb in host_batches]
    outs = [dict(slot=torch.empty(N_RAYS, dtype=torch.int32, device=dev),
                 t=torch.empty(N_RAYS, device=dev), u=torch.empty(N_RAYS, device=dev),
                 v=torch.empty(N_RAYS, device=dev)) for _ in range(N_BATCHES)]
    torch.cuda.synchronize()

    # Algorithmic bytes of one launch (gpugi's own fetch pattern), from the
    # device-side walk counters averaged over the batches.
    alg = [cuda.algorithmic_bytes(cuda.trace_stats_device(ctx, ds, bt), N_RAYS) for bt in batches]
    alg_bytes = float(np.mean(alg))

    # Steps alternate between several streams (gpugi_trace_closest_device_async):
    # independent batches, so the walker tail of step k (its few deepest
    # rays) overlaps the filter and walk of the next steps; each stream-ordered
    # walk launches a share of the persistent grid (--walker-share, the
    # library's default 50 %), so two or more walks run side by side. The same
    # K steps as synchronous calls on the context's stream, with the full
    # grid, are timed too ("single_stream").
    qstreams = [torch.cuda.Stream(device=dev) for _ in range(args.streams)]
    ctx.set_async_walker_share(args.walker_share)

    def issue(k):
        s = qstreams[k % len(qstreams)]
        cuda.trace_closest_device_async(ctx, ds, batches[k % N_BATCHES], outs[k % N_BATCHES], s.cuda_stream)
        return s

    for k in range(max(args.warmup, len(qstreams))):
        issue(k)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    t_begin = torch.cuda.Event(enable_timing=True)
    t_end = [torch.cuda.Event(enable_timing=True) for _ in qstreams]
    with ClockSampler(local) as clk:
        # about a second of the same untimed steps right before the timed
        # region, so the clock record (100 ms samples) sees the GPU under
        # this load: the timed region itself lasts a few milliseconds
        t_soak = time.perf_counter()
        k = 0
        while time.perf_counter() - t_soak < 1.0:
            issue(k)
            k += 1
            if k % 64 == 0:
                torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        t_begin.record(qstreams[0])
        for s in qstreams[1:]:
            s.wait_event(t_begin)
        for k in range(args.steps):
            s = qstreams[k % len(qstreams)]
            starts[k].record(s)
            issue(k)
            ends[k].record(s)
        for e, s in zip(t_end, qstreams):
            e.record(s)
        torch.cuda.synchronize()
        barrier(world)
    per_launch_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = max(t_begin.elapsed_time(e) for e in t_end)
    total_ms = reduce_max(total_ms, world, dev)
    value = world * args.steps * N_RAYS / (total_ms / 1e3) / 1e6

    # the same steps on the context stream, one after another
    for k in range(args.warmup):
        cuda.trace_closest_device(ctx, ds, batches[k % N_BATCHES], outs[k % N_BATCHES])
    ctx.sync()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    single_launch = []
    with torch.cuda.stream(stream):
        s0.record(stream)
        for k in range(args.steps):
            a, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            cuda.trace_closest_device(ctx, ds, batches[k % N_BATCHES], outs[k % N_BATCHES])
            b_.record(stream)
            single_launch.append((a, b_))
        s1.record(stream)
    ctx.sync()
    torch.cuda.synchronize()
    single_ms = reduce_max(s0.elapsed_time(s1), world, dev)
    single = {"value": world * args.steps * N_RAYS / (single_ms / 1e3) / 1e6, "unit": UNIT,
              "ms_per_step": single_ms / args.steps,
              "avg_launch_ms": float(np.mean([a.elapsed_time(b_) for a, b_ in single_launch]))}

    # The same steps with the watertight triangle test (an addition of the
    # library; the headline keeps the reference's test).
    ds.set_triangle_test(True)
    for k in range(args.warmup):
        cuda.trace_closest_device(ctx, ds, batches[k % N_BATCHES], outs[k % N_BATCHES])
    ctx.sync()
    w0, w1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        w0.record(stream)
        for k in range(args.steps):
            cuda.trace_closest_device(ctx, ds, batches[k % N_BATCHES], outs[k % N_BATCHES])
        w1.record(stream)
    ctx.sync()
    torch.cuda.synchronize()
    wt_ms = reduce_max(w0.elapsed_time(w1), world, dev)
    watertight = {"value": world * args.steps * N_RAYS / (wt_ms / 1e3) / 1e6, "unit": UNIT,
                  "ms_per_step": wt_ms / args.steps,
                  "test": "Woop-Benthin-Wald watertight triangle test + Ize robust box test, same walk"}
    ds.set_triangle_test(False)

    # End to end through the public C ABI with host buffers: every step copies
    # its rays from page-locked host memory and its results back. Steps are
    # issued with gpugi_trace_closest_async over several streams, so one
    # batch's results travel back while the next batch's rays travel in; the
    # synchronous call (gpugi_trace_closest, one batch at a time) is timed too.
    # The host rays of a batch are one page-locked structure-of-arrays block
    # (ox | oy | oz | dx | dy | dz | tmax) and its results another (slot | t
    # | u | v): the library moves evenly spaced columns with one copy each way.
    ns = max(1, args.e2e_streams)
    pin, res, blocks = [], [], []
    for rb in host_batches[:max(ns, 2)]:
        blk = torch.empty((len(cuda.RAY_KEYS), N_RAYS), dtype=torch.float32).pin_memory().numpy()
        for i, key in enumerate(cuda.RAY_KEYS):
            blk[i] = rb[key]
        pin.append({key: blk[i] for i, key in enumerate(cuda.RAY_KEYS)})
        blocks.append(blk)
    for k in range(max(ns, 2)):
        blk = torch.empty((4, N_RAYS), dtype=torch.float32).pin_memory().numpy()
        res.append(dict(slot=blk[0].view(np.int32), t=blk[1], u=blk[2], v=blk[3]))
        blocks[k] = (blocks[k], blk)
    lib = cuda.lib()
    lib.gpugi_trace_closest_async.argtypes = [ctypes.c_void_p] * 9 + [ctypes.c_uint64] + [ctypes.c_void_p] * 5
    estreams = [torch.cuda.Stream(device=dev) for _ in range(ns)]

    def e2e_issue(k):
        r, o, s = pin[k % ns], res[k % ns], estreams[k % ns]
        ctx.check(lib.gpugi_trace_closest_async(ctx.handle, ds.handle, *[cuda._ptr(r[key]) for key in cuda.RAY_KEYS],
                                                N_RAYS, cuda._ptr(o["slot"]), cuda._ptr(o["t"]), cuda._ptr(o["u"]),
                                                cuda._ptr(o["v"]), ctypes.c_void_p(s.cuda_stream)))

    def e2e_sync_step(k):
        r, o = pin[k % 2], res[k % 2]
        ctx.check(lib.gpugi_trace_closest(ctx.handle, ds.handle, *[cuda._ptr(r[key]) for key in cuda.RAY_KEYS],
                                          N_RAYS, cuda._ptr(o["slot"]), cuda._ptr(o["t"]), cuda._ptr(o["u"]),
                                          cuda._ptr(o["v"])))

    for k in range(max(args.warmup, ns)):
        e2e_issue(k)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_issue(k)
    for s in estreams:
        s.synchronize()
    e2e_s = reduce_max(time.perf_counter() - t0, world, dev)
    e2e_value = world * args.steps * N_RAYS / e2e_s / 1e6
    assert (res[0]["slot"] >= -1).all() and ctx.device_error_bits() == 0
    for k in range(args.warmup):
        e2e_sync_step(k)
    barrier(world)
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_sync_step(k)
    e2e_sync_s = reduce_max(time.perf_counter() - t0, world, dev)
    e2e_sync = {"value": world * args.steps * N_RAYS / e2e_sync_s / 1e6, "unit": UNIT,
                "call": "gpugi_trace_closest (synchronous, one batch at a time)"}
    link = link_bound(blocks[0][0], blocks[0][1], dev)

    peak, peak_src = peaks()
    avg_launch_s = float(np.mean(per_launch_ms)) / 1e3
    # Consecutive launches overlap (two streams), so a launch's own span
    # counts time it shares with its neighbours: the time per launch is the
    # timed region divided by the launches (the spans are reported beside).
    step_s = total_ms / 1e3 / args.steps
    achieved = alg_bytes / step_s / 1e9
    traffic = profile_traffic()
    l2 = l2_read_gbs(ctx)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(world),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": N_RAYS * 28,
                    "d2h_bytes_per_step": N_RAYS * 16,
                    "call": f"gpugi_trace_closest_async from page-locked host arrays over {ns} streams",
                    "synchronous": e2e_sync, "link_bound": link},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per step, read from "
                                           "the committed profiles/trace_closest_icosphere65536.md (DRAM counters "
                                           "need ncu and are not measured in this run)" if traffic else None,
                         "peak_source": f"{peak_src} hbm_gbs (MEASURED_PEAKS.json)" if peak_src == "measured"
                         else "fallback 6.8 TB/s",
                         "alg_bytes_per_launch": alg_bytes, "time_per_launch_ms": step_s * 1e3,
                         "avg_launch_span_ms": avg_launch_s * 1e3,
                         "launch_time": f"timed region / launches; steps alternate over {len(qstreams)} streams",
                         "kernel": KERNELS[args.trace_mode]},
            # the scene (5.4 MB) is L2-resident: the same algorithmic bytes against the L2
            "roofline_l2": {"achieved": achieved, "peak": l2, "unit": "GB/s", "frac": achieved / l2,
                            "peak_source": "measured in this run: L2 reads of an L2-resident 32 MiB buffer"},
            "streams": len(qstreams),
            "async_walker_share": args.walker_share,
            "single_stream": single,
            "watertight": watertight,
            "gpu_launches": args.steps * (2 if args.trace_mode >= 2 else 1),
            "clocks": dict(clk.summary(), window="1 s of the same untimed steps, then the timed region")}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(b, sc["positions"], host_batches, seconds=args.cpu_seconds)
    ds.close()
    ctx.close()
    if rank == 0 and world == 1 and not args.no_nrc:
        with ClockSampler(local) as nclk:
            line["nrc"] = nrc_headline(args)
        line["nrc"]["clocks"] = nclk.summary()
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_passes(args):
    """Per-pass throughput of the wavefront renderers on the Cornell workload:
    room of ~98k triangles (5 walls, 2 rotated boxes, level-6 sphere, 0.5 x
    0.5 ceiling light of radiance 10, albedos U[0.1, 0.9]), 512 x 512, 16 spp,
    depth 8, Russian roulette after depth 3. For PT, LT, BPT, the Whitted ray
    tracer, the photon mapper (2048 photons per light sample, radius
    0.01, one photon map per iteration), the importon map light tracer (2048
    photons per light sample, radius 0.005, one importon map per iteration)
    and the hierarchy-importance renderer
    (its own 4-vertex paths; the importance pass runs in the warm-up
    iteration and is timed there): samples/s
    (iterations x pixels per second) and Mrays/s (closest-hit + any-hit rays
    traced, counted on the device by the wavefront passes), CUDA events
    around 16 spp after one warm-up iteration. Beside each, the CPU
    restatement of the same pass on all host threads over a bounded sample
    (64 x 64, 2 iterations)."""
    import numpy as np
    import torch
    import oracle
    from gpugi_gb300 import bvh, cuda, render, scenes
    W = H = 512
    spp, depth, rr = 16, 8, 3
    ctx = cuda.Context(0)
    sc = scenes.cornell_room(seed=1)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", normals=sc["normals"])
    ds = ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]), sc["materials"])
    ds.set_hierarchy_ndf(b.sggx)
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    stream = torch.cuda.ExternalStream(ctx.stream)
    out = {}
    for pass_ in (args.passes.split(",") if args.passes else ("PT", "LT", "BPT", "WHITTED", "PM", "IM", "HIERARCHY")):
        hier = pass_ == "HIERARCHY"
        d = 4 if hier else depth
        img = render.Image(ctx, W, H)
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        render.render(ctx, ds, cam, img, pass_, max_path_length=d, samples=1, rr_start_depth=rr, rng_state=[1])
        e1.record(stream)
        e1.synchronize()
        first = e0.elapsed_time(e1)
        e0.record(stream)
        render.render(ctx, ds, cam, img, pass_, max_path_length=d, samples=spp, iteration=1, rr_start_depth=rr,
                      rng_state=[2])
        e1.record(stream)
        e1.synchronize()
        sec = e0.elapsed_time(e1) / 1e3
        closest, anyhit = render.ray_counts(ctx)
        img.close()
        # CPU restatement, bounded sample
        cw = ch = 64
        ccam = render.camera_lookat(*scenes.CORNELL_CAMERA, cw, ch)
        nls = render.DEFAULT_LIGHT_SAMPLES[pass_]
        st = [3]
        t0 = time.perf_counter()
        acc = None
        gbuf = np.zeros((ch, cw, 5), np.float32) if pass_ == "IM" else None  # the importon pass's G-buffer
        if hier:
            ls0 = render.generate_light_samples(ds, st, nls)
            imp, _ = oracle.hier_importance(b, sc, cw, ch, ccam.as_array(), ls0, iterations=10)
            mats = oracle.hier_materials(b, sc)
        for it in range(2):
            ls = ls0 if (hier and it == 0) else render.generate_light_samples(ds, st, nls)
            if hier:
                acc = oracle.render_hier(b, sc, cw, ch, ccam.as_array(), render.frame_seed(it), ls, imp, mats, b.sggx,
                                         max_path_length=d, accum=acc)
            else:
                acc = oracle.render(b, sc, pass_, cw, ch, ccam.as_array(), render.frame_seed(it), ls,
                                    max_path_length=depth, rr_start_depth=rr, accum=acc, gbuffer=gbuf)
        cpu = time.perf_counter() - t0
        out[pass_] = {"samples_per_s": W * H * spp / sec, "ms_per_iteration": sec / spp * 1e3,
                      "cpu_samples_per_s": cw * ch * 2 / cpu, "cpu_threads": os.cpu_count()}
        if hier:  # megakernel: no device ray counters; the warm-up iteration holds the importance pass
            out[pass_].update({"path_length": d, "first_iteration_ms": first})
        else:
            out[pass_].update({"mrays_per_s": (closest + anyhit) / sec / 1e6, "closest_rays": closest,
                               "any_hit_rays": anyhit})
    line = {"metric": "samples/s and Mrays/s per pass", "config": {
        "workload": "Cornell room ~98k tris, 512x512, 16 spp, depth 8, RR after depth 3", "parallelism": "single GPU"},
        "passes": out, "data": "synthetic", "dtype": "f32",
        "cpu_sample": "64x64, 2 iterations of the same pass on all host threads"}
    print(json.dumps(line), flush=True)
    ds.close()
    ctx.close()


def run_large(args):
    """Large workload: ~7.9M triangles (20k instances of displaced icospheres
    and boxes in a 100^3 volume), 64 materials (Lambertian / Phong exponent
    U[10, 1000]), 256 small area lights (radiance log-uniform [1, 100]),
    ellipsoid-bounded sweep hierarchy. Reports (1) closest-hit ray queries on
    2^22 rays (origins uniform in the volume, directions uniform), with the
    algorithmic-byte roofline fraction: the scene (~0.5 GB) exceeds L2;
    (2) BPT and PT at 1920 x 1080, 8 spp, depth 6: samples/s and Mrays/s."""
    import torch
    from gpugi_gb300 import bvh, cuda, render, scenes
    hbm, peak_src = peaks()
    ctx = cuda.Context(0)
    t0 = time.perf_counter()
    sc = scenes.large_instanced(seed=1)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", fit="ellipsoid")
    t_build = time.perf_counter() - t0
    ds = ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]), sc["materials"])
    stream = torch.cuda.ExternalStream(ctx.stream)

    def ev_time(fn, reps=1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    # (1) ray queries
    n = 1 << 22
    g = torch.Generator(device="cuda").manual_seed(5)
    o = torch.rand((3, n), device="cuda", generator=g) * 100.0
    d = torch.randn((3, n), device="cuda", generator=g)
    d /= d.norm(dim=0, keepdim=True)
    rays = {"ox": o[0].contiguous(), "oy": o[1].contiguous(), "oz": o[2].contiguous(), "dx": d[0].contiguous(),
            "dy": d[1].contiguous(), "dz": d[2].contiguous(), "tmax": torch.full((n,), 3.402823466e38, device="cuda")}
    out = dict(slot=torch.empty(n, dtype=torch.int32, device="cuda"), t=torch.empty(n, device="cuda"),
               u=torch.empty(n, device="cuda"), v=torch.empty(n, device="cuda"))
    torch.cuda.synchronize()
    cuda.trace_closest_device(ctx, ds, rays, out)
    ctx.sync()
    sec = ev_time(lambda: cuda.trace_closest_device(ctx, ds, rays, out), reps=5)
    sums = cuda.trace_stats_device(ctx, ds, rays)
    alg = cuda.algorithmic_bytes(sums, n)
    queries = {"mrays_per_s": n / sec / 1e6, "ms_per_launch": sec * 1e3, "rays": n,
               "roofline": {"bound": "hbm", "achieved": alg / sec / 1e9, "peak": hbm, "unit": "GB/s",
                            "frac": alg / sec / 1e9 / hbm, "peak_source": peak_src, "alg_bytes_per_launch": alg},
               "hit_fraction": float((out["slot"] >= 0).float().mean().item())}
    # (2) passes
    W, H, spp, depth = 1920, 1080, 8, 6
    cam = render.camera_lookat(*scenes.LARGE_CAMERA, W, H)
    passes = {}
    for pass_ in ("BPT", "PT"):
        img = render.Image(ctx, W, H)
        render.render(ctx, ds, cam, img, pass_, max_path_length=depth, samples=1, rng_state=[1])
        ctx.sync()
        sec = ev_time(lambda: render.render(ctx, ds, cam, img, pass_, max_path_length=depth, samples=spp,
                                            iteration=1, rng_state=[2]))
        closest, anyhit = render.ray_counts(ctx)
        passes[pass_] = {"samples_per_s": W * H * spp / sec, "mrays_per_s": (closest + anyhit) / sec / 1e6,
                         "s_per_frame_8spp": sec, "mean": float(img.read()[..., :3].mean() / spp)}
        img.close()
    line = {"metric": "large scene: closest-hit Mrays/s and BPT/PT samples/s", "queries": queries, "passes": passes,
            "config": {"workload": "~7.9M tris (20k instances, 100^3), 64 materials, 256 area lights, ellipsoid BVH; "
                                   "queries 2^22 random rays; passes 1920x1080 8 spp depth 6",
                       "triangles": int(sc["triangles"].shape[0]), "nodes": int(b.num_nodes),
                       "build_s": round(t_build, 1)}, "data": "synthetic", "dtype": "f32"}
    print(json.dumps(line), flush=True)
    ds.close()
    ctx.close()


def run_build(args):
    """Hierarchy build on the GPU (gpugi_scene_build, linear BVH) against the
    host build (bvhmake sweep SAH, then gpugi_scene_upload), on the large
    workload's ~7.9M triangles (AABB nodes) and on the 65,536-triangle
    icosphere of the headline. Build: wall time from host arrays to a
    traversable scene (after one untimed GPU build). Traversal: closest-hit
    Mrays/s on each tree (large: 2^22 random rays inside the volume;
    icosphere: the headline's 2^20 rays), CUDA events; the host LDS tree
    (bvhmake's largest-dimension split) traversed beside them."""
    import torch
    from gpugi_gb300 import bvh, cuda, scenes
    ctx = cuda.Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream)

    def ev_time(fn, reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        fn()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    def to_dev(r):
        return {k: torch.from_numpy(np.ascontiguousarray(r[k])).cuda() for k in cuda.RAY_KEYS}

    out = {}
    big = scenes.large_instanced(seed=1)
    n = 1 << 22
    g = torch.Generator(device="cuda").manual_seed(5)
    o = torch.rand((3, n), device="cuda", generator=g) * 100.0
    d = torch.randn((3, n), device="cuda", generator=g)
    d /= d.norm(dim=0, keepdim=True)
    big_rays = {"ox": o[0].contiguous(), "oy": o[1].contiguous(), "oz": o[2].contiguous(), "dx": d[0].contiguous(),
                "dy": d[1].contiguous(), "dz": d[2].contiguous(),
                "tmax": torch.full((n,), 3.402823466e38, device="cuda")}
    ico, _, batches = make_workload()
    ico_rays = to_dev(batches[0])
    for name, sc, rays in (("large", big, big_rays), ("icosphere", ico, ico_rays)):
        m = rays["ox"].numel()
        res = {"triangles": int(sc["triangles"].shape[0]), "rays": m}
        t0 = time.perf_counter()
        hb = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
        host = ctx.upload_scene(hb, sc["positions"])
        res["host_build_s"] = time.perf_counter() - t0
        ctx.build_scene(sc["positions"], sc["triangles"]).close()
        ctx.sync()
        t0 = time.perf_counter()
        gpu = ctx.build_scene(sc["positions"], sc["triangles"])
        res["gpu_build_s"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        lb = bvh.build_bvh(sc["positions"], sc["triangles"], method="lds")
        res["host_lds_build_s"] = time.perf_counter() - t0
        lds = ctx.upload_scene(lb, sc["positions"])
        res["nodes"] = {"host_sweep": host.num_nodes, "host_lds": lds.num_nodes, "gpu_lbvh": gpu.num_nodes}
        outs = dict(slot=torch.empty(m, dtype=torch.int32, device="cuda"), t=torch.empty(m, device="cuda"),
                    u=torch.empty(m, device="cuda"), v=torch.empty(m, device="cuda"))
        torch.cuda.synchronize()
        for key, ds in (("host_sweep", host), ("host_lds", lds), ("gpu_lbvh", gpu)):
            sec = ev_time(lambda: cuda.trace_closest_device(ctx, ds, rays, outs), 5)
            res[f"{key}_mrays_per_s"] = m / sec / 1e6
        out[name] = res
        for x in (host, lds, gpu):
            x.close()
    line = {"metric": "hierarchy build time, GPU linear BVH vs host sweep SAH", "unit": "s", "results": out,
            "config": {"workload": "large: ~7.9M tris (20k instances in 100^3); icosphere: 65,536 tris (headline)",
                       "leaf_size": 8, "bounds": "AABB"}, "data": "synthetic", "dtype": "f32"}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_batch(args):
    """Batched rendering workload: 8 scenes of instanced icospheres, boxes and
    tori (triangle counts log-uniform in [10k, 2M]), each with a random
    resolution in {256^2, 512^2, 768^2, 1024^2} and spp in {4, 16, 64}, PT,
    LT and BPT at depth 8 (24 jobs). One gpugi_render_batch call (all 24 jobs
    in one two-phase wavefront replayed as a CUDA graph per round) against
    the same jobs as 24 gpugi_render calls; also each pass's 8 jobs alone,
    and 64 small mixed jobs. Wall time of synchronised calls; samples =
    pixels x spp summed over jobs."""
    from gpugi_gb300 import bvh, cuda, render, scenes
    rs = scenes.Stream(args.batch_seed, 23)
    ctx = cuda.Context(0)
    tris = np.exp(rs.uniform(8, math.log(1e4), math.log(2e6)))
    res = [256, 512, 768, 1024]
    spps = [4, 16, 64]
    specs, dss = [], []
    for k in range(8):
        sc = scenes.instanced_scene(seed=100 + k, num_triangles=int(tris[k]))
        b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
        ds = ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]), sc["materials"])
        dss.append(ds)
        r = res[int(rs.u64(1)[0] % 4)]
        spp = spps[int(rs.u64(1)[0] % 3)]
        cam = render.camera_lookat((0.0, 1.0, 7.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 45.0, r, r)
        specs.append((ds, cam, r, spp, sc["triangles"].shape[0]))

    def make_jobs(passes=("PT", "LT", "BPT")):
        jobs = []
        for k, (ds, cam, r, spp, _) in enumerate(specs):
            for pass_ in passes:
                jobs.append(dict(scene=ds, camera=cam, image=render.Image(ctx, r, r), pass_=pass_, samples=spp,
                                 max_path_length=8, rng_state=[1000 + k]))
        return jobs

    def timed(fn):
        ctx.sync()
        t0 = time.perf_counter()
        fn()
        ctx.sync()
        return time.perf_counter() - t0

    def run_single(jobs):
        for j in jobs:
            render.render(ctx, j["scene"], j["camera"], j["image"], j["pass_"], max_path_length=j["max_path_length"],
                          samples=j["samples"], rng_state=j["rng_state"])

    def samples(jobs):
        return sum(j["image"].width * j["image"].height * j["samples"] for j in jobs)

    def measure(fn, make):
        warm = make()
        fn(warm)  # buffers, graph capture
        for j in warm:
            j["image"].close()
        jobs = make()
        t = timed(lambda: fn(jobs))
        for j in jobs:
            j["image"].close()
        return t, samples(jobs)

    result = {}
    for name, fn in (("batch", lambda js: render.render_batch(ctx, js)), ("single", run_single)):
        t, n = measure(fn, make_jobs)
        result[name] = {"all_s": round(t, 4), "all_samples_per_s": n / t}
        if name == "batch":  # rays the batched walkers traced (device counters of the call)
            closest, anyhit = render.ray_counts(ctx)
            result[name].update({"closest_rays": closest, "any_hit_rays": anyhit,
                                 "mrays_per_s": (closest + anyhit) / t / 1e6})
        for pass_ in ("PT", "LT", "BPT"):
            t, n = measure(fn, lambda: make_jobs((pass_,)))
            result[name][pass_ + "_s"] = round(t, 4)
            result[name][pass_ + "_samples_per_s"] = n / t
    # many small jobs: 64 jobs of 128 x 128 at 4 spp over the same 8 scenes, PT / LT / BPT in turn
    def small_jobs():
        return [dict(scene=specs[k % 8][0], camera=render.camera_lookat((0.0, 1.0, 7.0), (0.0, 0.0, 0.0),
                                                                        (0.0, 1.0, 0.0), 45.0, 128, 128),
                     image=render.Image(ctx, 128, 128), pass_=("PT", "LT", "BPT")[k % 3], samples=4,
                     max_path_length=8, rng_state=[2000 + k]) for k in range(64)]
    small = {}
    for name, fn in (("batch", lambda js: render.render_batch(ctx, js)), ("single", run_single)):
        t, n = measure(fn, small_jobs)
        small[name] = {"s": round(t, 5), "samples_per_s": n / t}
    result["small_jobs_64x128x128x4spp_mixed"] = small
    line = {"metric": "samples/s, 24 jobs of 8 scenes: batched vs one call per job",
            "value": result["batch"]["all_samples_per_s"], "unit": "samples/s", "higher_is_better": True,
            "speedup_batched": result["single"]["all_s"] / result["batch"]["all_s"],
            "small_jobs_speedup_batched": small["single"]["s"] / small["batch"]["s"], "runs": result,
            "config": {"workload": "8 instanced scenes, tris log-uniform [10k, 2M], res {256..1024}^2, "
                                   "spp {4,16,64}, PT+LT+BPT depth 8",
                       "scenes": [{"tris": t, "res": r, "spp": s_} for (_, _, r, s_, t) in specs],
                       "paths_per_round": 16 << 20},
            "data": "synthetic", "dtype": "f32"}
    print(json.dumps(line), flush=True)
    for ds in dss:
        ds.close()
    ctx.close()


def run_mlp(args):
    """The radiance cache's MLP kernels alone, both kernel sets (tcgen05 and
    the warp-level mma.sync one): a training step (forward, backward, weight
    gradients, Adam) on 65,536 samples and inference of 921,600 queries (the
    cache lookups of one 1280 x 720 frame). CUDA events on the library's
    stream around --steps queued calls after --warmup. Tensor work per
    sample: forward 2 x 17,408 flops; training adds the backward products of
    layers 4-1 (2 x 13,312) and the weight gradients (2 x 17,408); reported
    against the measured dense bf16 peak (f16 runs at the same rate)."""
    import torch
    from gpugi_gb300 import cuda, nrc
    ctx = cuda.Context(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    rng = np.random.default_rng(1)

    def queries(n):
        q = np.concatenate([rng.uniform(-1, 1, (n, 3)), rng.normal(size=(n, 3)), rng.normal(size=(n, 3)),
                            rng.uniform(0.1, 0.9, (n, 3))], 1).astype(np.float32)
        q[:, 3:6] /= np.linalg.norm(q[:, 3:6], axis=1, keepdims=True)
        q[:, 6:9] /= np.linalg.norm(q[:, 6:9], axis=1, keepdims=True)
        return q

    nt, ni = 65536, 921600
    qt = queries(nt)
    samples = torch.from_numpy(np.concatenate([qt, rng.uniform(0, 2, (nt, 3)).astype(np.float32)], 1)).to(dev)
    qi = torch.from_numpy(queries(ni)).to(dev)
    out = torch.empty((ni, 3), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    L = nrc._declare()
    peak = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["bf16_tflops"] if (ROOT / "MEASURED_PEAKS.json").exists() \
        else 1900.0
    res = {}
    for k in ("tcgen05", "mma_sync"):
        c = nrc.RadianceCache(ctx, (-1, -1, -1), (1, 1, 1), seed=3)
        c.set_kernels(k)

        def timed(fn):
            for _ in range(args.warmup):
                fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ctx.sync()
            e0.record(stream)
            for _ in range(args.steps):
                fn()
            e1.record(stream)
            e1.synchronize()
            return e0.elapsed_time(e1) / args.steps * 1e3  # us

        t_train = timed(lambda: ctx.check(L.gpugi_nrc_train_device(ctx.handle, c.handle, cuda._ptr(samples), nt,
                                                                   None)))
        t_inf = timed(lambda: ctx.check(L.gpugi_nrc_infer_device(ctx.handle, c.handle, cuda._ptr(qi), ni,
                                                                 cuda._ptr(out))))
        f_train = 2.0 * nt * (17408 + 13312 + 17408)
        f_inf = 2.0 * ni * 17408
        res[k] = {"train_step_us": round(t_train, 2), "train_tflops": round(f_train / t_train / 1e6, 2),
                  "train_frac_of_peak": round(f_train / t_train / 1e6 / peak, 4),
                  "infer_us": round(t_inf, 2), "infer_tflops": round(f_inf / t_inf / 1e6, 2),
                  "infer_frac_of_peak": round(f_inf / t_inf / 1e6 / peak, 4)}
        c.close()
    assert ctx.device_error_bits() == 0
    print(json.dumps({"metric": "radiance-cache MLP: us per training step (65,536 samples) and per inference of "
                                "921,600 queries", "results": res, "peak_tflops": peak,
                      "peak_source": "MEASURED_PEAKS.json bf16_tflops (dense)", "steps": args.steps,
                      "warmup": args.warmup, "data": "synthetic", "dtype": "f16 weights/activations, f32 accumulate"}),
          flush=True)
    ctx.close()


NRC_WORKLOAD_PT = "heightfield 512x512 fBm (amplitude 0.2) + 500 boxes, sun 5, sky 0.5, depth 8"


class NrcSetup:
    """Scene, camera and FP64 reference image of a time-to-equal-RMSE run.
    PT: the heightfield workload (522k-triangle fBm terrain + 500 boxes, sun
    of irradiance 5, sky 0.5, Lambertian albedos U[0.1, 0.8], depth 8). BPT:
    the large workload (~7.9M triangles in 20k instances, 64 Lambertian /
    Phong materials, 256 area lights, ellipsoid hierarchy, depth 6), with
    eye paths that stop at the cache vertex. The reference is the plain pass
    accumulated in FP64 over ref_spp samples; its noise adds the same
    variance to both renderers' MSE, so it cancels out of the equal-RMSE
    comparison."""

    def __init__(self, pass_, W, H, ref_spp, rr, unbiased=1.0 / 16, lanes=2):
        from gpugi_gb300 import bvh, cuda, render, scenes
        self.pass_, self.W, self.H, self.rr, self.ref_spp = pass_, W, H, rr, ref_spp
        self.unbiased, self.lanes = unbiased, lanes
        self.ctx = cuda.Context(0)
        if pass_ == "PT":
            self.depth, self.sky = 8, (0.5, 0.5, 0.5)
            sc = scenes.heightfield_boxes(seed=1)
            b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
            self.box = ((-1.05, -0.25, -1.05), (1.05, 0.35, 1.05))
            cam_args = scenes.HEIGHTFIELD_CAMERA
            self.workload = NRC_WORKLOAD_PT
        else:
            self.depth, self.sky = 6, (0.0, 0.0, 0.0)
            sc = scenes.large_instanced(seed=1)
            b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", fit="ellipsoid")
            self.box = ((-3.0, -3.0, -3.0), (103.0, 103.0, 103.0))
            cam_args = scenes.LARGE_CAMERA
            self.workload = ("~7.9M tris (20k instances in 100^3), 64 Lambertian/Phong materials, 256 area lights, "
                             "ellipsoid BVH, depth 6")
        self.ds = self.ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]),
                                        sc["materials"])
        if pass_ == "PT":
            render.add_directional_light(self.ds, scenes.HEIGHTFIELD_SUN, (5.0, 5.0, 5.0))
        self.cam = render.camera_lookat(*cam_args, W, H)
        conv = render.Image(self.ctx, W, H, fp64=True)
        self.t_ref = self.timed(lambda: render.render(self.ctx, self.ds, self.cam, conv, pass_,
                                                      max_path_length=self.depth, samples=ref_spp,
                                                      iteration=1 << 24, rng_state=[99], sky=self.sky,
                                                      rr_start_depth=rr))
        self.ref = (conv.read64() / ref_spp).astype(np.float32)
        conv.close()

    def timed(self, fn):
        """Host clock around a synchronised call (the renderers queue work on
        the library's stream; both sides synchronise)."""
        self.ctx.sync()
        t0 = time.perf_counter()
        fn()
        self.ctx.sync()
        return time.perf_counter() - t0

    def rmse(self, img, n):
        return float(np.sqrt(img.mse(n, self.ref, use_fp64=True)))

    def plain(self, spp=1024):
        """The plain pass to spp samples in doubling chunks: (time, final
        RMSE = the target, curve of (spp, s, RMSE))."""
        from gpugi_gb300 import render
        pt = render.Image(self.ctx, self.W, self.H, fp64=True)
        t, n, curve = 0.0, 0, []
        chunks = [1, 1] + [1 << k for k in range(1, 20) if (1 << k) < spp]
        for c in chunks:
            c = min(c, spp - n)
            if c <= 0:
                break
            t += self.timed(lambda: render.render(self.ctx, self.ds, self.cam, pt, self.pass_,
                                                  max_path_length=self.depth, samples=c, iteration=n,
                                                  rng_state=[7 + n], sky=self.sky, rr_start_depth=self.rr))
            n += c
            curve.append((n, round(t, 5), round(self.rmse(pt, n), 6)))
        pt.close()
        return t, curve[-1][2], curve

    def cache_run(self, t_pt, target, td, spf, steps, tl, spread, warmup, train_fraction=0.0, limit=3.0,
                  at_frames=64):
        """The cache renderer from a fresh network: `warmup` frames train
        (timed, not accumulated), then frames accumulate until the RMSE
        reaches the target or the time exceeds limit x t_pt."""
        from gpugi_gb300 import nrc, render
        W, H = self.W, self.H
        # training paths: about 1.5 x 65,536 vertices per frame (3 per path)
        tf = train_fraction or min(0.05, 1.5 * 65536 / (3.0 * W * H * spf))
        cache = nrc.RadianceCache(self.ctx, *self.box, seed=5)
        opts = dict(max_path_length=self.depth, sky=self.sky, terminate_depth=td, train_fraction=tf,
                    train_steps=steps, samples_per_frame=spf, rr_start_depth=self.rr, pass_=self.pass_,
                    train_length=tl, terminate_spread=spread, unbiased_fraction=self.unbiased, lanes=self.lanes)
        t_nrc = 0.0
        if warmup:
            scratch = render.Image(self.ctx, W, H)
            t_nrc = self.timed(lambda: nrc.render_nrc(self.ctx, self.ds, self.cam, scratch, cache,
                                                      samples=warmup * spf, iteration=1 << 20, rng_state=[11],
                                                      **opts))
            scratch.close()
        t_warm = t_nrc
        img = render.Image(self.ctx, W, H, fp64=True)
        frames, curve, reached, at_equal_time, at_n, chunk = 0, [], None, None, None, 1
        while t_nrc < limit * t_pt and frames * spf < 8192:
            t_nrc += self.timed(lambda: nrc.render_nrc(self.ctx, self.ds, self.cam, img, cache,
                                                       samples=chunk * spf, iteration=frames * spf,
                                                       rng_state=[13 + frames], **opts))
            frames += chunk
            r = self.rmse(img, frames * spf)
            curve.append((frames * spf, round(t_nrc, 5), round(r, 6)))
            if at_equal_time is None and t_nrc >= t_pt:
                at_equal_time = r
            if at_n is None and frames >= at_frames:
                at_n = {"frames": frames, "s": round(t_nrc, 5), "rmse": round(r, 6)}
            if r <= target:
                reached = t_nrc
                break
            chunk = min(chunk * 2, max(1, 64 // spf), max(1, at_frames - frames) if at_n is None else 1 << 30)
        img.close()
        cache.close()
        return {"value": (reached / t_pt) if reached else None, "t_nrc_s": round(reached, 4) if reached else None,
                "t_nrc_warmup_s": round(t_warm, 4), "nrc_rmse_at_equal_time": at_equal_time,
                f"after_{at_frames}_frames": at_n,
                "nrc": {"terminate_depth": td, "train_fraction": round(tf, 5), "train_steps": steps,
                        "train_length": tl, "unbiased_fraction": self.unbiased if tl else None,
                        "terminate_spread": spread, "samples_per_frame": spf, "warmup_frames": warmup,
                        "lanes": self.lanes,
                        "max_train_samples": 65536, "ema": 0.99,
                        "mlp": "64-64x4-3 ReLU fp16, fp32 accumulate, Adam lr 1e-2"},
                "nrc_curve": curve}

    def fixed_budget(self, spp, td, spf, steps, tl, spread, warmup, train_fraction=0.0):
        """The cache renderer at a fixed sample budget (after `warmup`
        training frames, timed) against the plain pass run until it reaches
        the same RMSE: (plain time to the cache's RMSE) / (cache time)."""
        from gpugi_gb300 import nrc, render
        W, H = self.W, self.H
        tf = train_fraction or min(0.05, 1.5 * 65536 / (3.0 * W * H * spf))
        cache = nrc.RadianceCache(self.ctx, *self.box, seed=5)
        opts = dict(max_path_length=self.depth, sky=self.sky, terminate_depth=td, train_fraction=tf,
                    train_steps=steps, samples_per_frame=spf, rr_start_depth=self.rr, pass_=self.pass_,
                    train_length=tl, terminate_spread=spread, unbiased_fraction=self.unbiased, lanes=self.lanes)
        t_nrc = 0.0
        if warmup:
            scratch = render.Image(self.ctx, W, H)
            t_nrc = self.timed(lambda: nrc.render_nrc(self.ctx, self.ds, self.cam, scratch, cache,
                                                      samples=warmup * spf, iteration=1 << 20, rng_state=[11],
                                                      **opts))
            scratch.close()
        img = render.Image(self.ctx, W, H, fp64=True)
        t_nrc += self.timed(lambda: nrc.render_nrc(self.ctx, self.ds, self.cam, img, cache, samples=spp,
                                                   iteration=0, rng_state=[13], **opts))
        r_nrc = self.rmse(img, spp)
        img.close()
        cache.close()
        pt = render.Image(self.ctx, W, H, fp64=True)
        t, n, curve, reached, at_equal_time = 0.0, 0, [], None, None
        c = 1
        while n < 64 * spp and reached is None:
            t += self.timed(lambda: render.render(self.ctx, self.ds, self.cam, pt, self.pass_,
                                                  max_path_length=self.depth, samples=c, iteration=n,
                                                  rng_state=[7 + n], sky=self.sky, rr_start_depth=self.rr))
            n += c
            r = self.rmse(pt, n)
            curve.append((n, round(t, 5), round(r, 6)))
            if at_equal_time is None and t >= t_nrc:
                at_equal_time = r
            if r <= r_nrc:
                reached = t
            c = n  # doubling
        pt.close()
        return {"value": (reached / t_nrc) if reached else None, "unit": "speed-up (plain time to the cache's RMSE / cache time)",
                "nrc_spp": spp, "t_nrc_s": round(t_nrc, 4), "nrc_rmse": round(r_nrc, 6),
                "t_plain_to_equal_rmse_s": round(reached, 4) if reached else None,
                "plain_rmse_at_equal_time": at_equal_time, "plain_curve": curve,
                "nrc": {"terminate_depth": td, "train_fraction": round(tf, 5), "train_steps": steps,
                        "train_length": tl, "terminate_spread": spread, "samples_per_frame": spf,
                        "warmup_frames": warmup}}

    def close(self):
        self.ds.close()
        self.ctx.close()


def nrc_headline(args):
    """The second headline, time to equal RMSE of the radiance cache against
    plain PT on the heightfield workload at 1280 x 720, as the workload
    states it: 1 spp per frame, 65,536 training samples per frame, ratio =
    (cache time to the plain tracer's 1024-spp RMSE) / (plain time to 1024
    spp); null when the cache does not get there within 3x the plain
    time."""
    st = NrcSetup("PT", 1280, 720, args.nrc_ref_spp, args.nrc_rr, args.nrc_unbiased, args.nrc_lanes)
    try:
        t_pt, target, pt_curve = st.plain(1024)
        r = st.cache_run(t_pt, target, args.nrc_td, 1, args.nrc_train_steps, args.nrc_train_length,
                         args.nrc_spread, args.nrc_warmup)
        plain_at_64 = next(c for c in pt_curve if c[0] >= 64)
        out = {"metric": "time to the 1024-spp plain-PT RMSE, PT with the radiance cache / plain PT",
               "unit": "ratio", "higher_is_better": False, "value": r.pop("value"),
               "t_pt_s": round(t_pt, 4), "target_rmse": target, "plain_pt_at_64_spp": plain_at_64}
        out.update(r)
        out["config"] = {"workload": st.workload, "resolution": [1280, 720], "reference_spp": st.ref_spp,
                         "reference_s": round(st.t_ref, 2), "rr_start_depth": st.rr,
                         "timing": "host clock around synchronised calls"}
        out["pt_curve"] = pt_curve
        return out
    finally:
        st.close()


def run_nrc_frames(args):
    """Cache frames alone on the heightfield workload (1280 x 720, 1 spp per
    frame, the cache settings of the `nrc` options): --warmup frames, then
    --steps frames in one call, beside plain PT of --steps spp in one call
    and in 1-spp calls; ms per frame / spp, host clock around synchronised
    calls. For launch lists and per-frame costs."""
    from gpugi_gb300 import nrc, render
    st = NrcSetup("PT", 1280, 720, 1, args.nrc_rr, args.nrc_unbiased, args.nrc_lanes)
    tf = min(0.05, 1.5 * 65536 / (3.0 * 1280 * 720))
    cache = nrc.RadianceCache(st.ctx, *st.box, seed=5)
    img = render.Image(st.ctx, 1280, 720, fp64=True)
    opts = dict(max_path_length=st.depth, sky=st.sky, terminate_depth=args.nrc_td, train_fraction=tf,
                train_steps=args.nrc_train_steps, samples_per_frame=1, train_length=args.nrc_train_length,
                terminate_spread=args.nrc_spread, unbiased_fraction=args.nrc_unbiased, lanes=args.nrc_lanes)
    nrc.render_nrc(st.ctx, st.ds, st.cam, img, cache, samples=max(args.warmup, 1), iteration=0, rng_state=[1],
                   **opts)
    t_frames = st.timed(lambda: nrc.render_nrc(st.ctx, st.ds, st.cam, img, cache, samples=args.steps,
                                               iteration=1000, rng_state=[2], **opts))
    pt = render.Image(st.ctx, 1280, 720, fp64=True)
    render.render(st.ctx, st.ds, st.cam, pt, "PT", max_path_length=st.depth, samples=max(args.warmup, 1),
                  iteration=0, rng_state=[3], sky=st.sky)
    t_pt = st.timed(lambda: render.render(st.ctx, st.ds, st.cam, pt, "PT", max_path_length=st.depth,
                                          samples=args.steps, iteration=100, rng_state=[4], sky=st.sky))

    def single():
        for k in range(args.steps):
            render.render(st.ctx, st.ds, st.cam, pt, "PT", max_path_length=st.depth, samples=1,
                          iteration=10000 + k, rng_state=[5 + k], sky=st.sky)
    t_pt1 = st.timed(single)
    print(json.dumps({"metric": "ms per 1-spp cache frame and per plain PT sample, heightfield 1280 x 720",
                      "nrc_ms_per_frame": round(t_frames / args.steps * 1e3, 4),
                      "pt_ms_per_spp_one_call": round(t_pt / args.steps * 1e3, 4),
                      "pt_ms_per_spp_one_spp_calls": round(t_pt1 / args.steps * 1e3, 4),
                      "frames": args.steps, "warmup": args.warmup,
                      "nrc": {"terminate_depth": args.nrc_td, "train_steps": args.nrc_train_steps,
                              "train_length": args.nrc_train_length, "lanes": args.nrc_lanes},
                      "data": "synthetic"}), flush=True)
    for x in (img, pt, cache):
        x.close()
    st.close()


def run_nrc(args):
    """Time to equal RMSE, rendering with the radiance cache vs the plain
    renderer of the same pass (NrcSetup): the plain pass accumulates 1024
    spp (doubling chunks); its final RMSE is the target and its wall time
    T_plain. Each cache setting (--nrc-configs) first trains for
    --nrc-warmup frames (timed, not accumulated), then accumulates frames
    until its RMSE reaches the target or its time exceeds 3 T_plain."""
    pass_ = args.nrc_pass
    W, H = args.nrc_size if args.nrc_size else ((640, 360) if pass_ == "PT" else (480, 270))
    st = NrcSetup(pass_, W, H, args.nrc_ref_spp, args.nrc_rr, args.nrc_unbiased, args.nrc_lanes)

    def parse(c):
        v = [float(x) for x in c.split(",")]
        v += [args.nrc_train_length, args.nrc_spread][len(v) - 3:] if len(v) < 5 else []
        return int(v[0]), int(v[1]), int(v[2]), int(v[3]), v[4]

    configs = [parse(c) for c in args.nrc_configs.split(";")] if args.nrc_configs else \
        [(args.nrc_td, args.nrc_spf, args.nrc_train_steps, args.nrc_train_length, args.nrc_spread)]
    if args.nrc_budget:
        for td, spf, steps, tl, spread in configs:
            r = st.fixed_budget(args.nrc_budget, td, spf, steps, tl, spread, args.nrc_warmup,
                                train_fraction=args.nrc_train_fraction)
            line = {"metric": f"{pass_} with the radiance cache at {args.nrc_budget} spp vs plain {pass_} at equal RMSE",
                    "higher_is_better": True}
            line.update(r)
            line["config"] = {"workload": st.workload, "pass": pass_, "rr_start_depth": st.rr, "resolution": [W, H],
                              "reference_spp": st.ref_spp, "reference_s": round(st.t_ref, 2), "nrc": line.pop("nrc")}
            line.update({"data": "synthetic", "dtype": "f32 paths, f16 MLP"})
            print(json.dumps(line), flush=True)
        st.close()
        return
    t_pt, target, pt_curve = st.plain(1024)
    for td, spf, steps, tl, spread in configs:
        r = st.cache_run(t_pt, target, td, spf, steps, tl, spread, args.nrc_warmup,
                         train_fraction=args.nrc_train_fraction)
        line = {"metric": f"time to the 1024-spp plain-{pass_} RMSE, {pass_} with the radiance cache vs plain {pass_}",
                "unit": "ratio", "value": r.pop("value"), "higher_is_better": False,
                "t_pt_s": round(t_pt, 4), "target_rmse": target}
        line.update(r)
        line["config"] = {"workload": st.workload, "pass": pass_, "rr_start_depth": st.rr, "resolution": [W, H],
                          "reference_spp": st.ref_spp, "reference_s": round(st.t_ref, 2), "nrc": line.pop("nrc")}
        line.update({"pt_curve": pt_curve, "data": "synthetic", "dtype": "f32 paths, f16 MLP"})
        print(json.dumps(line), flush=True)
    st.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-nrc", action="store_true",
                    help="leave out the radiance-cache time-to-equal-RMSE key of the default line")
    ap.add_argument("--passes", default=None,
                    help="passes workload: comma-separated subset of PT,LT,BPT,WHITTED,PM,IM,HIERARCHY")
    ap.add_argument("--shared-nodes", type=int, default=0,
                    help="top-of-tree nodes staged in shared memory by the walkers")
    ap.add_argument("--streams", type=int, default=4,
                    help="caller streams the headline steps alternate over (1 = no overlap)")
    ap.add_argument("--walker-share", type=int, default=50,
                    help="percent of the persistent walker grid a stream-ordered device-array query launches")
    ap.add_argument("--e2e-streams", type=int, default=3,
                    help="streams the end-to-end host-buffer steps alternate over")
    ap.add_argument("--trace-mode", type=int, default=3,
                    help="0: thread per ray, 1: persistent lane refill, 2: root prefilter + persistent, "
                         "3/4/5: root prefilter + 8/4/16-lane group walker")
    ap.add_argument("--batch-seed", type=int, default=1)
    ap.add_argument("--host-parts", type=int, default=2,
                    help="parts of a host-pointer query whose copies and traversal overlap")
    ap.add_argument("--zero-copy", action="store_true",
                    help="kernels read and write the page-locked host arrays directly instead of staging")
    ap.add_argument("--workload", choices=["trace", "nrc", "passes", "batch", "large", "build", "mlp", "nrc-frames"], default="trace",
                    help="trace: the closest-hit headline; nrc: time-to-equal-RMSE of the radiance cache; "
                         "passes: samples/s and Mrays/s of PT, LT and BPT; batch: batched vs per-job rendering; "
                         "large: the 7.9M-triangle workload; build: GPU vs host hierarchy build; "
                         "mlp: the radiance-cache MLP kernels alone; nrc-frames: 1-spp cache frames alone")
    ap.add_argument("--nrc-pass", choices=["PT", "BPT"], default="PT",
                    help="PT: heightfield workload; BPT: large workload (eye paths stop at the cache vertex)")
    ap.add_argument("--nrc-size", type=int, nargs=2, default=None, help="default 640 360 (PT), 480 270 (BPT)")
    ap.add_argument("--nrc-ref-spp", type=int, default=8192)
    ap.add_argument("--nrc-spf", type=int, default=16, help="samples per cache frame")
    ap.add_argument("--nrc-warmup", type=int, default=32, help="training frames before accumulation")
    ap.add_argument("--nrc-train-fraction", type=float, default=0.0,
                    help="share of training paths (0: about 98k training vertices per frame)")
    ap.add_argument("--nrc-configs", default="",
                    help="'td,spf,steps[,train_length[,spread]];...' several cache settings in one run")
    ap.add_argument("--nrc-train-steps", type=int, default=2)
    ap.add_argument("--nrc-train-length", type=int, default=3,
                    help="self-training: training paths take the cache's radiance at this vertex (0: off)")
    ap.add_argument("--nrc-spread", type=float, default=0.0,
                    help="path-spread termination constant c (0: stop at --nrc-td)")
    ap.add_argument("--nrc-td", type=int, default=3, help="path vertex where render paths query the cache")
    ap.add_argument("--nrc-unbiased", type=float, default=1.0 / 16,
                    help="self-training: share of training paths that run to their end")
    ap.add_argument("--nrc-lanes", type=int, default=4, help="cache frames in flight (wavefront lanes)")
    ap.add_argument("--nrc-budget", type=int, default=0,
                    help="cache renderer at this many spp against the plain pass at equal RMSE (0: time to the "
                         "plain 1024-spp RMSE)")
    ap.add_argument("--nrc-rr", type=int, default=0, help="Russian roulette start depth of both tracers")
    args = ap.parse_args()
    if args.workload != "trace":
        from __graft_entry__ import build
        build()
        {"nrc": run_nrc, "passes": run_passes, "batch": run_batch, "large": run_large,
         "build": run_build, "mlp": run_mlp, "nrc-frames": run_nrc_frames}[args.workload](args)
        return
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        from __graft_entry__ import build
        if rank == 0:
            build()
        barrier(world)
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
