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


def make_workload():
    from gpugi_gb300 import bvh, scenes
    sc = scenes.displaced_icosphere(65536, seed=1)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", leaf_size=8)
    batches = [scenes.random_rays(N_RAYS, seed=100 + k) for k in range(N_BATCHES)]
    return sc, b, batches


def cpu_baseline(b, positions, batches, seconds=10.0, threads=None):
    """The oracle (C++ restatement of the shaders) on the host cores, over a
    bounded sample of the same workload: whole 2^20-ray batches until
    `seconds` of wall time have passed."""
    import oracle
    nthreads = threads or os.cpu_count() or 1
    oracle.trace_closest(b, positions, batches[0], num_threads=nthreads)  # warm-up, builds the library
    rays = 0
    t0 = time.perf_counter()
    k = 0
    while True:
        oracle.trace_closest(b, positions, batches[k % len(batches)], num_threads=nthreads)
        rays += N_RAYS
        k += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return {"value": rays / el / 1e6, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{k} batches of 2^20 rays of this workload ({rays} rays, {el:.1f} s wall) on {nthreads} threads"}


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
    import oracle
    for k in range(args.warmup):
        oracle.trace_closest(b, sc["positions"], batches[k % N_BATCHES], num_threads=nthreads)
    t0 = time.perf_counter()
    for k in range(args.steps):
        oracle.trace_closest(b, sc["positions"], batches[k % N_BATCHES], num_threads=nthreads)
    el = time.perf_counter() - t0
    value = args.steps * N_RAYS / el / 1e6
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "parallelism": "host threads"}, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": f"{args.steps} steps x 2^20 rays on {nthreads} threads (the reference's "
                                       "GLSL path cannot run on this box: no OpenGL; the oracle restatement "
                                       "of its shaders stands in)"},
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

    for k in range(args.warmup):
        cuda.trace_closest_device(ctx, ds, batches[k % N_BATCHES], outs[k % N_BATCHES])
    ctx.sync()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        time.sleep(0.3)
        barrier(world)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                starts[k].record(stream)
                cuda.trace_closest_device(ctx, ds, batches[k % N_BATCHES], outs[k % N_BATCHES])
                ends[k].record(stream)
        ctx.sync()
        torch.cuda.synchronize()
        barrier(world)
    per_launch_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = starts[0].elapsed_time(ends[-1])
    total_ms = reduce_max(total_ms, world, dev)
    value = world * args.steps * N_RAYS / (total_ms / 1e3) / 1e6

    # End to end through the public C ABI with host buffers: every step copies
    # its rays from pinned host memory and its results back.
    pin = [{k: torch.from_numpy(rb[k]).pin_memory().numpy() for k in cuda.RAY_KEYS} for rb in host_batches[:2]]
    res = [dict(slot=torch.empty(N_RAYS, dtype=torch.int32).pin_memory().numpy(),
                t=torch.empty(N_RAYS).pin_memory().numpy(), u=torch.empty(N_RAYS).pin_memory().numpy(),
                v=torch.empty(N_RAYS).pin_memory().numpy()) for _ in range(2)]
    lib = cuda.lib()

    def e2e_step(k):
        r, o = pin[k % 2], res[k % 2]
        ctx.check(lib.gpugi_trace_closest(ctx.handle, ds.handle, *[cuda._ptr(r[key]) for key in cuda.RAY_KEYS],
                                          N_RAYS, cuda._ptr(o["slot"]), cuda._ptr(o["t"]), cuda._ptr(o["u"]),
                                          cuda._ptr(o["v"])))

    for k in range(args.warmup):
        e2e_step(k)
    barrier(world)
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_step(k)
    e2e_s = reduce_max(time.perf_counter() - t0, world, dev)
    e2e_value = world * args.steps * N_RAYS / e2e_s / 1e6
    assert (res[0]["slot"] >= -1).all()

    peak, peak_src = peaks()
    avg_launch_s = float(np.mean(per_launch_ms)) / 1e3
    achieved = alg_bytes / avg_launch_s / 1e9
    traffic = profile_traffic()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "l2": "inputs larger than L2: 8 rotating ray batches (8 x 44 MB rays+results)",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": N_RAYS * 28,
                    "d2h_bytes_per_step": N_RAYS * 16},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_source": f"{peak_src} hbm_gbs (MEASURED_PEAKS.json)" if peak_src == "measured"
                         else "fallback 6.8 TB/s",
                         "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": avg_launch_s * 1e3,
                         "kernel": KERNELS[args.trace_mode]},
            "gpu_launches": args.steps * (2 if args.trace_mode >= 2 else 1),
            "clocks": clk.summary()}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(b, sc["positions"], host_batches, seconds=args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ds.close()
    ctx.close()


def run_nrc(args):
    """Time to equal RMSE, path tracing with the radiance cache vs plain path
    tracing, on the heightfield workload (522k-triangle fBm terrain + 500
    boxes, sun of irradiance 5, sky 0.5, Lambertian albedos U[0.1, 0.8],
    depth 8). RMSE is TextureMSE's, in FP64, against an FP64-accumulated
    plain-PT image of --nrc-ref-spp samples. Plain PT accumulates 1024 spp
    (doubling chunks); its final RMSE is the target and its wall time T_pt.
    The cache path tracer first trains for --nrc-warmup frames (timed, not
    accumulated), then accumulates frames until its RMSE reaches the target
    or its time exceeds 3 T_pt. Wall times: host clock around synchronised
    calls (both renderers synchronise internally)."""
    from gpugi_gb300 import bvh, cuda, nrc, render, scenes
    W, H = args.nrc_size
    depth, sky = 8, (0.5, 0.5, 0.5)
    ctx = cuda.Context(0)
    sc = scenes.heightfield_boxes(seed=1)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]), sc["materials"])
    render.add_directional_light(ds, scenes.HEIGHTFIELD_SUN, (5.0, 5.0, 5.0))
    cam = render.camera_lookat(*scenes.HEIGHTFIELD_CAMERA, W, H)

    def timed(fn):
        ctx.sync()
        t0 = time.perf_counter()
        fn()
        ctx.sync()
        return time.perf_counter() - t0

    conv = render.Image(ctx, W, H, fp64=True)
    t_ref = timed(lambda: render.render(ctx, ds, cam, conv, "PT", max_path_length=depth, samples=args.nrc_ref_spp,
                                        iteration=1 << 24, rng_state=[99], sky=sky))
    ref = (conv.read64() / args.nrc_ref_spp).astype(np.float32)
    conv.close()

    def rmse(img, n):
        return float(np.sqrt(img.mse(n, ref, use_fp64=True)))

    pt = render.Image(ctx, W, H, fp64=True)
    t_pt, spp, pt_curve = 0.0, 0, []
    for c in [1, 1, 2, 4, 8, 16, 32, 64, 128, 256, 512]:
        t_pt += timed(lambda: render.render(ctx, ds, cam, pt, "PT", max_path_length=depth, samples=c, iteration=spp,
                                            rng_state=[7 + spp], sky=sky))
        spp += c
        pt_curve.append((spp, round(t_pt, 5), round(rmse(pt, spp), 6)))
    target = pt_curve[-1][2]
    pt.close()

    box = ((-1.05, -0.25, -1.05), (1.05, 0.35, 1.05))
    configs = [tuple(int(x) for x in c.split(",")) for c in args.nrc_configs.split(";")] if args.nrc_configs else \
        [(args.nrc_td, args.nrc_spf, args.nrc_train_steps)]
    for td, spf, steps in configs:
        # training paths: about 1.5 x 65,536 vertices per frame (3 per path)
        tf = args.nrc_train_fraction or min(0.05, 1.5 * 65536 / (3.0 * W * H * spf))
        cache = nrc.RadianceCache(ctx, *box, seed=5)
        opts = dict(max_path_length=depth, sky=sky, terminate_depth=td, train_fraction=tf, train_steps=steps,
                    samples_per_frame=spf)
        scratch = render.Image(ctx, W, H)
        t_nrc = timed(lambda: nrc.render_nrc(ctx, ds, cam, scratch, cache, samples=args.nrc_warmup * spf,
                                             iteration=1 << 20, rng_state=[11], **opts))
        t_warm = t_nrc
        scratch.close()
        img = render.Image(ctx, W, H, fp64=True)
        frames, nrc_curve, reached, at_equal_time, chunk = 0, [], None, None, 1
        while t_nrc < 3.0 * t_pt and frames * spf < 8192:
            t_nrc += timed(lambda: nrc.render_nrc(ctx, ds, cam, img, cache, samples=chunk * spf,
                                                  iteration=frames * spf, rng_state=[13 + frames], **opts))
            frames += chunk
            r = rmse(img, frames * spf)
            nrc_curve.append((frames * spf, round(t_nrc, 5), round(r, 6)))
            if at_equal_time is None and t_nrc >= t_pt:
                at_equal_time = r
            if r <= target:
                reached = t_nrc
                break
            chunk = min(chunk * 2, max(1, 64 // spf))
        line = {"metric": "time to the 1024-spp plain-PT RMSE, NRC path tracing vs plain PT", "unit": "ratio",
                "value": (reached / t_pt) if reached else None, "higher_is_better": False,
                "t_pt_s": round(t_pt, 4), "t_nrc_s": round(reached, 4) if reached else None,
                "t_nrc_warmup_s": round(t_warm, 4), "target_rmse": target,
                "nrc_rmse_at_equal_time": at_equal_time,
                "config": {"workload": "heightfield 512x512 fBm (amplitude 0.2) + 500 boxes, sun 5, sky 0.5, depth 8",
                           "resolution": [W, H], "reference_spp": args.nrc_ref_spp, "reference_s": round(t_ref, 2),
                           "nrc": {"terminate_depth": td, "train_fraction": round(tf, 5), "train_steps": steps,
                                   "samples_per_frame": spf, "warmup_frames": args.nrc_warmup,
                                   "max_train_samples": 65536, "ema": 0.99,
                                   "mlp": "64-64x4-3 ReLU fp16, fp32 accumulate, Adam lr 1e-2"}},
                "pt_curve": pt_curve, "nrc_curve": nrc_curve, "data": "synthetic", "dtype": "f32 paths, f16 MLP"}
        print(json.dumps(line), flush=True)
        img.close()
        cache.close()
    ds.close()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--shared-nodes", type=int, default=0,
                    help="top-of-tree nodes staged in shared memory by the walkers")
    ap.add_argument("--trace-mode", type=int, default=3,
                    help="0: thread per ray, 1: persistent lane refill, 2: root prefilter + persistent, "
                         "3/4: root prefilter + 8/4-lane group walker")
    ap.add_argument("--workload", choices=["trace", "nrc"], default="trace",
                    help="trace: the closest-hit headline; nrc: time-to-equal-RMSE of the radiance cache")
    ap.add_argument("--nrc-size", type=int, nargs=2, default=[640, 360])
    ap.add_argument("--nrc-ref-spp", type=int, default=16384)
    ap.add_argument("--nrc-spf", type=int, default=16, help="samples per cache frame")
    ap.add_argument("--nrc-warmup", type=int, default=16, help="training frames before accumulation")
    ap.add_argument("--nrc-train-fraction", type=float, default=0.0,
                    help="share of training paths (0: about 98k training vertices per frame)")
    ap.add_argument("--nrc-configs", default="", help="'td,spf,steps;...' several cache settings in one run")
    ap.add_argument("--nrc-train-steps", type=int, default=4)
    ap.add_argument("--nrc-td", type=int, default=2, help="path vertex where render paths query the cache")
    args = ap.parse_args()
    if args.workload == "nrc":
        from __graft_entry__ import build
        build()
        run_nrc(args)
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
