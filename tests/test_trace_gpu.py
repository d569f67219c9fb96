"""GPU traversal parity: the sm_103a kernels against the oracle, through the C ABI.

Bar (bit-exact for index work): hit slot identical, t identical to the bit
(the spec allows 2 ulp; the kernels reproduce the exact IEEE sequence),
barycentrics identical, any-hit flags identical.
"""
import math

import numpy as np
import pytest

import oracle
from gpugi_gb300 import bvh, cuda, scenes

pytestmark = pytest.mark.gpu

T_ULP_TOL = 2  # spec tolerance on t; the implementation is expected to be exact


def _bits(a):
    return np.asarray(a, np.float32).view(np.int32)


def _compare_closest(g, o):
    assert np.array_equal(g["slot"], o["slot"]), f"{(g['slot'] != o['slot']).sum()} slot mismatches"
    dt = np.abs(_bits(g["t"]).astype(np.int64) - _bits(o["t"]).astype(np.int64))
    assert dt.max() <= T_ULP_TOL
    assert (dt == 0).all(), "t differs in the last bits"
    hit = o["slot"] >= 0
    assert np.array_equal(_bits(g["u"])[hit], _bits(o["u"])[hit])
    assert np.array_equal(_bits(g["v"])[hit], _bits(o["v"])[hit])


@pytest.fixture(scope="module")
def icosphere_65536():
    sc = scenes.displaced_icosphere(65536, seed=1)
    return sc


@pytest.mark.parametrize("method,leaf", [("sweep", 8), ("kdtree", 8), ("sweep", 2), ("lds", 8)])
def test_closest_and_any_match_oracle(cuda_ctx, icosphere_65536, method, leaf):
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method=method, leaf_size=leaf)
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    try:
        for mode in (0, 1, 2, 3, 4, 5):  # thread per ray / lane refill / root prefilter + persistent / + 8-, 4-, 16-lane groups
            cuda_ctx.set_trace_config(mode=mode)
            for rays in (scenes.random_rays(1 << 18, seed=3), scenes.aimed_rays(1 << 18, sc["positions"], seed=4)):
                g = cuda.trace_closest(cuda_ctx, ds, rays)
                o = oracle.trace_closest(b, sc["positions"], rays)
                _compare_closest(g, o)
                occ = cuda.trace_any(cuda_ctx, ds, rays)
                oa = oracle.trace_any(b, sc["positions"], rays)["occluded"]
                assert np.array_equal(occ, oa)
    finally:
        cuda_ctx.set_trace_config(mode=3)
    ds.close()


@pytest.mark.parametrize("method", ["kdtree", "sweep"])
def test_ellipsoid_bounds_match_oracle_and_bruteforce(cuda_ctx, method):
    """Ellipsoid nodes (the BVH kind of the large BDPT workload): the walk
    over fitted ellipsoids is bit-exact against the oracle and finds the same
    closest hits as brute force (the fit contains every triangle)."""
    sc = scenes.displaced_icosphere(6000, seed=9)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method=method, fit="ellipsoid")
    assert b.bounds_kind == 1
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    for mode in (0, 1, 2, 3, 4, 5):
        cuda_ctx.set_trace_config(mode=mode)
        for rays in (scenes.aimed_rays(40_000, sc["positions"], seed=13), scenes.random_rays(40_000, seed=14)):
            g = cuda.trace_closest(cuda_ctx, ds, rays)
            _compare_closest(g, oracle.trace_closest(b, sc["positions"], rays))
            assert np.array_equal(cuda.trace_any(cuda_ctx, ds, rays),
                                  oracle.trace_any(b, sc["positions"], rays)["occluded"])
            bf = oracle.bruteforce_closest(b.slots, sc["positions"], rays)
            assert (g["t"].view(np.uint32) == bf["t"].view(np.uint32)).mean() > 0.999
    cuda_ctx.set_trace_config(mode=3)
    ds.close()


@pytest.mark.parametrize("shared_nodes", [0, 3, 64, 2048, 7000])
def test_staged_layouts_give_identical_results(cuda_ctx, icosphere_65536, shared_nodes):
    """The breadth-first top-level layout and its shared-memory staging change
    node addresses only: every mode returns the oracle's results."""
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    cuda_ctx.set_scene_layout(shared_nodes, shared_nodes)
    try:
        ds = cuda_ctx.upload_scene(b, sc["positions"])
        rays = scenes.aimed_rays(1 << 17, sc["positions"], seed=77, spread=2.5)
        o = oracle.trace_closest(b, sc["positions"], rays)
        oa = oracle.trace_any(b, sc["positions"], rays)["occluded"]
        for mode in (0, 1, 2, 3, 4, 5):
            cuda_ctx.set_trace_config(mode=mode)
            _compare_closest(cuda.trace_closest(cuda_ctx, ds, rays), o)
            assert np.array_equal(cuda.trace_any(cuda_ctx, ds, rays), oa)
        ds.close()
    finally:
        cuda_ctx.set_trace_config(mode=3)
        cuda_ctx.set_scene_layout(0, 0)


def test_full_size_properties(cuda_ctx, icosphere_65536):
    """2^20 rays of the closest-hit workload: exact against the oracle, and
    size-independent checks (any-hit == closest-hit hit mask, t > 1e-4)."""
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    rays = scenes.random_rays(1 << 20, seed=1)
    g = cuda.trace_closest(cuda_ctx, ds, rays)
    o = oracle.trace_closest(b, sc["positions"], rays)
    _compare_closest(g, o)
    occ = cuda.trace_any(cuda_ctx, ds, rays)
    assert np.array_equal(occ.astype(bool), g["slot"] >= 0)
    assert (g["t"][g["slot"] >= 0] > 1e-4).all()
    assert np.isinf(g["t"][g["slot"] < 0]).all()
    ds.close()


def test_device_entry_points(cuda_ctx, icosphere_65536):
    import torch
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    rays = scenes.aimed_rays(100_003, sc["positions"], seed=12)
    dr = {k: torch.from_numpy(rays[k]).cuda() for k in cuda.RAY_KEYS}
    n = rays["ox"].shape[0]
    out = dict(slot=torch.empty(n, dtype=torch.int32, device="cuda"), t=torch.empty(n, device="cuda"),
               u=torch.empty(n, device="cuda"), v=torch.empty(n, device="cuda"))
    torch.cuda.synchronize()
    cuda.trace_closest_device(cuda_ctx, ds, dr, out)
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    cuda.trace_any_device(cuda_ctx, ds, dr, occ)
    cuda_ctx.sync()
    g = {k: v.cpu().numpy() for k, v in out.items()}
    o = oracle.trace_closest(b, sc["positions"], rays)
    _compare_closest(g, o)
    assert np.array_equal(occ.cpu().numpy(), oracle.trace_any(b, sc["positions"], rays)["occluded"])
    ds.close()


def test_walk_statistics_match_oracle_counters(cuda_ctx, icosphere_65536):
    """The device fetch counters (used for the roofline's algorithmic bytes)
    equal the oracle's TRACERAY_DEBUG_VARS-style counters."""
    import torch
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    for any_hit in (False, True):
        for rays in (scenes.random_rays(50_000, seed=31), scenes.aimed_rays(50_000, sc["positions"], seed=32)):
            dr = {k: torch.from_numpy(rays[k]).cuda() for k in cuda.RAY_KEYS}
            sums = cuda.trace_stats_device(cuda_ctx, ds, dr, any_hit=any_hit)
            f = oracle.trace_any if any_hit else oracle.trace_closest
            c = f(b, sc["positions"], rays, counters=True)["counters"].astype(np.uint64).sum(0)
            assert np.array_equal(sums, c), (any_hit, sums, c)
            assert cuda.algorithmic_bytes(sums, 50_000, any_hit) == int(
                oracle.algorithmic_bytes(f(b, sc["positions"], rays, counters=True)["counters"], any_hit).sum())
    ds.close()


def test_triangle_known_answers_gpu(cuda_ctx):
    import json
    from pathlib import Path
    cases = json.loads((Path(__file__).resolve().parent / "golden" / "kat_triangles.json").read_text())["cases"]
    for c in cases:
        positions = np.array(c["triangle"], dtype=np.float32)
        tri = np.array([[0, 1, 2, 0]], dtype=np.uint32)
        b = bvh.build_bvh(positions, tri)
        ds = cuda_ctx.upload_scene(b, positions)
        rays = {k: np.array([v], np.float32) for k, v in zip(("ox", "oy", "oz"), c["origin"])}
        rays.update({k: np.array([v], np.float32) for k, v in zip(("dx", "dy", "dz"), c["direction"])})
        rays["tmax"] = np.array([c["tmax"] if c["tmax"] is not None else math.inf], np.float32)
        g = cuda.trace_closest(cuda_ctx, ds, rays)
        assert (g["slot"][0] >= 0) == c["walk_hit"], c["name"]
        if c["walk_hit"]:
            assert g["t"][0] == np.float32(c["t"]) and g["u"][0] == np.float32(c["u"]), c["name"]
            assert g["v"][0] == np.float32(c["v"]), c["name"]
        ds.close()


def test_edge_rays(cuda_ctx):
    """Axis-parallel directions (inf*0 = NaN slabs), origins inside the mesh,
    on bounding planes, zero-length tmax, NaN-free misses, n = 0."""
    sc = scenes.displaced_icosphere(5000, seed=3)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", leaf_size=4)
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    dirs = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                     [0.6, 0.8, 0], [0, 0.6, -0.8], [-0.6, 0, 0.8]], np.float32)
    lo, hi = sc["positions"].min(0), sc["positions"].max(0)
    origins = [np.zeros(3), (lo + hi) / 2, lo, hi, np.array([lo[0], 0.5, 0.5]), np.array([2.0, 0.5, 0.5]),
               np.array([0.5, 0.5, 0.5]), np.array([0.5, 0.5, -3.0])]
    o = np.array([oo for oo in origins for _ in dirs], np.float32)
    d = np.array([dd for _ in origins for dd in dirs], np.float32)
    rays = dict(ox=o[:, 0].copy(), oy=o[:, 1].copy(), oz=o[:, 2].copy(), dx=d[:, 0].copy(), dy=d[:, 1].copy(),
                dz=d[:, 2].copy())
    for tm in (math.inf, 3.402823466e38, 0.3, 0.0, 1e-4):
        rays["tmax"] = np.full(o.shape[0], tm, np.float32)
        g = cuda.trace_closest(cuda_ctx, ds, rays)
        orc = oracle.trace_closest(b, sc["positions"], rays)
        _compare_closest(g, orc)
        assert np.array_equal(cuda.trace_any(cuda_ctx, ds, rays), oracle.trace_any(b, sc["positions"], rays)["occluded"])
    empty = {k: np.zeros(0, np.float32) for k in cuda.RAY_KEYS}
    g = cuda.trace_closest(cuda_ctx, ds, empty)
    assert g["slot"].shape == (0,)
    ds.close()


@pytest.mark.parametrize("ntri", [1, 3, 8, 9])
def test_tiny_scenes(cuda_ctx, ntri):
    sc = scenes.displaced_icosphere(ntri, seed=2)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    rays = scenes.aimed_rays(20000, sc["positions"], seed=5, spread=3.0)
    _compare_closest(cuda.trace_closest(cuda_ctx, ds, rays), oracle.trace_closest(b, sc["positions"], rays))
    ds.close()


def test_rejects_malformed_hierarchy(cuda_ctx):
    sc = scenes.displaced_icosphere(512, seed=2)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    bad = bvh.BVH(b.hierarchy.copy(), b.slots.copy(), b.parents, b.leaf_size, 0, b.max_depth)
    esc = bad.hierarchy[:, 7].view(np.uint32)
    esc[5] = 2  # an escape pointing backwards would loop
    with pytest.raises(cuda.GpugiError) as e:
        cuda_ctx.upload_scene(bad, sc["positions"])
    assert e.value.status == 2
    bad = bvh.BVH(b.hierarchy.copy(), b.slots.copy(), b.parents, b.leaf_size, 0, b.max_depth)
    bad.slots[3, 2] = 10 ** 7
    with pytest.raises(cuda.GpugiError):
        cuda_ctx.upload_scene(bad, sc["positions"])
    bad = bvh.BVH(b.hierarchy.copy(), b.slots.copy(), b.parents, b.leaf_size, 0, b.max_depth)
    fc = bad.hierarchy[:, 3].view(np.uint32)
    leaf = np.nonzero(fc & 0x80000000)[0][0]
    fc[leaf] = 0x80000000 | 0x7FFFFFF
    with pytest.raises(cuda.GpugiError):
        cuda_ctx.upload_scene(bad, sc["positions"])
    assert cuda_ctx.device_error_bits() == 0


@pytest.mark.parametrize("parts,pinned", [(1, False), (2, False), (3, False), (8, False), (2, True)])
def test_host_paths_give_identical_results(cuda_ctx, icosphere_65536, parts, pinned):
    """Host-pointer queries: staged and split into overlapping parts (copies
    in, traversal, copies out on three streams), or on page-locked arrays
    read and written by the kernels directly; both return the oracle's
    results, including a ray count that is not a multiple of the part size."""
    import torch
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    cuda_ctx.set_host_pipeline(parts, zero_copy=True)
    try:
        rays = scenes.aimed_rays(300_001, sc["positions"], seed=21, spread=2.5)
        if pinned:
            rays = {k: torch.from_numpy(np.ascontiguousarray(v, dtype=np.float32)).pin_memory().numpy()
                    for k, v in rays.items()}
            n = rays["ox"].shape[0]
            out = dict(slot=torch.empty(n, dtype=torch.int32).pin_memory().numpy(),
                       t=torch.empty(n).pin_memory().numpy(), u=torch.empty(n).pin_memory().numpy(),
                       v=torch.empty(n).pin_memory().numpy())
            cuda_ctx.check(cuda.lib().gpugi_trace_closest(
                cuda_ctx.handle, ds.handle, *[cuda._ptr(rays[k]) for k in cuda.RAY_KEYS], n,
                *[cuda._ptr(out[k]) for k in ("slot", "t", "u", "v")]))
            g = out
            occ = torch.empty(n, dtype=torch.uint8).pin_memory().numpy()
            cuda_ctx.check(cuda.lib().gpugi_trace_any(cuda_ctx.handle, ds.handle,
                                                      *[cuda._ptr(rays[k]) for k in cuda.RAY_KEYS], n, cuda._ptr(occ)))
        else:
            g = cuda.trace_closest(cuda_ctx, ds, rays)
            occ = cuda.trace_any(cuda_ctx, ds, rays)
        _compare_closest(g, oracle.trace_closest(b, sc["positions"], rays))
        assert np.array_equal(occ, oracle.trace_any(b, sc["positions"], rays)["occluded"])
    finally:
        cuda_ctx.set_host_pipeline(2)
        ds.close()


@pytest.mark.parametrize("parts,pad,pinned", [(1, 0, True), (2, 0, True), (3, 5, True), (2, 1000, True),
                                             (1, 0, False)])
def test_host_soa_blocks(cuda_ctx, icosphere_65536, parts, pad, pinned):
    """Rays and results in structure-of-arrays blocks (evenly spaced
    columns, packed or with a gap between them: one 2D copy each way) give
    the oracle's results through the synchronous call (staged in parts) and
    the stream-ordered call."""
    import ctypes as C

    import torch
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    n = 200_003
    w = n + pad
    rays = scenes.aimed_rays(n, sc["positions"], seed=23, spread=2.5)

    def block(rows):
        a = torch.empty(rows * w, dtype=torch.float32)
        return (a.pin_memory() if pinned else a).numpy()

    rb, ob, occb = block(7), block(4), block(1)
    cols = {k: rb[i * w:i * w + n] for i, k in enumerate(cuda.RAY_KEYS)}
    for k in cuda.RAY_KEYS:
        cols[k][:] = rays[k]
    out = dict(slot=ob[0:n].view(np.int32), t=ob[w:w + n], u=ob[2 * w:2 * w + n], v=ob[3 * w:3 * w + n])
    occ = occb.view(np.uint8)[:n]
    want = oracle.trace_closest(b, sc["positions"], rays)
    want_occ = oracle.trace_any(b, sc["positions"], rays)["occluded"]
    L = cuda.lib()
    cuda_ctx.set_host_pipeline(parts)
    try:
        cuda_ctx.check(L.gpugi_trace_closest(cuda_ctx.handle, ds.handle, *[cuda._ptr(cols[k]) for k in cuda.RAY_KEYS],
                                             n, *[cuda._ptr(out[k]) for k in ("slot", "t", "u", "v")]))
        _compare_closest(out, want)
        cuda_ctx.check(L.gpugi_trace_any(cuda_ctx.handle, ds.handle, *[cuda._ptr(cols[k]) for k in cuda.RAY_KEYS], n,
                                         cuda._ptr(occ)))
        assert np.array_equal(occ, want_occ)
        ob[:] = np.nan
        occ[:] = 7
        L.gpugi_trace_closest_async.argtypes = [C.c_void_p] * 9 + [C.c_uint64] + [C.c_void_p] * 5
        L.gpugi_trace_any_async.argtypes = [C.c_void_p] * 9 + [C.c_uint64, C.c_void_p, C.c_void_p]
        st = torch.cuda.Stream()
        cuda_ctx.check(L.gpugi_trace_closest_async(cuda_ctx.handle, ds.handle,
                                                   *[cuda._ptr(cols[k]) for k in cuda.RAY_KEYS], n,
                                                   *[cuda._ptr(out[k]) for k in ("slot", "t", "u", "v")],
                                                   C.c_void_p(st.cuda_stream)))
        cuda_ctx.check(L.gpugi_trace_any_async(cuda_ctx.handle, ds.handle, *[cuda._ptr(cols[k]) for k in cuda.RAY_KEYS],
                                               n, cuda._ptr(occ), C.c_void_p(st.cuda_stream)))
        st.synchronize()
        assert cuda_ctx.device_error_bits() == 0
        _compare_closest(out, want)
        assert np.array_equal(occ, want_occ)
    finally:
        cuda_ctx.set_host_pipeline(2)
        ds.close()


@pytest.mark.parametrize("parts,zero_copy", [(1, False), (2, False), (1, True)])
def test_device_guard_bits_reach_the_caller(cuda_ctx, icosphere_65536, parts, zero_copy):
    """A guard bit set on the device (here by the test-support call, as a
    guard would) fails the next host-pointer query with GPUGI_ERROR_DEVICE
    once, whatever path the query takes, and is cleared for the next call."""
    import torch
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    n = 1 << 17
    rays = scenes.random_rays(n, seed=21)
    # page-locked inputs and outputs, so zero copy applies when enabled
    r = {k: torch.from_numpy(np.ascontiguousarray(rays[k], dtype=np.float32)).pin_memory().numpy()
         for k in cuda.RAY_KEYS}
    out = dict(slot=torch.empty(n, dtype=torch.int32).pin_memory().numpy(), t=torch.empty(n).pin_memory().numpy(),
               u=torch.empty(n).pin_memory().numpy(), v=torch.empty(n).pin_memory().numpy())

    def query():
        cuda_ctx.check(cuda.lib().gpugi_trace_closest(cuda_ctx.handle, ds.handle,
                                                      *[cuda._ptr(r[k]) for k in cuda.RAY_KEYS], n,
                                                      *[cuda._ptr(out[k]) for k in ("slot", "t", "u", "v")]))

    cuda_ctx.set_host_pipeline(parts, zero_copy)
    try:
        cuda_ctx.debug_raise_device_error(0x2)
        with pytest.raises(cuda.GpugiError) as e:
            query()
        assert e.value.status == 5 and "0x2" in str(e.value)
        query()  # the bits were cleared
        _compare_closest(out, oracle.trace_closest(b, sc["positions"], rays))
        assert cuda_ctx.device_error_bits() == 0
    finally:
        cuda_ctx.set_host_pipeline(2, False)
    ds.close()


def test_l2_bandwidth_measurement(cuda_ctx):
    """The second roofline's denominator: L2 reads of an L2-resident buffer
    run faster than the HBM copy rate; bad sizes are refused."""
    import ctypes as C
    lib = cuda.lib()
    lib.gpugi_measure_l2_bandwidth.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.POINTER(C.c_double)]
    g = C.c_double()
    cuda_ctx.check(lib.gpugi_measure_l2_bandwidth(cuda_ctx.handle, 32 << 20, 50, C.byref(g)))
    assert g.value > 1000.0
    with pytest.raises(cuda.GpugiError):
        cuda_ctx.check(lib.gpugi_measure_l2_bandwidth(cuda_ctx.handle, 1000, 1, C.byref(g)))


@pytest.mark.parametrize("share", [50, 100, 1])
def test_stream_ordered_queries_overlap_and_match(cuda_ctx, icosphere_65536, share):
    """gpugi_trace_*_device_async on several caller streams: batches issued
    alternately on three streams (and one on the context stream, NULL) give
    the results of the context-stream calls, whatever share of the walker
    grid the stream-ordered walks launch; a larger batch on a stream grows
    its scratch."""
    import torch
    for bad in (0, 101):
        with pytest.raises(cuda.GpugiError):
            cuda_ctx.set_async_walker_share(bad)
    cuda_ctx.set_async_walker_share(share)
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    streams = [torch.cuda.Stream() for _ in range(3)]
    sizes = [1 << 14, 3 << 14, 50001, 1 << 18, 1 << 16, 7]
    host = [scenes.random_rays(n, seed=300 + i) for i, n in enumerate(sizes)]
    dev = [{k: torch.from_numpy(r[k]).cuda() for k in cuda.RAY_KEYS} for r in host]
    outs = [dict(slot=torch.empty(n, dtype=torch.int32, device="cuda"), t=torch.empty(n, device="cuda"),
                 u=torch.empty(n, device="cuda"), v=torch.empty(n, device="cuda")) for n in sizes]
    occ = [torch.empty(n, dtype=torch.uint8, device="cuda") for n in sizes]
    torch.cuda.synchronize()
    for i in range(len(sizes)):
        s = streams[i % 3].cuda_stream if i != 4 else 0
        cuda.trace_closest_device_async(cuda_ctx, ds, dev[i], outs[i], s)
        cuda.trace_any_device_async(cuda_ctx, ds, dev[i], occ[i], s)
    torch.cuda.synchronize()
    cuda_ctx.sync()
    for i in range(len(sizes)):
        g = {k: v.cpu().numpy() for k, v in outs[i].items()}
        _compare_closest(g, cuda.trace_closest(cuda_ctx, ds, host[i]))
        assert np.array_equal(occ[i].cpu().numpy(), cuda.trace_any(cuda_ctx, ds, host[i]))
    assert cuda_ctx.device_error_bits() == 0
    cuda_ctx.set_async_walker_share(50)
    ds.close()


def test_stream_ordered_host_queries(cuda_ctx, icosphere_65536):
    """gpugi_trace_closest_async / gpugi_trace_any_async with page-locked host
    arrays on three streams equal the synchronous host calls."""
    import ctypes as C

    import torch
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    L = cuda.lib()
    L.gpugi_trace_closest_async.argtypes = [C.c_void_p] * 9 + [C.c_uint64] + [C.c_void_p] * 5
    L.gpugi_trace_any_async.argtypes = [C.c_void_p] * 9 + [C.c_uint64, C.c_void_p, C.c_void_p]
    streams = [torch.cuda.Stream() for _ in range(3)]
    sizes = [1 << 16, 12345, 1 << 18, 3, 1 << 16, 40000]
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()
    host = [{k: pin(v) for k, v in scenes.random_rays(n, seed=400 + i).items()} for i, n in enumerate(sizes)]
    outs = [dict(slot=pin(np.empty(n, np.int32)), t=pin(np.empty(n, np.float32)), u=pin(np.empty(n, np.float32)),
                 v=pin(np.empty(n, np.float32)), occ=pin(np.empty(n, np.uint8))) for n in sizes]
    for i, n in enumerate(sizes):
        s = C.c_void_p(streams[i % 3].cuda_stream)
        r, o = host[i], outs[i]
        cuda_ctx.check(L.gpugi_trace_closest_async(cuda_ctx.handle, ds.handle, *[cuda._ptr(r[k]) for k in cuda.RAY_KEYS],
                                                   n, *[cuda._ptr(o[k]) for k in ("slot", "t", "u", "v")], s))
        cuda_ctx.check(L.gpugi_trace_any_async(cuda_ctx.handle, ds.handle, *[cuda._ptr(r[k]) for k in cuda.RAY_KEYS],
                                               n, cuda._ptr(o["occ"]), s))
    for s in streams:
        s.synchronize()
    assert cuda_ctx.device_error_bits() == 0
    for i in range(len(sizes)):
        _compare_closest({k: outs[i][k] for k in ("slot", "t", "u", "v")}, cuda.trace_closest(cuda_ctx, ds, host[i]))
        assert np.array_equal(outs[i]["occ"], cuda.trace_any(cuda_ctx, ds, host[i]))
    ds.close()


@pytest.mark.parametrize("watertight", [False, True])
def test_oriented_box_hierarchy_bit_exact(cuda_ctx, icosphere_65536, watertight):
    """GPUGI_BOUNDS_OBOX scenes (48-B nodes, the reference's OBOX_BVH walk):
    bit-exact against the oracle in every trace mode, in both triangle tests,
    through the stream-ordered query too."""
    import torch
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", fit="obox")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    ds.set_triangle_test(watertight)
    try:
        for rays in (scenes.random_rays(1 << 18, seed=61), scenes.aimed_rays(1 << 17, sc["positions"], seed=62)):
            o = oracle.trace_closest(b, sc["positions"], rays, watertight=watertight)
            oa = oracle.trace_any(b, sc["positions"], rays, watertight=watertight)["occluded"]
            for mode in (0, 1, 2, 3, 4, 5):
                cuda_ctx.set_trace_config(mode=mode)
                _compare_closest(cuda.trace_closest(cuda_ctx, ds, rays), o)
                assert np.array_equal(cuda.trace_any(cuda_ctx, ds, rays), oa)
            cuda_ctx.set_trace_config(mode=3)
            dev = {k: torch.from_numpy(rays[k]).cuda() for k in cuda.RAY_KEYS}
            n = rays["ox"].shape[0]
            out = dict(slot=torch.empty(n, dtype=torch.int32, device="cuda"), t=torch.empty(n, device="cuda"),
                       u=torch.empty(n, device="cuda"), v=torch.empty(n, device="cuda"))
            s = torch.cuda.Stream()
            torch.cuda.synchronize()
            cuda.trace_closest_device_async(cuda_ctx, ds, dev, out, s.cuda_stream)
            s.synchronize()
            _compare_closest({k: v.cpu().numpy() for k, v in out.items()}, o)
        stats = cuda.trace_stats_device(cuda_ctx, ds, {k: torch.from_numpy(v).cuda() for k, v in rays.items()})
        oc = oracle.trace_closest(b, sc["positions"], rays, counters=True, watertight=watertight)["counters"]
        assert np.array_equal(np.asarray(stats, np.int64), oc.astype(np.int64).sum(0))
    finally:
        cuda_ctx.set_trace_config(mode=3)
    assert cuda_ctx.device_error_bits() == 0
    exported = ds.export()
    assert np.array_equal(exported.hierarchy.view(np.uint32)[:, 8:], b.hierarchy.view(np.uint32)[:, 8:])
    ds.close()


def test_stream_ordered_queries_on_many_streams(cuda_ctx, icosphere_65536):
    """More caller streams than scratch sets (GPUGI_MAX_QUERY_STREAMS = 8):
    the least recently used set is taken over once its work has finished;
    every batch still gets its own results."""
    import torch
    sc = icosphere_65536
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    streams = [torch.cuda.Stream() for _ in range(13)]
    host = [scenes.random_rays(20000 + 1000 * i, seed=700 + i) for i in range(13)]
    dev = [{k: torch.from_numpy(r[k]).cuda() for k in cuda.RAY_KEYS} for r in host]
    outs = [dict(slot=torch.empty(r["ox"].shape[0], dtype=torch.int32, device="cuda"),
                 t=torch.empty(r["ox"].shape[0], device="cuda"), u=torch.empty(r["ox"].shape[0], device="cuda"),
                 v=torch.empty(r["ox"].shape[0], device="cuda")) for r in host]
    torch.cuda.synchronize()
    for rep in range(2):
        for i, s in enumerate(streams):
            cuda.trace_closest_device_async(cuda_ctx, ds, dev[i], outs[i], s.cuda_stream)
        torch.cuda.synchronize()
        for i in range(len(streams)):
            _compare_closest({k: v.cpu().numpy() for k, v in outs[i].items()}, cuda.trace_closest(cuda_ctx, ds, host[i]))
    assert cuda_ctx.device_error_bits() == 0
    ds.close()
