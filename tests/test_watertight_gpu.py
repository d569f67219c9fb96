"""Watertight triangle-test mode of the ray queries, GPU against the oracle.

gpugi_scene_set_triangle_test(GPUGI_TRIANGLE_WATERTIGHT) switches a scene's
ray queries to the watertight test of Woop, Benthin and Wald (JCGT 2013)
with the robust box test of Ize (JCGT 2013); the walk and its acceptance rule
stay the reference's. Bars: slot, t, u, v and any-hit flags bit-identical to
the oracle's watertight restatement in every trace mode; on a closed mesh
every ray from its centre through a vertex or an edge midpoint hits (the
reference test lets a share of those through); switching back restores the
reference results.
"""
import numpy as np
import pytest

import oracle
from gpugi_gb300 import bvh, cuda, scenes

pytestmark = pytest.mark.gpu


def _same(g, o):
    assert np.array_equal(g["slot"], o["slot"]), (g["slot"] != o["slot"]).sum()
    assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
    hit = o["slot"] >= 0
    assert np.array_equal(g["u"].view(np.uint32)[hit], o["u"].view(np.uint32)[hit])
    assert np.array_equal(g["v"].view(np.uint32)[hit], o["v"].view(np.uint32)[hit])


@pytest.fixture(scope="module")
def closed_mesh(cuda_ctx):
    sc = scenes.closed_icosphere(4, seed=1)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    yield sc, b, ds
    ds.close()


def test_crack_rays_all_hit(cuda_ctx, closed_mesh):
    sc, b, ds = closed_mesh
    rays = scenes.crack_rays(sc)
    ref = cuda.trace_closest(cuda_ctx, ds, rays)
    _same(ref, oracle.trace_closest(b, sc["positions"], rays))
    assert (ref["slot"] < 0).sum() > 100  # the reference test is not watertight
    ds.set_triangle_test(True)
    try:
        for mode in (0, 1, 2, 3, 4, 5):
            cuda_ctx.set_trace_config(mode=mode)
            g = cuda.trace_closest(cuda_ctx, ds, rays)
            assert (g["slot"] >= 0).all(), (mode, (g["slot"] < 0).sum())
            _same(g, oracle.trace_closest(b, sc["positions"], rays, watertight=True))
            assert cuda.trace_any(cuda_ctx, ds, rays).all()
    finally:
        cuda_ctx.set_trace_config(mode=3)
        ds.set_triangle_test(False)
    _same(cuda.trace_closest(cuda_ctx, ds, rays), oracle.trace_closest(b, sc["positions"], rays))


@pytest.mark.parametrize("fit", ["aabox", "ellipsoid"])
def test_watertight_bit_exact_on_query_workload(cuda_ctx, fit):
    """The closest-hit query workload (65,536-triangle displaced icosphere,
    sweep hierarchy, 2^20 rays) and its ellipsoid variant."""
    sc = scenes.displaced_icosphere(65536, seed=1)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", fit=fit)
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    ds.set_triangle_test(True)
    rays = scenes.random_rays(1 << 20, seed=100)
    o = oracle.trace_closest(b, sc["positions"], rays, watertight=True)
    oa = oracle.trace_any(b, sc["positions"], rays, watertight=True)["occluded"]
    try:
        for mode in ((0, 1, 2, 3, 4, 5) if fit == "aabox" else (0, 3)):
            cuda_ctx.set_trace_config(mode=mode)
            _same(cuda.trace_closest(cuda_ctx, ds, rays), o)
            assert np.array_equal(cuda.trace_any(cuda_ctx, ds, rays), oa)
    finally:
        cuda_ctx.set_trace_config(mode=3)
    assert cuda_ctx.device_error_bits() == 0
    ds.close()


def test_watertight_no_alloc_and_stats(cuda_ctx, closed_mesh):
    """The allocation-free query and the walk statistics follow the scene's
    triangle test too."""
    import ctypes as C

    import torch
    sc, b, ds = closed_mesh
    rays = scenes.crack_rays(sc)
    L = cuda.lib()
    P, U64 = C.c_void_p, C.c_uint64
    L.gpugi_trace_closest_noalloc.argtypes = [P, P] + [P] * 7 + [U64] + [P] * 4
    ds.set_triangle_test(True)
    try:
        dev = {k: torch.from_numpy(v).cuda() for k, v in rays.items()}
        n = rays["ox"].shape[0]
        out = dict(slot=torch.empty(n, dtype=torch.int32, device="cuda"), t=torch.empty(n, device="cuda"),
                   u=torch.empty(n, device="cuda"), v=torch.empty(n, device="cuda"))
        torch.cuda.synchronize()
        cuda_ctx.check(L.gpugi_trace_closest_noalloc(cuda_ctx.handle, ds.handle,
                                                     *[cuda._ptr(dev[k]) for k in cuda.RAY_KEYS], n,
                                                     *[cuda._ptr(out[k]) for k in ("slot", "t", "u", "v")]))
        cuda_ctx.sync()
        g = {k: v.cpu().numpy() for k, v in out.items()}
        _same(g, oracle.trace_closest(b, sc["positions"], rays, watertight=True))
        stats = cuda.trace_stats_device(cuda_ctx, ds, dev)
        o = oracle.trace_closest(b, sc["positions"], rays, counters=True, watertight=True)["counters"]
        assert np.array_equal(np.asarray(stats, np.int64), o.astype(np.int64).sum(0))
    finally:
        ds.set_triangle_test(False)


def test_triangle_test_validation(cuda_ctx, closed_mesh):
    sc, b, ds = closed_mesh
    assert cuda.lib().gpugi_scene_set_triangle_test(cuda_ctx.handle, ds.handle, 2) == 1  # invalid argument
    assert cuda.lib().gpugi_scene_set_triangle_test(cuda_ctx.handle, None, 1) == 1
