"""Parity on the workload scenes themselves, not reduced stand-ins.

* Plain path tracer workload: the enclosed room of ~98k triangles
  (5 walls, 2 rotated boxes, a level-6 sphere, the 0.5 x 0.5 ceiling light
  of radiance 10, albedos U[0.1, 0.9]) at its defaults, PCG streams, Russian
  roulette after depth 3, rendered at 64 x 64 (the workload's 512 x 512
  reduced so the oracle finishes in seconds): depth-1 images agree per pixel
  to 1e-4 of the maximum, depth-8 images by mean and 8x8-block statistics.
* Large BDPT workload's hierarchy kind: instanced displaced icospheres and
  boxes (~520k triangles) under ellipsoid-fitted node bounds; closest and
  any hits bit-exact against the oracle in every trace mode, and the closest
  hits equal brute force (the fitted ellipsoids contain their triangles).
"""
import numpy as np
import pytest

import oracle
from gpugi_gb300 import bvh, cuda, render, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def room_full(cuda_ctx):
    sc = scenes.cornell_room(seed=1)
    assert sc["triangles"].shape[0] > 90_000
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]),
                               sc["materials"])
    yield sc, b, ds
    ds.close()


def _light_sets(ds, n_sets, n, seed=321):
    state = [seed]
    return np.stack([render.generate_light_samples(ds, state, n) for _ in range(n_sets)])


def _oracle(b, sc, W, H, cam, ls, iters, **kw):
    acc = None
    for s in range(iters):
        acc = oracle.render(b, sc, "PT", W, H, cam.as_array(), render.frame_seed(s), ls[s], accum=acc, **kw)
    return acc


def test_room_workload_direct_light_per_pixel(cuda_ctx, room_full):
    sc, b, ds = room_full
    W = H = 64
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(ds, 4, 128)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img, "PT", max_path_length=1, samples=4, light_samples=ls, rr_start_depth=3)
    g = img.read()[..., :3]
    o = _oracle(b, sc, W, H, cam, ls, 4, max_path_length=1, rr_start_depth=3)[..., :3]
    assert np.abs(g - o).max() <= 1e-4 * np.abs(o).max() + 1e-6
    img.close()


def test_room_workload_full_depth(cuda_ctx, room_full):
    """Depth 8, Russian roulette after depth 3 (the workload's settings):
    the GPU batches and the oracle draw the same streams, so the block
    means agree well inside their batch noise."""
    sc, b, ds = room_full
    W = H = 64
    iters, K = 16, 4
    per = iters // K
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(ds, iters, 128)
    batches = []
    for k in range(K):
        img = render.Image(cuda_ctx, W, H)
        render.render(cuda_ctx, ds, cam, img, "PT", max_path_length=8, samples=per, iteration=k * per,
                      light_samples=ls[k * per:(k + 1) * per], rr_start_depth=3)
        batches.append(img.read()[..., :3] / per)
        img.close()
    o = _oracle(b, sc, W, H, cam, ls, iters, max_path_length=8, rr_start_depth=3)[..., :3] / iters
    g = np.stack(batches)
    assert abs(g.mean() / o.mean() - 1) < 0.02, (g.mean(), o.mean())
    blk = lambda a: a.reshape(*a.shape[:-3], H // 8, 8, W // 8, 8, 3).mean((-4, -2))
    gb = blk(g)
    se = gb.std(0, ddof=1) / np.sqrt(K)
    d = np.abs(gb.mean(0) - blk(o[None])[0])
    assert (d <= 6 * np.sqrt(2) * se + 1e-3 * np.abs(gb.mean(0)) + 1e-5).mean() > 0.97
    assert cuda_ctx.device_error_bits() == 0


@pytest.fixture(scope="module")
def instanced_ellipsoids(cuda_ctx):
    sc = scenes.large_instanced(seed=5, num_instances=1300, volume=40.0, num_lights=32)
    assert sc["triangles"].shape[0] >= 500_000
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", fit="ellipsoid")
    assert b.bounds_kind == 1
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    yield sc, b, ds
    ds.close()


def _volume_rays(n, seed, lo=0.0, hi=40.0):
    rays = scenes.random_rays(n, seed=seed, origin_lo=lo, origin_hi=hi)
    return rays


def test_instanced_ellipsoid_hierarchy_bit_exact(cuda_ctx, instanced_ellipsoids):
    sc, b, ds = instanced_ellipsoids
    rays = _volume_rays(1 << 16, seed=31)
    o = oracle.trace_closest(b, sc["positions"], rays)
    oa = oracle.trace_any(b, sc["positions"], rays)["occluded"]
    assert (o["slot"] >= 0).mean() > 0.5
    try:
        for mode in (0, 1, 2, 3, 4, 5):
            cuda_ctx.set_trace_config(mode=mode)
            g = cuda.trace_closest(cuda_ctx, ds, rays)
            assert np.array_equal(g["slot"], o["slot"]), (mode, (g["slot"] != o["slot"]).sum())
            assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32)), mode
            hit = o["slot"] >= 0
            assert np.array_equal(g["u"].view(np.uint32)[hit], o["u"].view(np.uint32)[hit])
            assert np.array_equal(g["v"].view(np.uint32)[hit], o["v"].view(np.uint32)[hit])
            assert np.array_equal(cuda.trace_any(cuda_ctx, ds, rays), oa), mode
    finally:
        cuda_ctx.set_trace_config(mode=3)
    assert cuda_ctx.device_error_bits() == 0


def test_instanced_ellipsoid_hierarchy_contains_hits(cuda_ctx, instanced_ellipsoids):
    sc, b, ds = instanced_ellipsoids
    rays = _volume_rays(1024, seed=32)
    g = cuda.trace_closest(cuda_ctx, ds, rays)
    bf = oracle.bruteforce_closest(b.slots, sc["positions"], rays)
    assert (g["t"].view(np.uint32) == bf["t"].view(np.uint32)).mean() > 0.999
