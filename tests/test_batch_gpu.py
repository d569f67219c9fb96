"""Batched rendering (gpugi_render_batch): several jobs with their own
scenes, cameras, resolutions, sample counts and path lengths in one
wavefront, replayed as a CUDA graph per round. Every job's image must equal
gpugi_render's for the same arguments (path tracing is deterministic given
the seeds and light samples; only the order of the atomic adds differs).
"""
import numpy as np
import pytest

from gpugi_gb300 import bvh, cuda, render, scenes

pytestmark = pytest.mark.gpu


def _upload(ctx, sc):
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    return ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]), sc["materials"])


@pytest.fixture(scope="module")
def scenes3(cuda_ctx):
    a = _upload(cuda_ctx, scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8))
    b = _upload(cuda_ctx, scenes.cornell_room(seed=7, sphere_level=2, wall_grid=4, light_radiance=25.0))
    c = _upload(cuda_ctx, scenes.cornell_room(seed=3, sphere_level=4, wall_grid=2))
    yield a, b, c
    for x in (a, b, c):
        x.close()


def _jobs(cuda_ctx, scs):
    spec = [  # (scene, W, H, samples, depth, camera)
        (scs[0], 32, 32, 4, 6, scenes.CORNELL_CAMERA),
        (scs[1], 48, 24, 3, 3, ((0.3, 1.2, 3.0), (0.0, 0.8, 0.0), (0.0, 1.0, 0.0), 50.0)),
        (scs[2], 16, 16, 7, 8, ((-0.5, 1.5, 2.5), (0.0, 1.0, 0.0), (0.0, 1.0, 0.0), 35.0)),
    ]
    jobs = []
    for i, (ds, W, H, spp, depth, cam) in enumerate(spec):
        state = [100 + i]
        ls = np.stack([render.generate_light_samples(ds, state, 128) for _ in range(spp)])
        jobs.append(dict(scene=ds, camera=render.camera_lookat(*cam, W, H), image=render.Image(cuda_ctx, W, H),
                         samples=spp, max_path_length=depth, light_samples=ls, iteration=10 * i))
    return jobs


def _single(cuda_ctx, j):
    img = render.Image(cuda_ctx, j["image"].width, j["image"].height)
    render.render(cuda_ctx, j["scene"], j["camera"], img, "PT", max_path_length=j["max_path_length"],
                  samples=j["samples"], iteration=j["iteration"], light_samples=j["light_samples"])
    out = img.read()
    img.close()
    return out


@pytest.mark.parametrize("paths_per_round,use_graph", [(16 << 20, True), (2048, True), (2048, False)])
def test_batch_equals_single_renders(cuda_ctx, scenes3, paths_per_round, use_graph):
    render.set_batch_config(cuda_ctx, paths_per_round, use_graph)
    try:
        jobs = _jobs(cuda_ctx, scenes3)
        render.render_batch(cuda_ctx, jobs)
        for j in jobs:
            got = j["image"].read()
            expect = _single(cuda_ctx, j)
            assert got.shape == expect.shape
            assert np.allclose(got, expect, rtol=1e-5, atol=1e-6 * np.abs(expect).max()), \
                np.abs(got - expect).max()
            assert got[..., :3].mean() > 0
        assert cuda_ctx.device_error_bits() == 0
    finally:
        render.set_batch_config(cuda_ctx)
        for j in jobs:
            j["image"].close()


def test_batch_runs_other_passes_and_validates(cuda_ctx, scenes3):
    ds = scenes3[0]
    W = H = 16
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    state = [5]
    ls = np.stack([render.generate_light_samples(ds, state, 256) for _ in range(2)])
    lt = render.Image(cuda_ctx, W, H)
    render.render_batch(cuda_ctx, [dict(scene=ds, camera=cam, image=lt, pass_="LT", samples=2, max_path_length=4,
                                         light_samples=ls)])
    ref = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, ref, "LT", max_path_length=4, samples=2, light_samples=ls)
    assert np.allclose(lt.read(), ref.read(), rtol=1e-5, atol=1e-6 * np.abs(ref.read()).max())
    # an image larger than the path queue is refused
    render.set_batch_config(cuda_ctx, 1024, True)
    big = render.Image(cuda_ctx, 64, 64)
    with pytest.raises(cuda.GpugiError):
        render.render_batch(cuda_ctx, [dict(scene=ds, camera=render.camera_lookat(*scenes.CORNELL_CAMERA, 64, 64),
                                            image=big, rng_state=[1])])
    render.set_batch_config(cuda_ctx)
    for x in (lt, ref, big):
        x.close()


def test_autotune_picks_a_candidate_and_keeps_results(cuda_ctx, scenes3):
    import oracle
    sc = scenes.displaced_icosphere(20000, seed=4)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"])
    try:
        t = cuda_ctx.autotune(ds, trace=True)
        assert (t["traceMode"], t["traceBlock"]) in {(0, 64), (0, 128), (0, 256), (1, 128), (2, 128), (3, 128), (4, 128), (5, 128)}
        assert t["traceMraysPerSecond"] > 0
        rays = scenes.aimed_rays(50_000, sc["positions"], seed=8)
        g = cuda.trace_closest(cuda_ctx, ds, rays)
        o = oracle.trace_closest(b, sc["positions"], rays)
        assert np.array_equal(g["slot"], o["slot"])
        assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
        tb = cuda_ctx.autotune(scenes3[0], trace=False, batch=True)
        assert tb["batchPaths"] in {256 << 10, 1 << 20, 4 << 20, 16 << 20} and tb["batchMpathsPerSecond"] > 0
    finally:
        cuda_ctx.set_trace_config(3, 128)
        render.set_batch_config(cuda_ctx)
        ds.close()
