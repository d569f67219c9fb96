"""Batched rendering (gpugi_render_batch): several jobs with their own
scenes, cameras, resolutions, sample counts, path lengths and passes (PT,
LT, BPT) in one wavefront, replayed as a CUDA graph per round. Every PT and
LT job's image must equal gpugi_render's for the same arguments (the passes
are deterministic given the seeds and light samples; only the order of the
atomic adds differs). So must a BPT job's at path length 1: its eye vertices
connect only to the light samples, which sit at fixed cache slots. Deeper BPT
connections pick cache entries whose slots follow the atomic order, so there
the batched and the single-call images agree in distribution.
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


def _jobs(cuda_ctx, scs, passes=("PT",), bpt_depth=1):
    spec = [  # (scene, W, H, samples, depth, camera)
        (scs[0], 32, 32, 4, 6, scenes.CORNELL_CAMERA),
        (scs[1], 48, 24, 3, 3, ((0.3, 1.2, 3.0), (0.0, 0.8, 0.0), (0.0, 1.0, 0.0), 50.0)),
        (scs[2], 16, 16, 7, 8, ((-0.5, 1.5, 2.5), (0.0, 1.0, 0.0), (0.0, 1.0, 0.0), 35.0)),
    ]
    jobs = []
    for i, (ds, W, H, spp, depth, cam) in enumerate(spec):
        for k, pass_ in enumerate(passes):
            nls = 128 if pass_ == "PT" else 16
            state = [100 + i + 10 * k]
            ls = np.stack([render.generate_light_samples(ds, state, nls) for _ in range(spp)])
            jobs.append(dict(scene=ds, camera=render.camera_lookat(*cam, W, H), image=render.Image(cuda_ctx, W, H),
                             pass_=pass_, samples=spp, max_path_length=bpt_depth if pass_ == "BPT" else depth,
                             num_light_samples=nls, light_samples=ls, iteration=10 * i + k))
    return jobs


def _single(cuda_ctx, j):
    img = render.Image(cuda_ctx, j["image"].width, j["image"].height)
    render.render(cuda_ctx, j["scene"], j["camera"], img, j["pass_"], max_path_length=j["max_path_length"],
                  samples=j["samples"], iteration=j["iteration"], num_light_samples=j["num_light_samples"],
                  light_samples=j["light_samples"])
    out = img.read()
    img.close()
    return out


@pytest.mark.parametrize("paths_per_round,use_graph", [(16 << 20, True), (4096, True), (4096, False)])
def test_batch_equals_single_renders(cuda_ctx, scenes3, paths_per_round, use_graph):
    render.set_batch_config(cuda_ctx, paths_per_round, use_graph)
    jobs = _jobs(cuda_ctx, scenes3, passes=("PT", "LT", "BPT"))
    try:
        render.render_batch(cuda_ctx, jobs)
        for j in jobs:
            got = j["image"].read()
            expect = _single(cuda_ctx, j)
            assert got.shape == expect.shape
            assert np.allclose(got, expect, rtol=1e-5, atol=1e-6 * np.abs(expect).max()), \
                (j["pass_"], np.abs(got - expect).max())
            assert got[..., :3].mean() > 0, j["pass_"]
        assert cuda_ctx.device_error_bits() == 0
    finally:
        render.set_batch_config(cuda_ctx)
        for j in jobs:
            j["image"].close()


def test_batch_bpt_agrees_with_single_renders(cuda_ctx, scenes3):
    """BPT at path length 6 in a batch with PT and LT jobs: over 6 independent
    iterations, the batched and the single-call estimates of every 8 x 8
    block and of the image mean agree within 5 standard errors."""
    render.set_batch_config(cuda_ctx, 1 << 20, True)
    runs = {"batch": [], "single": []}
    try:
        for it in range(6):
            jobs = _jobs(cuda_ctx, scenes3, passes=("PT", "LT", "BPT"), bpt_depth=6)
            for j in jobs:
                j["iteration"] += 1000 * it
            render.render_batch(cuda_ctx, jobs)
            j = jobs[2]  # the 32 x 32 BPT job
            assert j["pass_"] == "BPT"
            runs["batch"].append(j["image"].read()[..., :3])
            runs["single"].append(_single(cuda_ctx, j)[..., :3])
            for x in jobs:
                x["image"].close()
        assert cuda_ctx.device_error_bits() == 0
    finally:
        render.set_batch_config(cuda_ctx)

    def stats(imgs):
        b = np.stack(imgs).astype(np.float64)  # (K, 32, 32, 3)
        blocks = b.reshape(b.shape[0], 4, 8, 4, 8, 3).mean((2, 4))
        whole = b.mean((1, 2))
        se = lambda x: x.std(0, ddof=1) / np.sqrt(x.shape[0])
        return blocks.mean(0), se(blocks), whole.mean(0), se(whole)

    mb, sb, wb, swb = stats(runs["batch"])
    ms, ss, ws, sws = stats(runs["single"])
    assert wb.min() > 0
    z_blocks = np.abs(mb - ms) / np.sqrt(sb ** 2 + ss ** 2 + 1e-30)
    z_whole = np.abs(wb - ws) / np.sqrt(swb ** 2 + sws ** 2)
    assert z_blocks.max() < 5.0, z_blocks.max()
    assert z_whole.max() < 5.0, (wb, ws)


def test_batch_runs_other_passes_and_validates(cuda_ctx, scenes3):
    ds = scenes3[0]
    W = H = 16
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    state = [5]
    ls = np.stack([render.generate_light_samples(ds, state, 256) for _ in range(2)])
    # the Whitted ray tracer runs after the fused jobs, one call per job
    wt = render.Image(cuda_ctx, W, H)
    render.render_batch(cuda_ctx, [dict(scene=ds, camera=cam, image=wt, pass_="WHITTED", samples=2,
                                         max_path_length=4, num_light_samples=256, light_samples=ls)])
    ref = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, ref, "WHITTED", max_path_length=4, samples=2, num_light_samples=256,
                  light_samples=ls)
    assert np.allclose(wt.read(), ref.read(), rtol=1e-5, atol=1e-6 * np.abs(ref.read()).max())
    assert wt.read()[..., :3].mean() > 0
    # so does the importon map light tracer, from its cleared G-buffer at iteration 0
    lsi = np.ascontiguousarray(ls[:, :128])
    im = render.Image(cuda_ctx, W, H)
    render.render_batch(cuda_ctx, [dict(scene=ds, camera=cam, image=im, pass_="IM", samples=2, max_path_length=4,
                                         num_light_samples=128, light_samples=lsi)])
    refi = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, refi, "IM", max_path_length=4, samples=2, num_light_samples=128,
                  light_samples=lsi)
    assert np.allclose(im.read(), refi.read(), rtol=1e-4, atol=1e-5 * np.abs(refi.read()).max())
    assert im.read()[..., :3].mean() > 0
    # an image larger than the path queue is refused
    render.set_batch_config(cuda_ctx, 1024, True)
    big = render.Image(cuda_ctx, 64, 64)
    with pytest.raises(cuda.GpugiError):
        render.render_batch(cuda_ctx, [dict(scene=ds, camera=render.camera_lookat(*scenes.CORNELL_CAMERA, 64, 64),
                                            image=big, rng_state=[1])])
    # so is an LT sample whose particles and light-sample connections do not fit
    # (16 light samples x 64 particles + 16 camera connections > 1024)
    with pytest.raises(cuda.GpugiError):
        render.render_batch(cuda_ctx, [dict(scene=ds, camera=cam, image=wt, pass_="LT", num_light_samples=16,
                                            rng_state=[1])])
    render.set_batch_config(cuda_ctx)
    for x in (wt, ref, big):
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
