"""Path tracing with the radiance cache (gpugi_render_nrc) on the GPU.

The reference has no radiance cache; the cache is checked against the plain
path tracer (itself checked against the oracle in test_render_gpu.py):
  * with no cache lookups the pass is exactly the path tracer, whether the
    paths are render paths or training paths (atomic splat order aside);
  * on a sky-lit floor whose reflected radiance is known in closed form
    (albedo x sky, every training target is exact) the trained cache
    reproduces it to 5 %;
  * on the Cornell room (light out of view), after online training, 4
    frames with the cache have a lower RMSE against a converged plain-PT
    image than 4 spp of plain PT, and the cache's bias stays small.
"""
import numpy as np
import pytest

from gpugi_gb300 import bvh, cuda, nrc, render, scenes

pytestmark = pytest.mark.gpu

ROOM_BOX = ((-1.05, -0.05, -1.05), (1.05, 2.05, 1.05))


@pytest.fixture(scope="module")
def room(cuda_ctx):
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]),
                               sc["materials"])
    yield sc, b, ds
    ds.close()


def _light_sets(ds, n_sets, n=128, seed=123):
    state = [seed]
    return np.stack([render.generate_light_samples(ds, state, n) for _ in range(n_sets)])


@pytest.mark.parametrize("train_fraction,lanes", [(0.0, 2), (1.0, 2), (1.0, 1), (1.0, 3)])
def test_without_lookups_the_pass_is_plain_pt(cuda_ctx, room, train_fraction, lanes):
    sc, b, ds = room
    W = H = 32
    frames = 4
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(ds, frames)
    ref = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, ref, "PT", max_path_length=6, samples=frames, light_samples=ls)
    cache = nrc.RadianceCache(cuda_ctx, *ROOM_BOX, seed=2)
    img = render.Image(cuda_ctx, W, H)
    # terminate_depth beyond the path length: no render path ever queries
    nrc.render_nrc(cuda_ctx, ds, cam, img, cache, max_path_length=6, samples=frames, light_samples=ls,
                   terminate_depth=6, train_fraction=train_fraction, train=False, lanes=lanes)
    a, r = img.read()[..., :3], ref.read()[..., :3]
    assert np.abs(a - r).max() <= 1e-5 * np.abs(r).max() + 1e-6
    assert cuda_ctx.device_error_bits() == 0
    for x in (img, ref, cache):
        x.close()


def _floor_scene(n=8, albedos=((0.8, 0.4, 0.2), (0.2, 0.5, 0.7))):
    v, f, nrm = scenes._grid_quad((-1.0, 0.0, 1.0), (2.0, 0.0, 0.0), (0.0, 0.0, -2.0), n)
    cell = np.arange(f.shape[0]) % (n * n)
    mat_ids = ((cell // n) + (cell % n)) % 2
    mats = np.stack([scenes.lambert(a) for a in albedos])
    return scenes._pack(v.astype(np.float32), f, mats, material_ids=mat_ids, normals=nrm.astype(np.float32))


def test_cache_learns_sky_lit_floor(cuda_ctx):
    """Lambertian floor under a constant sky: the radiance reflected at any
    floor point is albedo x sky, and every training path's target is
    exactly that (one diffuse bounce, then the sky)."""
    sc = _floor_scene()
    assert np.allclose(sc["normals"][:, 1], 1.0)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]),
                               sc["materials"])
    W = H = 48
    sky = (0.5, 0.7, 1.0)
    cam = render.camera_lookat((0.0, 1.6, 1.2), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0, W, H)
    # one directional light shining from below the floor: never contributes
    ls = np.zeros((1, 4, 8), np.float32)
    ls[..., 1] = -1.0
    ls[..., 7] = 3.0
    ref = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, ref, "PT", max_path_length=2, rr_start_depth=2, samples=1, sky=sky,
                  num_light_samples=4, light_samples=ls)
    expect = ref.read()[..., :3]
    floor = np.abs(expect - np.asarray(sky)).max(-1) > 1e-3
    assert floor.mean() > 0.5
    cache = nrc.RadianceCache(cuda_ctx, (-1.1, -0.1, -1.1), (1.1, 1.1, 1.1), seed=4)
    frames = 150
    nrc.render_nrc(cuda_ctx, ds, cam, render.Image(cuda_ctx, W, H), cache, max_path_length=2, rr_start_depth=2,
                   samples=frames, sky=sky, num_light_samples=4, light_samples=np.repeat(ls, frames, 0),
                   terminate_depth=5, train_fraction=1.0, train_steps=4)
    img = render.Image(cuda_ctx, W, H)
    nrc.render_nrc(cuda_ctx, ds, cam, img, cache, max_path_length=2, rr_start_depth=2, samples=1, sky=sky,
                   num_light_samples=4, light_samples=ls, terminate_depth=0, train_fraction=0.0, train=False)
    got = img.read()[..., :3]
    rel = np.abs(got - expect)[floor] / expect[floor]
    assert np.median(rel) < 0.02 and np.percentile(rel, 95) < 0.05, (np.median(rel), np.percentile(rel, 95))
    assert np.allclose(got[~floor], expect[~floor], rtol=1e-6)
    for x in (img, ref, cache, ds):
        x.close()


def test_cache_beats_plain_pt_at_equal_samples(cuda_ctx, room):
    """Camera looking down at the floor (the light is out of view: directly
    seen emitter edges would dominate both RMSEs with pixel-jitter noise
    that no cache can remove)."""
    sc, b, ds = room
    W = H = 64
    depth = 8
    cam = render.camera_lookat((0.0, 1.2, 2.0), (0.0, 0.0, -0.3), (0.0, 1.0, 0.0), 40.0, W, H)
    conv = render.Image(cuda_ctx, W, H, fp64=True)
    n_ref = 4096
    render.render(cuda_ctx, ds, cam, conv, "PT", max_path_length=depth, samples=n_ref, iteration=1000,
                  rng_state=[99])
    reference = (conv.read64() / n_ref).astype(np.float32)

    spp = 4
    pt = render.Image(cuda_ctx, W, H, fp64=True)
    render.render(cuda_ctx, ds, cam, pt, "PT", max_path_length=depth, samples=spp, rng_state=[7])
    rmse_pt = np.sqrt(pt.mse(spp, reference, use_fp64=True))

    cache = nrc.RadianceCache(cuda_ctx, *ROOM_BOX, seed=5)
    warm = render.Image(cuda_ctx, W, H)
    nrc.render_nrc(cuda_ctx, ds, cam, warm, cache, max_path_length=depth, samples=200, iteration=10000,
                   rng_state=[11], terminate_depth=1, train_fraction=0.25, train_steps=4)
    img = render.Image(cuda_ctx, W, H, fp64=True)
    nrc.render_nrc(cuda_ctx, ds, cam, img, cache, max_path_length=depth, samples=spp, iteration=20000,
                   rng_state=[13], terminate_depth=1, train_fraction=0.25, train_steps=4)
    rmse_nrc = np.sqrt(img.mse(spp, reference, use_fp64=True))
    assert rmse_nrc < 0.85 * rmse_pt, (rmse_nrc, rmse_pt)
    # bias: the cache image's mean stays within 5 % of the converged mean
    mean_nrc = img.read64().mean() / spp
    assert abs(mean_nrc / reference.mean() - 1) < 0.05, (mean_nrc, reference.mean())
    assert cuda_ctx.device_error_bits() == 0
    for x in (conv, pt, warm, img, cache):
        x.close()


def test_spread_termination_brackets_fixed_depth(cuda_ctx, room):
    """Path-spread termination (terminate_spread = c): a vanishing c stops
    every render path at the first vertex it may (vertex 1), a huge c never
    fires, leaving the terminate_depth cap; both equal the fixed-depth pass
    with the same (untrained) cache."""
    sc, b, ds = room
    W = H = 32
    frames = 4
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(ds, frames)
    cache = nrc.RadianceCache(cuda_ctx, *ROOM_BOX, seed=3)

    def run(td, spread):
        img = render.Image(cuda_ctx, W, H)
        nrc.render_nrc(cuda_ctx, ds, cam, img, cache, max_path_length=6, samples=frames, light_samples=ls,
                       terminate_depth=td, train_fraction=0.0, train=False, terminate_spread=spread)
        out = img.read()[..., :3]
        img.close()
        return out

    for a, r in ((run(5, 1e-30), run(1, 0.0)), (run(3, 1e30), run(3, 0.0))):
        assert np.abs(a - r).max() <= 1e-5 * np.abs(r).max() + 1e-6
    mid = run(5, 0.01)  # the paper's c: most paths stop at vertex 1, a few later
    assert np.isfinite(mid).all() and mid.mean() > 0
    assert cuda_ctx.device_error_bits() == 0
    cache.close()


@pytest.mark.parametrize("train_length,unbiased", [(0, 0.0), (2, 1.0 / 16), (2, 0.0)])
def test_self_training_keeps_the_cache_unbiased(cuda_ctx, room, train_length, unbiased):
    """Self-training (training paths take the cache's radiance at vertex
    train_length, 1/16 of them run to the end): the trained cache's image
    keeps its mean near converged PT: within 5 % with full training paths,
    within 10 % with self-training, whose targets inherit the cache's own
    error (6 % low on this room after 300 frames). Dropping or misrouting
    the self-training queries loses the radiance of every bounce after
    train_length at the vertices the render paths query: 15-20 % here."""
    sc, b, ds = room
    W = H = 64
    depth = 8
    cam = render.camera_lookat((0.0, 1.2, 2.0), (0.0, 0.0, -0.3), (0.0, 1.0, 0.0), 40.0, W, H)
    conv = render.Image(cuda_ctx, W, H, fp64=True)
    n_ref = 2048
    render.render(cuda_ctx, ds, cam, conv, "PT", max_path_length=depth, samples=n_ref, iteration=1000,
                  rng_state=[99])
    reference = conv.read64() / n_ref
    cache = nrc.RadianceCache(cuda_ctx, *ROOM_BOX, seed=5)
    opts = dict(max_path_length=depth, terminate_depth=1, train_fraction=0.25, train_steps=4,
                train_length=train_length, unbiased_fraction=unbiased)
    warm = render.Image(cuda_ctx, W, H)
    nrc.render_nrc(cuda_ctx, ds, cam, warm, cache, samples=300, iteration=10000, rng_state=[11], **opts)
    img = render.Image(cuda_ctx, W, H, fp64=True)
    spp = 64
    nrc.render_nrc(cuda_ctx, ds, cam, img, cache, samples=spp, iteration=20000, rng_state=[13], **opts)
    mean_nrc = img.read64().mean() / spp
    assert abs(mean_nrc / reference.mean() - 1) < (0.05 if train_length == 0 else 0.1), (mean_nrc, reference.mean())
    assert cuda_ctx.device_error_bits() == 0
    for x in (conv, warm, img, cache):
        x.close()


def test_cache_bias_stays_below_the_plain_1024_spp_rmse(cuda_ctx, room):
    """The cached image's bias against converged PT (the cache trained, then
    frozen) stays below the RMSE of 1024 spp of plain PT on the same view:
    two independent 256-spp cache images A and B give
    bias^2 = MSE(A) - MSE(A - B) / 2 (the variance of one image is half the
    expected squared difference of two), the reference's own noise
    (16,384 spp) being negligible beside both."""
    sc, b, ds = room
    W = H = 64
    depth = 8
    cam = render.camera_lookat((0.0, 1.2, 2.0), (0.0, 0.0, -0.3), (0.0, 1.0, 0.0), 40.0, W, H)
    conv = render.Image(cuda_ctx, W, H, fp64=True)
    render.render(cuda_ctx, ds, cam, conv, "PT", max_path_length=depth, samples=16384, iteration=1 << 20,
                  rng_state=[99])
    reference = conv.read64() / 16384
    pt = render.Image(cuda_ctx, W, H, fp64=True)
    render.render(cuda_ctx, ds, cam, pt, "PT", max_path_length=depth, samples=1024, iteration=0, rng_state=[7])
    target = np.sqrt(((pt.read64() / 1024 - reference) ** 2).sum(-1).mean())
    cache = nrc.RadianceCache(cuda_ctx, *ROOM_BOX, seed=5)
    opts = dict(max_path_length=depth, terminate_depth=2, train_fraction=0.25, train_steps=4, samples_per_frame=4)
    warm = render.Image(cuda_ctx, W, H)
    nrc.render_nrc(cuda_ctx, ds, cam, warm, cache, samples=1200, iteration=10000, rng_state=[11], **opts)
    spp = 256
    imgs = []
    for k in range(2):
        img = render.Image(cuda_ctx, W, H, fp64=True)
        nrc.render_nrc(cuda_ctx, ds, cam, img, cache, samples=spp, iteration=20000 + 10000 * k, rng_state=[13 + k],
                       train=False, **dict(opts, train_fraction=0.0))
        imgs.append(img.read64() / spp)
        img.close()
    a, bb = imgs
    mse_a = ((a - reference) ** 2).sum(-1).mean()
    var_a = ((a - bb) ** 2).sum(-1).mean() / 2
    bias = np.sqrt(max(mse_a - var_a, 0.0))
    assert bias < target, (bias, target, np.sqrt(mse_a))
    assert cuda_ctx.device_error_bits() == 0
    for x in (conv, pt, warm, cache):
        x.close()
