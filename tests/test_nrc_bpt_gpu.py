"""Bidirectional path tracing with the radiance cache (gpugi_render_nrc with
the BPT pass) on the GPU.

Render eye paths stop at vertex terminateDepth. Paths with at most that
many bounces keep every BPT strategy and its MIS weight (light-cache
connections and the light tracer's camera splats are limited to that
length); the radiance of all longer paths comes from the cache query at
the last vertex, weighted by the eye throughput without MIS factors.
Training paths are extra PT paths that only feed the cache. The reference
has no radiance cache; the pass is checked against the estimators that are
themselves checked against the oracle (test_render_gpu.py):
  * terminateDepth >= maxPathLength: no query, the pass is BPT;
  * a zero cache at terminateDepth k: BPT with the cache and PT with the
    cache both estimate the image of paths with at most k bounces, each
    with its own strategies; their ratio is that of plain BPT and PT (the
    reference's BPT weights are heuristic, so that ratio is not 1);
  * after online training the cache supplies the energy of the longer
    paths: the mean is within 5 % of converged BPT, where the zero cache
    misses a large share.
The light cache is filled by atomic appends, so BPT images vary with the
append order: comparisons are statistical, by block means over independent
batches.
"""
import numpy as np
import pytest

from gpugi_gb300 import bvh, cuda, nrc, render, scenes

pytestmark = pytest.mark.gpu

ROOM_BOX = ((-1.05, -0.05, -1.05), (1.05, 2.05, 1.05))
W = H = 32
BLOCK = 8


@pytest.fixture(scope="module")
def room(cuda_ctx):
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]),
                               sc["materials"])
    yield ds
    ds.close()


def _blocks(rgb):
    """Luminance-weighted block means of an (H, W, 3) image."""
    lum = rgb @ np.array([0.2126, 0.7152, 0.0722])
    return lum.reshape(H // BLOCK, BLOCK, W // BLOCK, BLOCK).mean((1, 3)).ravel()


def _batches(ctx, draw, n_batches, spp):
    """Block means of n_batches independent renders of spp samples each."""
    out = []
    for k in range(n_batches):
        img = render.Image(ctx, W, H, fp64=True)
        draw(img, k)
        out.append(_blocks(img.read64() / spp))
        img.close()
    return np.array(out)


def _agree(a, b, z_max=5.0):
    """Block means of two estimators agree within z_max of their batch noise."""
    ma, mb = a.mean(0), b.mean(0)
    se = np.sqrt(a.var(0, ddof=1) / a.shape[0] + b.var(0, ddof=1) / b.shape[0]) + 1e-12
    z = (ma - mb) / se
    assert np.abs(z).max() < z_max, (z, ma, mb)
    assert abs(ma.mean() / mb.mean() - 1.0) < 0.03, (ma.mean(), mb.mean())


def test_without_lookups_the_pass_is_bpt(cuda_ctx, room):
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    cache = nrc.RadianceCache(cuda_ctx, *ROOM_BOX, seed=2)
    spp, depth = 32, 6

    def bpt(img, k):
        render.render(cuda_ctx, room, cam, img, "BPT", max_path_length=depth, samples=spp, iteration=1000 * k,
                      rng_state=[100 + k])

    def nrc_bpt(img, k):
        nrc.render_nrc(cuda_ctx, room, cam, img, cache, pass_="BPT", max_path_length=depth, samples=spp,
                       iteration=1000 * k, rng_state=[100 + k], terminate_depth=depth, train=False,
                       samples_per_frame=8)

    _agree(_batches(cuda_ctx, nrc_bpt, 8, spp), _batches(cuda_ctx, bpt, 8, spp))
    assert cuda_ctx.device_error_bits() == 0
    cache.close()


@pytest.mark.parametrize("td", [1, 2])
def test_zero_cache_keeps_bpt_for_paths_up_to_the_terminating_vertex(cuda_ctx, room, td):
    """With the cache returning 0, BPT with the cache renders the paths of at
    most td bounces with BPT's strategies, PT with the cache the same paths
    with PT's (emission and NEE up to vertex td). The reference's BPT uses
    heuristic MIS weights (InitialMIS = 1, lightcache.glsl:58-88), so plain
    BPT and plain PT differ by a few percent here; the truncated passes must
    keep that same ratio. A missing cap (longer paths added on top of the
    cache) or a cap one vertex short (strategies of td-bounce paths lost)
    would move it by 10 % or more."""
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    cache = nrc.RadianceCache(cuda_ctx, *ROOM_BOX, seed=3)
    cache.set_weights(np.zeros(nrc.PARAMS, np.float32))
    spp, depth = 32, 8

    def plain(pass_):
        def draw(img, k):
            render.render(cuda_ctx, room, cam, img, pass_, max_path_length=depth, samples=spp, iteration=1000 * k,
                          rng_state=[5 + k])
        return draw

    def truncated(pass_):
        def draw(img, k):
            nrc.render_nrc(cuda_ctx, room, cam, img, cache, pass_=pass_, max_path_length=depth, samples=spp,
                           iteration=5000 + 1000 * k, rng_state=[300 + k], terminate_depth=td, train=False,
                           train_fraction=0.0, samples_per_frame=8)
        return draw

    ratio_plain = _batches(cuda_ctx, plain("BPT"), 8, spp).mean() / _batches(cuda_ctx, plain("PT"), 8, spp).mean()
    bpt_td = _batches(cuda_ctx, truncated("BPT"), 8, spp).mean()
    pt_td = _batches(cuda_ctx, truncated("PT"), 8, spp).mean()
    assert abs(bpt_td / pt_td - ratio_plain) < 0.02, (bpt_td / pt_td, ratio_plain)
    # and the truncation removes a large share of the energy at vertex 1
    if td == 1:
        full = _batches(cuda_ctx, plain("PT"), 4, spp).mean()
        assert pt_td < 0.9 * full, (pt_td, full)
    assert cuda_ctx.device_error_bits() == 0
    cache.close()


def test_trained_cache_restores_the_longer_paths(cuda_ctx, room):
    """Camera looking down at the floor, the light out of view, where
    indirect light is a large share of the image."""
    cam = render.camera_lookat((0.0, 1.2, 2.0), (0.0, 0.0, -0.3), (0.0, 1.0, 0.0), 40.0, W, H)
    depth, td, spp = 8, 1, 16
    conv = render.Image(cuda_ctx, W, H, fp64=True)
    n_ref = 1024
    render.render(cuda_ctx, room, cam, conv, "BPT", max_path_length=depth, samples=n_ref, iteration=1 << 20,
                  rng_state=[99])
    ref_mean = _blocks(conv.read64() / n_ref).mean()

    cache = nrc.RadianceCache(cuda_ctx, *ROOM_BOX, seed=5)
    opts = dict(pass_="BPT", max_path_length=depth, terminate_depth=td, samples_per_frame=4)
    zero = render.Image(cuda_ctx, W, H, fp64=True)
    cache_zero = nrc.RadianceCache(cuda_ctx, *ROOM_BOX, seed=5)
    cache_zero.set_weights(np.zeros(nrc.PARAMS, np.float32))
    nrc.render_nrc(cuda_ctx, room, cam, zero, cache_zero, samples=spp, iteration=30000, rng_state=[21],
                   train=False, **opts)
    zero_mean = _blocks(zero.read64() / spp).mean()

    warm = render.Image(cuda_ctx, W, H)
    nrc.render_nrc(cuda_ctx, room, cam, warm, cache, samples=800, iteration=10000, rng_state=[11],
                   train_fraction=1.0, train_steps=4, **opts)
    img = render.Image(cuda_ctx, W, H, fp64=True)
    nrc.render_nrc(cuda_ctx, room, cam, img, cache, samples=spp, iteration=20000, rng_state=[13], train=False,
                   **opts)
    got_mean = _blocks(img.read64() / spp).mean()
    assert zero_mean < 0.85 * ref_mean, (zero_mean, ref_mean)
    assert abs(got_mean / ref_mean - 1.0) < 0.05, (got_mean, ref_mean, zero_mean)
    assert cuda_ctx.device_error_bits() == 0
    for x in (conv, zero, warm, img, cache, cache_zero):
        x.close()


def test_bpt_cache_rejects_other_passes(cuda_ctx, room):
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    cache = nrc.RadianceCache(cuda_ctx, *ROOM_BOX, seed=2)
    img = render.Image(cuda_ctx, W, H)
    with pytest.raises(ValueError):
        nrc.render_nrc(cuda_ctx, room, cam, img, cache, pass_="LT")
    for x in (img, cache):
        x.close()
