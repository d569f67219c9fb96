"""GPU wavefront renderers (PT, LT, BPT) against the oracle, through the C ABI.

The oracle and the kernels draw the same per-path RNG streams in the same
order (PCG by default; wanghash seeds + xorshift32 in the reference mode) on
bit-identical hierarchies, and take the
same light-sample arrays. Shading uses CUDA's sinf/cosf/powf instead of the C
library's, so values differ in the last bits and a path may eventually branch
differently; the bars are therefore:
  * depth-1 PT (emission + NEE at the first hit): per-pixel relative error
    below 1e-4 of the image maximum (near bit-identical paths);
  * full-depth PT / LT / BPT: image means within 2 %, 8x8-block means within
    a statistical bound estimated from four independent batches;
  * the Whitted ray tracer (every pixel of a frame on the same RNG stream,
    specular/glossy bounces until the first diffuse decision, two NEE
    samples there): per-pixel agreement on a room with a glossy sphere and
    box, as for depth-1 PT except for the few pixels whose glossy bounce the
    rounding of powf/sinf diverts.
"""
import numpy as np
import pytest

import oracle
from gpugi_gb300 import bvh, cuda, render, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def room(cuda_ctx):
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]),
                               sc["materials"])
    yield sc, b, ds
    ds.close()


def _light_sets(ds, n_sets, n, seed=123):
    state = [seed]
    return np.stack([render.generate_light_samples(ds, state, n) for _ in range(n_sets)])


def _oracle(b, sc, pass_, W, H, cam, ls, iters, first=0, rng="pcg", **kw):
    acc = None
    for s in range(iters):
        acc = oracle.render(b, sc, pass_, W, H, cam.as_array(), render.frame_seed(first + s, rng), ls[s], accum=acc,
                            rng=rng, **kw)
    return acc


def test_light_sampler_matches_scene_lights(cuda_ctx, room):
    sc, b, ds = room
    ls = render.generate_light_samples(ds, [123], 128)
    assert np.all(ls[:, 7] < 1.5)  # area-light samples (normal.z of a downward light is 0)
    assert np.allclose(ls[:, 1], 1.999 - 1e-4, atol=1e-6)
    assert (np.abs(ls[:, 0]) <= 0.25 + 1e-6).all() and (np.abs(ls[:, 2]) <= 0.25 + 1e-6).all()
    # each sample carries luminance * area / n = 10 * 0.25 / 128
    assert np.allclose(ls[:, 4:7], 10.0 * 0.25 / 128, rtol=1e-5)


@pytest.mark.parametrize("rng", ["pcg", "reference"])
def test_pt_direct_light_matches_oracle(cuda_ctx, room, rng):
    sc, b, ds = room
    W = H = 48
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(ds, 4, 128)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img, "PT", max_path_length=1, samples=4, iteration=0, light_samples=ls, rng=rng)
    g = img.read()
    o = _oracle(b, sc, "PT", W, H, cam, ls, 4, max_path_length=1, rng=rng)
    err = np.abs(g[..., :3] - o[..., :3])
    assert err.max() <= 1e-4 * np.abs(o[..., :3]).max() + 1e-6
    img.close()


def _stat_compare(g_batches, o_img, tol_mean=0.02, z=6.0):
    """g_batches: (K, H, W, 3) per-batch means; o_img: oracle mean image."""
    g = g_batches.mean(0)
    assert abs(g.mean() / o_img.mean() - 1) < tol_mean, (g.mean(), o_img.mean())
    K = g_batches.shape[0]
    H, W = g.shape[:2]
    blk = lambda a: a[..., : H // 8 * 8, : W // 8 * 8, :].reshape(*a.shape[:-3], H // 8, 8, W // 8, 8, 3).mean((-4, -2))
    gb = blk(g_batches)                          # (K, h, w, 3)
    se = gb.std(0, ddof=1) / np.sqrt(K)          # standard error of the GPU block mean
    d = np.abs(gb.mean(0) - blk(o_img[None])[0])
    assert (d <= z * np.sqrt(2) * se + 1e-3 * np.abs(gb.mean(0)) + 1e-5).mean() > 0.97


@pytest.mark.parametrize("pass_,iters,rng", [("PT", 32, "pcg"), ("BPT", 32, "pcg"), ("LT", 48, "pcg"),
                                             ("PT", 32, "reference"), ("BPT", 32, "reference"),
                                             ("LT", 48, "reference")])
def test_full_depth_passes_match_oracle(cuda_ctx, room, pass_, iters, rng):
    sc, b, ds = room
    W = H = 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    nls = render.DEFAULT_LIGHT_SAMPLES[pass_]
    ls = _light_sets(ds, iters, nls)
    K = 4
    per = iters // K
    batches = []
    for k in range(K):
        img = render.Image(cuda_ctx, W, H)
        render.render(cuda_ctx, ds, cam, img, pass_, max_path_length=6, samples=per, iteration=k * per,
                      light_samples=ls[k * per:(k + 1) * per], rng=rng)
        batches.append(img.read()[..., :3] / per)
        img.close()
    o = _oracle(b, sc, pass_, W, H, cam, ls, iters, max_path_length=6, rng=rng)[..., :3] / iters
    _stat_compare(np.stack(batches), o, tol_mean=0.03)
    assert cuda_ctx.device_error_bits() == 0


def test_bpt_counts_iterations_in_alpha(cuda_ctx, room):
    sc, b, ds = room
    W = H = 16
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img, "BPT", max_path_length=4, samples=3, rng_state=[7])
    assert np.all(img.read()[..., 3] == 3.0)  # pathtracer_bidir.comp:248 writes vec4(color, 1)
    img.close()


def test_fp64_accumulation_and_mse(cuda_ctx, room):
    sc, b, ds = room
    W = H = 24
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    img = render.Image(cuda_ctx, W, H, fp64=True)
    render.render(cuda_ctx, ds, cam, img, "PT", max_path_length=4, samples=16, rng_state=[5])
    f32 = img.read()[..., :3].astype(np.float64)
    f64 = img.read64()
    assert np.allclose(f32, f64, rtol=1e-4, atol=1e-5)
    ref = (f64 / 16 * 0.9).astype(np.float32)
    expect = ((f64 / 16 - ref.astype(np.float64)) ** 2).sum(-1).mean()
    assert abs(img.mse(16, ref, use_fp64=True) / expect - 1) < 1e-9
    assert abs(img.mse(16, ref, use_fp64=False) / expect - 1) < 1e-3
    img.close()


def test_ray_counts_and_rr(cuda_ctx, room):
    sc, b, ds = room
    W = H = 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img, "PT", max_path_length=8, samples=2, rng_state=[3])
    closest, shadow = render.ray_counts(cuda_ctx)
    assert closest >= 2 * W * H and closest <= 8 * 2 * W * H
    assert 0 < shadow <= closest
    # Russian roulette only after depth 3 keeps more paths alive
    render.render(cuda_ctx, ds, cam, img, "PT", max_path_length=8, samples=2, rr_start_depth=3, rng_state=[3])
    closest_rr3, _ = render.ray_counts(cuda_ctx)
    assert closest_rr3 > closest
    img.close()


@pytest.mark.parametrize("pass_", ["PT", "BPT", "LT"])
def test_converged_image_matches_oracle_per_pixel(cuda_ctx, pass_):
    """Per-pixel radiance parity: the GPU's FP64-accumulated 65,536-iteration
    image against the oracle's 2,048-iteration estimate, in 32 batches whose
    spread gives each pixel's standard error. Pixel values are heavy-tailed
    (NEE near the light, partly covered light pixels), so the statistics are
    robust ones: for unbiased renderers the median of z^2 is about 0.45 (a
    bias of one standard error everywhere would make it about 1.4), and
    fewer than 2 % of the pixel channels lie beyond 4.5 sigma."""
    sc = scenes.cornell_room(seed=4, sphere_level=2, wall_grid=4)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]), sc["materials"])
    W = H = 12
    depth = 5
    cam = render.camera_lookat((0.0, 1.0, 3.0), (0.0, 0.9, 0.0), (0.0, 1.0, 0.0), 45.0, W, H)
    n_gpu = 65536
    img = render.Image(cuda_ctx, W, H, fp64=True)
    render.render(cuda_ctx, ds, cam, img, pass_, max_path_length=depth, samples=n_gpu, iteration=1 << 20,
                  rng_state=[77])
    g = img.read64() / n_gpu
    nls = render.DEFAULT_LIGHT_SAMPLES[pass_]
    K, per = 32, 64
    st = [5]
    batches = []
    for k in range(K):
        acc = None
        for s in range(per):
            ls = render.generate_light_samples(ds, st, nls)
            acc = oracle.render(b, sc, pass_, W, H, cam.as_array(), render.frame_seed(k * per + s), ls,
                                max_path_length=depth, accum=acc)
        batches.append(acc[..., :3].astype(np.float64) / per)
    batches = np.stack(batches)
    o = batches.mean(0)
    se = batches.std(0, ddof=1) / np.sqrt(K)
    live = se > 0  # channels that receive light
    z = (g - o)[live] / se[live]
    assert np.median(z ** 2) < 1.0, np.median(z ** 2)
    assert (np.abs(z) > 4.5).mean() < 0.02, (np.abs(z) > 4.5).mean()
    assert abs(g.mean() / o.mean() - 1) < 0.03, (g.mean(), o.mean())
    img.close()
    ds.close()


@pytest.fixture(scope="module")
def glossy_room(cuda_ctx):
    """The Cornell room with a glossy sphere (specular 0.8, exponent ~1100)
    and a glossy tall box (specular 0.5, exponent 25)."""
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8)
    mats = sc["materials"].reshape(-1, 24).copy()
    mats[7] = scenes.material_record(albedo=(0.1, 0.1, 0.1), specular=(0.8, 0.8, 0.8), roughness=0.03)
    mats[5] = scenes.material_record(albedo=(0.3, 0.4, 0.5), specular=(0.5, 0.5, 0.5), roughness=0.2)
    sc = dict(sc, materials=mats)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]), mats)
    yield sc, b, ds
    ds.close()


def test_whitted_matches_oracle_per_pixel(cuda_ctx, glossy_room):
    sc, b, ds = glossy_room
    W = H = 48
    iters = 8
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(ds, iters, 128)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img, "WHITTED", max_path_length=6, samples=iters, iteration=0,
                  light_samples=ls)
    g = img.read()
    o = _oracle(b, sc, "WHITTED", W, H, cam, ls, iters, max_path_length=6)
    assert np.all(g[..., 3] == iters) and np.all(o[..., 3] == iters)  # vec4(color, 1.0) per iteration
    close = np.abs(g[..., :3] - o[..., :3]) <= 1e-4 * np.abs(o[..., :3]).max() + 1e-6
    assert close.all(-1).mean() > 0.97, close.all(-1).mean()
    assert abs(g[..., :3].mean() / o[..., :3].mean() - 1) < 0.01
    # the glossy bounces are taken: some paths end on a diffuse decision after
    # a specular one (the sphere shows the room)
    img2 = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img2, "WHITTED", max_path_length=1, samples=iters, iteration=0,
                  light_samples=ls)
    assert np.abs(img2.read()[..., :3] - g[..., :3]).max() > 1e-3
    assert cuda_ctx.device_error_bits() == 0
    for x in (img, img2):
        x.close()


def test_photon_mapper_matches_oracle_per_pixel(cuda_ctx, glossy_room):
    """PhotonMapper (photondistribution.comp + gather.comp) at its defaults,
    2048 photons per light sample and query radius 0.01: the GPU and the
    oracle trace the same photons (same seeds, bit-identical walks) into the
    same grid cells; a gather sums a handful of photons, so a pixel differs
    when rounding diverts one of them."""
    sc, b, ds = glossy_room
    W = H = 48
    iters = 4
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(ds, iters, 128)
    render.set_photon_config(cuda_ctx, 2048, 0.01)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img, "PM", max_path_length=6, samples=iters, iteration=0, light_samples=ls)
    g = img.read()
    o = _oracle(b, sc, "PM", W, H, cam, ls, iters, max_path_length=6)
    assert np.all(g[..., 3] == iters) and np.all(o[..., 3] == iters)
    close = np.abs(g[..., :3] - o[..., :3]) <= 1e-3 * np.abs(o[..., :3]).max() + 1e-5
    assert close.all(-1).mean() > 0.9, close.all(-1).mean()
    assert abs(g[..., :3].mean() / o[..., :3].mean() - 1) < 0.02, (g[..., :3].mean(), o[..., :3].mean())
    assert cuda_ctx.device_error_bits() == 0
    img.close()


def test_photon_mapper_converges_to_path_tracing(cuda_ctx, room):
    """On the diffuse room the photon-map estimate (radius 0.02, 4096 photons
    per light sample) approaches the path-traced image: a density estimate
    biased by its kernel, so image means agree to a few percent."""
    sc, b, ds = room
    W = H = 32
    cam = render.camera_lookat((0.0, 1.2, 2.0), (0.0, 0.0, -0.3), (0.0, 1.0, 0.0), 40.0, W, H)
    render.set_photon_config(cuda_ctx, 4096, 0.02)
    pm = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, pm, "PM", max_path_length=8, samples=32, rng_state=[3])
    pt = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, pt, "PT", max_path_length=8, samples=256, rng_state=[4])
    a, r = pm.read()[..., :3].mean() / 32, pt.read()[..., :3].mean() / 256
    assert abs(a / r - 1) < 0.08, (a, r)
    render.set_photon_config(cuda_ctx)
    for x in (pm, pt):
        x.close()


def _oracle_im(b, sc, W, H, cam, ls, iters, **kw):
    acc, gbuf = None, np.zeros((H, W, 5), np.float32)
    for s in range(iters):
        acc = oracle.render(b, sc, "IM", W, H, cam.as_array(), render.frame_seed(s), ls[s], accum=acc, gbuffer=gbuf,
                            **kw)
    return acc


def test_importon_map_matches_oracle_per_pixel(cuda_ctx, glossy_room):
    """PixelMapLighttracer (importondistribution.comp + photontracing.comp)
    at its defaults, 2048 photons per light sample and query radius 0.005:
    the eye paths store the same importons (bit-identical walks, the same
    packed throughputs and directions), the photons gather them and
    reproject against the same G-buffer; a pixel differs when rounding
    diverts a photon, so most pixels agree to 1e-3 of the image maximum."""
    sc, b, ds = glossy_room
    W = H = 48
    iters = 4
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(ds, iters, 128)
    render.set_importon_config(cuda_ctx, 2048, 0.005)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img, "IM", max_path_length=6, samples=iters, iteration=0, light_samples=ls)
    g = img.read()
    o = _oracle_im(b, sc, W, H, cam, ls, iters, max_path_length=6, photons_per_light_sample=2048,
                   query_radius=0.005)
    assert np.all(g[..., 3] == iters) and np.all(o[..., 3] == iters)
    close = np.abs(g[..., :3] - o[..., :3]) <= 1e-3 * np.abs(o[..., :3]).max() + 1e-5
    assert close.all(-1).mean() > 0.9, close.all(-1).mean()
    assert abs(g[..., :3].mean() / o[..., :3].mean() - 1) < 0.02, (g[..., :3].mean(), o[..., :3].mean())
    assert cuda_ctx.device_error_bits() == 0
    img.close()


def test_importon_map_converges_to_path_tracing(cuda_ctx, glossy_room):
    """On the glossy room the importon-map image (reprojected light paths
    plus importons behind the glossy bounces, radius 0.02) approaches the
    path-traced image: image means within a few percent."""
    sc, b, ds = glossy_room
    W = H = 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    render.set_importon_config(cuda_ctx, 4096, 0.02)
    im = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, im, "IM", max_path_length=8, samples=32, rng_state=[3])
    pt = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, pt, "PT", max_path_length=8, samples=256, rng_state=[4])
    a, r = im.read()[..., :3].mean() / 32, pt.read()[..., :3].mean() / 256
    assert abs(a / r - 1) < 0.08, (a, r)
    render.set_importon_config(cuda_ctx)
    assert cuda_ctx.device_error_bits() == 0
    for x in (im, pt):
        x.close()


def test_importon_share_matches_oracle(cuda_ctx, glossy_room):
    """The light the importons carry (the image with a radius that finds
    importons minus the image with one that finds none, on the same seeds
    and light samples) equals the oracle's share on the same inputs: a pass
    that dropped or misplaced importon gathers (wrong cell, side test or
    pixel unpacking) would lose most of it."""
    sc, b, ds = glossy_room
    W = H = 32
    iters = 4
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(ds, iters, 128, seed=77)
    means = {}
    for radius in (0.02, 1e-6):  # 1e-6: no importon within reach
        render.set_importon_config(cuda_ctx, 1024, radius)
        img = render.Image(cuda_ctx, W, H)
        render.render(cuda_ctx, ds, cam, img, "IM", max_path_length=8, samples=iters, iteration=0, light_samples=ls)
        g = img.read()[..., :3].mean()
        img.close()
        o = _oracle_im(b, sc, W, H, cam, ls, iters, max_path_length=8, photons_per_light_sample=1024,
                       query_radius=radius)[..., :3].mean()
        means[radius] = (g, o)
    render.set_importon_config(cuda_ctx)
    share_g = 1 - means[1e-6][0] / means[0.02][0]
    share_o = 1 - means[1e-6][1] / means[0.02][1]
    assert share_o > 0.005, share_o  # the importons carry light on this scene
    assert abs(share_g - share_o) < 0.1 * share_o + 1e-3, (share_g, share_o)
    assert cuda_ctx.device_error_bits() == 0


def test_importon_config_validation_and_progressive_radius(cuda_ctx, room):
    sc, b, ds = room
    for bad in ((0, 0.01), (1 << 21, 0.01), (2048, 0.0), (2048, float("nan"))):
        with pytest.raises(cuda.GpugiError):
            render.set_importon_config(cuda_ctx, *bad)
    W = H = 24
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    render.set_importon_config(cuda_ctx, 512, 0.05, progressive=True)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img, "IM", max_path_length=4, samples=6, iteration=3, rng_state=[1])
    g = img.read()
    assert np.all(g[..., 3] == 6) and np.isfinite(g).all() and g[..., :3].mean() > 0
    assert cuda_ctx.device_error_bits() == 0
    render.set_importon_config(cuda_ctx)
    img.close()


def test_photon_config_validation_and_progressive_radius(cuda_ctx, room):
    sc, b, ds = room
    for bad in ((0, 0.01), (1 << 21, 0.01), (2048, 0.0), (2048, float("nan"))):
        with pytest.raises(cuda.GpugiError):
            render.set_photon_config(cuda_ctx, *bad)
    W = H = 24
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    render.set_photon_config(cuda_ctx, 512, 0.05, progressive=True)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img, "PM", max_path_length=4, samples=6, iteration=3, rng_state=[1])
    g = img.read()
    assert np.all(g[..., 3] == 6) and np.isfinite(g).all() and g[..., :3].mean() > 0
    assert cuda_ctx.device_error_bits() == 0
    render.set_photon_config(cuda_ctx)
    img.close()


def test_passes_on_oriented_box_hierarchy(cuda_ctx):
    """The passes walk an oriented-box hierarchy (OBOX_BVH) like a box one:
    depth-1 PT equals the oracle per pixel, and full-depth PT and LT images
    equal those of the box hierarchy of the same scene (same seeds and light
    samples; the closest hits are the same triangles)."""
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8)
    bo = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", fit="obox")
    ba = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    vi = cuda.vertex_info(sc["normals"], sc["texcoords"])
    do = cuda_ctx.upload_scene(bo, sc["positions"], vi, sc["materials"])
    da = cuda_ctx.upload_scene(ba, sc["positions"], vi, sc["materials"])
    W = H = 40
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(do, 4, 128)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, do, cam, img, "PT", max_path_length=1, samples=4, light_samples=ls)
    g = img.read()
    o = _oracle(bo, sc, "PT", W, H, cam, ls, 4, max_path_length=1)
    assert np.abs(g[..., :3] - o[..., :3]).max() <= 1e-4 * np.abs(o[..., :3]).max() + 1e-6
    img.close()
    for pass_ in ("PT", "LT"):
        nls = render.DEFAULT_LIGHT_SAMPLES[pass_]
        ls = _light_sets(do, 8, nls, seed=9)
        imgs = []
        for ds in (do, da):
            im = render.Image(cuda_ctx, W, H)
            render.render(cuda_ctx, ds, cam, im, pass_, max_path_length=6, samples=8, light_samples=ls)
            imgs.append(im.read()[..., :3])
            im.close()
        close = np.abs(imgs[0] - imgs[1]) <= 1e-3 * np.abs(imgs[1]).max() + 1e-5
        assert close.all(-1).mean() > 0.98, (pass_, close.all(-1).mean())
        assert abs(imgs[0].mean() / imgs[1].mean() - 1) < 0.01
    assert cuda_ctx.device_error_bits() == 0
    do.close()
    da.close()
