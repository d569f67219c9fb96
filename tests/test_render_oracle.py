"""Analytic checks of the oracle's restated rendering passes (CPU only).

The reference has no image tests; these pin the restated shader math against
closed-form radiometry on tiny scenes:
  * a camera looking straight at an emissive quad sees its emissivity
    (pathtracer.comp:77-78: emission counts before any NEE);
  * a Lambertian floor under a point light shows albedo/pi * I cos / d^2
    (lightsource.glsl:25-55 with BSDF = albedo/pi);
  * the light tracer, path tracer and BPT converge to the same image on a
    diffuse room (the reference's renderer-comparison practice);
  * the Whitted ray tracer on that floor (a diffuse decision at the first
    hit, two NEE samples weighted 128 / 2) shows the same radiance, with its
    pixel jitter in [x, x + 1) (whittedraytracer.comp:24, no -0.5);
  * the importon map light tracer on that floor (no importons: the eye
    paths end at their first, diffuse, hit) is the photons' reprojection
    alone, and the G-buffer plane test passes every visible floor point.
"""
import math

import numpy as np
import pytest

import oracle
from gpugi_gb300 import bvh, render, scenes


def _quad_scene(albedo=0.5, emission=0.0, size=4.0):
    v, f, n = scenes._grid_quad((-size / 2, 0.0, -size / 2), (0, 0, size), (size, 0, 0), 8)  # y = 0, normal +y
    mat = scenes.material_record(albedo=(albedo,) * 3, specular=(0.0, 0.0, 0.0), emissivity=(emission,) * 3)
    return scenes._pack(v, f, [mat], normals=n)


def _point_light_samples(pos, intensity, n=128):
    """Light samples of one point light, as LightSampler writes them
    (lightsampler.cpp:77-94: normalThetaCos = 2, intensity / (n * 1))."""
    ls = np.zeros((n, 8), np.float32)
    ls[:, 0:3] = pos
    ls[:, 4:7] = np.asarray(intensity, np.float32) / n
    ls[:, 7] = 2.0
    return ls


def test_direct_emission_seen_by_camera(built):
    sc = _quad_scene(albedo=0.0, emission=3.0)
    b = bvh.build_bvh(sc["positions"], sc["triangles"])
    cam = render.camera_lookat((0.0, 1.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 30.0, 16, 16)
    ls = np.zeros((128, 8), np.float32)  # black dummy lights
    img = oracle.render(b, sc, "PT", 16, 16, cam.as_array(), render.frame_seed(0), ls, max_path_length=4)
    assert np.allclose(img[..., :3], 3.0, rtol=1e-6)


def test_point_light_on_lambert_floor(built):
    albedo, I, h = 0.6, 5.0, 1.5
    sc = _quad_scene(albedo=albedo)
    b = bvh.build_bvh(sc["positions"], sc["triangles"])
    W = H = 24
    cam = render.camera_lookat((0.0, 3.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 40.0, W, H)
    ls = _point_light_samples((0.0, h, 0.0), (I, I, I))
    # depth 1: only the first hit's NEE contributes (no emission anywhere)
    acc = None
    iters = 16
    for it in range(iters):
        acc = oracle.render(b, sc, "PT", W, H, cam.as_array(), render.frame_seed(it), ls, max_path_length=1, accum=acc)
    img = acc[..., 0] / iters
    # expected radiance at the floor point seen through each pixel centre (jitter averages out)
    c = cam.as_array()
    U, V, Wd, P = c[0:3], c[3:6], c[6:9], c[9:12]
    ys, xs = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    sx = xs / W * 2 - 1
    sy = ys / H * 2 - 1
    d = sx[..., None] * U + sy[..., None] * V + Wd
    t = -P[1] / d[..., 1]
    p = P + t[..., None] * d
    r2 = p[..., 0] ** 2 + (h - p[..., 1]) ** 2 + p[..., 2] ** 2 + 1e-5
    cos = h / np.sqrt(r2)
    expected = albedo / math.pi * I * cos / r2
    inner = (np.abs(p[..., 0]) < 1.5) & (np.abs(p[..., 2]) < 1.5)
    rel = np.abs(img - expected)[inner] / expected[inner]
    assert np.median(rel) < 0.02
    assert rel.max() < 0.15  # pixel footprint averaging


def test_whitted_point_light_on_lambert_floor(built):
    albedo, I, h = 0.6, 5.0, 1.5
    sc = _quad_scene(albedo=albedo)
    b = bvh.build_bvh(sc["positions"], sc["triangles"])
    W = H = 24
    cam = render.camera_lookat((0.0, 3.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 40.0, W, H)
    ls = _point_light_samples((0.0, h, 0.0), (I, I, I))
    acc = None
    iters = 32
    for it in range(iters):
        acc = oracle.render(b, sc, "WHITTED", W, H, cam.as_array(), render.frame_seed(it), ls, max_path_length=4,
                            accum=acc)
    assert np.all(acc[..., 3] == iters)
    img = acc[..., 0] / iters
    c = cam.as_array()
    U, V, Wd, P = c[0:3], c[3:6], c[6:9], c[9:12]
    ys, xs = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    sx = (xs + 0.5) / W * 2 - 1
    sy = (ys + 0.5) / H * 2 - 1
    d = sx[..., None] * U + sy[..., None] * V + Wd
    t = -P[1] / d[..., 1]
    p = P + t[..., None] * d
    r2 = p[..., 0] ** 2 + (h - p[..., 1]) ** 2 + p[..., 2] ** 2 + 1e-5
    cos = h / np.sqrt(r2)
    expected = albedo / math.pi * I * cos / r2
    inner = (np.abs(p[..., 0]) < 1.5) & (np.abs(p[..., 2]) < 1.5)
    rel = np.abs(img - expected)[inner] / expected[inner]
    assert np.median(rel) < 0.02
    assert rel.max() < 0.15


def test_estimators_agree_on_diffuse_room(built):
    """The camera does not see the emitter: LT shows directly visible light
    samples at 1/(2 pi) of their radiance (showlightcaches.comp:41), which the
    restatement keeps, so only indirectly lit pixels are comparable."""
    sc = scenes.cornell_room(seed=3, sphere_level=2, wall_grid=2)
    b = bvh.build_bvh(sc["positions"], sc["triangles"])
    W = H = 16
    cam = render.camera_lookat((0.0, 1.0, 2.5), (0.0, 0.2, 0.0), (0.0, 1.0, 0.0), 40.0, W, H)
    # light samples uniformly over the ceiling quad (area 0.25, L = 10)
    rng = np.random.default_rng(0)
    means = {}
    for p, iters in (("PT", 64), ("BPT", 64), ("LT", 128)):
        acc = None
        for it in range(iters):
            n = 256 if p == "LT" else 128
            ls = np.zeros((n, 8), np.float32)
            ls[:, 0] = rng.uniform(-0.25, 0.25, n)
            ls[:, 2] = rng.uniform(-0.25, 0.25, n)
            ls[:, 1] = 1.999 - 1e-4
            ls[:, 3] = math.atan2(-1.0, 0.0)
            ls[:, 4:7] = 10.0 * 0.25 / n
            ls[:, 7] = 0.0
            acc = oracle.render(b, sc, p, W, H, cam.as_array(), render.frame_seed(it), ls, max_path_length=4, accum=acc)
        means[p] = acc[..., :3].mean() / iters
    assert abs(means["BPT"] / means["PT"] - 1) < 0.05, means
    assert abs(means["LT"] / means["PT"] - 1) < 0.06, means


def test_photon_map_point_light_on_lambert_floor(built):
    """Photon mapping on the floor under a point light: the density
    estimate over the query disc (radius 0.05 here) converges to the same
    irradiance as NEE, up to the kernel's blur of the smooth falloff."""
    albedo, I, h = 0.6, 5.0, 1.5
    sc = _quad_scene(albedo=albedo)
    b = bvh.build_bvh(sc["positions"], sc["triangles"])
    W = H = 16
    cam = render.camera_lookat((0.0, 3.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 30.0, W, H)
    ls = _point_light_samples((0.0, h, 0.0), (I, I, I), n=16)
    acc = None
    iters = 24
    for it in range(iters):
        acc = oracle.render(b, sc, "PM", W, H, cam.as_array(), render.frame_seed(it), ls, max_path_length=1,
                            accum=acc, photons_per_light_sample=1 << 14, query_radius=0.05)
    assert np.all(acc[..., 3] == iters)
    img = acc[..., 0] / iters
    c = cam.as_array()
    U, V, Wd, P = c[0:3], c[3:6], c[6:9], c[9:12]
    ys, xs = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    d = ((xs + 0.5) / W * 2 - 1)[..., None] * U + ((ys + 0.5) / H * 2 - 1)[..., None] * V + Wd
    p = P + (-P[1] / d[..., 1])[..., None] * d
    r2 = p[..., 0] ** 2 + (h - p[..., 1]) ** 2 + p[..., 2] ** 2 + 1e-5
    expected = albedo / math.pi * I * (h / np.sqrt(r2)) / r2
    rel = np.abs(img - expected) / expected
    assert np.median(rel) < 0.05, np.median(rel)
    assert abs(img.mean() / expected.mean() - 1) < 0.03


def test_importon_map_point_light_on_lambert_floor(built):
    """PixelMapLighttracer on the floor under a point light: the eye paths
    store no importon (their first hit is diffuse), so the image is the
    reprojection of the photons' first hits (photontracing.comp with
    REPROJECT), whose G-buffer occlusion test must accept the floor it
    stands on; the image mean converges to the NEE irradiance of the floor."""
    albedo, I, h = 0.6, 5.0, 1.5
    sc = _quad_scene(albedo=albedo)
    b = bvh.build_bvh(sc["positions"], sc["triangles"])
    W = H = 16
    cam = render.camera_lookat((0.0, 3.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 30.0, W, H)
    ls = _point_light_samples((0.0, h, 0.0), (I, I, I), n=16)
    acc, gbuf = None, np.zeros((H, W, 5), np.float32)
    iters = 16
    for it in range(iters):
        acc = oracle.render(b, sc, "IM", W, H, cam.as_array(), render.frame_seed(it), ls, max_path_length=1,
                            accum=acc, gbuffer=gbuf, photons_per_light_sample=1 << 14, query_radius=0.05)
    assert np.all(acc[..., 3] == iters)
    assert np.allclose(gbuf[..., 1], 0.0, atol=1e-5)  # first hits on the floor y = 0
    # packed geometry normal facing the camera, +y: (phi, z) = (pi / 2, 0)
    assert np.allclose(gbuf[..., 3], 0.0, atol=1e-6) and np.allclose(gbuf[..., 4], math.pi / 2, atol=1e-6)
    img = acc[..., 0] / iters
    c = cam.as_array()
    U, V, Wd, P = c[0:3], c[3:6], c[6:9], c[9:12]
    ys, xs = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    d = ((xs + 0.5) / W * 2 - 1)[..., None] * U + ((ys + 0.5) / H * 2 - 1)[..., None] * V + Wd
    p = P + (-P[1] / d[..., 1])[..., None] * d
    r2 = p[..., 0] ** 2 + (h - p[..., 1]) ** 2 + p[..., 2] ** 2 + 1e-5
    expected = albedo / math.pi * I * (h / np.sqrt(r2)) / r2
    # border pixels collect half a pixel's splats (nearest-pixel rounding at the image edge, as in the
    # reference's light tracer), so compare the interior
    img, expected = img[1:-1, 1:-1], expected[1:-1, 1:-1]
    assert np.median(np.abs(img - expected) / expected) < 0.06
    assert abs(img.mean() / expected.mean() - 1) < 0.02, (img.mean(), expected.mean())


def test_pcg_seed_hash_and_streams(built):
    """PCG-RXS-M-XS-32 as the oracle restates it equals an independent
    integer restatement (the hash that seeds a path and the stream that
    follows), and its draws behave like uniform variates in [0, 1)."""
    import ctypes as C
    L = oracle.lib()
    L.oracle_pcg_hash.argtypes = [C.c_uint32]
    L.oracle_pcg_hash.restype = C.c_uint32
    for x in (0, 1, 2, 61, 12345, 0x7FFFFFFF, 0x80000000, 0xFFFFFFFF):
        assert L.oracle_pcg_hash(x) == render.pcg_hash(x)
    # the stream: state = state * 747796405 + 2891336453, output permutation RXS-M-XS
    state = np.uint64(render.pcg_hash(render.pcg_hash(7) + 1234))
    mask = np.uint64(0xFFFFFFFF)
    draws = np.empty(1 << 16, np.float64)
    for i in range(draws.size):
        state = (state * np.uint64(747796405) + np.uint64(2891336453)) & mask
        s = int(state)
        w = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & 0xFFFFFFFF
        draws[i] = (((w >> 22) ^ w) >> 8) / 16777216.0
    assert draws.min() >= 0.0 and draws.max() < 1.0
    assert abs(draws.mean() - 0.5) < 0.005
    hist = np.histogram(draws, bins=64, range=(0, 1))[0]
    chi2 = ((hist - draws.size / 64) ** 2 / (draws.size / 64)).sum()
    assert chi2 < 120  # 63 degrees of freedom: p < 1e-5 beyond this


@pytest.mark.parametrize("rng", ["pcg", "reference"])
def test_rng_modes_agree_in_distribution(built, rng):
    """Both random streams estimate the same radiance: the point-lit floor
    seen at depth 1 gives the closed-form mean in either mode."""
    sc = _quad_scene(albedo=0.5)
    b = bvh.build_bvh(sc["positions"], sc["triangles"])
    W = H = 16
    cam = render.camera_lookat((0.0, 2.0, 0.001), (0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 20.0, W, H)
    ls = _point_light_samples((0.0, 1.0, 0.0), (5.0, 5.0, 5.0))
    acc = None
    for it in range(8):
        acc = oracle.render(b, sc, "PT", W, H, cam.as_array(), render.frame_seed(it, rng), ls, max_path_length=1,
                            accum=acc, rng=rng)
    img = acc[..., :3] / 8
    # the floor right under the light: albedo / pi * I / d^2 at normal incidence
    centre = img[H // 2 - 1:H // 2 + 1, W // 2 - 1:W // 2 + 1].mean()
    assert abs(centre / (0.5 / math.pi * 5.0) - 1) < 0.02, centre


def test_light_sampler_restatement(built):
    """oracle/lights.cpp: area samples lie on the ceiling light, carry
    luminance x area / n each (lightsampler.cpp:36,72), and a point light
    takes the share of its log flux (scene.cpp:295-307)."""
    sc = scenes.cornell_room(seed=1, sphere_level=2, wall_grid=2)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ls = oracle.light_samples(sc["positions"], b.slots, sc["materials"], 128, [123])
    assert np.allclose(ls[:, 1], 1.999 - 1e-4, atol=1e-6)
    assert (np.abs(ls[:, 0]) <= 0.25 + 1e-6).all() and (np.abs(ls[:, 2]) <= 0.25 + 1e-6).all()
    assert np.allclose(ls[:, 4:7], 10.0 * 0.25 / 128, rtol=1e-5)
    both = oracle.light_samples(sc["positions"], b.slots, sc["materials"], 128, [123],
                                point_lights=[((0.0, 1.0, 0.0), (1000.0, 1000.0, 1000.0))])
    area_flux = 10.0 * 0.25 * math.pi
    point_flux = math.log(1.0 + 1000.0 * 4 * math.pi)
    assert (both[:, 7] == 2.0).sum() == int(point_flux / (point_flux + area_flux) * 128)


def test_texture_sampling_is_glsl_bilinear_repeat(built):
    """The oracle's textureLod(.., 0) of a material texture: bilinear with
    REPEAT wrapping (OpenGL 4.5 8.14.2, the reference's sampler,
    scene.cpp:15-20), against a float64 restatement of that formula."""
    import ctypes as C
    rng = np.random.default_rng(3)
    texs = [rng.uniform(0, 1, (5, 7, 4)).astype(np.float32), rng.uniform(0, 2, (1, 3, 4)).astype(np.float32)]
    oracle.set_textures(texs, np.array([[0, -1, 1, -1]], np.int32))
    try:
        L = oracle.lib()
        L.oracle_eval.argtypes = [C.c_int, C.c_uint64, C.c_void_p, C.c_void_p]
        n = 2000
        tex = rng.integers(0, 2, n)
        tc = rng.uniform(-3, 3, (n, 2))
        tc[:10] = [[0, 0], [1, 1], [0.5, 0.5], [-1e-7, 0.25], [0.999999, 0.1], [2.0, -2.0], [1e6, 3.25], [0.1, 0.0],
                   [1 / 14, 1 / 10], [0.5 / 7, 0.5 / 5]]
        inp = np.concatenate([tex[:, None], tc], 1).astype(np.float32)
        out = np.zeros((n, 4), np.float32)
        assert L.oracle_eval(11, n, inp.ctypes.data, out.ctypes.data) == 0
        for i in range(n):
            t = texs[tex[i]].astype(np.float64)
            h, w = t.shape[:2]
            u = float(np.float32(inp[i, 1])) * w - 0.5
            v = float(np.float32(inp[i, 2])) * h - 0.5
            i0, j0 = math.floor(u), math.floor(v)
            a, b = u - i0, v - j0
            x0, y0, x1, y1 = i0 % w, j0 % h, (i0 + 1) % w, (j0 + 1) % h
            want = ((1 - a) * (1 - b) * t[y0, x0] + a * (1 - b) * t[y0, x1] + (1 - a) * b * t[y1, x0]
                    + a * b * t[y1, x1])
            assert np.allclose(out[i], want, rtol=1e-5, atol=1e-5), (i, inp[i], out[i], want)
    finally:
        oracle.set_textures(None, None)
