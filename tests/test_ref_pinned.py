"""The oracle pinned to the reference's own shader text (CPU only).

oracle/ref_build.py compiles gpugi's GLSL (traceray.glsl,
intersectiontests.glsl, random.glsl, helper.glsl, and pathtracer.comp with
everything it includes: scenedata, materials, lightsource, globaluniforms)
as C++ into oracle/_ref/libgpugi_ref.so. These tests run it beside the
oracle's restatement on the same inputs and require identical bits:
  * TraceRay / TraceRayAnyHit on the closest-hit query workload (2^20 rays,
    65,536-triangle displaced icosphere, bvhmake sweep hierarchy with 8-slot
    leaves), on a 2-slot-leaf tree, on an oriented-box tree (OBOX_BVH) and
    on axis-parallel and box-plane rays
    with the tmax edge cases (the hit Triangle record, t, both barycentrics,
    the any-hit flag);
  * the random.glsl / helper.glsl functions on random inputs;
  * whole path-traced images (pathtracer.comp's main per pixel) on the
    Cornell room and on a room with glossy surfaces, depth 1 and depth 8,
    with the reference's random streams and Russian roulette;
  * whole light-traced images (LightPathtracer::Draw: lighttracer.comp,
    then showlightcaches.comp) and bidirectional images
    (BidirectionalPathtracer::Draw: lighttracer.comp with SAVE_LIGHT_CACHE,
    then pathtracer_bidir.comp per pixel) on the same rooms; both sides run
    their invocations in order on one thread, so the atomic image sums and
    the light-cache order are the same.
The GPU kernels are in turn checked against the oracle (tests/test_trace_gpu.py:
bit-exact traversal; tests/test_render_gpu.py: images). The tests skip where
the reference tree is absent and the library was not built.
"""
import math

import numpy as np
import pytest

import oracle
from gpugi_gb300 import bvh, render, scenes

ref = pytest.importorskip("oracle.ref")
pytestmark = pytest.mark.skipif(not ref.available(), reason="oracle/_ref not built (reference tree absent)")


def _same_closest(b, o, r):
    slots = np.asarray(b.slots).reshape(-1, 4)
    otri = np.where(o["slot"][:, None] >= 0, slots[np.maximum(o["slot"], 0)], -1)
    assert np.array_equal(otri, r["triangle"]), (otri != r["triangle"]).any(1).sum()
    assert np.array_equal(o["t"].view(np.uint32), r["t"].view(np.uint32))
    hit = o["slot"] >= 0
    assert np.array_equal(o["u"][hit].view(np.uint32), r["u"][hit].view(np.uint32))
    assert np.array_equal(o["v"][hit].view(np.uint32), r["v"][hit].view(np.uint32))


@pytest.fixture(scope="module")
def icosphere():
    sc = scenes.displaced_icosphere(65536, seed=1)
    return sc, bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", leaf_size=8)


def test_traversal_query_workload(icosphere):
    sc, b = icosphere
    rays = scenes.random_rays(1 << 20, seed=100)
    r = ref.trace_closest(b, sc["positions"], rays)
    o = oracle.trace_closest(b, sc["positions"], rays)
    assert (o["slot"] >= 0).sum() > 10_000
    _same_closest(b, o, r)
    assert np.array_equal(ref.trace_any(b, sc["positions"], rays), oracle.trace_any(b, sc["positions"], rays)["occluded"])


def test_traversal_aimed_rays_and_two_slot_leaves():
    sc = scenes.displaced_icosphere(8192, seed=7)
    for leaf in (8, 2):
        b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", leaf_size=leaf)
        rays = scenes.aimed_rays(100_000, sc["positions"], seed=8)
        _same_closest(b, oracle.trace_closest(b, sc["positions"], rays), ref.trace_closest(b, sc["positions"], rays))
        assert np.array_equal(ref.trace_any(b, sc["positions"], rays),
                              oracle.trace_any(b, sc["positions"], rays)["occluded"])


def test_traversal_oriented_boxes():
    """traceray.glsl with OBOX_BVH (FetchIntersectOBoxNode, rotate) over the
    fitted oriented-box hierarchy: identical to the oracle's walk."""
    sc = scenes.displaced_icosphere(16384, seed=21)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", fit="obox")
    assert b.bounds_kind == 2
    for rays in (scenes.random_rays(1 << 18, seed=22), scenes.aimed_rays(100_000, sc["positions"], seed=23)):
        _same_closest(b, oracle.trace_closest(b, sc["positions"], rays), ref.trace_closest(b, sc["positions"], rays))
        assert np.array_equal(ref.trace_any(b, sc["positions"], rays),
                              oracle.trace_any(b, sc["positions"], rays)["occluded"])


def test_traversal_edge_rays():
    """Axis-parallel rays, rays starting on the scene box's faces and corners
    (inf * 0 = NaN slabs), and tmax = inf, RAY_MAX, finite, 0, 1e-4."""
    sc = scenes.displaced_icosphere(5000, seed=3)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", leaf_size=8)
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
        _same_closest(b, oracle.trace_closest(b, sc["positions"], rays), ref.trace_closest(b, sc["positions"], rays))
        assert np.array_equal(ref.trace_any(b, sc["positions"], rays),
                              oracle.trace_any(b, sc["positions"], rays)["occluded"])


@pytest.mark.parametrize("kind", list(ref.EVAL_KINDS))
def test_random_and_helper_functions(kind):
    rng = np.random.default_rng(11)
    k, win, wout, dt = ref.EVAL_KINDS[kind]
    n = 20_000
    if kind in ("wanghash", "random_uint", "random", "init_random_seed"):
        inp = rng.integers(0, 2 ** 32, (n, win), dtype=np.uint64).astype(np.uint32)
        inp[:8] = np.array([0, 1, 61, 0xFFFFFFFF, 0x80000000, 123, 2 ** 16, 2 ** 31 - 1], np.uint32)[:, None]
    else:
        inp = rng.uniform(0, 1, (n, win)).astype(np.float32)
        if kind in ("sample_hemisphere_cosine", "sample_phong_lobe", "create_onb", "pack_normal", "luminance"):
            nn = rng.normal(size=(n, 3))
            nn /= np.linalg.norm(nn, axis=1, keepdims=True)
            nn[:6] = [[0, 1, 0], [0, -1, 0], [1, 0, 0], [0, 0, 1], [0, 0.99999, 0.0001], [0, 0, -1]]
            inp[:, -3:] = nn
        if kind == "sample_phong_lobe":
            inp[:, 2] = rng.uniform(1, 2000, n)
        if kind == "unpack_normal":
            inp[:, 0] = rng.uniform(-math.pi, math.pi, n)
            inp[:, 1] = rng.uniform(-1, 1, n)
    a = ref.evaluate(kind, inp)
    b = ref.evaluate_oracle(kind, inp)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), kind


def _glossy_room():
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8)
    mats = sc["materials"].reshape(-1, 24).copy()
    mats[7] = scenes.material_record(albedo=(0.1, 0.1, 0.1), specular=(0.8, 0.8, 0.8), roughness=0.03)
    mats[5] = scenes.material_record(albedo=(0.3, 0.4, 0.5), specular=(0.5, 0.5, 0.5), roughness=0.2,
                                     opacity=(0.4, 0.4, 0.4), refraction_index=1.4)
    return dict(sc, materials=mats)


@pytest.mark.parametrize("room,depth,sky", [("diffuse", 1, 0.0), ("diffuse", 8, 0.0), ("glossy", 8, 0.0),
                                             ("glossy", 6, 0.25)])
def test_path_tracer_images(room, depth, sky):
    """pathtracer.comp (the reference's text) and the oracle's PT restatement
    render identical images, iteration by iteration."""
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8) if room == "diffuse" else _glossy_room()
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    W, H = 40, 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H).as_array()
    acc_r = acc_o = None
    st = [123]
    for it in range(3):
        ls = oracle.light_samples(sc["positions"], b.slots, sc["materials"], 128, st)
        fs = render.frame_seed(it, "reference")
        acc_r = ref.render_pt(b, sc, W, H, cam, fs, ls, max_path_length=depth, sky=(sky,) * 3, accum=acc_r)
        acc_o = oracle.render(b, sc, "PT", W, H, cam, fs, ls, max_path_length=depth, sky=(sky,) * 3, accum=acc_o,
                              rng="reference")
        assert np.array_equal(acc_r.view(np.uint32), acc_o.view(np.uint32)), (it, np.abs(acc_r - acc_o).max())
    assert acc_r[..., :3].mean() > 0


@pytest.mark.parametrize("pass_", ["LT", "BPT"])
@pytest.mark.parametrize("room,depth", [("diffuse", 1), ("diffuse", 6), ("glossy", 8)])
def test_light_and_bidirectional_images(room, depth, pass_):
    """lighttracer.comp + showlightcaches.comp, and the light-cache pass +
    pathtracer_bidir.comp (the reference's text), against the oracle's LT and
    BPT restatements: identical images, iteration by iteration."""
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8) if room == "diffuse" else _glossy_room()
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    W, H = 40, 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H).as_array()
    acc_r = acc_o = None
    st = [321]
    for it in range(2):
        ls = oracle.light_samples(sc["positions"], b.slots, sc["materials"], render.DEFAULT_LIGHT_SAMPLES[pass_], st)
        fs = render.frame_seed(it, "reference")
        acc_r = ref.render_lt(b, sc, W, H, cam, fs, ls, max_path_length=depth, accum=acc_r, bidir=pass_ == "BPT")
        acc_o = oracle.render(b, sc, pass_, W, H, cam, fs, ls, max_path_length=depth, accum=acc_o, rng="reference",
                              num_threads=1)
        assert np.array_equal(acc_r.view(np.uint32), acc_o.view(np.uint32)), (it, np.abs(acc_r - acc_o).max())
    assert acc_r[..., :3].mean() > 0


@pytest.mark.parametrize("room,depth", [("diffuse", 6), ("glossy", 8)])
def test_whitted_images(room, depth):
    """whittedraytracer.comp (the reference's text, with the
    STOP_ON_DIFFUSE_BOUNCE define its renderer adds) against the oracle's
    Whitted restatement: identical images, iteration by iteration."""
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8) if room == "diffuse" else _glossy_room()
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    W, H = 40, 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H).as_array()
    acc_r = acc_o = None
    st = [5]
    for it in range(2):
        ls = oracle.light_samples(sc["positions"], b.slots, sc["materials"], 128, st)
        fs = render.frame_seed(it, "reference")
        acc_r = ref.render_whitted(b, sc, W, H, cam, fs, ls, max_path_length=depth, accum=acc_r)
        acc_o = oracle.render(b, sc, "WHITTED", W, H, cam, fs, ls, max_path_length=depth, accum=acc_o,
                              rng="reference", num_threads=1)
        assert np.array_equal(acc_r.view(np.uint32), acc_o.view(np.uint32)), (it, np.abs(acc_r - acc_o).max())
    assert acc_r[..., :3].mean() > 0


@pytest.mark.parametrize("room", ["diffuse", "glossy"])
def test_photon_map_and_importon_map_images(room):
    """The photon mapper's and the importon map light tracer's shaders (the
    reference's text) against the oracle's PM and IM restatements: identical
    images, iteration by iteration (the importon map carries its position
    texture and the image's alpha, the first hit's packed normal x, between
    iterations; the oracle carries its G-buffer)."""
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8) if room == "diffuse" else _glossy_room()
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    W, H = 40, 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H).as_array()
    st = [7]
    acc_r = acc_o = None
    for it in range(2):
        ls = oracle.light_samples(sc["positions"], b.slots, sc["materials"], 32, st)
        fs = render.frame_seed(it, "reference")
        acc_r = ref.render_pm(b, sc, W, H, cam, fs, ls, max_path_length=6, accum=acc_r, photons_per_light_sample=256,
                              query_radius=0.05)
        acc_o = oracle.render(b, sc, "PM", W, H, cam, fs, ls, max_path_length=6, accum=acc_o, rng="reference",
                              num_threads=1, photons_per_light_sample=256, query_radius=0.05)
        assert np.array_equal(acc_r.view(np.uint32), acc_o.view(np.uint32)), (it, np.abs(acc_r - acc_o).max())
    assert acc_r[..., :3].mean() > 0
    st = [9]
    acc_r, pos_r = np.zeros((H, W, 4), np.float32), np.zeros((H, W, 4), np.float32)
    acc_o, gbuf = None, np.zeros((H, W, 5), np.float32)
    for it in range(3):
        ls = oracle.light_samples(sc["positions"], b.slots, sc["materials"], 32, st)
        fs = render.frame_seed(it, "reference")
        ref.render_im(b, sc, W, H, cam, fs, ls, acc_r, pos_r, max_path_length=6, photons_per_light_sample=256,
                      query_radius=0.03)
        acc_o = oracle.render(b, sc, "IM", W, H, cam, fs, ls, max_path_length=6, accum=acc_o, rng="reference",
                              num_threads=1, photons_per_light_sample=256, query_radius=0.03, gbuffer=gbuf)
        assert np.array_equal(acc_r[..., :3].view(np.uint32), acc_o[..., :3].view(np.uint32)), \
            (it, np.abs(acc_r[..., :3] - acc_o[..., :3]).max())
    assert acc_r[..., :3].mean() > 0



@pytest.mark.parametrize("room", ["diffuse", "glossy"])
def test_hierarchy_path_tracer_images(room):
    """hierarchypathtracer.comp (the reference's text) against the oracle's
    restatement over the importance that the oracle's acquisition and
    propagation passes produce (so some nodes are cut short and shade their
    node materials and NDFs): identical images, iteration by iteration."""
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8) if room == "diffuse" else _glossy_room()
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", normals=sc["normals"])
    W, H = 40, 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H).as_array()
    st = [11]
    ls = oracle.light_samples(sc["positions"], b.slots, sc["materials"], 128, st)
    imp, _ = oracle.hier_importance(b, sc, W, H, cam, ls, iterations=4)
    mats = oracle.hier_materials(b, sc)
    acc_r = acc_o = None
    for it in range(3):
        ls = oracle.light_samples(sc["positions"], b.slots, sc["materials"], 128, st)
        fs = render.frame_seed(it, "reference")
        acc_r = ref.render_hier(b, sc, W, H, cam, fs, ls, imp, mats, b.sggx, accum=acc_r)
        acc_o = oracle.render_hier(b, sc, W, H, cam, fs, ls, imp, mats, b.sggx, accum=acc_o, num_threads=1,
                                   rng="reference")
        assert np.array_equal(acc_r.view(np.uint32), acc_o.view(np.uint32)), (it, np.abs(acc_r - acc_o).max())
    assert acc_r[..., :3].mean() > 0


@pytest.mark.parametrize("room", ["diffuse", "glossy"])
def test_hierarchy_importance_and_materials(room):
    """acquisition2.comp + the two propagation shaders, and
    sampleleafmaterials.comp + pullmaterials.comp (the reference's text),
    against the oracle's restatements: identical importance {x, y}, subtree
    importance and packed node materials."""
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8) if room == "diffuse" else _glossy_room()
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", normals=sc["normals"])
    W, H = 40, 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H).as_array()
    ls = oracle.light_samples(sc["positions"], b.slots, sc["materials"], 128, [13])
    imp_r, sub_r = ref.hier_importance(b, sc, W, H, cam, ls, iterations=3)
    imp_o, sub_o = oracle.hier_importance(b, sc, W, H, cam, ls, iterations=3, num_threads=1)
    assert imp_r[0, 0] > 0 and (sub_r > 0).all()
    assert np.array_equal(imp_r.view(np.uint32), imp_o.view(np.uint32)), np.abs(imp_r - imp_o).max()
    assert np.array_equal(sub_r.view(np.uint32), sub_o.view(np.uint32))
    mat_r, mat_o = ref.hier_materials(b, sc), oracle.hier_materials(b, sc)
    assert np.array_equal(mat_r, mat_o), np.argwhere(mat_r != mat_o)[:5]
