"""GPU hierarchy builder (gpugi_scene_build, a linear BVH) on the GPU.

The reference builds on the host (bvhmake); the GPU builder must emit a tree
in the same layout with the same invariants (test_bvhmake._check_tree: the
escape rules of bvhbuilder.cpp:710-722, every triangle in exactly one leaf
slot, padding at the end of a block, boxes containing their triangles), the
traversal over it must be bit-exact against the oracle walking the exported
tree, and closest hits must be those of brute force.
"""
import numpy as np
import pytest

import oracle
from gpugi_gb300 import bvh, cuda, render, scenes
from test_bvhmake import _check_tree
from test_trace_gpu import _compare_closest

pytestmark = pytest.mark.gpu


def _built(ctx, sc, leaf_size=8, **kw):
    ds = ctx.build_scene(sc["positions"], sc["triangles"], leaf_size=leaf_size, **kw)
    return ds, ds.export()


@pytest.mark.parametrize("ntri,leaf", [(1, 8), (7, 8), (8, 8), (9, 8), (17, 8), (1000, 8), (65536, 8),
                                       (3000, 1), (3000, 2), (3000, 32)])
def test_tree_invariants(cuda_ctx, ntri, leaf):
    sc = scenes.displaced_icosphere(ntri, seed=3)
    ds, b = _built(cuda_ctx, sc, leaf)
    _check_tree(b, sc["triangles"], sc["positions"])
    assert b.num_nodes == 2 * (b.num_slots // leaf) - 1
    if ntri <= leaf:
        assert b.num_nodes == 1
    ds.close()


def test_equal_morton_codes(cuda_ctx):
    """Many triangles with the same box centre (equal codes, ordered by
    index) and a flat scene (zero extent on one axis)."""
    base = scenes.displaced_icosphere(40, seed=8)
    pos = np.concatenate([base["positions"]] * 50)
    tris = np.concatenate([base["triangles"] + np.array([k * base["positions"].shape[0]] * 3 + [0], np.uint32)
                           for k in range(50)])
    ds, b = _built(cuda_ctx, {"positions": pos, "triangles": tris})
    _check_tree(b, tris, pos)
    ds.close()
    v, f, n = scenes._grid_quad((-1.0, 0.0, -1.0), (2.0, 0.0, 0.0), (0.0, 0.0, 2.0), 40)
    flat = scenes._pack(v.astype(np.float32), f, np.stack([scenes.lambert((0.5, 0.5, 0.5))]))
    ds, b = _built(cuda_ctx, flat)
    _check_tree(b, flat["triangles"], flat["positions"])
    ds.close()


@pytest.mark.parametrize("leaf", [8, 2])
def test_traversal_matches_oracle_and_bruteforce(cuda_ctx, leaf):
    sc = scenes.displaced_icosphere(65536, seed=1)
    ds, b = _built(cuda_ctx, sc, leaf)
    try:
        for mode in (0, 2, 3, 5):
            cuda_ctx.set_trace_config(mode=mode)
            for rays in (scenes.random_rays(1 << 17, seed=3), scenes.aimed_rays(1 << 17, sc["positions"], seed=4)):
                g = cuda.trace_closest(cuda_ctx, ds, rays)
                _compare_closest(g, oracle.trace_closest(b, sc["positions"], rays))
                assert np.array_equal(cuda.trace_any(cuda_ctx, ds, rays),
                                      oracle.trace_any(b, sc["positions"], rays)["occluded"])
        rays = scenes.aimed_rays(20_000, sc["positions"], seed=5)
        g = cuda.trace_closest(cuda_ctx, ds, rays)
        bf = oracle.bruteforce_closest(b.slots, sc["positions"], rays)
        assert (g["t"].view(np.uint32) == bf["t"].view(np.uint32)).mean() > 0.999
    finally:
        cuda_ctx.set_trace_config(mode=3)
    ds.close()


def test_render_equals_host_built_scene(cuda_ctx):
    """Closest hits do not depend on the tree (ties aside), so a path-traced
    image over the GPU-built hierarchy equals the one over bvhmake's."""
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8)
    vi = cuda.vertex_info(sc["normals"], sc["texcoords"])
    hb = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    host = cuda_ctx.upload_scene(hb, sc["positions"], vi, sc["materials"])
    gpu = cuda_ctx.build_scene(sc["positions"], sc["triangles"], vi, sc["materials"])
    W = H = 48
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    state = [5]
    ls = np.stack([render.generate_light_samples(host, state, 128) for _ in range(4)])
    imgs = []
    for ds in (host, gpu):
        img = render.Image(cuda_ctx, W, H)
        render.render(cuda_ctx, ds, cam, img, "PT", max_path_length=6, samples=4, light_samples=ls)
        imgs.append(img.read()[..., :3])
        img.close()
    diff = np.abs(imgs[0] - imgs[1]).max(-1)
    assert (diff <= 1e-4 * np.abs(imgs[0]).max() + 1e-6).mean() > 0.995
    assert abs(imgs[1].mean() / imgs[0].mean() - 1) < 1e-3
    # light tables of the GPU-built scene (its emissive triangles): the same
    # total flux per sample, positions on the ceiling light
    a = render.generate_light_samples(host, [9], 512)
    b = render.generate_light_samples(gpu, [9], 512)
    assert np.allclose(a[:, 4:7], b[:, 4:7], rtol=1e-6)
    assert np.allclose(b[:, 1], a[:, 1], atol=1e-6)  # the ceiling light's plane (the sampler's 1e-4 offset included)
    assert (np.abs(b[:, [0, 2]]) <= 0.25 + 1e-6).all()
    for x in (host, gpu):
        x.close()


def test_rejects_bad_triangles(cuda_ctx):
    sc = scenes.displaced_icosphere(64, seed=1)
    bad = sc["triangles"].copy()
    bad[3, 1] = 10 ** 6
    with pytest.raises(cuda.GpugiError):
        cuda_ctx.build_scene(sc["positions"], bad)
    bad = sc["triangles"].copy()
    bad[5, 1] = bad[5, 0]
    with pytest.raises(cuda.GpugiError):
        cuda_ctx.build_scene(sc["positions"], bad)
    with pytest.raises(cuda.GpugiError):
        cuda_ctx.build_scene(sc["positions"], sc["triangles"], leaf_size=33)
    bad = sc["triangles"].copy()
    bad[7, 3] = 1
    with pytest.raises(cuda.GpugiError):
        cuda_ctx.build_scene(sc["positions"], bad, materials=scenes.lambert((0.5, 0.5, 0.5))[None])
    ds = cuda_ctx.build_scene(sc["positions"], sc["triangles"])  # the context stays usable
    ds.close()
