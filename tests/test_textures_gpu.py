"""Textured materials (gpugi_scene_set_textures) in the rendering passes
against the oracle's SampleMaterialData (materials.glsl:19-30) with the
same textures: a Cornell room whose floor, back and left walls carry a
diffuse map, whose back wall carries a reflectiveness map and whose light
carries an emissivity map, texcoords running over [-0.25, 1.75] so the
REPEAT wrap is crossed in both directions.

Bars as for the untextured passes: depth-1 PT per pixel within 1e-4 of the
image maximum, full depth PT / LT / BPT image and block means.
"""
import numpy as np
import pytest

import oracle
from gpugi_gb300 import bvh, cuda, render, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def textured_room(cuda_ctx):
    sc = scenes.cornell_room(seed=2, sphere_level=3, wall_grid=8, textured=True)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]),
                               sc["materials"])
    ds.set_textures(sc["textures"], sc["material_textures"])
    oracle.set_textures(sc["textures"], sc["material_textures"])
    yield sc, b, ds
    oracle.set_textures(None, None)
    ds.close()


def _light_sets(ds, n_sets, n, seed=321):
    state = [seed]
    return np.stack([render.generate_light_samples(ds, state, n) for _ in range(n_sets)])


def _oracle(b, sc, pass_, W, H, cam, ls, iters, **kw):
    acc = None
    for s in range(iters):
        acc = oracle.render(b, sc, pass_, W, H, cam.as_array(), render.frame_seed(s), ls[s], accum=acc, **kw)
    return acc


def test_depth1_pt_samples_textures_like_oracle(cuda_ctx, textured_room):
    sc, b, ds = textured_room
    W = H = 48
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(ds, 4, 128)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img, "PT", max_path_length=1, samples=4, iteration=0, light_samples=ls)
    g = img.read()
    o = _oracle(b, sc, "PT", W, H, cam, ls, 4, max_path_length=1)
    err = np.abs(g[..., :3] - o[..., :3])
    assert err.max() <= 1e-4 * np.abs(o[..., :3]).max() + 1e-6
    img.close()

    # the textures change the picture: the same scene without them differs
    ds.set_textures([], None)
    try:
        plain = render.Image(cuda_ctx, W, H)
        render.render(cuda_ctx, ds, cam, plain, "PT", max_path_length=1, samples=4, iteration=0, light_samples=ls)
        p = plain.read()
        plain.close()
    finally:
        ds.set_textures(sc["textures"], sc["material_textures"])
    assert np.abs(p[..., :3] - g[..., :3]).max() > 0.05 * np.abs(g[..., :3]).max()
    # the light's emissivity map: its pixels (direct hits) are texel blends in [5, 15], not the constant 10
    lit = g[..., :3].max(-1) / 4 > 4.5
    assert lit.any() and not np.allclose(g[lit, 0] / 4, 10.0, rtol=1e-3)


@pytest.mark.parametrize("pass_,iters", [("PT", 32), ("BPT", 32), ("LT", 48)])
def test_full_depth_textured_passes_match_oracle(cuda_ctx, textured_room, pass_, iters):
    sc, b, ds = textured_room
    W = H = 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    ls = _light_sets(ds, iters, render.DEFAULT_LIGHT_SAMPLES[pass_])
    K = 4
    per = iters // K
    batches = []
    for k in range(K):
        img = render.Image(cuda_ctx, W, H)
        render.render(cuda_ctx, ds, cam, img, pass_, max_path_length=6, samples=per, iteration=k * per,
                      light_samples=ls[k * per:(k + 1) * per])
        batches.append(img.read()[..., :3] / per)
        img.close()
    g = np.stack(batches)
    o = _oracle(b, sc, pass_, W, H, cam, ls, iters, max_path_length=6)[..., :3] / iters
    assert abs(g.mean() / o.mean() - 1) < 0.03, (g.mean(), o.mean())
    blk = lambda a: a.reshape(*a.shape[:-3], 4, 8, 4, 8, 3).mean((-4, -2))
    gb = blk(g)
    se = gb.std(0, ddof=1) / np.sqrt(K)
    d = np.abs(gb.mean(0) - blk(o[None])[0])
    assert (d <= 6 * np.sqrt(2) * se + 1e-3 * np.abs(gb.mean(0)) + 1e-5).mean() > 0.97
    assert cuda_ctx.device_error_bits() == 0


def test_texture_arguments_are_checked(cuda_ctx, textured_room):
    sc, b, ds = textured_room
    mt = sc["material_textures"].copy()
    mt[0, 0] = 3  # only three textures
    with pytest.raises(cuda.GpugiError, match="out of range"):
        ds.set_textures(sc["textures"], mt)
    with pytest.raises(cuda.GpugiError, match="texels"):
        ds.set_textures([np.zeros((0, 4, 4), np.float32)], sc["material_textures"])
    ds.set_textures(sc["textures"], sc["material_textures"])
