"""Hierarchy-importance renderer on the CPU: the builder's node NDFs
(bvhmake's approx_sggx) and the oracle's restatement of the importance
acquisition, propagation, node materials and path tracer
(gpugi/renderer/hierarchyimportance.cpp, gpugi/shader/hierarchy/*).

The reference ships no values for any of these, so the checks are
invariants: a flat scene's NDF is its normal, the propagation's sums, an
area-weighted material of one material is that material, and a hierarchy
that is never cut short renders what the path tracer renders.
"""
import numpy as np
import pytest

import oracle
from gpugi_gb300 import bvh, render, scenes


def _flat(n=24, seed=0):
    v, f, nrm = scenes._grid_quad((-1.0, 0.0, -1.0), (0.0, 0.0, 2.0), (2.0, 0.0, 0.0), n)  # y = 0, normal +y
    mat = scenes.material_record(albedo=(0.5, 0.5, 0.5), specular=(0.0, 0.0, 0.0), emissivity=(0.0, 0.0, 0.0))
    return scenes._pack(v, f, [mat], normals=nrm)


def _area_lights(n=128, seed=3):
    """Samples of a 0.5 x 0.5 ceiling light facing down (Lambertian, normal packed as {phi, cos theta})."""
    rng = np.random.default_rng(seed)
    ls = np.zeros((n, 8), np.float32)
    ls[:, 0] = rng.uniform(-0.25, 0.25, n)
    ls[:, 1] = 1.99
    ls[:, 2] = rng.uniform(-0.25, 0.25, n)
    ls[:, 3] = np.arctan2(-1.0, 0.0)
    ls[:, 7] = 0.0
    ls[:, 4:7] = 10.0 * 0.25 / n * np.pi
    return ls


def test_half_conversion_rounds_to_nearest_even():
    x = np.random.default_rng(1).standard_normal(100_000).astype(np.float32) * np.float32(300)
    x = np.concatenate([x, np.float32([65504, 65519.99, 65520, 6e-8, 2.9802322e-8, 2.9802326e-8, -0.0, 1e-5,
                                       6.1035156e-05, 6.103515e-05, np.inf, -np.inf])])
    with np.errstate(over="ignore"):
        ref = x.astype(np.float16).view(np.uint16)
    assert np.array_equal(oracle.float_to_half(x), ref)
    h = np.arange(65536, dtype=np.uint16)
    ref = h.view(np.float16).astype(np.float32)
    got = oracle.half_to_float(h)
    ok = np.isnan(ref) & np.isnan(got) | (got.view(np.uint32) == ref.view(np.uint32))
    assert ok.all()


def test_flat_scene_ndf_is_the_normal():
    sc = _flat()
    b = bvh.build_bvh(sc["positions"], sc["triangles"], normals=sc["normals"])
    s = b.sggx.astype(np.int64)
    assert s.shape == (b.num_nodes, 6)
    # S = n n^T with n = +y: sigma = (0, 1, 0), r = 0 (stored 32767)
    assert (s[:, 0] == 0).all() and (s[:, 2] == 0).all()
    assert (s[:, 1] >= 65534).all()
    assert (s[:, 3:] == 32767).all()


def test_ndf_values_and_file_chunk(tmp_path):
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], normals=sc["normals"])
    sig = b.sggx[:, :3].astype(np.float64) / 65535
    # sigma^2 are the diagonal of a matrix whose eigenvalues are mean |q . n|
    # over unit normals: each in [0, 1], trace >= 1
    assert ((sig ** 2).sum(1) >= 0.999 - 1e-3).all()
    path = tmp_path / "room.bim"
    bvh.write_bvh_file(sc["positions"], sc["triangles"], path, normals=sc["normals"])
    rb = bvh.read_bvh_file(path)
    assert rb.sggx is not None and np.array_equal(rb.sggx, b.sggx)
    # no normals, no chunk
    bvh.write_bvh_file(sc["positions"], sc["triangles"], tmp_path / "plain.bim")
    assert bvh.read_bvh_file(tmp_path / "plain.bim").sggx is None


def _room(seed=1):
    sc = scenes.cornell_room(seed=seed, sphere_level=2, wall_grid=4)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], normals=sc["normals"])
    return sc, b


def test_propagation_sums():
    sc, b = _room()
    W = H = 24
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H).as_array()
    imp, sub = oracle.hier_importance(b, sc, W, H, cam, _area_lights(), iterations=4)
    nn = b.num_nodes
    assert np.isfinite(imp[:, 0]).all() and (imp[:, 0] >= 0).all()
    assert imp[0, 0] > 0  # every camera ray enters the root
    fc = b.first_child
    esc = b.escape
    hier = b.hierarchy
    for i in range(nn):
        c = fc[i]
        if c & 0x80000000:
            blk = c & 0x7FFFFFFF
            s = np.float32(0)
            for k in range(b.leaf_size):
                s = np.float32(s + imp[nn + blk * b.leaf_size + k, 0])
            s = np.float32(s / np.float32(4))
            assert sub[i] == max(s, np.float32(1.19e-07))
            children = s
        else:
            children = np.float32(np.float32(0) + sub[c]) + sub[esc[c]]
            assert sub[i] == children
        with np.errstate(divide="ignore", invalid="ignore"):
            a = np.float32(imp[i, 0] / children)
        sides = hier[i, 4:7] - hier[i, 0:3]
        area = np.float32(np.float32(np.float32(sides[0] * sides[1] + sides[0] * sides[2]) + sides[1] * sides[2])
                          * np.float32(2)) / np.float32(6)
        y = np.float32(np.float32(a * a) * area)
        assert imp[i, 1] == y or (np.isnan(imp[i, 1]) and np.isnan(y)), i
    # the propagation alone reproduces the full pass's values
    raw = imp.copy()
    raw[:nn, 0] *= 4  # x was divided by the (power-of-two) iteration count
    imp2, sub2 = oracle.hier_propagate(b, raw, 4)
    assert np.array_equal(imp2.view(np.uint32), imp.view(np.uint32))
    assert np.array_equal(sub2, sub)


def test_single_material_node_materials():
    sc = _flat()
    b = bvh.build_bvh(sc["positions"], sc["triangles"], normals=sc["normals"])
    m = oracle.hier_materials(b, sc)
    h = oracle.half_to_float(m.view(np.uint16)).reshape(b.num_nodes, 24)
    rec = sc["materials"][0]
    diffuse = np.float16(rec[0:3]).astype(np.float32)
    assert np.allclose(h[:, 8:11], diffuse, rtol=2e-3)  # {Diffuse.xy}, {Diffuse.z, 0}
    # root area: the whole quad (2 x 2) in half precision
    assert abs(h[0, 7] - 4.0) < 4.0 * 2e-3


def test_unbroken_hierarchy_renders_like_the_path_tracer():
    """With importance y = +inf no node is cut short: the hierarchy path
    tracer is then a path tracer with adjoint BSDF sampling (the same for
    Lambertian surfaces), no -0.5 pixel offset and Russian roulette from the
    first vertex, so its image mean is the path tracer's."""
    sc, b = _room()
    W = H = 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H).as_array()
    ls = _area_lights()
    imp = np.zeros((b.num_nodes + b.num_slots, 2), np.float32)
    imp[:, 1] = np.inf
    mats = oracle.hier_materials(b, sc)
    acc_h = acc_p = None
    n = 24
    for it in range(n):
        acc_h = oracle.render_hier(b, sc, W, H, cam, render.frame_seed(it), ls, imp, mats, b.sggx, accum=acc_h)
        acc_p = oracle.render(b, sc, "PT", W, H, cam, render.frame_seed(it + 1000), ls, max_path_length=4, accum=acc_p)
    assert np.all(acc_h[..., 3] == n)
    mh, mp = acc_h[..., :3].mean() / n, acc_p[..., :3].mean() / n
    assert mh > 0 and abs(mh / mp - 1) < 0.05, (mh, mp)


def test_cut_hierarchy_stays_finite():
    """A zero importance cuts every node (y = 0 <= threshold x entry): the
    walk stops at the first node entered and shades its node material."""
    sc, b = _room()
    W = H = 16
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H).as_array()
    imp = np.zeros((b.num_nodes + b.num_slots, 2), np.float32)
    mats = oracle.hier_materials(b, sc)
    acc = oracle.render_hier(b, sc, W, H, cam, 7, _area_lights(), imp, mats, b.sggx)
    assert np.isfinite(acc).all() and acc[..., :3].sum() > 0
