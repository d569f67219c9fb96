"""The bvhmake restatement produces a valid escape tree in gpugi's layout.

Checks the invariants bvhmake asserts or relies on (bvhmake/bvhbuilder.cpp:
551, 699-722; buildmethods/*): preorder with the root at 0, every triangle in
exactly one leaf slot, padding only at the end of a block, escape(left) =
right, escape(right) = parent's escape, escape(root) = 0, and bounds that
contain every triangle below them.
"""
import numpy as np
import pytest

from gpugi_gb300 import bvh, scenes


def _check_tree(b, tris, positions):
    n = b.num_nodes
    fc = b.first_child
    esc = b.escape
    L = b.leaf_size
    assert esc[0] == 0
    seen = np.zeros(tris.shape[0], dtype=np.int64)
    tri_key = {tuple(t): i for i, t in enumerate(tris.tolist())}
    # subtree triangle boxes, bottom-up
    lo = np.full((n, 3), np.inf, np.float32)
    hi = np.full((n, 3), -np.inf, np.float32)
    for i in range(n - 1, -1, -1):
        c = int(fc[i])
        if c & 0x80000000:
            blk = c & 0x7FFFFFFF
            block = b.slots[blk * L:(blk + 1) * L]
            valid = block[:, 0] != block[:, 1]
            k = int(valid.sum())
            assert k >= 1 and valid[:k].all() and not valid[k:].any()  # padding at the end only
            assert (block[~valid] == 0).all()
            for t in block[valid]:
                seen[tri_key[tuple(int(x) for x in t)]] += 1
                p = positions[t[:3]]
                lo[i] = np.minimum(lo[i], p.min(0))
                hi[i] = np.maximum(hi[i], p.max(0))
        else:
            assert i < c < n, "left child follows its parent (preorder)"
            r = int(esc[c])
            assert c < r < n, "escape(left) is the right sibling"
            assert esc[r] == esc[i], "escape(right) is the parent's escape"
            assert b.parents[c] == i and b.parents[r] == i
            lo[i] = np.minimum(lo[c], lo[r])
            hi[i] = np.maximum(hi[c], hi[r])
    assert (seen == 1).all(), "every triangle appears in exactly one leaf slot"
    if b.bounds_kind == 0:
        assert (b.hierarchy[:, 0:3] <= lo).all() and (b.hierarchy[:, 4:7] >= hi).all()
    elif b.bounds_kind == 2:  # oriented box: every vertex below inside, in the shader's float rotation
        _check_oboxes(b, positions)
    else:  # ellipsoid contains the box corners of everything below
        c, r = b.hierarchy[:, 0:3].astype(np.float64), b.hierarchy[:, 4:7].astype(np.float64)
        for corner in range(8):
            sel = [(corner >> k) & 1 for k in range(3)]
            p = np.where(np.array(sel, bool)[None, :], hi, lo).astype(np.float64)
            q = ((p - c) / r) ** 2
            inside = q.sum(1)
            # leaves may be tighter than the box ellipsoid: check vertices instead below
        for i in range(n):
            ci = int(fc[i])
            if ci & 0x80000000:
                blk = ci & 0x7FFFFFFF
                block = b.slots[blk * L:(blk + 1) * L]
                block = block[block[:, 0] != block[:, 1]]
                p = positions[block[:, :3].reshape(-1)].astype(np.float64)
                assert (((p - c[i]) / r[i]) ** 2).sum(1).max() <= 1.0 + 1e-6


def _qrotate(x, q):
    """rotate(x, q) of intersectiontests.glsl:82-89 in float32, the shader's order."""
    f = np.float32
    x = x.astype(f)
    qx, qy, qz, qw = (np.asarray(q[..., k], f)[..., None] for k in range(4))
    t = np.stack([qy[..., 0] * x[..., 2] - qz[..., 0] * x[..., 1], qz[..., 0] * x[..., 0] - qx[..., 0] * x[..., 2],
                  qx[..., 0] * x[..., 1] - qy[..., 0] * x[..., 0]], -1).astype(f)
    u = np.stack([(qw[..., 0] * t[..., 0] + qy[..., 0] * t[..., 2]) - qz[..., 0] * t[..., 1],
                  (qw[..., 0] * t[..., 1] + qz[..., 0] * t[..., 0]) - qx[..., 0] * t[..., 2],
                  (qw[..., 0] * t[..., 2] + qx[..., 0] * t[..., 1]) - qy[..., 0] * t[..., 0]], -1).astype(f)
    return (x + f(2.0) * u).astype(f)


def _check_oboxes(b, positions):
    """Every vertex below a node lies inside its oriented box, with the
    rotation computed as the walk computes it; the quaternions are unit."""
    H = b.hierarchy
    assert H.shape[1] == 12
    assert np.allclose((H[:, 8:12].astype(np.float64) ** 2).sum(1), 1.0, atol=1e-5)
    fc = b.first_child
    n, L = b.num_nodes, b.leaf_size
    blo = np.zeros(n, np.int64)
    bhi = np.zeros(n, np.int64)
    for i in range(n - 1, -1, -1):
        c = int(fc[i])
        if c & 0x80000000:
            blo[i] = bhi[i] = c & 0x7FFFFFFF
        else:
            r = int(b.escape[c])
            blo[i], bhi[i] = min(blo[c], blo[r]), max(bhi[c], bhi[r])
    for i in range(n):
        block = b.slots[blo[i] * L:(bhi[i] + 1) * L]
        block = block[block[:, 0] != block[:, 1]]
        p = positions[block[:, :3].reshape(-1)].astype(np.float32)
        local = _qrotate(p - H[i, 0:3], H[i, 8:12])
        assert (np.abs(local) <= H[i, 4:7]).all(), i


@pytest.mark.parametrize("method", ["sweep", "kdtree", "lds"])
def test_oriented_box_fit(built, method):
    sc = scenes.displaced_icosphere(3000, seed=6)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method=method, fit="obox")
    assert b.bounds_kind == 2 and b.hierarchy.shape == (b.num_nodes, 12)
    _check_tree(b, sc["triangles"], sc["positions"])
    # the topology is the method's own; only the bounds differ from the box fit
    a = bvh.build_bvh(sc["positions"], sc["triangles"], method=method)
    assert np.array_equal(a.first_child, b.first_child) and np.array_equal(a.escape, b.escape)
    assert np.array_equal(a.slots, b.slots)


def test_oriented_box_file_round_trip(built, tmp_path):
    sc = scenes.displaced_icosphere(1500, seed=3)
    p = tmp_path / "obox.bim"
    bvh.write_bvh_file(sc["positions"], sc["triangles"], str(p), method="sweep", fit="obox")
    b = bvh.read_bvh_file(str(p))
    ref = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", fit="obox")
    assert b.bounds_kind == 2
    assert np.array_equal(b.hierarchy.view(np.uint32), ref.hierarchy.view(np.uint32))
    assert np.array_equal(b.slots, ref.slots)


@pytest.mark.parametrize("method", ["sweep", "kdtree", "lds"])
@pytest.mark.parametrize("leaf_size", [1, 2, 8])
def test_escape_tree_invariants(built, method, leaf_size):
    sc = scenes.displaced_icosphere(2000, seed=5)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method=method, leaf_size=leaf_size)
    _check_tree(b, sc["triangles"], sc["positions"])


def test_ellipsoid_bounds_contain_leaves(built):
    sc = scenes.displaced_icosphere(600, seed=7)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="kdtree", fit="ellipsoid")
    assert b.bounds_kind == 1
    _check_tree(b, sc["triangles"], sc["positions"])


@pytest.mark.parametrize("ntri", [1, 7, 8, 9, 17])
def test_small_scenes(built, ntri):
    sc = scenes.displaced_icosphere(ntri, seed=2)
    for method in ("sweep", "kdtree", "lds"):
        b = bvh.build_bvh(sc["positions"], sc["triangles"], method=method)
        _check_tree(b, sc["triangles"], sc["positions"])
        if ntri <= 8:
            assert b.num_nodes == 1 and (b.first_child[0] & 0x80000000)


@pytest.mark.parametrize("method", ["sweep", "lds"])
def test_deterministic(built, method):
    sc = scenes.displaced_icosphere(3000, seed=11)
    a = bvh.build_bvh(sc["positions"], sc["triangles"], method=method)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method=method)
    assert np.array_equal(a.hierarchy.view(np.uint32), b.hierarchy.view(np.uint32))
    assert np.array_equal(a.slots, b.slots)


def test_lds_splits_along_the_principal_axis(built):
    """A long thin slab along a diagonal: the largest-dimension split follows
    the diagonal, so the root's children separate the two ends, and the SAH
    sweep keeps the tree within a few percent of the sweep builder's cost."""
    rng = np.random.default_rng(4)
    n = 512
    t = np.sort(rng.uniform(0, 1, n)).astype(np.float32)
    axis = np.array([1.0, 1.0, 0.0], np.float32) / np.sqrt(2)
    base = t[:, None] * axis[None] * 10
    off = rng.uniform(-0.01, 0.01, (n, 3, 3)).astype(np.float32)
    pos = (base[:, None, :] + off).reshape(-1, 3).astype(np.float32)
    tris = np.concatenate([np.arange(3 * n, dtype=np.uint32).reshape(n, 3), np.zeros((n, 1), np.uint32)], 1)
    b = bvh.build_bvh(pos, tris, method="lds")
    _check_tree(b, tris, pos)
    left = int(b.first_child[0])
    right = int(b.escape[left])
    cl = (b.hierarchy[left, 0:3] + b.hierarchy[left, 4:7]) / 2
    cr = (b.hierarchy[right, 0:3] + b.hierarchy[right, 4:7]) / 2
    d = cr - cl
    assert abs(d[0]) > 2 and abs(d[1]) > 2 and abs(d[2]) < 0.1  # split across the diagonal


def test_rejects_bad_input(built):
    sc = scenes.displaced_icosphere(64, seed=1)
    with pytest.raises(ValueError):
        bvh.build_bvh(sc["positions"], sc["triangles"][:0])
    bad = sc["triangles"].copy()
    bad[3, 1] = 10 ** 6
    with pytest.raises(ValueError):
        bvh.build_bvh(sc["positions"], bad)
    bad = sc["triangles"].copy()
    bad[5, 1] = bad[5, 0]
    with pytest.raises(ValueError):
        bvh.build_bvh(sc["positions"], bad)


def test_file_round_trip(built, tmp_path):
    sc = scenes.displaced_icosphere(1500, seed=3)
    p = tmp_path / "scene.bim"
    bvh.write_bvh_file(sc["positions"], sc["triangles"], str(p), method="sweep", leaf_size=4)
    b = bvh.read_bvh_file(str(p))
    ref = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep", leaf_size=4)
    assert b.leaf_size == 4
    assert np.array_equal(b.hierarchy.view(np.uint32), ref.hierarchy.view(np.uint32))
    assert np.array_equal(b.slots, ref.slots)
    assert np.array_equal(b.positions, sc["positions"])


def test_file_carries_vertex_attributes_and_materials(built, tmp_path):
    sc = scenes.cornell_room(seed=2, sphere_level=1, wall_grid=2)
    p = tmp_path / "room.bim"
    bvh.write_bvh_file(sc["positions"], sc["triangles"], str(p), normals=sc["normals"], texcoords=sc["texcoords"],
                       materials=sc["materials"], method="sweep", leaf_size=8)
    b = bvh.read_bvh_file(str(p))
    assert np.array_equal(b.normals, sc["normals"])
    assert np.array_equal(b.texcoords, sc["texcoords"])
    assert np.array_equal(b.materials, sc["materials"].reshape(-1, 24))
    # without attributes the file still round-trips, with zero attributes and no materials
    bvh.write_bvh_file(sc["positions"], sc["triangles"], str(p), method="sweep", leaf_size=8)
    b = bvh.read_bvh_file(str(p))
    assert not b.normals.any() and b.materials.shape == (0, 24)


SCENE_JSON = """{
  "scene": "room.bim", "accelerator": "aabox",
  "materials": {
    "Matte":  {"type": "legacy", "albedo": [0.25, 0.5, 0.75], "roughness": [0.5], "opacity": [1]},
    "Coated": {"albedo": [0.1, 0.1, 0.1], "specularColor": [0.2, 0.3, 0.4], "roughness": 0.1,
               "opacity": [0.0, 0.0, 0.0], "refractionIndex": 1.33},
    "Lamp":   {"emissivity": [10, 20, 30], "reflectiveness": [0.5, 0.6, 0.7]},
    "Textured": {"albedo": "wood.png"}
  },
  "lights": {}, "cameras": {}
}"""


def test_material_json_uses_load_material_mapping(built):
    """Scene::LoadMaterial (gpugi/scene/scene.cpp:132-180): fresnel0 defaults
    to 0.03, fresnel1 = 1 - fresnel0, exponent = 1 / (roughness^2 + 1e-20),
    scalar parameters read the first array element, reflectiveness.w is the
    exponent, unset values take the defaults."""
    m = bvh.materials_from_json(SCENE_JSON, ["Lamp", "Matte", "Coated"])
    f = np.float32
    lamp, matte, coated = m
    assert np.allclose(lamp[0:3], 0.5) and lamp[3] == f(1.5) and np.allclose(lamp[4:7], 1.0)
    assert np.allclose(lamp[8:11], [0.5, 0.6, 0.7]) and lamp[11] == f(1.0) / (f(1.0) + f(1e-20))
    assert np.allclose(lamp[12:15], [10, 20, 30]) and np.allclose(lamp[16:19], 0.03)
    assert np.allclose(lamp[20:23], 0.97)
    assert np.allclose(matte[0:3], [0.25, 0.5, 0.75]) and matte[11] == f(1.0) / (f(0.25) + f(1e-20))
    assert np.allclose(coated[16:19], [0.2, 0.3, 0.4]) and np.allclose(coated[20:23], [0.8, 0.7, 0.6])
    assert np.allclose(coated[4:7], 0.0) and coated[3] == f(1.33)
    assert np.isclose(coated[11], 1.0 / (0.1 * 0.1))


@pytest.mark.parametrize("text,names", [(SCENE_JSON, ["Textured"]), (SCENE_JSON, ["Missing"]),
                                        ('{"materials": {', ["Matte"]), ("[1, 2]", ["Matte"])])
def test_material_json_errors(built, text, names):
    with pytest.raises(ValueError):
        bvh.materials_from_json(text, names)


def test_file_carries_material_names(built, tmp_path):
    sc = scenes.displaced_icosphere(500, seed=5)
    p = tmp_path / "named.bim"
    bvh.write_bvh_file(sc["positions"], sc["triangles"], str(p), material_names=["Matte", "Coated"])
    b = bvh.read_bvh_file(str(p))
    assert b.material_names == ["Matte", "Coated"]
    with pytest.raises(ValueError):
        bvh.write_bvh_file(sc["positions"], sc["triangles"], str(p), material_names=["x" * 40])
