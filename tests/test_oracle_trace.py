"""The oracle's traversal against brute force and analytic known answers.

The reference ships no golden vectors, so the oracle is checked two ways:
  * its BVH walk returns exactly the triangle and t that an O(N) scan with the
    same triangle test and the same strict '<' finds (ties aside);
  * the triangle test reproduces the hand-derived cases in
    tests/golden/kat_triangles.json (exact rational arithmetic, see
    tests/golden/make_kat.py).
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import oracle
from gpugi_gb300 import bvh, scenes

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("method,leaf", [("sweep", 8), ("kdtree", 8), ("sweep", 2), ("kdtree", 1), ("lds", 8)])
def test_walk_matches_bruteforce(built, method, leaf):
    sc = scenes.displaced_icosphere(4096, seed=21)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method=method, leaf_size=leaf)
    # Rays aimed at the object so most of them hit.
    rays = scenes.aimed_rays(6000, sc["positions"], seed=4)
    o = oracle.trace_closest(b, sc["positions"], rays)
    bf = oracle.bruteforce_closest(b.slots, sc["positions"], rays)
    hit = bf["slot"] >= 0
    assert hit.mean() > 0.3
    same_t = o["t"].view(np.uint32) == bf["t"].view(np.uint32)
    assert same_t.all()
    # slots may differ only where two triangles report bit-identical t
    diff = o["slot"] != bf["slot"]
    assert diff.sum() <= max(2, int(0.001 * len(diff)))
    occ = oracle.trace_any(b, sc["positions"], rays)["occluded"]
    assert np.array_equal(occ.astype(bool), hit)


def test_tmax_limits_hits(built):
    sc = scenes.displaced_icosphere(2048, seed=8)
    b = bvh.build_bvh(sc["positions"], sc["triangles"])
    rays = scenes.aimed_rays(3000, sc["positions"], seed=9)
    full = oracle.trace_closest(b, sc["positions"], rays)
    half = dict(rays)
    cut = np.where(full["slot"] >= 0, full["t"] * 0.5, np.float32(np.inf)).astype(np.float32)
    half["tmax"] = cut
    r = oracle.trace_closest(b, sc["positions"], half)
    assert (r["slot"][full["slot"] >= 0] == -1).all()
    assert np.array_equal(r["t"][full["slot"] >= 0], cut[full["slot"] >= 0])
    # any-hit with tmax exactly at the hit distance is not occluded (strict '<')
    at = dict(rays)
    at["tmax"] = np.where(full["slot"] >= 0, full["t"], np.float32(np.inf)).astype(np.float32)
    occ = oracle.trace_any(b, sc["positions"], at)["occluded"]
    first = oracle.bruteforce_closest(b.slots, sc["positions"], at)
    assert np.array_equal(occ.astype(bool), first["slot"] >= 0)


def test_counters_and_bytes(built):
    sc = scenes.displaced_icosphere(4096, seed=1)
    b = bvh.build_bvh(sc["positions"], sc["triangles"])
    rays = scenes.random_rays(2000, seed=2)
    o = oracle.trace_closest(b, sc["positions"], rays, counters=True)
    c = o["counters"]
    assert (c[:, 0] >= 1).all()  # the root is always tested
    assert (c[:, 2] <= c[:, 1]).all()
    by = oracle.algorithmic_bytes(c)
    assert (by >= 24 + 16 + 32).all()


def _kat_scene(p0, p1, p2):
    positions = np.array([p0, p1, p2], dtype=np.float32)
    tri = np.array([[0, 1, 2, 0]], dtype=np.uint32)
    return positions, tri


def test_triangle_known_answers(built):
    cases = json.loads((GOLDEN / "kat_triangles.json").read_text())["cases"]
    assert len(cases) >= 8
    for c in cases:
        positions, tri = _kat_scene(*c["triangle"])
        b = bvh.build_bvh(positions, tri)
        rays = {k: np.array([v], np.float32) for k, v in zip(("ox", "oy", "oz"), c["origin"])}
        rays.update({k: np.array([v], np.float32) for k, v in zip(("dx", "dy", "dz"), c["direction"])})
        rays["tmax"] = np.array([c["tmax"] if c["tmax"] is not None else math.inf], np.float32)
        # the bare triangle test (brute force has no box test)
        bf = oracle.bruteforce_closest(b.slots, positions, rays)
        assert (bf["slot"][0] >= 0) == c["hit"], c["name"]
        if c["hit"]:
            assert bf["t"][0] == np.float32(c["t"]), c["name"]
        # the full walk: box test of the node, then the triangle
        o = oracle.trace_closest(b, positions, rays)
        assert (o["slot"][0] >= 0) == c["walk_hit"], c["name"]
        if c["walk_hit"]:
            assert o["t"][0] == np.float32(c["t"]), c["name"]
            assert o["u"][0] == np.float32(c["u"]) and o["v"][0] == np.float32(c["v"]), c["name"]


def test_watertight_oracle_closes_cracks():
    """The watertight restatement (Woop, Benthin and Wald 2013, with the robust
    box test of Ize 2013) hits a closed mesh with every ray from its centre
    through its vertices and edge midpoints, in the walk and by brute force;
    the reference's Moeller-Trumbore test lets a share of them slip through
    (it is not watertight, intersectiontests.glsl:55-79)."""
    sc = scenes.closed_icosphere(4, seed=1)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    rays = scenes.crack_rays(sc)
    wt = oracle.trace_closest(b, sc["positions"], rays, watertight=True)
    assert (wt["slot"] >= 0).all()
    assert (oracle.bruteforce_closest(b.slots, sc["positions"], rays, watertight=True)["slot"] >= 0).all()
    assert oracle.trace_any(b, sc["positions"], rays, watertight=True)["occluded"].all()
    ref = oracle.trace_closest(b, sc["positions"], rays)
    assert (ref["slot"] < 0).sum() > 100


def test_watertight_oracle_matches_bruteforce_and_reference_hits():
    """Away from edges both tests find the same triangles: the walk equals brute
    force in watertight mode, and its hits agree with the reference test's on
    almost every random ray (t within a few ulp: the two tests round
    differently)."""
    sc = scenes.displaced_icosphere(4096, seed=3)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    rays = scenes.aimed_rays(20000, sc["positions"], seed=4)
    wt = oracle.trace_closest(b, sc["positions"], rays, watertight=True)
    bf = oracle.bruteforce_closest(b.slots, sc["positions"], rays, watertight=True)
    assert (wt["t"].view(np.uint32) == bf["t"].view(np.uint32)).mean() > 0.999
    ref = oracle.trace_closest(b, sc["positions"], rays)
    assert (wt["slot"] == ref["slot"]).mean() > 0.995
    both = (wt["slot"] >= 0) & (wt["slot"] == ref["slot"])
    dt = np.abs(wt["t"][both].view(np.int32).astype(np.int64) - ref["t"][both].view(np.int32).astype(np.int64))
    assert np.median(dt) <= 2
    hit = wt["slot"] >= 0
    assert np.allclose(wt["u"][both], ref["u"][both], atol=1e-4)
    assert hit.mean() > 0.3


@pytest.mark.parametrize("method", ["sweep", "kdtree"])
def test_oriented_box_walk_matches_bruteforce(method):
    """The oracle's OBOX_BVH walk (FetchIntersectOBoxNode) over the fitted
    oriented boxes finds the brute-force closest hits, the same ones as the
    box hierarchy of the same topology, while testing fewer triangles."""
    sc = scenes.displaced_icosphere(8192, seed=12)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method=method, fit="obox")
    a = bvh.build_bvh(sc["positions"], sc["triangles"], method=method)
    rays = scenes.aimed_rays(30000, sc["positions"], seed=13)
    o = oracle.trace_closest(b, sc["positions"], rays, counters=True)
    bf = oracle.bruteforce_closest(b.slots, sc["positions"], rays)
    assert (o["t"].view(np.uint32) == bf["t"].view(np.uint32)).mean() > 0.999
    oa = oracle.trace_closest(a, sc["positions"], rays, counters=True)
    assert (o["t"].view(np.uint32) == oa["t"].view(np.uint32)).mean() > 0.999
    assert o["counters"][:, 2].sum() < oa["counters"][:, 2].sum()
    occ = oracle.trace_any(b, sc["positions"], rays)["occluded"]
    assert np.array_equal(occ.astype(bool), o["slot"] >= 0)
