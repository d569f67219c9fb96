"""Generate tests/golden/kat_triangles.json: known answers for gpugi's
ray-triangle test (gpugi/shader/intersectiontests.glsl:63-79) derived with
exact rational arithmetic, independent of any implementation in this repo.

Every case uses dyadic coordinates so that each intermediate value of the
shader's formula is exactly representable in float32; the script asserts it.
Then the float32 computation has no rounding at all and the expected t, u, v
are exact. Run: python tests/golden/make_kat.py
"""
import json
from fractions import Fraction as Fr
from pathlib import Path

import numpy as np

INF = None


def f32_exact(x):
    if x is None:
        return True
    return Fr(float(np.float32(float(x)))) == x


def sub(a, b): return [a[i] - b[i] for i in range(3)]
def dot(a, b): return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]
def cross(a, b): return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def box_hit(p0, p1, p2, o, d, tmax):
    """IntersectBox (intersectiontests.glsl:9-20) on the triangle's bounding
    box, in float32 with IEEE minNum/maxNum (np.fmin/np.fmax) so that a ray
    lying in a face plane with a zero direction component yields the NaN slab
    the shader produces."""
    f = np.float32
    lo = np.minimum(np.minimum(np.array(p0, f), np.array(p1, f)), np.array(p2, f))
    hi = np.maximum(np.maximum(np.array(p0, f), np.array(p1, f)), np.array(p2, f))
    o, d = np.array(o, f), np.array(d, f)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = f(1.0) / d
        tbot = inv * (lo - o)
        ttop = inv * (hi - o)
    tmin, tmx = np.fmin(ttop, tbot), np.fmax(ttop, tbot)
    first = np.fmax(f(0), np.fmax(np.fmax(tmin[0], tmin[1]), np.fmax(tmin[0], tmin[2])))
    last = np.fmin(np.fmin(tmx[0], tmx[1]), np.fmin(tmx[0], tmx[2]))
    limit = f(np.inf) if tmax is None else f(tmax)
    return bool(first <= last and first <= limit)


def evaluate(p0, p1, p2, o, d, tmax):
    p0, p1, p2, o, d = ([Fr(x) for x in v] for v in (p0, p1, p2, o, d))
    e0, e1 = sub(p1, p0), sub(p0, p2)
    n = cross(e1, e0)
    nd = dot(n, d)
    inter = [*e0, *e1, *n, nd]
    if nd == 0:
        return dict(hit=False, exact=all(f32_exact(x) for x in inter))
    r = 1 / nd
    e2 = [r * x for x in sub(p0, o)]
    i = cross(d, e2)
    by, bz = dot(i, e1), dot(i, e0)
    bx = 1 - (bz + by)
    t = dot(n, e2)
    inter += [r, *e2, *i, by, bz, bx, t, by + bz]
    hit = t > Fr(1, 10000) and bx >= 0 and by >= 0 and bz >= 0 and (tmax is None or t < Fr(tmax))
    return dict(hit=hit, t=float(t), u=float(by), v=float(bz), exact=all(f32_exact(x) for x in inter))


T = ([0, 0, 0], [1, 0, 0], [0, 1, 0])
CASES = [
    ("center_front", T, [0.25, 0.25, 1], [0, 0, -1], INF),
    ("center_back_side", T, [0.25, 0.25, -2], [0, 0, 1], INF),
    ("on_edge_u0", T, [0.5, 0, 1], [0, 0, -1], INF),
    ("on_vertex_p0", T, [0, 0, 1], [0, 0, -1], INF),
    ("on_hypotenuse", T, [0.5, 0.5, 1], [0, 0, -1], INF),
    ("outside_u", T, [0.75, 0.5, 1], [0, 0, -1], INF),
    ("outside_negative", T, [-0.25, 0.25, 1], [0, 0, -1], INF),
    ("pointing_away", T, [0.25, 0.25, 1], [0, 0, 1], INF),
    ("parallel", T, [0.25, 0.25, 1], [1, 0, 0], INF),
    ("tmax_before_hit", T, [0.25, 0.25, 1], [0, 0, -1], 0.5),
    ("tmax_equal_hit", T, [0.25, 0.25, 1], [0, 0, -1], 1.0),
    ("tmax_after_hit", T, [0.25, 0.25, 1], [0, 0, -1], 1.5),
    ("oblique", ([0, 0, 0], [4, 0, 0], [0, 4, 0]), [0, 0, 2], [0.5, 0.5, -1], INF),
    ("scaled_far", ([-8, -8, 16], [8, -8, 16], [0, 8, 16]), [0, 0, 0], [0, 0, 2], INF),
    ("behind_origin_close", T, [0.25, 0.25, 0.0625], [0, 0, -1], INF),
    ("on_edge_oblique", T, [0.5, -0.5, 1], [0, 0.5, -1], INF),
    ("on_vertex_oblique", T, [-0.5, -0.5, 1], [0.5, 0.5, -1], INF),
    ("box_face_plane_axis_parallel", T, [0.25, 0, 1], [0, 0, -1], INF),
]


def main():
    out = []
    for name, (p0, p1, p2), o, d, tmax in CASES:
        r = evaluate(p0, p1, p2, o, d, tmax)
        assert r.pop("exact"), f"{name}: an intermediate value is not exact in float32"
        # walk_hit: what the full traversal returns over a one-node hierarchy
        # (the triangle test gated by the box test of the node).
        r["walk_hit"] = bool(r["hit"] and box_hit(p0, p1, p2, o, d, tmax))
        out.append(dict(name=name, triangle=[p0, p1, p2], origin=o, direction=d, tmax=tmax, **r))
    path = Path(__file__).resolve().parent / "kat_triangles.json"
    path.write_text(json.dumps(dict(
        source="gpugi/shader/intersectiontests.glsl:63-79, exact rational evaluation (make_kat.py)",
        cases=out), indent=1))
    print(f"wrote {len(out)} cases to {path}")


if __name__ == "__main__":
    main()
