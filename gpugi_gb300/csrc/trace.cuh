// Stackless escape-pointer BVH walk and its intersection tests (device code).
//
// Same walk as gpugi's TraceRay/TraceRayAnyHit (gpugi/shader/traceray.glsl:
// 25-180): nodes are visited in preorder; a node whose bounds are hit with
// firstHit <= rayLength descends into firstChild (or tests the leaf block and
// then continues at escape), a missed node continues at escape, and escape 0
// ends the walk. Leaf slots are tested in order and a triangle is accepted
// when hit < rayLength (strict, so ties keep the first slot found). The
// node/leaf state machine of the shader is written here as two nested loops
// that perform the same sequence of tests.
#pragma once
#include "common.cuh"
#include "scene.cuh"

namespace gpugi {

// IntersectBox (intersectiontests.glsl:9-20). min/max are IEEE minNum/maxNum
// (fminf/fmaxf): an axis-parallel ray produces inf*0 = NaN slabs that drop out
// (a ray lying in a face plane of the box then misses it).
// ROBUST is the box test of the watertight mode (an addition): a slab of a
// ray that lies in one of its bounding planes (a NaN slab value) does not
// constrain the ray, and the exit distance is widened by 1 + 2 gamma(3),
// rounded up to 1 + 2^-21 (Ize, "Robust BVH Ray Traversal", JCGT 2(2),
// 2013), so that rounding never culls a box whose surface the ray touches:
// a ray through a vertex or edge on the box boundary still reaches the
// triangles there.
template <bool ROBUST = false>
GPUGI_D bool intersect_box(float3 o, float3 inv, float4 lo, float4 hi, float& firstHit) {
    // x and y slabs as packed pairs (add.f32x2 / mul.f32x2: per component
    // the same IEEE round-to-nearest results as the scalar operations;
    // lo - o as lo + (-o), exact for every input including signed zeros)
    const float2 no = make_float2(-o.x, -o.y), ixy = make_float2(inv.x, inv.y);
    const float2 b2 = __fmul2_rn(__fadd2_rn(make_float2(lo.x, lo.y), no), ixy);
    const float2 t2 = __fmul2_rn(__fadd2_rn(make_float2(hi.x, hi.y), no), ixy);
    float tbx = b2.x, tby = b2.y, tbz = X::mul(inv.z, X::sub(lo.z, o.z));
    float ttx = t2.x, tty = t2.y, ttz = X::mul(inv.z, X::sub(hi.z, o.z));
    float mnx = fminf(ttx, tbx), mny = fminf(tty, tby), mnz = fminf(ttz, tbz);
    float mxx = fmaxf(ttx, tbx), mxy = fmaxf(tty, tby), mxz = fmaxf(ttz, tbz);
    if (ROBUST) {
        const float inf = __int_as_float(0x7f800000);
        if (isnan(tbx) || isnan(ttx)) mnx = -inf, mxx = inf;
        if (isnan(tby) || isnan(tty)) mny = -inf, mxy = inf;
        if (isnan(tbz) || isnan(ttz)) mnz = -inf, mxz = inf;
    }
    // max(max(mnx, mny), max(mnx, mnz)) of the shader is the maximum of the
    // three (NaNs ignored either way); likewise for the minimum
    firstHit = fmaxf(0.0f, max3f(mnx, mny, mnz));
    float lastHit = min3f(mxx, mxy, mxz);
    if (ROBUST) lastHit = X::mul(lastHit, 0x1.000008p+0f);
    return firstHit <= lastHit;
}

// Ray against a stored axis-aligned ellipsoid. The node holds {center,
// ir = 1 / (radii + 1e-15)} (reciprocals taken at upload; the guard is the
// one of IntersectVirtualEllipsoid, intersectiontests.glsl:26-52). The steps
// are that function's: advance the ray to its closest approach to the centre
// for stability, scale into the unit sphere and solve the quadratic; the
// scaling multiplies by ir and the two quotients by ddotd share one
// reciprocal, so a node costs one correctly rounded reciprocal and one sqrt
// instead of eight divisions and a sqrt. The reference never walks
// ellipsoids, so this test defines the node kind; the oracle restates it
// operation for operation.
GPUGI_D bool intersect_ellipsoid(float3 ro, float3 rd, float4 c, float4 ir, float& firstHit) {
    float3 o = X::sub3(ro, xyz(c));
    const float t = fmaxf(0.0f, -X::dot(o, rd));
    o = X::add3(o, X::scale(t, rd));
    o = X::mul3(o, xyz(ir));
    const float3 d = X::mul3(rd, xyz(ir));
    const float odoto = X::dot(o, o), odotd = X::dot(o, d), ddotd = X::dot(d, d);
    const float inv = X::rcp(ddotd);
    const float phalf = X::mul(odotd, inv);
    const float q = X::mul(X::sub(odoto, 1.0f), inv);
    float rad = X::sub(X::mul(phalf, phalf), q);
    if (rad < 0.0f) return false;
    rad = __fsqrt_rn(rad);
    firstHit = fmaxf(0.0f, X::add(X::sub(-phalf, rad), t));
    return X::add(X::add(-phalf, rad), t) >= 0.0f;
}

// rotate(x, q) (intersectiontests.glsl:82-89) in the shader's operation order.
GPUGI_D float3 qrotate(float3 x, float4 q) {
    const float3 t = X::cross(make_float3(q.x, q.y, q.z), x);
    const float3 u = make_float3(X::sub(X::add(X::mul(q.w, t.x), X::mul(q.y, t.z)), X::mul(q.z, t.y)),
                                 X::sub(X::add(X::mul(q.w, t.y), X::mul(q.z, t.x)), X::mul(q.x, t.z)),
                                 X::sub(X::add(X::mul(q.w, t.z), X::mul(q.x, t.y)), X::mul(q.y, t.x)));
    return X::add3(x, X::scale(2.0f, u));
}

// FetchIntersectOBoxNode (intersectiontests.glsl:114-128) on the 48-B node
// {center | child}, {sidesHalf | escape}, rotationInv: the ray is rotated
// into the box frame (origin relative to the centre), its direction
// inverted there, and the box [-sidesHalf, sidesHalf] tested with
// IntersectBox (ROBUST: the watertight mode's box test).
template <bool ROBUST = false>
GPUGI_D bool intersect_obox(float3 ro, float3 rd, float4 a, float4 b, float4 rotationInv, float& firstHit) {
    const float3 o = qrotate(X::sub3(ro, xyz(a)), rotationInv);
    const float3 d = qrotate(rd, rotationInv);
    const float3 inv = make_float3(X::rcp(d.x), X::rcp(d.y), X::rcp(d.z));
    return intersect_box<ROBUST>(o, inv, make_float4(-b.x, -b.y, -b.z, 0.0f), b, firstHit);
}

// Node layouts: AABB and ellipsoid nodes take 2 float4, oriented boxes 3.
template <int BOUNDS>
constexpr uint32_t node_stride() {
    return BOUNDS == 2 ? 3u : 2u;
}
// The bounds test of a node kind (0 box, 1 ellipsoid, 2 oriented box); c is
// the oriented box's third texel (unused otherwise).
template <int BOUNDS, bool ROBUST>
GPUGI_D bool bounds_test(float3 o, float3 d, float3 inv, float4 a, float4 b, float4 c, float& firstHit) {
    if (BOUNDS == 0) return intersect_box<ROBUST>(o, inv, a, b, firstHit);
    if (BOUNDS == 1) return intersect_ellipsoid(o, d, a, b, firstHit);
    return intersect_obox<ROBUST>(o, d, a, b, c, firstHit);
}

// IntersectTriangle (intersectiontests.glsl:63-79) on the precomputed record
// {p0, e0, e1, n}. Returns hit distance and the two barycentrics (y, z).
GPUGI_D bool intersect_triangle_v(float3 o, float3 d, float4 a, float4 b, float4 c, float& hit, float& by,
                                  float& bz) {
    float3 p0 = make_float3(a.x, a.y, a.z);
    float3 e0 = make_float3(a.w, b.x, b.y);
    float3 e1 = make_float3(b.z, b.w, c.x);
    float3 n = make_float3(c.y, c.z, c.w);
    float3 e2 = X::scale(X::rcp(X::dot(n, d)), X::sub3(p0, o));
    float3 i = X::cross(d, e2);
    by = X::dot(i, e1);
    bz = X::dot(i, e0);
    float bx = X::sub(1.0f, X::add(bz, by));
    hit = X::dot(n, e2);
    return (hit > 0.0001f) && bx >= 0.0f && by >= 0.0f && bz >= 0.0f;
}
GPUGI_D bool intersect_triangle(float3 o, float3 d, const float4* rec, float& hit, float& by, float& bz) {
    return intersect_triangle_v(o, d, __ldg(rec), __ldg(rec + 1), __ldg(rec + 2), hit, by, bz);
}

// Watertight ray/triangle test (an addition; the reference's test above is
// not watertight): Woop, Benthin and Wald, "Watertight Ray/Triangle
// Intersection", JCGT 2(1), 2013. Per ray, the axis kz of the largest
// |direction| component becomes the ray's z axis (kx, ky follow cyclically,
// swapped when d[kz] < 0 to keep the winding) and the shear
// S = (d[kx] / d[kz], d[ky] / d[kz], 1 / d[kz]) maps the ray onto +z. Per
// triangle, the vertices relative to the origin are sheared into that frame
// and the three 2D edge functions U, V, W are evaluated; an edge function
// that comes out exactly 0 is evaluated again in double precision (products
// of two floats are exact there), so rays through shared edges and vertices
// of a closed mesh see consistent signs and never slip through. Two-sided:
// U, V, W must not have mixed signs and det = U + V + W must not be 0; then
// t = T / det with T = U Az + V Bz + W Cz. The hit rule of the reference
// test is kept: t > 1e-4 (INTERSECT_EPSILON), and the walk accepts
// t < rayLength. Barycentrics (u, v) = (V, W) / det, the weights of p1 and
// p2 as in gpugi's convention. Records hold the exact vertices
// {p0.xyz p1.x | p1.yz p2.xy | p2.z 0 0 0} (48 B, like the reference records).
struct WtRay {
    float Sx, Sy, Sz;
    uint32_t kx, ky, kz;
};
GPUGI_D float comp3(float3 v, uint32_t k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
GPUGI_D WtRay wt_setup(float3 d) {
    WtRay w;
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    w.kz = ax >= ay ? (ax >= az ? 0u : 2u) : (ay >= az ? 1u : 2u);
    w.kx = w.kz == 2u ? 0u : w.kz + 1u;
    w.ky = w.kx == 2u ? 0u : w.kx + 1u;
    const float dz = comp3(d, w.kz);
    if (dz < 0.0f) {
        const uint32_t t = w.kx;
        w.kx = w.ky;
        w.ky = t;
    }
    w.Sx = X::div(comp3(d, w.kx), dz);
    w.Sy = X::div(comp3(d, w.ky), dz);
    w.Sz = X::rcp(dz);
    return w;
}
GPUGI_D float wt_edge(float ax, float ay, float bx, float by) {  // ax * by - ay * bx
    return X::sub(X::mul(ax, by), X::mul(ay, bx));
}
GPUGI_D float wt_edge64(float ax, float ay, float bx, float by) {
    return __double2float_rn(__dsub_rn(__dmul_rn((double)ax, (double)by), __dmul_rn((double)ay, (double)bx)));
}
GPUGI_D bool intersect_triangle_wt_v(float3 o, const WtRay& w, float4 ra, float4 rb, float4 rc, float& hit,
                                     float& by, float& bz) {
    const float3 A = X::sub3(make_float3(ra.x, ra.y, ra.z), o);
    const float3 B = X::sub3(make_float3(ra.w, rb.x, rb.y), o);
    const float3 C = X::sub3(make_float3(rb.z, rb.w, rc.x), o);
    const float Akz = comp3(A, w.kz), Bkz = comp3(B, w.kz), Ckz = comp3(C, w.kz);
    const float Ax = X::sub(comp3(A, w.kx), X::mul(w.Sx, Akz)), Ay = X::sub(comp3(A, w.ky), X::mul(w.Sy, Akz));
    const float Bx = X::sub(comp3(B, w.kx), X::mul(w.Sx, Bkz)), By = X::sub(comp3(B, w.ky), X::mul(w.Sy, Bkz));
    const float Cx = X::sub(comp3(C, w.kx), X::mul(w.Sx, Ckz)), Cy = X::sub(comp3(C, w.ky), X::mul(w.Sy, Ckz));
    float U = wt_edge(Cx, Cy, Bx, By), V = wt_edge(Ax, Ay, Cx, Cy), W = wt_edge(Bx, By, Ax, Ay);
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = wt_edge64(Cx, Cy, Bx, By);
        V = wt_edge64(Ax, Ay, Cx, Cy);
        W = wt_edge64(Bx, By, Ax, Ay);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = X::add(X::add(U, V), W);
    if (det == 0.0f) return false;
    const float T = X::add(X::add(X::mul(U, X::mul(w.Sz, Akz)), X::mul(V, X::mul(w.Sz, Bkz))),
                           X::mul(W, X::mul(w.Sz, Ckz)));
    const float rcpDet = X::rcp(det);
    hit = X::mul(T, rcpDet);
    by = X::mul(V, rcpDet);
    bz = X::mul(W, rcpDet);
    return hit > 0.0001f;
}
// The triangle test of a leaf slot: TRI 0 = the reference's, 1 = watertight.
template <int TRI>
GPUGI_D bool slot_test(const DevScene& s, float3 o, float3 d, const WtRay& w, uint32_t k, float& hit, float& by,
                       float& bz) {
    if (TRI == 0) return intersect_triangle(o, d, s.tris + 3 * (size_t)k, hit, by, bz);
    const float4* rec = s.wtris + 3 * (size_t)k;
    return intersect_triangle_wt_v(o, w, __ldg(rec), __ldg(rec + 1), __ldg(rec + 2), hit, by, bz);
}

struct TraceResult {
    int32_t slot;  // -1 = miss
    float t;
    float u, v;
};

// Fetch counters of one walk, the analogue of TRACERAY_DEBUG_VARS
// (traceray.glsl:59-61,131-133): node fetches, leaf slot fetches (the shader
// also fetches the first invalid slot of a block before leaving it) and
// valid triangles tested.
struct WalkCounters {
    uint32_t nodes = 0, slots = 0, tris = 0;
};

// The walk. ANY_HIT returns at the first accepted triangle (result.slot set
// to the accepting slot). Every loop is bounded: a validated hierarchy
// strictly increases the node index, so numNodes visits always suffice; the
// cap only guards against device memory corruption and reports
// DEVERR_TRAVERSAL_CAP instead of spinning.
template <bool ANY_HIT, int BOUNDS, bool COUNT = false, int TRI = 0>
GPUGI_D TraceResult trace_ray(const DevScene& s, float3 o, float3 d, float rayLength, uint32_t* errWord,
                              WalkCounters* cnt = nullptr) {
    TraceResult r;
    r.slot = -1;
    r.u = r.v = 0.0f;
    const float3 inv = make_float3(X::rcp(d.x), X::rcp(d.y), X::rcp(d.z));
    const WtRay wt = TRI ? wt_setup(d) : WtRay{};
    uint32_t node = 0;
    uint32_t budget = s.numNodes;
    const float4* __restrict__ nodes = s.nodes;
    while (true) {
        if (budget-- == 0) {
            raise_error(errWord, DEVERR_TRAVERSAL_CAP);
            break;
        }
        if (kChecked && node >= s.numNodes) {
            raise_error(errWord, DEVERR_BOUNDS);
            break;
        }
        if (COUNT) ++cnt->nodes;
        const float4* nd = nodes + node_stride<BOUNDS>() * (size_t)node;
        const float4 a = __ldg(nd);
        const float4 b = __ldg(nd + 1);
        const float4 c = BOUNDS == 2 ? __ldg(nd + 2) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const uint32_t child = __float_as_uint(a.w);
        const uint32_t escape = __float_as_uint(b.w);
        float firstHit;
        const bool hit = bounds_test<BOUNDS, TRI != 0>(o, d, inv, a, b, c, firstHit);
        if (hit && firstHit <= rayLength) {
            if (child & LEAF_FLAG) {
                const uint32_t count = (child >> LEAF_COUNT_SHIFT) & LEAF_COUNT_MASK;
                const uint32_t slot0 = (child & LEAF_BLOCK_MASK) * s.leafSize;
                if (kChecked && (uint64_t)slot0 + count > s.numSlots) {
                    raise_error(errWord, DEVERR_BOUNDS);
                    break;
                }
                if (COUNT) cnt->slots += count < s.leafSize ? count + 1 : count;
                for (uint32_t k = 0; k < count; ++k) {
                    if (COUNT) ++cnt->tris;
                    float h, by, bz;
                    if (slot_test<TRI>(s, o, d, wt, slot0 + k, h, by, bz) && h < rayLength) {
                        rayLength = h;
                        r.slot = (int32_t)(slot0 + k);
                        r.u = by;
                        r.v = bz;
                        if (ANY_HIT) {
                            // the shader stops fetching at the accepting slot
                            if (COUNT) cnt->slots -= (count < s.leafSize ? count + 1 : count) - (k + 1);
                            r.t = rayLength;
                            return r;
                        }
                    }
                }
                node = escape;
            } else {
                node = child;
            }
        } else {
            node = escape;
        }
        if (node == 0) break;
    }
    r.t = rayLength;
    return r;
}

// One ray's walk as a resumable state machine, advanced one test at a time.
// The sequence of node and triangle tests is the same as trace_ray's; the
// state lets a persistent warp refill a finished lane with the next ray
// instead of idling until the warp's longest walk ends. (Testing a whole
// leaf block per step, four triangles at a time, was measured 18 % slower on
// the 65,536-triangle icosphere: lanes of a warp then diverge between node
// steps and leaf loops of different lengths.)
struct WalkState {
    float3 o, d, inv;
    WtRay wt;  // used by the watertight test only
    float len;
    uint32_t node;  // next node to test, NODE_DONE when the escape chain ended
    uint32_t cur, end;  // leaf slots still to test
    uint32_t budget;
    int32_t slot;
    float u, v;
};
constexpr uint32_t NODE_DONE = 0xFFFFFFFFu;

GPUGI_D void walk_begin(WalkState& w, const DevScene& s, float3 o, float3 d, float tmax) {
    w.o = o;
    w.d = d;
    w.inv = make_float3(X::rcp(d.x), X::rcp(d.y), X::rcp(d.z));
    w.wt = wt_setup(d);  // dead code unless a watertight walker reads it
    w.len = tmax;
    w.node = 0;
    w.cur = w.end = 0;
    w.budget = s.numNodes;
    w.slot = -1;
    w.u = w.v = 0.0f;
}

// Copy the first `count` nodes (the top tree levels, see DevScene::topNodes)
// into shared memory. Called by every thread of a block before its walks.
GPUGI_D void stage_top_nodes(const DevScene& s, float4* smem, uint32_t count) {
    // oriented-box scenes stage nothing (their upload keeps the preorder layout)
    for (uint32_t i = threadIdx.x; i < 2 * count; i += blockDim.x) smem[i] = __ldg(s.nodes + i);
    __syncthreads();
}

// Perform one test. Returns true when the walk is over (for ANY_HIT also
// when a triangle was accepted). Nodes below topCount come from `top`.
// Node and triangle steps share one fetch (the record address depends on the
// step kind), so the lanes of a warp that are at different kinds of step
// wait for one memory round trip per step instead of one per kind.
template <bool ANY_HIT, int BOUNDS, int TRI = 0>
GPUGI_D bool walk_step(WalkState& w, const DevScene& s, uint32_t* errWord, const float4* top = nullptr,
                       uint32_t topCount = 0) {
    const bool isTri = w.cur < w.end;
    if (!isTri && w.budget-- == 0) {
        raise_error(errWord, DEVERR_TRAVERSAL_CAP);
        w.node = NODE_DONE;
        return true;
    }
    if (kChecked && (isTri ? w.cur >= s.numSlots : w.node >= s.numNodes)) {
        raise_error(errWord, DEVERR_BOUNDS);
        w.cur = w.end;
        w.node = NODE_DONE;
        return true;
    }
    float4 a, b, c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    constexpr uint32_t NS = node_stride<BOUNDS>();
    if (!isTri && w.node < topCount) {
        a = top[NS * w.node];
        b = top[NS * w.node + 1];
        if (BOUNDS == 2) c = top[NS * w.node + 2];
    } else {
        const float4* src =
            isTri ? (TRI ? s.wtris : s.tris) + 3 * (size_t)w.cur : s.nodes + NS * (size_t)w.node;
        a = __ldg(src);
        b = __ldg(src + 1);
        if (isTri || BOUNDS == 2) c = __ldg(src + 2);
    }
    if (isTri) {
        float h, by, bz;
        const bool ok = TRI ? intersect_triangle_wt_v(w.o, w.wt, a, b, c, h, by, bz)
                            : intersect_triangle_v(w.o, w.d, a, b, c, h, by, bz);
        if (ok && h < w.len) {
            w.len = h;
            w.slot = (int32_t)w.cur;
            w.u = by;
            w.v = bz;
            if (ANY_HIT) return true;
        }
        ++w.cur;
    } else {
        const uint32_t child = __float_as_uint(a.w);
        const uint32_t escape = __float_as_uint(b.w);
        float firstHit;
        const bool hit = bounds_test<BOUNDS, TRI != 0>(w.o, w.d, w.inv, a, b, c, firstHit);
        if (hit && firstHit <= w.len) {
            if (child & LEAF_FLAG) {
                w.cur = (child & LEAF_BLOCK_MASK) * s.leafSize;
                w.end = w.cur + ((child >> LEAF_COUNT_SHIFT) & LEAF_COUNT_MASK);
                w.node = escape ? escape : NODE_DONE;
            } else {
                w.node = child;
            }
        } else {
            w.node = escape ? escape : NODE_DONE;
        }
    }
    return w.cur >= w.end && w.node == NODE_DONE;
}

// ---------------------------------------------------------------- group walk
// G lanes walk one ray together (G = 4, 8 or 16; every lane of the group
// holds the same state and calls group_step with it). A node round tests
// the G consecutive nodes [node, node + G) of the node array (one coalesced
// load), then resolves which of them the sequential walk visits by pointer
// jumping over the successors inside the window (log2 G shuffles): the walk
// leaves the window at a node outside it, at the end of the escape chain or
// at a hit leaf. A leaf round tests G slots of the leaf block at once and
// applies the sequential acceptance rule: a slot is accepted when
// hit < rayLength, so the result is the first slot reaching the minimum (any
// hit: the first accepted slot). Every node decision uses trace_ray's
// arithmetic with the same rayLength, so results are identical; tests of
// nodes the walk skips are discarded. Successors may point backwards (the
// breadth-first top-level layout): they simply end the round.
struct GroupWalk {
    float3 o, d, inv;
    WtRay wt;  // used by the watertight test only
    float len, u, v;
    int32_t slot;
    uint32_t node, cur, end, resume, budget;
};
constexpr uint32_t kGroupDone = 0xFFFFFFFFu, kGroupLeaf = 0x80000000u;

GPUGI_D void group_begin(GroupWalk& g, const DevScene& s, float3 o, float3 d, float tmax) {
    g.o = o;
    g.d = d;
    g.inv = make_float3(X::rcp(d.x), X::rcp(d.y), X::rcp(d.z));
    g.wt = wt_setup(d);  // dead code unless a watertight walker reads it
    g.len = tmax;
    g.u = g.v = 0.0f;
    g.slot = -1;
    g.node = 0;
    g.cur = g.end = 0;
    g.resume = kGroupDone;
    g.budget = s.numNodes;
}

// One round; returns true when the walk is over. gl = lane in the group,
// gbase = first lane of the group, gmask = the group's lanes.
template <bool ANY_HIT, int BOUNDS, int G, int TRI = 0>
GPUGI_D bool group_step(GroupWalk& g, const DevScene& s, uint32_t* err, unsigned gl, unsigned gbase,
                        unsigned gmask) {
    static_assert(G == 4 || G == 8 || G == 16, "group size");
    if (g.cur < g.end) {
        const uint32_t k = g.cur + gl;
        float h = 0.0f, by = 0.0f, bz = 0.0f;
        bool ok = false;
        if (k < g.end) ok = slot_test<TRI>(s, g.o, g.d, g.wt, k, h, by, bz) && h < g.len;
        if (ANY_HIT) {
            const uint32_t key = __reduce_min_sync(gmask, ok ? k : kGroupDone);
            if (key != kGroupDone) {
                g.slot = (int32_t)key;
                return true;
            }
        } else {
            // minimum hit distance (positive floats order like their bits),
            // then the lowest slot reaching it
            const uint32_t hb = __reduce_min_sync(gmask, ok ? __float_as_uint(h) : kGroupDone);
            const unsigned tie = __ballot_sync(gmask, ok && __float_as_uint(h) == hb);
            const unsigned src = tie ? (unsigned)(__ffs(tie) - 1) : gbase;
            const float wu = __shfl_sync(gmask, by, src), wv = __shfl_sync(gmask, bz, src);
            if (tie) {
                g.slot = (int32_t)(g.cur + (src - gbase));
                g.len = __uint_as_float(hb);
                g.u = wu;
                g.v = wv;
            }
        }
        g.cur = min(g.cur + G, g.end);
        if (g.cur >= g.end) {
            g.node = g.resume;
            if (g.node == kGroupDone) return true;
        }
        return false;
    }
    if (g.budget-- == 0) {
        raise_error(err, DEVERR_TRAVERSAL_CAP);
        return true;
    }
    if (kChecked && g.node >= s.numNodes) {
        raise_error(err, DEVERR_BOUNDS);
        return true;
    }
    const uint32_t p = g.node + gl;
    uint32_t next = kGroupDone, child = 0, escape = 0;
    if (p < s.numNodes) {
        const float4* nd = s.nodes + node_stride<BOUNDS>() * (size_t)p;
        const float4 a = __ldg(nd), b = __ldg(nd + 1);
        const float4 c = BOUNDS == 2 ? __ldg(nd + 2) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        child = __float_as_uint(a.w);
        escape = __float_as_uint(b.w);
        float firstHit;
        const bool hit = bounds_test<BOUNDS, TRI != 0>(g.o, g.d, g.inv, a, b, c, firstHit);
        if (hit && firstHit <= g.len) next = (child & LEAF_FLAG) ? (kGroupLeaf | gl) : child;
        else next = escape ? escape : kGroupDone;
    }
#pragma unroll
    for (int r = 1; r < G; r <<= 1) {
        const bool chase = next < kGroupLeaf && next - g.node < (uint32_t)G;
        const uint32_t w = __shfl_sync(gmask, next, gbase + (chase ? next - g.node : gl));
        next = chase ? w : next;
    }
    const uint32_t r0 = __shfl_sync(gmask, next, gbase);
    if (r0 == kGroupDone) return true;
    if (r0 & kGroupLeaf) {
        const unsigned src = gbase + (r0 & (kGroupLeaf - 1u));
        const uint32_t lc = __shfl_sync(gmask, child, src), le = __shfl_sync(gmask, escape, src);
        g.cur = (lc & LEAF_BLOCK_MASK) * s.leafSize;
        g.end = g.cur + ((lc >> LEAF_COUNT_SHIFT) & LEAF_COUNT_MASK);
        g.resume = le ? le : kGroupDone;
        if (kChecked && g.end > s.numSlots) {
            raise_error(err, DEVERR_BOUNDS);
            return true;
        }
        if (g.cur >= g.end) {  // empty leaf block
            g.node = g.resume;
            return g.node == kGroupDone;
        }
        return false;
    }
    g.node = r0;
    return false;
}

// Persistent loop of group walks over n work items. Group k of the grid
// takes item k first, then, whenever its walk ends, item (groups in the
// grid) + the value of one atomic increment of *work (which starts at 0).
// load(i, o, d, tmax) fills the ray of item i; finish(i, walk) runs in the
// group's first lane. With MULTI the rays belong to different scenes: load
// returns the item's scene and its bounds kind selects the node test per
// round; otherwise every ray walks `scene` with the BOUNDS test.
template <bool ANY_HIT, int BOUNDS, int G, bool MULTI, int TRI, typename Load, typename Finish>
GPUGI_D void group_walks_impl(const DevScene& scene, uint64_t n, unsigned long long* work, uint32_t* err, Load load,
                              Finish finish) {
    // The loop has no warp-wide synchronisation: all shuffles stay inside
    // the group, and a group leaves once the items are exhausted. The first
    // item needs no atomic, so a launch does not start with one increment
    // per group queued on the same counter (tens of thousands of them
    // serialise in L2 for ~10 us); small launches cost no atomics at all.
    const unsigned lane = threadIdx.x & 31u;
    const unsigned gl = lane & (G - 1), gbase = lane & ~(unsigned)(G - 1);
    const unsigned gmask = ((1u << G) - 1u) << gbase;
    const uint64_t perBlock = blockDim.x / G;
    const uint64_t groups = (uint64_t)gridDim.x * perBlock;
    GroupWalk g;
    DevScene sc;  // MULTI: the ray's scene, copied at its walk's start (fields stay in registers)
    for (uint64_t my = (uint64_t)blockIdx.x * perBlock + threadIdx.x / G; my < n;) {
        float3 o, d;
        float tmax;
        if constexpr (MULTI) {
            sc = *load(my, o, d, tmax);
            group_begin(g, sc, o, d, tmax);
        } else {
            load(my, o, d, tmax);
            group_begin(g, scene, o, d, tmax);
        }
        bool done = false;
        while (!done) {
            if constexpr (MULTI)
                done = sc.boundsKind == GPUGI_BOUNDS_ELLIPSOID ? group_step<ANY_HIT, 1, G>(g, sc, err, gl, gbase, gmask)
                       : sc.boundsKind == GPUGI_BOUNDS_OBOX    ? group_step<ANY_HIT, 2, G>(g, sc, err, gl, gbase, gmask)
                                                               : group_step<ANY_HIT, 0, G>(g, sc, err, gl, gbase, gmask);
            else
                done = group_step<ANY_HIT, BOUNDS, G, TRI>(g, scene, err, gl, gbase, gmask);
        }
        if (gl == 0) finish(my, g);
        unsigned long long next = 0;
        if (gl == 0) next = atomicAdd(work, 1ull);
        my = groups + __shfl_sync(gmask, next, gbase);
    }
}

template <bool ANY_HIT, int BOUNDS, int G, int TRI = 0, typename Load, typename Finish>
GPUGI_D void group_walks(const DevScene& scene, uint64_t n, unsigned long long* work, uint32_t* err, Load load,
                         Finish finish) {
    group_walks_impl<ANY_HIT, BOUNDS, G, false, TRI>(scene, n, work, err, load, finish);
}

template <bool ANY_HIT, int G, typename Load, typename Finish>
GPUGI_D void group_walks_multi(uint64_t n, unsigned long long* work, uint32_t* err, Load load, Finish finish) {
    group_walks_impl<ANY_HIT, 0, G, true, 0>(DevScene{}, n, work, err, load, finish);
}

}  // namespace gpugi
