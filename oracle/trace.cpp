// ORACLE — test infrastructure only (see glsl.hpp for the parity status).
//
// CPU restatement of gpugi's stackless BVH traversal and its intersection
// tests:
//   IntersectBox            gpugi/shader/intersectiontests.glsl:9-20
//   IntersectTriangle       gpugi/shader/intersectiontests.glsl:63-79
//   FetchIntersectBoxNode   gpugi/shader/intersectiontests.glsl:100-111
//   IntersectVirtualEllipsoid gpugi/shader/intersectiontests.glsl:26-52 (restated
//                           for a stored {center, radii} node, see below)
//   TraceRay/TraceRayAnyHit gpugi/shader/traceray.glsl:18-180
// plus a brute-force O(N) closest-hit search used to check the walk itself.
#include "oracle.hpp"
#include <cstring>
#include <limits>

using namespace glsl;

namespace oracle {

static const float INTERSECT_EPSILON = 0.0001f;  // intersectiontests.glsl:1

// intersectiontests.glsl:9-20
static bool IntersectBox(vec3 rayOrigin, vec3 invRayDir, vec3 aabbMin, vec3 aabbMax,
                         float& firstHit, float& lastHit) {
    vec3 tbot = invRayDir * (aabbMin - rayOrigin);
    vec3 ttop = invRayDir * (aabbMax - rayOrigin);
    vec3 tmin = min(ttop, tbot);
    vec3 tmax = max(ttop, tbot);
    vec2 t = max(vec2(tmin.x, tmin.x), vec2(tmin.y, tmin.z));
    firstHit = max(0.0f, max(t.x, t.y));
    t = min(vec2(tmax.x, tmax.x), vec2(tmax.y, tmax.z));
    lastHit = min(t.x, t.y);
    return firstHit <= lastHit;
}

// The box test of the watertight mode (the library's addition): IntersectBox
// where a slab with a NaN value (the ray lies in one of its planes) does not
// constrain the ray, and the exit distance is widened by 1 + 2 gamma(3)
// rounded up to 1 + 2^-21 (Ize, "Robust BVH Ray Traversal", JCGT 2013).
static bool IntersectBoxRobust(vec3 rayOrigin, vec3 invRayDir, vec3 aabbMin, vec3 aabbMax, float& firstHit) {
    vec3 tbot = invRayDir * (aabbMin - rayOrigin);
    vec3 ttop = invRayDir * (aabbMax - rayOrigin);
    vec3 tmin = min(ttop, tbot);
    vec3 tmax = max(ttop, tbot);
    const float inf = std::numeric_limits<float>::infinity();
    for (int k = 0; k < 3; ++k)
        if (std::isnan(tbot[k]) || std::isnan(ttop[k])) {
            tmin[k] = -inf;
            tmax[k] = inf;
        }
    firstHit = max(0.0f, max(max(tmin.x, tmin.y), max(tmin.x, tmin.z)));
    float lastHit = min(min(tmax.x, tmax.y), min(tmax.x, tmax.z));
    return firstHit <= lastHit * 0x1.000008p+0f;
}

// Ray against a stored axis-aligned ellipsoid {center, radii} (bvhmake's
// "bounding_ellipsoid" chunk, bvhmake/bvhbuilder.cpp:586-588). The reference
// never traverses ellipsoids (its IntersectVirtualEllipsoid,
// intersectiontests.glsl:26-52, is unused), so the node test is the
// library's own: that function's steps (closest approach, scaling into the
// unit sphere, quadratic) with ir = 1 / (radii + 1e-15) (the shader's guard,
// taken once per node) multiplied in, and one reciprocal of ddotd shared by
// both quotients.
static bool IntersectEllipsoid(const Ray& ray, vec3 center, vec3 radiiIn, float& firstHit) {
    const vec3 ir = 1.0f / (radiiIn + 1e-15f);
    vec3 o = ray.Origin - center;
    float t = dot(o, ray.Direction);
    t = max(0.0f, -t);
    o += ray.Direction * t;
    o *= ir;
    float odoto = dot(o, o);
    vec3 d = ray.Direction * ir;
    float odotd = dot(o, d);
    float ddotd = dot(d, d);
    float inv = 1.0f / ddotd;
    float phalf = odotd * inv;
    float q = (odoto - 1.0f) * inv;
    float rad = phalf * phalf - q;
    if (rad < 0.0f) return false;
    rad = sqrt(rad);
    firstHit = max(0.0f, -phalf - rad + t);
    return -phalf + rad + t >= 0.0f;
}

// intersectiontests.glsl:63-79 (OptiX-style branchless Moeller-Trumbore)
static bool IntersectTriangle(const Ray& ray, vec3 p0, vec3 p1, vec3 p2, float& hit,
                              vec3& barycentricCoord, vec3& triangleNormal) {
    const vec3 e0 = p1 - p0;
    const vec3 e1 = p0 - p2;
    triangleNormal = cross(e1, e0);
    const vec3 e2 = (1.0f / dot(triangleNormal, ray.Direction)) * (p0 - ray.Origin);
    const vec3 i = cross(ray.Direction, e2);
    barycentricCoord.y = dot(i, e1);
    barycentricCoord.z = dot(i, e0);
    barycentricCoord.x = 1.0f - (barycentricCoord.z + barycentricCoord.y);
    hit = dot(triangleNormal, e2);
    return (hit > INTERSECT_EPSILON) && all_ge0(barycentricCoord);
}

// Watertight test (an addition of the library, not in the reference):
// Woop, Benthin and Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1),
// 2013, section 3 and its pseudocode, two-sided, with the reference's hit
// rule t > INTERSECT_EPSILON and its barycentric convention (y, z = the
// weights of p1, p2). kz is the axis of the largest |d| component (x, then
// y, then z on ties); an edge function that is exactly 0 in float is
// recomputed in double from the same float operands.
struct WatertightRay {
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
static WatertightRay WatertightSetup(vec3 d) {
    WatertightRay w;
    float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    w.kz = ax >= ay ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
    w.kx = (w.kz + 1) % 3;
    w.ky = (w.kx + 1) % 3;
    if (d[w.kz] < 0.0f) {
        int t = w.kx;
        w.kx = w.ky;
        w.ky = t;
    }
    w.Sx = d[w.kx] / d[w.kz];
    w.Sy = d[w.ky] / d[w.kz];
    w.Sz = 1.0f / d[w.kz];
    return w;
}
static bool IntersectTriangleWatertight(const Ray& ray, const WatertightRay& w, vec3 p0, vec3 p1, vec3 p2,
                                        float& hit, vec3& barycentricCoord) {
    const vec3 A = p0 - ray.Origin;
    const vec3 B = p1 - ray.Origin;
    const vec3 C = p2 - ray.Origin;
    const float Ax = A[w.kx] - w.Sx * A[w.kz];
    const float Ay = A[w.ky] - w.Sy * A[w.kz];
    const float Bx = B[w.kx] - w.Sx * B[w.kz];
    const float By = B[w.ky] - w.Sy * B[w.kz];
    const float Cx = C[w.kx] - w.Sx * C[w.kz];
    const float Cy = C[w.ky] - w.Sy * C[w.kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float Az = w.Sz * A[w.kz];
    const float Bz = w.Sz * B[w.kz];
    const float Cz = w.Sz * C[w.kz];
    const float T = U * Az + V * Bz + W * Cz;
    const float rcpDet = 1.0f / det;
    hit = T * rcpDet;
    barycentricCoord.y = V * rcpDet;
    barycentricCoord.z = W * rcpDet;
    barycentricCoord.x = 1.0f - (barycentricCoord.z + barycentricCoord.y);
    return hit > INTERSECT_EPSILON;
}

static inline vec3 Position(const Scene& s, int32_t idx) {
    const float* p = s.positions + 3 * (int64_t)idx;
    return vec3(p[0], p[1], p[2]);
}

// rotate(x, q) (intersectiontests.glsl:82-89)
static vec3 Rotate(vec3 x, vec4 q) {
    vec3 t = cross(vec3(q.x, q.y, q.z), x);
    return x + 2.0f * vec3(q.w * t.x + q.y * t.z - q.z * t.y, q.w * t.y + q.z * t.x - q.x * t.z,
                           q.w * t.z + q.x * t.y - q.y * t.x);
}

// FetchIntersectBoxNode (intersectiontests.glsl:100-111), FetchIntersectOBoxNode
// (:114-128; 48-B nodes {center, firstChild}, {sidesHalf, escape}, rotationInv:
// the ray goes into the box frame and meets the box [-sidesHalf, sidesHalf])
// and the ellipsoid node of this library.
static inline bool FetchIntersectNode(const Scene& s, const Ray& ray, vec3 invRayDir, int nodeIdx,
                                      float& newHit, uint& childCode, int& escape) {
    const int stride = s.boundsKind == BOUNDS_OBOX ? 3 : 2;
    vec4 a = s.hierarchy[stride * nodeIdx];
    vec4 b = s.hierarchy[stride * nodeIdx + 1];
    childCode = floatBitsToUint(a.w);
    escape = floatBitsToInt(b.w);
    if (s.boundsKind == BOUNDS_ELLIPSOID) return IntersectEllipsoid(ray, a.xyz(), b.xyz(), newHit);
    if (s.boundsKind == BOUNDS_OBOX) {
        vec4 rotationInv = s.hierarchy[3 * nodeIdx + 2];
        vec3 o = Rotate(ray.Origin - a.xyz(), rotationInv);
        vec3 d = Rotate(ray.Direction, rotationInv);
        vec3 inv = vec3(1.0f) / d;
        float exitDist;
        if (s.triangleTest) return IntersectBoxRobust(o, inv, -b.xyz(), b.xyz(), newHit);
        return IntersectBox(o, inv, -b.xyz(), b.xyz(), newHit, exitDist);
    }
    float exitDist;
    if (s.triangleTest) return IntersectBoxRobust(ray.Origin, invRayDir, a.xyz(), b.xyz(), newHit);
    return IntersectBox(ray.Origin, invRayDir, a.xyz(), b.xyz(), newHit, exitDist);
}

// traceray.glsl:18-180. One body serves both variants, like the shader's
// double include with and without ANY_HIT (stdheader.glsl:24-28).
template <bool ANY_HIT>
static bool TraceImpl(const Scene& s, const Ray& ray, float& rayLength, HitRecord* out,
                      TraceCounters* cnt) {
    const int TRIANGLES_PER_LEAF = (int)s.leafSize;
    int currentNodeIndex = 0;
    int currentLeafIndex = 0;
    vec3 invRayDir = 1.0f / ray.Direction;
    const WatertightRay wt = WatertightSetup(ray.Direction);
    bool nextIsLeafNode = false;
    if (s.numNodes == 0) return false;
    // Iteration guard: a well-formed escape tree visits every node at most
    // once and every slot at most once.
    uint64_t guard = (uint64_t)s.numNodes + (uint64_t)s.numSlots + 2;
    do {
        if (guard-- == 0) return false;
        if (!nextIsLeafNode) {
            if (cnt) ++cnt->nodesVisited;
            float newHit;
            uint childCode;
            int escape;
            if (FetchIntersectNode(s, ray, invRayDir, currentNodeIndex, newHit, childCode, escape) &&
                newHit <= rayLength) {
                // Most significant bit tells us if this is a leaf.
                currentNodeIndex = int(childCode & uint(0x7FFFFFFF));
                nextIsLeafNode = (uint)currentNodeIndex != childCode;
                if (nextIsLeafNode) {
                    currentLeafIndex = int(TRIANGLES_PER_LEAF * currentNodeIndex);
                    currentNodeIndex = escape;
                }
            } else {
                currentNodeIndex = escape;
            }
        }
        if (nextIsLeafNode) {
            if (cnt) ++cnt->slotsFetched;
            ivec4 triangle = s.triangles[currentLeafIndex];
            if (triangle.x == triangle.y) {
                nextIsLeafNode = false;
            } else {
                if (cnt) ++cnt->trianglesTested;
                vec3 p0 = Position(s, triangle.x), p1 = Position(s, triangle.y), p2 = Position(s, triangle.z);
                vec3 newTriangleNormal, newBarycentricCoord;
                float newHit;
                const bool isHit = s.triangleTest
                                       ? IntersectTriangleWatertight(ray, wt, p0, p1, p2, newHit, newBarycentricCoord)
                                       : IntersectTriangle(ray, p0, p1, p2, newHit, newBarycentricCoord,
                                                           newTriangleNormal);
                if (isHit && newHit < rayLength) {
                    if (ANY_HIT) return true;
                    rayLength = newHit;
                    out->slot = currentLeafIndex;
                    out->triangle = triangle;
                    out->bary = newBarycentricCoord;
                    out->normal = newTriangleNormal;
                }
                ++currentLeafIndex;
                nextIsLeafNode = (currentLeafIndex % TRIANGLES_PER_LEAF) != 0;
            }
        }
    } while (currentNodeIndex != 0 || nextIsLeafNode);
    return false;
}

bool FetchIntersectBoxNode(const Scene& s, vec3 origin, vec3 invRayDir, int nodeIdx, float& firstHit,
                           float& lastHit, uint& childCode, int& escape, float& nodeSizeSq) {
    vec4 a = s.hierarchy[2 * nodeIdx];
    vec4 b = s.hierarchy[2 * nodeIdx + 1];
    childCode = floatBitsToUint(a.w);
    escape = floatBitsToInt(b.w);
    vec3 ext = b.xyz() - a.xyz();
    nodeSizeSq = dot(ext, ext);
    return IntersectBox(origin, invRayDir, a.xyz(), b.xyz(), firstHit, lastHit);
}

bool IntersectSlot(const Scene& s, const Ray& ray, int slot, float& hit, vec3& bary, ivec4& triangle) {
    triangle = s.triangles[slot];
    vec3 p0 = Position(s, triangle.x), p1 = Position(s, triangle.y), p2 = Position(s, triangle.z);
    vec3 normal;
    return IntersectTriangle(ray, p0, p1, p2, hit, bary, normal);
}

void TraceRay(const Scene& s, const Ray& ray, float& rayLength, HitRecord& hit, TraceCounters* c) {
    hit.slot = -1;
    TraceImpl<false>(s, ray, rayLength, &hit, c);
    hit.t = rayLength;
}

bool TraceRayAnyHit(const Scene& s, const Ray& ray, float rayLength, TraceCounters* c) {
    return TraceImpl<true>(s, ray, rayLength, nullptr, c);
}

}  // namespace oracle

// ---------------------------------------------------------------------------
// C API for ctypes (tests and the CPU baseline).
// ---------------------------------------------------------------------------
using namespace oracle;

// Triangle test of the following query calls (0 reference, 1 watertight);
// the oracle serves one caller at a time.
static uint32_t g_triangleTest = 0;

static Scene MakeScene(const float* hierarchy, uint32_t numNodes, uint32_t boundsKind,
                       const int32_t* slots, uint32_t numSlots, uint32_t leafSize,
                       const float* positions, uint32_t numVertices) {
    Scene s;
    s.hierarchy = reinterpret_cast<const vec4*>(hierarchy);
    s.numNodes = numNodes;
    s.boundsKind = boundsKind;
    s.triangles = reinterpret_cast<const ivec4*>(slots);
    s.numSlots = numSlots;
    s.leafSize = leafSize;
    s.positions = positions;
    s.numVertices = numVertices;
    s.triangleTest = g_triangleTest;
    return s;
}

extern "C" {

void oracle_set_triangle_test(int watertight) { g_triangleTest = watertight ? 1u : 0u; }

// Closest-hit queries over SoA rays. Outputs per ray: slot (-1 = miss), t,
// u = bary.y, v = bary.z, and optional fetch counters (3 uint32 per ray).
int oracle_trace_closest(const float* hierarchy, uint32_t numNodes, uint32_t boundsKind,
                         const int32_t* slots, uint32_t numSlots, uint32_t leafSize,
                         const float* positions, uint32_t numVertices,
                         const float* ox, const float* oy, const float* oz,
                         const float* dx, const float* dy, const float* dz, const float* tmax,
                         uint64_t n, int32_t* outSlot, float* outT, float* outU, float* outV,
                         uint32_t* outCounters, int numThreads) {
    Scene s = MakeScene(hierarchy, numNodes, boundsKind, slots, numSlots, leafSize, positions, numVertices);
    ParallelFor(n, numThreads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            Ray r{vec3(ox[i], oy[i], oz[i]), vec3(dx[i], dy[i], dz[i])};
            float len = tmax[i];
            HitRecord h;
            TraceCounters c;
            TraceRay(s, r, len, h, outCounters ? &c : nullptr);
            outSlot[i] = h.slot;
            outT[i] = h.t;
            outU[i] = h.slot >= 0 ? h.bary.y : 0.0f;
            outV[i] = h.slot >= 0 ? h.bary.z : 0.0f;
            if (outCounters) {
                outCounters[3 * i + 0] = c.nodesVisited;
                outCounters[3 * i + 1] = c.slotsFetched;
                outCounters[3 * i + 2] = c.trianglesTested;
            }
        }
    });
    return 0;
}

int oracle_trace_any(const float* hierarchy, uint32_t numNodes, uint32_t boundsKind,
                     const int32_t* slots, uint32_t numSlots, uint32_t leafSize,
                     const float* positions, uint32_t numVertices,
                     const float* ox, const float* oy, const float* oz,
                     const float* dx, const float* dy, const float* dz, const float* tmax,
                     uint64_t n, uint8_t* outOccluded, uint32_t* outCounters, int numThreads) {
    Scene s = MakeScene(hierarchy, numNodes, boundsKind, slots, numSlots, leafSize, positions, numVertices);
    ParallelFor(n, numThreads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            Ray r{vec3(ox[i], oy[i], oz[i]), vec3(dx[i], dy[i], dz[i])};
            TraceCounters c;
            outOccluded[i] = TraceRayAnyHit(s, r, tmax[i], outCounters ? &c : nullptr) ? 1 : 0;
            if (outCounters) {
                outCounters[3 * i + 0] = c.nodesVisited;
                outCounters[3 * i + 1] = c.slotsFetched;
                outCounters[3 * i + 2] = c.trianglesTested;
            }
        }
    });
    return 0;
}

// Brute force: every valid slot is tested with the same triangle test and
// the same strict '<' acceptance, in slot order. Used to check that the BVH
// walk finds the same closest triangle (ties aside).
int oracle_bruteforce_closest(const int32_t* slots, uint32_t numSlots, const float* positions,
                              const float* ox, const float* oy, const float* oz,
                              const float* dx, const float* dy, const float* dz, const float* tmax,
                              uint64_t n, int32_t* outSlot, float* outT, int numThreads) {
    Scene s = MakeScene(nullptr, 0, 0, slots, numSlots, 8, positions, 0);
    ParallelFor(n, numThreads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            Ray r{vec3(ox[i], oy[i], oz[i]), vec3(dx[i], dy[i], dz[i])};
            const WatertightRay wt = WatertightSetup(r.Direction);
            float len = tmax[i];
            int32_t best = -1;
            for (uint32_t k = 0; k < numSlots; ++k) {
                const ivec4 tri = s.triangles[k];
                if (tri.x == tri.y) continue;
                vec3 bc, nrm;
                float h;
                const vec3 p0 = Position(s, tri.x), p1 = Position(s, tri.y), p2 = Position(s, tri.z);
                const bool isHit = s.triangleTest ? IntersectTriangleWatertight(r, wt, p0, p1, p2, h, bc)
                                                  : IntersectTriangle(r, p0, p1, p2, h, bc, nrm);
                if (isHit && h < len) {
                    len = h;
                    best = (int32_t)k;
                }
            }
            outSlot[i] = best;
            outT[i] = len;
        }
    });
    return 0;
}

}  // extern "C"
