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

static inline vec3 Position(const Scene& s, int32_t idx) {
    const float* p = s.positions + 3 * (int64_t)idx;
    return vec3(p[0], p[1], p[2]);
}

// FetchIntersectBoxNode (intersectiontests.glsl:100-111) and its ellipsoid twin.
static inline bool FetchIntersectNode(const Scene& s, const Ray& ray, vec3 invRayDir, int nodeIdx,
                                      float& newHit, uint& childCode, int& escape) {
    vec4 a = s.hierarchy[2 * nodeIdx];
    vec4 b = s.hierarchy[2 * nodeIdx + 1];
    childCode = floatBitsToUint(a.w);
    escape = floatBitsToInt(b.w);
    if (s.boundsKind == BOUNDS_ELLIPSOID) return IntersectEllipsoid(ray, a.xyz(), b.xyz(), newHit);
    float exitDist;
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
                if (IntersectTriangle(ray, p0, p1, p2, newHit, newBarycentricCoord, newTriangleNormal) &&
                    newHit < rayLength) {
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
    return s;
}

extern "C" {

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
            float len = tmax[i];
            int32_t best = -1;
            for (uint32_t k = 0; k < numSlots; ++k) {
                const ivec4 tri = s.triangles[k];
                if (tri.x == tri.y) continue;
                vec3 bc, nrm;
                float h;
                if (IntersectTriangle(r, Position(s, tri.x), Position(s, tri.y), Position(s, tri.z), h, bc, nrm) &&
                    h < len) {
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
