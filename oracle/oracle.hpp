// ORACLE — test infrastructure only (see glsl.hpp for the parity status).
//
// Scene buffers exactly as gpugi binds them to its shaders
// (gpugi/renderer/renderersystem.cpp:138-147, gpugi/shader/scenedata.glsl:21-51):
//   HierachyBuffer        2 texels (vec4) per node: {min.xyz | firstChild bits},
//                         {max.xyz | escape bits}   (gpugi/scene/scene.hpp:30-38)
//                         ellipsoid bounds use {center.xyz | firstChild},
//                         {radii.xyz | escape} with the same stride; oriented
//                         boxes 3 texels {center | firstChild}, {sidesHalf |
//                         escape}, rotationInv (scene.hpp:40-49).
//   TriangleBuffer        one ivec4 {v0, v1, v2, material} per leaf slot,
//                         leafSize slots per leaf block  (scene.hpp:64-68)
//   VertexPositionBuffer  tightly packed RGB32F, 12 bytes per vertex (scene.cpp:87)
//   VertexInfoBuffer      vec4 {atan2(n.y,n.x), n.z, u, v} per vertex (scene.cpp:79-84)
#pragma once
#include <cstdint>
#include "glsl.hpp"

namespace oracle {

enum BoundsKind : uint32_t { BOUNDS_AABB = 0, BOUNDS_ELLIPSOID = 1, BOUNDS_OBOX = 2 };

struct Scene {
    const glsl::vec4* hierarchy = nullptr;
    uint32_t numNodes = 0;
    const glsl::ivec4* triangles = nullptr;
    uint32_t numSlots = 0;
    uint32_t leafSize = 8;
    const float* positions = nullptr;
    uint32_t numVertices = 0;
    const glsl::vec4* vertexInfo = nullptr;
    uint32_t boundsKind = BOUNDS_AABB;
    uint32_t triangleTest = 0;  // 0: IntersectTriangle as the reference writes it, 1: watertight
};

struct Ray {
    glsl::vec3 Origin;
    glsl::vec3 Direction;
};

// Per-ray fetch counters, the analogue of TRACERAY_DEBUG_VARS
// (gpugi/shader/traceray.glsl:59-61,131-133).
struct TraceCounters {
    uint32_t nodesVisited = 0;     // node fetch + bounds test
    uint32_t slotsFetched = 0;     // leaf slot (16-byte triangle index) fetches
    uint32_t trianglesTested = 0;  // valid triangles: 3 vertex fetches + test
};

struct HitRecord {
    int32_t slot = -1;             // leaf slot index of the closest hit, -1 = miss
    float t = 0.0f;                // final rayLength
    glsl::vec3 bary;               // (1-u-v, u, v)
    glsl::ivec4 triangle{0, 0, 0, 0};
    glsl::vec3 normal;             // unnormalised cross(e1, e0) (TRINORMAL_OUTPUT)
};

// Closest hit: restates TraceRay (traceray.glsl:25-180 without ANY_HIT).
// rayLength is both the initial limit and, on return, the hit distance.
void TraceRay(const Scene& s, const Ray& ray, float& rayLength, HitRecord& hit,
              TraceCounters* counters);
// Any hit: restates TraceRayAnyHit (traceray.glsl:18-23 with ANY_HIT).
bool TraceRayAnyHit(const Scene& s, const Ray& ray, float rayLength, TraceCounters* counters);

// FetchIntersectBoxNode (intersectiontests.glsl:100-111) of an AABB node:
// entry and exit distances, child code, escape and the squared diagonal.
bool FetchIntersectBoxNode(const Scene& s, glsl::vec3 origin, glsl::vec3 invRayDir, int nodeIdx, float& firstHit,
                           float& lastHit, uint32_t& childCode, int& escape, float& nodeSizeSq);
// IntersectTriangle (intersectiontests.glsl:63-79) with the triangle of a leaf slot.
bool IntersectSlot(const Scene& s, const Ray& ray, int slot, float& hit, glsl::vec3& bary, glsl::ivec4& triangle);

// Thread pool helper: runs fn(begin, end) over [0, n) split into contiguous ranges.
template <typename F>
void ParallelFor(uint64_t n, int numThreads, F fn);

}  // namespace oracle

#include <thread>
#include <vector>
namespace oracle {
template <typename F>
void ParallelFor(uint64_t n, int numThreads, F fn) {
    if (numThreads <= 0) numThreads = (int)std::thread::hardware_concurrency();
    if (numThreads < 1) numThreads = 1;
    if ((uint64_t)numThreads > n) numThreads = (int)(n ? n : 1);
    if (numThreads == 1) { fn(0, n); return; }
    std::vector<std::thread> pool;
    uint64_t chunk = (n + numThreads - 1) / numThreads;
    for (int t = 0; t < numThreads; ++t) {
        uint64_t b = (uint64_t)t * chunk, e = b + chunk < n ? b + chunk : n;
        if (b >= e) break;
        pool.emplace_back([=]() { fn(b, e); });
    }
    for (auto& th : pool) th.join();
}
}  // namespace oracle
