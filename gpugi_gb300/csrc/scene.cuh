// Device-resident scene: the data layout in HBM.
//
//   nodes      2 x float4 per node (32 B, 32-B aligned): {min.xyz | child},
//              {max.xyz | escape}; ellipsoid bounds store {center | child},
//              {1 / (radii + 1e-15) | escape}. Same stride and words as gpugi's
//              HierachyBuffer (scene.hpp:30-38) except that a leaf child
//              also carries the count of leading valid slots (common.cuh).
//   tris       3 x float4 per leaf slot (48 B): p0, e0 = p1-p0, e1 = p0-p2,
//              n = cross(e1, e0), precomputed once with the exact operation
//              order of IntersectTriangle (intersectiontests.glsl:66-68), so a
//              test needs one 48-B read instead of an index fetch plus three
//              dependent vertex fetches.
//   slots      int4 per leaf slot {v0, v1, v2, material} (TriangleBuffer)
//   positions  3 floats per vertex (VertexPositionBuffer)
//   vinfo      float4 per vertex {normal angles, uv} (VertexInfoBuffer)
//   materials  6 x float4 per material (gpugi_material)
#pragma once
#include "common.cuh"

namespace gpugi {

struct DevScene {
    const float4* nodes = nullptr;
    const float4* tris = nullptr;
    // watertight test records {p0.xyz p1.x | p1.yz p2.xy | p2.z 0 0 0} per leaf
    // slot, made on demand (gpugi_scene_set_triangle_test); null otherwise
    const float4* wtris = nullptr;
    const int4* slots = nullptr;
    const float* positions = nullptr;
    const float4* vinfo = nullptr;
    const float4* materials = nullptr;
    uint32_t numNodes = 0;
    uint32_t numSlots = 0;
    uint32_t leafSize = 8;
    uint32_t boundsKind = 0;
    uint32_t numVertices = 0;
    uint32_t numMaterials = 0;
    // Nodes are stored with the top tree levels first (breadth-first), the
    // rest in preorder; persistent walkers stage nodes [0, topNodes) in
    // shared memory. Node 0 is the root; an escape of 0 still ends the walk.
    uint32_t topNodes = 0;
    // Triangle test of the ray queries: 0 = the reference's (IntersectTriangle),
    // 1 = watertight (wtris holds its records).
    uint32_t triangleTest = 0;
};

// Material view (constant-valued MaterialData, materials.glsl:9-30).
struct MaterialData {
    float4 Reflectiveness;
    float3 Opacity;
    float3 Diffuse;
    float3 Emissivity;
    float3 Fresnel0;
    float RefractionIndexAvg;
    float3 Fresnel1;
};

GPUGI_D MaterialData load_material(const DevScene& s, int id) {
    const float4* m = s.materials + 6 * id;
    float4 a = __ldg(m), b = __ldg(m + 1), c = __ldg(m + 2), d = __ldg(m + 3), e = __ldg(m + 4),
           f = __ldg(m + 5);
    MaterialData md;
    md.Diffuse = xyz(a);
    md.RefractionIndexAvg = a.w;
    md.Opacity = xyz(b);
    md.Reflectiveness = c;
    md.Emissivity = xyz(d);
    md.Fresnel0 = xyz(e);
    md.Fresnel1 = xyz(f);
    return md;
}

}  // namespace gpugi
