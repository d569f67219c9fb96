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
    // Material textures (gpugi_scene_set_textures), null without: RGBA32F
    // texels of all textures, per texture {first texel, width, height, 0},
    // per material the texture of {reflectiveness, opacity, diffuse,
    // emissivity} or -1 for the record's constant.
    const float4* texels = nullptr;
    const uint4* texInfo = nullptr;
    const int4* matTex = nullptr;
    // The owning context's device error word: the checked library reports
    // out-of-range indexes met while shading this scene there.
    uint32_t* err = nullptr;
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

// textureLod(sampler2D(handle), texcoord, 0.0) of a material texture: the
// reference's sampler (scene.cpp:15-20: magnification LINEAR, wrap REPEAT;
// level 0 of a texture without mipmaps is magnified) filters bilinearly
// (OpenGL 4.5, 8.14.2: u = s w - 1/2, i0 = floor(u), weights from the
// fractional parts, REPEAT wraps i0 and i0 + 1). The weights are computed in
// float here (GL hardware quantises them to a few bits), with a fixed
// operation order that the oracle restates.
GPUGI_D float4 sample_texture(const DevScene& s, int tex, float2 tc) {
    const uint4 info = __ldg(s.texInfo + tex);
    const float w = (float)info.y, h = (float)info.z;
    float u = __fsub_rn(__fmul_rn(tc.x, w), 0.5f), v = __fsub_rn(__fmul_rn(tc.y, h), 0.5f);
    if (!isfinite(u)) u = 0.0f;
    if (!isfinite(v)) v = 0.0f;
    const float fu = floorf(u), fv = floorf(v);
    const float a = __fsub_rn(u, fu), b = __fsub_rn(v, fv);
    float i0 = fmodf(fu, w), j0 = fmodf(fv, h);  // exact for every float
    if (i0 < 0.0f) i0 = __fadd_rn(i0, w);
    if (j0 < 0.0f) j0 = __fadd_rn(j0, h);
    const uint32_t x0 = (uint32_t)i0 < info.y ? (uint32_t)i0 : 0u, y0 = (uint32_t)j0 < info.z ? (uint32_t)j0 : 0u;
    const uint32_t x1 = x0 + 1 == info.y ? 0u : x0 + 1, y1 = y0 + 1 == info.z ? 0u : y0 + 1;
    const float4* t = s.texels + info.x;
    const float4 t00 = __ldg(t + (size_t)y0 * info.y + x0), t10 = __ldg(t + (size_t)y0 * info.y + x1);
    const float4 t01 = __ldg(t + (size_t)y1 * info.y + x0), t11 = __ldg(t + (size_t)y1 * info.y + x1);
    const float na = __fsub_rn(1.0f, a), nb = __fsub_rn(1.0f, b);
    const float w00 = __fmul_rn(na, nb), w10 = __fmul_rn(a, nb), w01 = __fmul_rn(na, b), w11 = __fmul_rn(a, b);
    auto mix4 = [&](float c00, float c10, float c01, float c11) {
        return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w00, c00), __fmul_rn(w10, c10)), __fmul_rn(w01, c01)),
                         __fmul_rn(w11, c11));
    };
    return make_float4(mix4(t00.x, t10.x, t01.x, t11.x), mix4(t00.y, t10.y, t01.y, t11.y),
                       mix4(t00.z, t10.z, t01.z, t11.z), mix4(t00.w, t10.w, t01.w, t11.w));
}

// SampleMaterialData (materials.glsl:19-30): the four maps at the hit's
// texture coordinate (the record's constants where a material has no texture).
GPUGI_D MaterialData load_material(const DevScene& s, int id, float2 tc = make_float2(0.0f, 0.0f)) {
    if (kChecked && (id < 0 || (uint32_t)id >= s.numMaterials)) {
        raise_error(s.err, DEVERR_BOUNDS);
        id = 0;
    }
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
    if (s.matTex) {
        const int4 tx = __ldg(s.matTex + id);
        if (tx.x >= 0) md.Reflectiveness = sample_texture(s, tx.x, tc);
        if (tx.y >= 0) md.Opacity = xyz(sample_texture(s, tx.y, tc));
        if (tx.z >= 0) md.Diffuse = xyz(sample_texture(s, tx.z, tc));
        if (tx.w >= 0) md.Emissivity = xyz(sample_texture(s, tx.w, tc));
    }
    return md;
}

}  // namespace gpugi
