// Shared device helpers: vector math with a fixed IEEE operation order,
// error plumbing, and launch helpers.
//
// The traversal and intersection math uses __fmul_rn/__fadd_rn/__fsub_rn/
// __frcp_rn/__fdiv_rn: these are never contracted into FMAs, so every
// comparison the walk makes is the same IEEE sequence as gpugi's GLSL written
// out in order (dot = (x*x' + y*y') + z*z', cross component-wise, 1.0/x
// correctly rounded). That is what makes hit slots and t bit-exact.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define GPUGI_HD __host__ __device__ __forceinline__
#define GPUGI_D __device__ __forceinline__

namespace gpugi {

// ---------------- exact (non-contracted) float3 arithmetic -----------------
struct X {  // namespace-like holder so the names stay short at call sites
    static GPUGI_D float mul(float a, float b) { return __fmul_rn(a, b); }
    static GPUGI_D float add(float a, float b) { return __fadd_rn(a, b); }
    static GPUGI_D float sub(float a, float b) { return __fsub_rn(a, b); }
    static GPUGI_D float div(float a, float b) { return __fdiv_rn(a, b); }
    static GPUGI_D float rcp(float a) { return __frcp_rn(a); }
    static GPUGI_D float3 sub3(float3 a, float3 b) { return make_float3(sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)); }
    static GPUGI_D float3 add3(float3 a, float3 b) { return make_float3(add(a.x, b.x), add(a.y, b.y), add(a.z, b.z)); }
    static GPUGI_D float3 mul3(float3 a, float3 b) { return make_float3(mul(a.x, b.x), mul(a.y, b.y), mul(a.z, b.z)); }
    static GPUGI_D float3 div3(float3 a, float3 b) { return make_float3(div(a.x, b.x), div(a.y, b.y), div(a.z, b.z)); }
    static GPUGI_D float3 scale(float s, float3 a) { return make_float3(mul(s, a.x), mul(s, a.y), mul(s, a.z)); }
    static GPUGI_D float dot(float3 a, float3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
    static GPUGI_D float3 cross(float3 a, float3 b) {
        return make_float3(sub(mul(a.y, b.z), mul(a.z, b.y)), sub(mul(a.z, b.x), mul(a.x, b.z)),
                           sub(mul(a.x, b.y), mul(a.y, b.x)));
    }
    // normalize(v) = v / sqrt(dot(v, v)) with the correctly rounded sqrt
    static GPUGI_D float3 normalize(float3 v) {
        float l = __fsqrt_rn(dot(v, v));
        return make_float3(div(v.x, l), div(v.y, l), div(v.z, l));
    }
};

// Three-input IEEE minNum/maxNum (PTX min.f32 / max.f32 with three sources,
// sm_100 and later): NaN operands are ignored like fminf/fmaxf ignore them,
// so min3(a, b, c) = fminf(fminf(a, b), c) for every input, in one
// instruction.
GPUGI_D float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
GPUGI_D float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// ---------------- ordinary float3 helpers (shading; contraction allowed) ---
GPUGI_HD float3 f3(float a, float b, float c) { return make_float3(a, b, c); }
GPUGI_HD float3 f3(float s) { return make_float3(s, s, s); }
GPUGI_HD float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
GPUGI_HD float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
GPUGI_HD float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
GPUGI_HD float3 operator/(float3 a, float3 b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
GPUGI_HD float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
GPUGI_HD float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
GPUGI_HD float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
GPUGI_HD float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
GPUGI_HD float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
GPUGI_HD float3& operator*=(float3& a, float3 b) { a = a * b; return a; }
GPUGI_HD float3& operator*=(float3& a, float s) { a = a * s; return a; }
GPUGI_HD float3& operator/=(float3& a, float s) { a = a / s; return a; }
GPUGI_HD float dot(float3 a, float3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
GPUGI_HD float3 cross(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
GPUGI_HD float3 normalize(float3 v) { return v / sqrtf(dot(v, v)); }
GPUGI_HD float saturate(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
GPUGI_HD float3 saturate(float3 v) { return f3(saturate(v.x), saturate(v.y), saturate(v.z)); }
GPUGI_HD float3 fabs3(float3 v) { return f3(fabsf(v.x), fabsf(v.y), fabsf(v.z)); }
GPUGI_HD float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
GPUGI_HD float3 xyz(float4 v) { return make_float3(v.x, v.y, v.z); }

// Device error word bits (mirrors include/gpugi_cuda.h).
constexpr uint32_t DEVERR_TRAVERSAL_CAP = 0x1u;
constexpr uint32_t DEVERR_QUEUE_OVERFLOW = 0x2u;
constexpr uint32_t DEVERR_WAIT_TIMEOUT = 0x4u;
constexpr uint32_t DEVERR_BUILD = 0x8u;  // GPU hierarchy build: a walk to the root exceeded the tree depth bound
constexpr uint32_t DEVERR_HIERARCHY = 0x10u;  // hierarchy importance: a walk to the root exceeded the node count
constexpr uint32_t DEVERR_BOUNDS = 0x20u;  // checked builds: an index outside its array (the access was skipped)

// Bounds-checked builds (compiled with -DGPUGI_CHECKED=1 into
// libgpugi_cuda_checked.so): node, leaf-slot, vertex and material indexes
// are checked before every fetch; a bad index sets DEVERR_BOUNDS and the
// fetch is skipped (the walk or the shading of that item ends). The
// wavefront queues and light caches check their capacity in every build.
#ifdef GPUGI_CHECKED
constexpr bool kChecked = true;
#else
constexpr bool kChecked = false;
#endif

GPUGI_D void raise_error(uint32_t* word, uint32_t bits) {
    if (word) atomicOr(word, bits);
}

// Leaf encoding of the device node copy: bit 31 = leaf, bits 25..30 = number
// of leading valid slots in the block (0..32), bits 0..24 = leaf block.
constexpr uint32_t LEAF_FLAG = 0x80000000u;
constexpr uint32_t LEAF_BLOCK_MASK = 0x01FFFFFFu;
constexpr uint32_t LEAF_COUNT_SHIFT = 25;
constexpr uint32_t LEAF_COUNT_MASK = 0x3Fu;

}  // namespace gpugi
