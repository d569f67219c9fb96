// ORACLE — test infrastructure only. Not part of the product.
//
// GLSL built-ins and types in C++, so that gpugi's own shader text
// (gpugi/shader/*.glsl, *.comp), after the mechanical rewrite done by
// oracle/ref_build.py (qualifiers to references, float literals to float,
// swizzle reads to calls, layout/uniform wrappers stripped), compiles as
// C++ and runs on the CPU. The result is the reference's own code for the
// hot path, used to pin the oracle's restatement (oracle/*.cpp): same inputs,
// bit-identical outputs.
//
// This header defines only what GLSL itself defines (types, constructors,
// operators, built-in functions, texelFetch/texture/image access over plain
// arrays); every function of the reference comes from its own text. The
// arithmetic conventions are the ones the oracle fixes for what GLSL leaves
// open (compile with -ffp-contract=off):
//   dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z; cross component-wise;
//   min/max are IEEE minNum/maxNum (std::fmin/fmax); clamp = min(max(x, lo), hi);
//   1.0/x, sqrt correctly rounded; sin/cos/pow/atan/log2/exp2 from the C
//   library in single precision; round() and packSnorm ties to even.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace glslref {

typedef uint32_t uint;

// ------------------------------------------------------------------ vectors
#define GR_SW2(T, a, b) \
    T a##b() const { return T(a, b); }
#define GR_SW3(T, a, b, c) \
    T a##b##c() const { return T(a, b, c); }

struct vec2;
struct vec3;
struct vec4;
struct ivec2;
struct uvec2;
struct uvec3;

struct vec2 {
    union { float x, r; };
    union { float y, g; };
    vec2() : x(0), y(0) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    inline explicit vec2(const ivec2& v);
    float& operator[](int i) { return i == 0 ? x : y; }
    float operator[](int i) const { return i == 0 ? x : y; }
    GR_SW2(vec2, x, x) GR_SW2(vec2, x, y) GR_SW2(vec2, y, x) GR_SW2(vec2, y, y)
};
// `v.xy` / `v.zw` of a vec3 or vec4 as an lvalue (`mat.Opacity.xy += c`,
// pullmaterials.comp): reads as a vec2, assigns component by component.
struct VecSwizzle2 {
    float *a, *b;
    inline operator vec2() const { return vec2(*a, *b); }
    inline VecSwizzle2& operator=(const vec2& v) {
        *a = v.x, *b = v.y;
        return *this;
    }
    inline VecSwizzle2& operator+=(const vec2& v) {
        *a += v.x, *b += v.y;
        return *this;
    }
    inline VecSwizzle2& operator-=(const vec2& v) {
        *a -= v.x, *b -= v.y;
        return *this;
    }
};
struct vec3 {
    union { float x, r; };
    union { float y, g; };
    union { float z, b; };
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b_, float c) : x(a), y(b_), z(c) {}
    vec3(const vec2& v, float c) : x(v.x), y(v.y), z(c) {}
    vec3(float a, const vec2& v) : x(a), y(v.x), z(v.y) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    GR_SW2(vec2, x, x) GR_SW2(vec2, x, y) GR_SW2(vec2, x, z) GR_SW2(vec2, y, x) GR_SW2(vec2, y, y)
    GR_SW2(vec2, y, z) GR_SW2(vec2, z, x) GR_SW2(vec2, z, y) GR_SW2(vec2, z, z)
    GR_SW3(vec3, x, y, z) GR_SW3(vec3, z, y, x)
    VecSwizzle2 xy() { return VecSwizzle2{&x, &y}; }
};
// `v.xyz` of a vec4 as an lvalue (`color.xyz += c`, importondistribution.comp,
// screenreproject.glsl): reads as a vec3, assigns component by component.
struct VecSwizzle3 {
    float *a, *b, *c;
    inline operator vec3() const;
    inline VecSwizzle3& operator=(const vec3& v);
    inline VecSwizzle3& operator+=(const vec3& v);
    inline VecSwizzle3& operator-=(const vec3& v);
};
struct vec4 {
    union { float x, r; };
    union { float y, g; };
    union { float z, b; };
    union { float w, a; };
    vec4() : x(0), y(0), z(0), w(0) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a_, float b_, float c, float d) : x(a_), y(b_), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(const vec2& u, const vec2& v) : x(u.x), y(u.y), z(v.x), w(v.y) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    GR_SW2(vec2, x, y) GR_SW2(vec2, z, w) GR_SW2(vec2, x, z) GR_SW2(vec2, y, z) GR_SW2(vec2, y, w)
    GR_SW2(vec2, x, w)
    GR_SW3(vec3, x, y, z) GR_SW3(vec3, y, z, w)
    VecSwizzle3 xyz() { return VecSwizzle3{&x, &y, &z}; }
    VecSwizzle2 xy() { return VecSwizzle2{&x, &y}; }
    VecSwizzle2 zw() { return VecSwizzle2{&z, &w}; }
    vec3 rgb() const { return vec3(x, y, z); }
};
inline VecSwizzle3::operator vec3() const { return vec3(*a, *b, *c); }
inline VecSwizzle3& VecSwizzle3::operator=(const vec3& v) {
    *a = v.x, *b = v.y, *c = v.z;
    return *this;
}
inline VecSwizzle3& VecSwizzle3::operator+=(const vec3& v) {
    *a += v.x, *b += v.y, *c += v.z;
    return *this;
}
inline VecSwizzle3& VecSwizzle3::operator-=(const vec3& v) {
    *a -= v.x, *b -= v.y, *c -= v.z;
    return *this;
}
struct ivec2 {
    int32_t x, y;
    ivec2() : x(0), y(0) {}
    explicit ivec2(int32_t s) : x(s), y(s) {}
    ivec2(int32_t a, int32_t b) : x(a), y(b) {}
    inline explicit ivec2(const vec2& v);
    inline explicit ivec2(const uvec2& v);
};
struct uvec2 {
    uint x, y;
    uvec2() : x(0), y(0) {}
    uvec2(uint a, uint b) : x(a), y(b) {}
};
struct uvec3 {
    uint x, y, z;
    uvec3() : x(0), y(0), z(0) {}
    uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
    uvec2 xy() const { return uvec2(x, y); }
};
struct ivec3 {
    int32_t x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    ivec3(int32_t a, int32_t b, int32_t c) : x(a), y(b), z(c) {}
    ivec3(const ivec2& a, int32_t c) : x(a.x), y(a.y), z(c) {}
    explicit ivec3(const vec3& v) : x((int32_t)v.x), y((int32_t)v.y), z((int32_t)v.z) {}
};
inline ivec3 operator+(ivec3 a, ivec3 b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
// A three-component swizzle of an ivec4 that can be read or assigned
// (`HashMapData[i].yzw = v`, photonmapper/photondistribution.comp).
struct ivec4;
struct IvecSwizzle3 {
    int32_t *a, *b, *c;
    operator ivec3() const { return ivec3(*a, *b, *c); }
    IvecSwizzle3& operator=(const ivec3& v) {
        *a = v.x;
        *b = v.y;
        *c = v.z;
        return *this;
    }
};
struct ivec4 {
    int32_t x, y, z, w;
    ivec4() : x(0), y(0), z(0), w(0) {}
    ivec4(int32_t a, int32_t b, int32_t c, int32_t d) : x(a), y(b), z(c), w(d) {}
    ivec4(const ivec3& v, int32_t d) : x(v.x), y(v.y), z(v.z), w(d) {}
    IvecSwizzle3 xyz() { return IvecSwizzle3{&x, &y, &z}; }
    IvecSwizzle3 yzw() { return IvecSwizzle3{&y, &z, &w}; }
    ivec3 xyz() const { return ivec3(x, y, z); }
    ivec3 yzw() const { return ivec3(y, z, w); }
    ivec2 yz() const { return ivec2(y, z); }
};
struct bvec3 {
    bool x, y, z;
};
inline vec2::vec2(const ivec2& v) : x((float)v.x), y((float)v.y) {}
inline ivec2::ivec2(const vec2& v) : x((int32_t)v.x), y((int32_t)v.y) {}
inline ivec2::ivec2(const uvec2& v) : x((int32_t)v.x), y((int32_t)v.y) {}
struct mat4 {
    vec4 c[4];
};
// mat3x3: three columns; m[i][j] is column i, row j.
struct mat3x3 {
    vec3 c[3];
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};

// ---------------------------------------------------------------- operators
#define GR_BIN2(OP)                                                                          \
    inline vec2 operator OP(vec2 a, vec2 b) { return vec2(a.x OP b.x, a.y OP b.y); }          \
    inline vec2 operator OP(vec2 a, float s) { return vec2(a.x OP s, a.y OP s); }             \
    inline vec2 operator OP(float s, vec2 a) { return vec2(s OP a.x, s OP a.y); }             \
    inline vec2 operator OP(vec2 a, ivec2 b) { return a OP vec2(b); }                          \
    inline vec2 operator OP(ivec2 a, vec2 b) { return vec2(a) OP b; }
#define GR_BIN3(OP)                                                                                  \
    inline vec3 operator OP(vec3 a, vec3 b) { return vec3(a.x OP b.x, a.y OP b.y, a.z OP b.z); }      \
    inline vec3 operator OP(vec3 a, float s) { return vec3(a.x OP s, a.y OP s, a.z OP s); }           \
    inline vec3 operator OP(float s, vec3 a) { return vec3(s OP a.x, s OP a.y, s OP a.z); }
#define GR_BIN4(OP)                                                                                                \
    inline vec4 operator OP(vec4 a, vec4 b) { return vec4(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w); }        \
    inline vec4 operator OP(vec4 a, float s) { return vec4(a.x OP s, a.y OP s, a.z OP s, a.w OP s); }               \
    inline vec4 operator OP(float s, vec4 a) { return vec4(s OP a.x, s OP a.y, s OP a.z, s OP a.w); }
GR_BIN2(+) GR_BIN2(-) GR_BIN2(*) GR_BIN2(/)
GR_BIN3(+) GR_BIN3(-) GR_BIN3(*) GR_BIN3(/)
GR_BIN4(+) GR_BIN4(-) GR_BIN4(*) GR_BIN4(/)
#define GR_ASSIGN(T, OP)                                   \
    inline T& operator OP##=(T& a, T b) { return a = a OP b; } \
    inline T& operator OP##=(T& a, float s) { return a = a OP s; }
GR_ASSIGN(vec2, +) GR_ASSIGN(vec2, -) GR_ASSIGN(vec2, *) GR_ASSIGN(vec2, /)
GR_ASSIGN(vec3, +) GR_ASSIGN(vec3, -) GR_ASSIGN(vec3, *) GR_ASSIGN(vec3, /)
GR_ASSIGN(vec4, +) GR_ASSIGN(vec4, -) GR_ASSIGN(vec4, *) GR_ASSIGN(vec4, /)
inline vec2 operator-(vec2 a) { return vec2(-a.x, -a.y); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec4 operator-(vec4 a) { return vec4(-a.x, -a.y, -a.z, -a.w); }
inline bool operator==(vec3 a, vec3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(vec3 a, vec3 b) { return !(a == b); }
inline ivec2 operator+(ivec2 a, ivec2 b) { return ivec2(a.x + b.x, a.y + b.y); }
inline ivec2 operator-(ivec2 a, ivec2 b) { return ivec2(a.x - b.x, a.y - b.y); }
inline ivec2 operator*(ivec2 a, ivec2 b) { return ivec2(a.x * b.x, a.y * b.y); }

// ---------------------------------------------------------------- built-ins
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline vec2 min(vec2 a, vec2 b) { return vec2(min(a.x, b.x), min(a.y, b.y)); }
inline vec2 max(vec2 a, vec2 b) { return vec2(max(a.x, b.x), max(a.y, b.y)); }
inline vec3 min(vec3 a, vec3 b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(vec3 a, vec3 b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 min(vec3 a, float b) { return min(a, vec3(b)); }
inline vec3 max(vec3 a, float b) { return max(a, vec3(b)); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec2 clamp(vec2 x, vec2 lo, vec2 hi) { return min(max(x, lo), hi); }
inline vec3 clamp(vec3 x, vec3 lo, vec3 hi) { return min(max(x, lo), hi); }
inline vec4 clamp(vec4 x, vec4 lo, vec4 hi) {
    return vec4(clamp(x.x, lo.x, hi.x), clamp(x.y, lo.y, hi.y), clamp(x.z, lo.z, hi.z), clamp(x.w, lo.w, hi.w));
}
inline vec2 clamp(vec2 x, float lo, float hi) { return clamp(x, vec2(lo), vec2(hi)); }
inline vec3 clamp(vec3 x, float lo, float hi) { return clamp(x, vec3(lo), vec3(hi)); }
inline float abs(float x) { return std::fabs(x); }
inline vec3 abs(vec3 v) { return vec3(abs(v.x), abs(v.y), abs(v.z)); }
inline vec2 abs(vec2 v) { return vec2(abs(v.x), abs(v.y)); }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline vec3 sign(vec3 v) { return vec3(sign(v.x), sign(v.y), sign(v.z)); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline float sin(float x) { return std::sin(x); }
inline float cos(float x) { return std::cos(x); }
inline float tan(float x) { return std::tan(x); }
inline float acos(float x) { return std::acos(x); }
inline float atan(float y, float x) { return std::atan2(y, x); }
inline float atan(float x) { return std::atan(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float exp(float x) { return std::exp(x); }
inline float exp2(float x) { return std::exp2(x); }
inline float log(float x) { return std::log(x); }
inline float log2(float x) { return std::log2(x); }
inline float floor(float x) { return std::floor(x); }
inline float ceil(float x) { return std::ceil(x); }
inline float fract(float x) { return x - std::floor(x); }
inline float round(float x) { return std::nearbyint(x); }  // ties to even (default rounding mode)
inline vec2 floor(vec2 v) { return vec2(floor(v.x), floor(v.y)); }
inline vec3 floor(vec3 v) { return vec3(floor(v.x), floor(v.y), floor(v.z)); }
inline vec2 round(vec2 v) { return vec2(round(v.x), round(v.y)); }
inline float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline vec3 mix(vec3 a, vec3 b, float t) { return a * (1.0f - t) + b * t; }
inline float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot(vec4 a, vec4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
inline vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(vec3 v) { return sqrt(dot(v, v)); }
// the columns combined left to right: (c0 v.x + c1 v.y) + c2 v.z
inline vec3 operator*(const mat3x3& m, vec3 v) { return (m.c[0] * v.x + m.c[1] * v.y) + m.c[2] * v.z; }
inline float length(vec2 v) { return sqrt(dot(v, v)); }
inline vec3 normalize(vec3 v) { return v / sqrt(dot(v, v)); }
inline vec3 reflect(vec3 i, vec3 n) { return i - 2.0f * dot(n, i) * n; }
inline bvec3 lessThan(vec3 a, vec3 b) { return bvec3{a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bvec3 greaterThan(vec3 a, vec3 b) { return bvec3{a.x > b.x, a.y > b.y, a.z > b.z}; }
inline bvec3 lessThanEqual(vec3 a, vec3 b) { return bvec3{a.x <= b.x, a.y <= b.y, a.z <= b.z}; }
inline bvec3 greaterThanEqual(vec3 a, vec3 b) { return bvec3{a.x >= b.x, a.y >= b.y, a.z >= b.z}; }
inline bvec3 equal(vec3 a, vec3 b) { return bvec3{a.x == b.x, a.y == b.y, a.z == b.z}; }
inline bvec3 notEqual(vec3 a, vec3 b) { return bvec3{a.x != b.x, a.y != b.y, a.z != b.z}; }
inline bool all(bvec3 v) { return v.x && v.y && v.z; }
inline bool any(bvec3 v) { return v.x || v.y || v.z; }
inline bool isnan(float x) { return std::isnan(x); }
inline bool isinf(float x) { return std::isinf(x); }

inline uint floatBitsToUint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
inline int floatBitsToInt(float f) { int u; std::memcpy(&u, &f, 4); return u; }
inline float uintBitsToFloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }
inline float intBitsToFloat(int u) { float f; std::memcpy(&f, &u, 4); return f; }
inline ivec3 floatBitsToInt(vec3 v) { return ivec3(floatBitsToInt(v.x), floatBitsToInt(v.y), floatBitsToInt(v.z)); }
inline vec3 intBitsToFloat(ivec3 v) { return vec3(intBitsToFloat(v.x), intBitsToFloat(v.y), intBitsToFloat(v.z)); }
inline ivec2 floatBitsToInt(vec2 v) { return ivec2(floatBitsToInt(v.x), floatBitsToInt(v.y)); }
inline vec2 intBitsToFloat(ivec2 v) { return vec2(intBitsToFloat(v.x), intBitsToFloat(v.y)); }
inline vec3 ceil(vec3 v) { return vec3(ceil(v.x), ceil(v.y), ceil(v.z)); }
inline vec3 round(vec3 v) { return vec3(round(v.x), round(v.y), round(v.z)); }
// packSnorm2x16: round(clamp(c, -1, +1) * 32767.0), x in the low 16 bits
inline uint packSnorm2x16(vec2 v) {
    auto c = [](float f) { return (uint)(uint16_t)(int16_t)round(clamp(f, -1.0f, 1.0f) * 32767.0f); };
    return c(v.x) | (c(v.y) << 16);
}
inline vec2 unpackSnorm2x16(uint p) {
    auto u = [](uint b) { return clamp((float)(int16_t)(uint16_t)b / 32767.0f, -1.0f, 1.0f); };
    return vec2(u(p & 0xFFFFu), u(p >> 16));
}

// -------------------------------------------------- buffers, images, samplers
// texelFetch over a texture buffer: a plain array of texels. A float buffer
// holds `channels` floats per texel (4 for RGBA32F, 3 for the RGB32F vertex
// positions, gpugi/scene/scene.cpp:87) and reads back as vec4 (missing
// channels 0, alpha 1).
struct samplerBuffer {
    const float* data = nullptr;
    int channels = 4;
};
struct isamplerBuffer {
    const ivec4* texels = nullptr;
};
inline vec4 texelFetch(const samplerBuffer& b, int i) {
    const float* p = b.data + (int64_t)b.channels * i;
    return vec4(p[0], b.channels > 1 ? p[1] : 0.0f, b.channels > 2 ? p[2] : 0.0f, b.channels > 3 ? p[3] : 1.0f);
}
inline ivec4 texelFetch(const isamplerBuffer& b, int i) { return b.texels[i]; }

// Bindless textures of constant-valued materials: a handle indexes a table
// of colours; every lookup returns that colour.
struct sampler2D {
    uint handle;
    explicit sampler2D(uvec2 h) : handle(h.x) {}
};
extern const vec4* g_textureColours;
inline vec4 textureLod(sampler2D s, vec2, float) { return g_textureColours[s.handle]; }
inline vec4 texture(sampler2D s, vec2) { return g_textureColours[s.handle]; }

// Environment map of the passes: a constant radiance (black in the reference's default scenes).
struct samplerCubeArray {
    vec3 colour;
};
inline vec4 textureLod(const samplerCubeArray& s, vec4, float) { return vec4(s.colour, 1.0f); }

// image2D: RGBA32F texels, row-major, width x height. As in GL, a store
// outside the image is discarded and a load there returns zero.
struct image2D {
    vec4* texels = nullptr;
    int width = 0;
    int height = 0;
};
inline bool image_inside(const image2D& im, ivec2 p, int widthScale = 1) {
    return p.x >= 0 && p.y >= 0 && p.x < widthScale * im.width && p.y < im.height;
}
inline vec4 imageLoad(const image2D& im, ivec2 p) {
    return image_inside(im, p) ? im.texels[(int64_t)p.y * im.width + p.x] : vec4(0.0f);
}
inline void imageStore(image2D& im, ivec2 p, vec4 v) {
    if (image_inside(im, p)) im.texels[(int64_t)p.y * im.width + p.x] = v;
}
// The light tracer binds the same RGBA32F image as r32f, four floats per
// texel side by side (screenreproject.glsl:7, 44-47): the float at column x
// of row y. Atomic (a compare-and-swap loop on the bits); returns the old value.
inline float imageAtomicAdd(image2D& im, ivec2 p, float v) {
    if (!image_inside(im, p, 4)) return 0.0f;
    uint32_t* u = reinterpret_cast<uint32_t*>(reinterpret_cast<float*>(im.texels) + (int64_t)p.y * 4 * im.width + p.x);
    uint32_t old = __atomic_load_n(u, __ATOMIC_RELAXED), next;
    float f;
    do {
        std::memcpy(&f, &old, 4);
        const float n = f + v;
        std::memcpy(&next, &n, 4);
    } while (!__atomic_compare_exchange_n(u, &old, next, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED));
    return f;
}
// atomicAdd on a storage-buffer float (counthits.glsl's importance sums;
// GL_NV_shader_atomic_float). The passes that use it run their invocations
// one at a time, in order, so the sum is a plain add.
inline float atomicAdd(float& x, float v) {
    const float o = x;
    x = o + v;
    return o;
}
// packHalf2x16 / unpackHalf2x16 through the compiler's IEEE binary16 type
// (round to nearest even; GLSL leaves the rounding open, NVIDIA's converter
// rounds to nearest even).
inline uint packHalf2x16(vec2 v) {
    const _Float16 a = (_Float16)v.x, b = (_Float16)v.y;
    uint16_t ua, ub;
    std::memcpy(&ua, &a, 2);
    std::memcpy(&ub, &b, 2);
    return (uint)ua | ((uint)ub << 16);
}
inline vec2 unpackHalf2x16(uint p) {
    const uint16_t ua = (uint16_t)(p & 0xFFFFu), ub = (uint16_t)(p >> 16);
    _Float16 a, b;
    std::memcpy(&a, &ua, 2);
    std::memcpy(&b, &ub, 2);
    return vec2((float)a, (float)b);
}
// atomicAdd on a storage-buffer integer (the light cache's entry counter,
// lightcache.glsl:27-35): returns the old value.
inline int atomicAdd(int& x, int v) { return __atomic_fetch_add(&x, v, __ATOMIC_RELAXED); }
inline uint atomicAdd(uint& x, uint v) { return __atomic_fetch_add(&x, v, __ATOMIC_RELAXED); }
// the hash map's cell keys and list heads (maps/hashmap.glsl): return the old value
inline uint atomicCompSwap(uint& x, uint compare, uint data) {
    __atomic_compare_exchange_n(&x, &compare, data, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED);
    return compare;
}
inline uint atomicExchange(uint& x, uint data) { return __atomic_exchange_n(&x, data, __ATOMIC_RELAXED); }
// The lock image of the reference's commented-out spin lock (declared, unused).
struct uimage2D {
    uint32_t* texels = nullptr;
    int width = 0;
};

}  // namespace glslref
