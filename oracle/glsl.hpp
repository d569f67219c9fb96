// ORACLE — test infrastructure only. Not part of the product.
//
// A tiny C++ stand-in for the GLSL types and built-ins that gpugi's compute
// shaders use (gpugi/shader/*.glsl), so that the shader bodies can be restated
// in C++ almost line by line and run on the CPU as the checker for the CUDA
// path. Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg
// load the library built from these files.
//
// Parity status: UNPINNED. The reference ships no golden vectors, no tests and
// cannot be built or run here (its shaders need an OpenGL 4.5 context; its host
// code needs the missing epsilon/bim/glhelper submodules). This restatement is
// checked against brute force, analytic cases and physical invariants instead.
//
// Arithmetic conventions (fixed here because GLSL leaves them open):
//  * every file of the oracle is compiled with -ffp-contract=off: no FMA
//    contraction anywhere;
//  * dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z, evaluated left to right;
//  * cross(a, b) = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x);
//  * min/max follow IEEE-754 minNum/maxNum (a NaN operand yields the other
//    operand), as C's fminf/fmaxf do;
//  * 1.0/x is the correctly rounded IEEE quotient;
//  * sin/cos/pow/atan2/sqrt are the C library's single-precision functions.
#pragma once
#include <cmath>
#include <cstdint>

namespace glsl {

typedef uint32_t uint;

struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
};
struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};
struct vec4 {
    float x, y, z, w;
    vec4() : x(0), y(0), z(0), w(0) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec3 xyz() const { return vec3(x, y, z); }
};
struct ivec4 {
    int32_t x, y, z, w;
};

// vec2
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(vec2 a, vec2 b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator/(vec2 a, vec2 b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator*(float s, vec2 a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator-(vec2 a, float s) { return vec2(a.x - s, a.y - s); }
inline vec2 operator+(vec2 a, float s) { return vec2(a.x + s, a.y + s); }

// vec3
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator/(float s, vec3 a) { return vec3(s / a.x, s / a.y, s / a.z); }
inline vec3 operator+(vec3 a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(vec3 a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator-(float s, vec3 a) { return vec3(s - a.x, s - a.y, s - a.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3& operator+=(vec3& a, vec3 b) { a = a + b; return a; }
inline vec3& operator-=(vec3& a, vec3 b) { a = a - b; return a; }
inline vec3& operator*=(vec3& a, vec3 b) { a = a * b; return a; }
inline vec3& operator*=(vec3& a, float s) { a = a * s; return a; }
inline vec3& operator/=(vec3& a, float s) { a = a / s; return a; }
inline vec3& operator/=(vec3& a, vec3 b) { a = a / b; return a; }
inline vec4 operator+(vec4 a, vec4 b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(vec4 a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator/(vec4 a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }

inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline vec2 min(vec2 a, vec2 b) { return vec2(min(a.x, b.x), min(a.y, b.y)); }
inline vec2 max(vec2 a, vec2 b) { return vec2(max(a.x, b.x), max(a.y, b.y)); }
inline vec3 min(vec3 a, vec3 b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(vec3 a, vec3 b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float saturate(float x) { return clamp(x, 0.0f, 1.0f); }
inline vec3 saturate(vec3 v) { return vec3(saturate(v.x), saturate(v.y), saturate(v.z)); }
inline float abs(float x) { return std::fabs(x); }
inline vec3 abs(vec3 v) { return vec3(abs(v.x), abs(v.y), abs(v.z)); }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// normalize(v) = v / length(v), length = sqrt(dot(v, v))
inline vec3 normalize(vec3 v) { return v / sqrt(dot(v, v)); }
inline float length(vec3 v) { return sqrt(dot(v, v)); }
inline bool all_ge0(vec3 v) { return v.x >= 0.0f && v.y >= 0.0f && v.z >= 0.0f; }

inline uint floatBitsToUint(float f) { uint u; __builtin_memcpy(&u, &f, 4); return u; }
inline int floatBitsToInt(float f) { int u; __builtin_memcpy(&u, &f, 4); return u; }
inline float uintBitsToFloat(uint u) { float f; __builtin_memcpy(&f, &u, 4); return f; }

}  // namespace glsl
