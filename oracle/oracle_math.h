// oracle_math.h — scalar float32 restatement of the GLSL built-ins the
// ZillumGL shaders use, for the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY.  The oracle is the checker of the CUDA path: only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
// Parity against the reference is UNPINNED at the shader level: the
// reference's device code is GLSL that needs an OpenGL 4.5 context, which is
// unavailable on this machine, so every formula below is a restatement of the
// GLSL 4.50 built-in definitions, compiled with -ffp-contract=off so that no
// multiply-add is fused.
//
// Arithmetic rules (shared with the CUDA kernels by definition, not by code):
//   * all literals are float (GLSL literals are float);
//   * dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, left to right;
//   * cross(a,b) = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x);
//   * length(v) = sqrt(dot(v,v)); normalize(v) = v / length(v) per component;
//   * min/max follow IEEE minNum/maxNum (a NaN operand yields the other one),
//     with -0 ordered below +0;
//   * float->int conversion truncates and saturates (NaN -> 0).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

static inline float fmin_(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    if (a == b) return std::signbit(a) ? a : b;
    return a < b ? a : b;
}
static inline float fmax_(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    if (a == b) return std::signbit(a) ? b : a;
    return a > b ? a : b;
}

static inline int32_t f2i(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}
static inline uint32_t f2u(float x) {
    if (x != x) return 0u;
    if (x >= 4294967296.0f) return UINT32_MAX;
    if (x <= 0.0f) return 0u;
    return (uint32_t)x;
}
static inline int32_t fbits(float x) { int32_t i; std::memcpy(&i, &x, 4); return i; }
static inline float bitsf(int32_t i) { float x; std::memcpy(&x, &i, 4); return x; }

struct vec2 {
    float x, y;
    vec2() : x(0.0f), y(0.0f) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
};
struct vec3 {
    float x, y, z;
    vec3() : x(0.0f), y(0.0f), z(0.0f) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

static inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
static inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
static inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
static inline vec3 operator/(float s, vec3 a) { return vec3(s / a.x, s / a.y, s / a.z); }
static inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
static inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
static inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
static inline vec2 operator*(vec2 a, vec2 b) { return vec2(a.x * b.x, a.y * b.y); }
static inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
static inline vec2 operator/(vec2 a, vec2 b) { return vec2(a.x / b.x, a.y / b.y); }
static inline vec2 operator-(vec2 a, float s) { return vec2(a.x - s, a.y - s); }
static inline vec2 operator+(vec2 a, float s) { return vec2(a.x + s, a.y + s); }

static inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
static inline vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float length(vec3 v) { return std::sqrt(dot(v, v)); }
static inline float length(vec2 v) { return std::sqrt(dot(v, v)); }
static inline vec3 normalize(vec3 v) { return v / length(v); }
static inline float distance(vec3 a, vec3 b) { return length(a - b); }
static inline vec3 vmin(vec3 a, vec3 b) { return vec3(fmin_(a.x, b.x), fmin_(a.y, b.y), fmin_(a.z, b.z)); }
static inline vec3 vmax(vec3 a, vec3 b) { return vec3(fmax_(a.x, b.x), fmax_(a.y, b.y), fmax_(a.z, b.z)); }
static inline vec3 vabs(vec3 a) { return vec3(std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)); }

}  // namespace orc
