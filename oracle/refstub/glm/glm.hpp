// glm.hpp — the subset of glm that the reference's accelerator sources use
// (src/accelerator/AABB.h, AABB.cpp, BVH.h, BVH.cpp), written here because
// glm is not installed.  TEST INFRASTRUCTURE ONLY: it is copied beside the
// reference sources into oracle/_ref/ by oracle/build_oracle.py and never
// linked into the product.
//
// glm is an unvendored, unversioned dependency of the reference.  The
// semantics restated here are glm's published scalar definitions, which are
// also the GLSL 4.50 definitions of min and max:
//   * min(x, y) = (y < x) ? y : x   — x on ties, including +0 / -0;
//   * max(x, y) = (x < y) ? y : x   — x on ties;
//   * vector forms apply them per component; vec3 is the packed (non-SIMD)
//     three-float type, so no intrinsic min/max is involved;
//   * arithmetic operators are per component in float.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>

namespace glm {

struct vec3 {
    float x, y, z;
    vec3() : x(0.0f), y(0.0f), z(0.0f) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

inline float min(float x, float y) { return (y < x) ? y : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }

}  // namespace glm
