// glsl_shim.h — GLSL 4.50 types and built-ins for the reference's compute
// shaders compiled as C++ (oracle/glsl_to_cpp.py).
//
// TEST INFRASTRUCTURE ONLY.  It lets the reference's own shader source run on
// the CPU as a second checker beside the hand restatement in
// render_oracle.cpp.  Where GLSL leaves an operation to the implementation,
// this header uses the same definition as the restatement and the CUDA
// kernels (the "defined arithmetic"):
//   * literals are float (the transform adds the f suffix);
//   * dot sums left to right; length = sqrt(dot); normalize(v) = v / length(v);
//     distance(a, b) = length(a - b); mix(x, y, a) = x (1 - a) + y a;
//     reflect(I, N) = I - (2 dot(N, I)) N; mat3 * v sums the columns left to
//     right; inverse(mat3) by cofactors (orc::inverse of render_oracle.cpp is
//     the same formula);
//   * min / max return the non-NaN operand and order -0 below +0;
//   * sin, cos, atan, log, pow are oracle_transc.h's series, sqrt and / are
//     IEEE;
//   * texture() on a 2D sampler is level 0, GL_LINEAR, GL_REPEAT at texel
//     centres: mix(mix(t00, t10, a), mix(t01, t11, a), b); texture2DArray on
//     the sRGB albedo array decodes each texel and blends with the weights
//     (1-a)(1-b), a(1-b), (1-a)b, ab in that order.
// Constructors take any arithmetic arguments (GLSL converts them), so that the
// transform can turn every vector constructor into a braced list, which C++
// evaluates left to right as GLSL does (vec4(sample1D(s), sample1D(s), ...)).
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "oracle_math.h"
#include "oracle_transc.h"

namespace glsl {

using uint = uint32_t;

template <class T>
using arith = std::enable_if_t<std::is_arithmetic<T>::value, int>;

struct vec2;
struct vec3;
struct vec4;

struct ivec2 {
    int x = 0, y = 0;
    ivec2() = default;
    template <class A, class B, arith<A> = 0, arith<B> = 0>
    ivec2(A a, B b) : x((int)a), y((int)b) {}
    explicit ivec2(const vec2& v);
    ivec2 xy() const { return *this; }
};
struct ivec4 {
    int x = 0, y = 0, z = 0, w = 0;
};
struct uvec3 {
    uint x = 0, y = 0, z = 0;
};
struct uvec4 {
    uint x = 0, y = 0, z = 0, w = 0;
};

struct vec2 {
    float x = 0.0f, y = 0.0f;
    vec2() = default;
    template <class A, arith<A> = 0>
    explicit vec2(A s) : x((float)s), y((float)s) {}
    template <class A, class B, arith<A> = 0, arith<B> = 0>
    vec2(A a, B b) : x((float)a), y((float)b) {}
    explicit vec2(ivec2 v) : x((float)v.x), y((float)v.y) {}
    vec2 xy() const { return *this; }
    vec2 yx() const { return vec2{y, x}; }
};
struct vec3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    vec3() = default;
    template <class A, arith<A> = 0>
    explicit vec3(A s) : x((float)s), y((float)s), z((float)s) {}
    template <class A, class B, class C, arith<A> = 0, arith<B> = 0, arith<C> = 0>
    vec3(A a, B b, C c) : x((float)a), y((float)b), z((float)c) {}
    template <class B, arith<B> = 0>
    vec3(vec2 v, B b) : x(v.x), y(v.y), z((float)b) {}
    vec2 xy() const { return vec2{x, y}; }
    vec2 yz() const { return vec2{y, z}; }
    vec2 xz() const { return vec2{x, z}; }
    vec3 xyz() const { return *this; }
};
struct vec4 {
    float x = 0.0f, y = 0.0f, z = 0.0f, w = 0.0f;
    vec4() = default;
    template <class A, arith<A> = 0>
    explicit vec4(A s) : x((float)s), y((float)s), z((float)s), w((float)s) {}
    template <class A, class B, class C, class D, arith<A> = 0, arith<B> = 0, arith<C> = 0, arith<D> = 0>
    vec4(A a, B b, C c, D d) : x((float)a), y((float)b), z((float)c), w((float)d) {}
    template <class B, arith<B> = 0>
    vec4(vec3 v, B b) : x(v.x), y(v.y), z(v.z), w((float)b) {}
    vec2 xy() const { return vec2{x, y}; }
    vec2 zw() const { return vec2{z, w}; }
    vec2 yz() const { return vec2{y, z}; }
    vec3 xyz() const { return vec3{x, y, z}; }
};
inline ivec2::ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}

// gl_GlobalInvocationID (read as .x or converted as .xy to ivec2)
struct GlobalId {
    uint x = 0, y = 0, z = 0;
    ivec2 xy() const { return ivec2{x, y}; }
};

// ------------------------------------------------------------ arithmetic
#define ZGL_V2(op)                                                                                        \
    inline vec2 operator op(vec2 a, vec2 b) { return vec2{a.x op b.x, a.y op b.y}; }                      \
    inline vec2 operator op(vec2 a, float s) { return vec2{a.x op s, a.y op s}; }                         \
    inline vec2 operator op(float s, vec2 a) { return vec2{s op a.x, s op a.y}; }
#define ZGL_V3(op)                                                                                        \
    inline vec3 operator op(vec3 a, vec3 b) { return vec3{a.x op b.x, a.y op b.y, a.z op b.z}; }          \
    inline vec3 operator op(vec3 a, float s) { return vec3{a.x op s, a.y op s, a.z op s}; }               \
    inline vec3 operator op(float s, vec3 a) { return vec3{s op a.x, s op a.y, s op a.z}; }
#define ZGL_V4(op)                                                                                        \
    inline vec4 operator op(vec4 a, vec4 b) { return vec4{a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w}; } \
    inline vec4 operator op(vec4 a, float s) { return vec4{a.x op s, a.y op s, a.z op s, a.w op s}; }
ZGL_V2(+) ZGL_V2(-) ZGL_V2(*) ZGL_V2(/)
ZGL_V3(+) ZGL_V3(-) ZGL_V3(*) ZGL_V3(/)
ZGL_V4(+) ZGL_V4(-) ZGL_V4(*) ZGL_V4(/)
#undef ZGL_V2
#undef ZGL_V3
#undef ZGL_V4

inline vec2 operator-(vec2 a) { return vec2{-a.x, -a.y}; }
inline vec3 operator-(vec3 a) { return vec3{-a.x, -a.y, -a.z}; }
template <class V, class S>
inline V& operator+=(V& a, S b) { return a = a + b; }
template <class V, class S>
inline V& operator-=(V& a, S b) { return a = a - b; }
template <class S>
inline vec3& operator*=(vec3& a, S b) { return a = a * b; }
template <class S>
inline vec3& operator/=(vec3& a, S b) { return a = a / b; }
template <class S>
inline vec2& operator*=(vec2& a, S b) { return a = a * b; }

struct mat3 {
    vec3 c0, c1, c2;  // columns
    mat3() = default;
    mat3(vec3 a, vec3 b, vec3 c) : c0(a), c1(b), c2(c) {}
};
inline vec3 operator*(const mat3& m, vec3 v) {
    return vec3{m.c0.x * v.x + m.c1.x * v.y + m.c2.x * v.z, m.c0.y * v.x + m.c1.y * v.y + m.c2.y * v.z,
                m.c0.z * v.x + m.c1.z * v.y + m.c2.z * v.z};
}
inline mat3 inverse(const mat3& m) {
    float a00 = m.c0.x, a01 = m.c1.x, a02 = m.c2.x;
    float a10 = m.c0.y, a11 = m.c1.y, a12 = m.c2.y;
    float a20 = m.c0.z, a21 = m.c1.z, a22 = m.c2.z;
    float C00 = a11 * a22 - a12 * a21;
    float C10 = a02 * a21 - a01 * a22;
    float C20 = a01 * a12 - a02 * a11;
    float det = a00 * C00 + a10 * C10 + a20 * C20;
    float id = 1.0f / det;
    float i00 = C00 * id, i01 = C10 * id, i02 = C20 * id;
    float i10 = (a12 * a20 - a10 * a22) * id, i11 = (a00 * a22 - a02 * a20) * id, i12 = (a02 * a10 - a00 * a12) * id;
    float i20 = (a10 * a21 - a11 * a20) * id, i21 = (a01 * a20 - a00 * a21) * id, i22 = (a00 * a11 - a01 * a10) * id;
    return mat3(vec3{i00, i10, i20}, vec3{i01, i11, i21}, vec3{i02, i12, i22});
}

// ------------------------------------------------------------- built-ins
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) { return vec3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float sqrt(float x) { return std::sqrt(x); }
inline float length(vec2 v) { return std::sqrt(dot(v, v)); }
inline float length(vec3 v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(vec3 v) { return v / length(v); }
inline float distance(vec3 a, vec3 b) { return length(a - b); }
inline float abs(float x) { return std::fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline vec3 abs(vec3 v) { return vec3{std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)}; }
inline float min(float a, float b) { return orc::fmin_(a, b); }
inline float max(float a, float b) { return orc::fmax_(a, b); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline vec3 min(vec3 a, vec3 b) { return vec3{min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)}; }
inline vec3 max(vec3 a, vec3 b) { return vec3{max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)}; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec2 mix(vec2 x, vec2 y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(vec3 x, vec3 y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(vec3 x, vec3 y, vec3 a) { return x * (vec3(1.0f) - a) + y * a; }
inline float floor(float x) { return std::floor(x); }
inline float fract(float x) { return x - std::floor(x); }
inline vec2 fract(vec2 v) { return vec2{fract(v.x), fract(v.y)}; }
inline float sin(float x) { return orc::zsin(x); }
inline float cos(float x) { return orc::zcos(x); }
inline float atan(float y, float x) { return orc::zatan2(y, x); }
inline float asin(float x) { return std::asin(x); }  // only in helpers the compared paths never call
inline float log(float x) { return orc::zlog(x); }
inline float pow(float x, float y) { return orc::zpow(x, y); }
inline bool isnan(float x) { return x != x; }
inline vec3 reflect(vec3 I, vec3 N) { return I - (2.0f * dot(N, I)) * N; }

// --------------------------------------------------------------- samplers
// Buffer textures: `comps` components per texel; GL returns (x, 0, 0, 1)
// style defaults for missing components.
struct samplerBuffer {
    const float* data = nullptr;
    int comps = 4;
};
struct isamplerBuffer {
    const int32_t* data = nullptr;
    int comps = 4;
};
struct usamplerBuffer {
    const uint32_t* data = nullptr;
    int comps = 1;
};
inline vec4 texelFetch(const samplerBuffer& s, int i) {
    const float* p = s.data + (int64_t)i * s.comps;
    vec4 r{0.0f, 0.0f, 0.0f, 1.0f};
    r.x = p[0];
    if (s.comps > 1) r.y = p[1];
    if (s.comps > 2) r.z = p[2];
    if (s.comps > 3) r.w = p[3];
    return r;
}
inline ivec4 texelFetch(const isamplerBuffer& s, int i) {
    const int32_t* p = s.data + (int64_t)i * s.comps;
    ivec4 r{0, 0, 0, 1};
    r.x = p[0];
    if (s.comps > 1) r.y = p[1];
    if (s.comps > 2) r.z = p[2];
    if (s.comps > 3) r.w = p[3];
    return r;
}
inline uvec4 texelFetch(const usamplerBuffer& s, int i) {
    uvec4 r{0u, 0u, 0u, 1u};
    r.x = s.data[(int64_t)i * s.comps];
    return r;
}

// 2D textures (row-major, `comps` floats per texel)
struct sampler2D {
    const float* data = nullptr;
    int w = 0, h = 0, comps = 4;
};
struct isampler2D {
    const int32_t* data = nullptr;
    int w = 0, h = 0;
};
inline vec4 texel2D(const sampler2D& s, int x, int y) {
    x %= s.w;
    if (x < 0) x += s.w;
    y %= s.h;
    if (y < 0) y += s.h;
    const float* p = s.data + ((int64_t)y * s.w + x) * s.comps;
    vec4 r{0.0f, 0.0f, 0.0f, 1.0f};
    r.x = p[0];
    if (s.comps > 1) r.y = p[1];
    if (s.comps > 2) r.z = p[2];
    if (s.comps > 3) r.w = p[3];
    return r;
}
inline vec4 texelFetch(const sampler2D& s, ivec2 c, int) { return texel2D(s, c.x, c.y); }
inline ivec4 texelFetch(const isampler2D& s, ivec2 c, int) {
    ivec4 r{0, 0, 0, 1};
    r.x = s.data[(int64_t)c.y * s.w + c.x];
    return r;
}
inline ivec2 textureSize(const sampler2D& s, int) { return ivec2{s.w, s.h}; }
inline vec4 mix4(vec4 a, vec4 b, float t) {
    return vec4{a.x * (1.0f - t) + b.x * t, a.y * (1.0f - t) + b.y * t, a.z * (1.0f - t) + b.z * t,
                a.w * (1.0f - t) + b.w * t};
}
inline vec4 texture(const sampler2D& s, vec2 st) {
    float u = st.x * (float)s.w - 0.5f;
    float v = st.y * (float)s.h - 0.5f;
    float fu = std::floor(u), fv = std::floor(v);
    float au = u - fu, av = v - fv;
    int x0 = orc::f2i(fu), y0 = orc::f2i(fv);
    vec4 t00 = texel2D(s, x0, y0), t10 = texel2D(s, x0 + 1, y0);
    vec4 t01 = texel2D(s, x0, y0 + 1), t11 = texel2D(s, x0 + 1, y0 + 1);
    return mix4(mix4(t00, t10, au), mix4(t01, t11, au), av);
}

// sRGB8 texture array: `layers` x h x w texels of 3 bytes, each image in the
// top-left corner of its layer; `lut` maps an sRGB code to linear.
struct sampler2DArray {
    const uint8_t* data = nullptr;
    int w = 0, h = 0;
    const float* lut = nullptr;
};
inline vec4 texture2DArray(const sampler2DArray& s, vec3 c) {
    const int W = s.w, H = s.h, layer = (int)c.z;
    const float u = c.x * (float)W - 0.5f, v = c.y * (float)H - 0.5f;
    const float a = u - std::floor(u), b = v - std::floor(v);
    auto wrap = [](int i, int n) { return ((i % n) + n) % n; };
    const int i0 = wrap((int)std::floor(u), W), j0 = wrap((int)std::floor(v), H);
    const int i1 = wrap(i0 + 1, W), j1 = wrap(j0 + 1, H);
    auto T = [&](int i, int j, int k) { return s.lut[s.data[(((int64_t)layer * H + j) * W + i) * 3 + k]]; };
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    float r[3];
    for (int k = 0; k < 3; k++) r[k] = w00 * T(i0, j0, k) + w10 * T(i1, j0, k) + w01 * T(i0, j1, k) + w11 * T(i1, j1, k);
    return vec4{r[0], r[1], r[2], 1.0f};
}

// storage image: RGBA32F (comps 4) or R32F (comps 1), row-major
struct image2D {
    float* data = nullptr;
    int w = 0, h = 0, comps = 4;
};
inline vec4 imageLoad(const image2D& im, ivec2 c) {
    const float* p = im.data + (int64_t)im.comps * ((int64_t)c.y * im.w + c.x);
    if (im.comps == 1) return vec4{p[0], 0.0f, 0.0f, 1.0f};
    return vec4{p[0], p[1], p[2], p[3]};
}
inline void imageStore(const image2D& im, ivec2 c, vec4 v) {
    float* p = im.data + (int64_t)im.comps * ((int64_t)c.y * im.w + c.x);
    p[0] = v.x;
    if (im.comps == 1) return;
    p[1] = v.y;
    p[2] = v.z;
    p[3] = v.w;
}
// imageAtomicAdd on an R32F image; the driver runs the invocations that add
// into one image on one thread, in invocation order
inline float imageAtomicAdd(const image2D& im, ivec2 c, float v) {
    float* p = im.data + ((int64_t)c.y * im.w + c.x);
    float old = *p;
    *p = old + v;
    return old;
}

}  // namespace glsl
