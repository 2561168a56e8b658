// zmath.cuh — float32 vector math and transcendental functions shared by the
// host tables and the CUDA kernels.
//
// GLSL leaves the accuracy of sin/cos/atan/log/pow to the driver, so this
// library defines them and evaluates exactly the same float32 operations on
// host and device (the library is compiled with -fmad=false and
// -ffp-contract=off, IEEE division and square root), which makes results
// reproducible bit for bit.  Methods (textbook, written from the mathematics):
//   * sin/cos: Cody–Waite reduction by pi/2 with a three-part constant, Taylor
//     series on [-pi/4, pi/4] (sin to x^13, cos to x^14);
//   * atan: |x| reduced to <= tan(pi/8) with atan(x) = pi/4 + atan((x-1)/(x+1))
//     and atan(x) = pi/2 - atan(1/x), Taylor series to x^23;
//   * log: x = m 2^e, m in [sqrt(1/2), sqrt(2)), log m = 2 atanh((m-1)/(m+1))
//     by its series to s^15, e ln2 with a two-part constant;
//   * exp2: 2^x = 2^n exp(f ln2), |f| <= 1/2, Taylor to degree 10;
//   * pow(x, y) = exp2(y log2 x), the GLSL 4.50 definition.
// Vector built-ins follow the GLSL 4.50 formulas evaluated left to right:
// dot = (x*x' + y*y') + z*z', normalize(v) = v / length(v), mix = x(1-a) + ya,
// reflect(I, N) = I - (2 dot(N, I)) N; min/max return the non-NaN operand and
// order -0 below +0.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#define ZHD __host__ __device__ __forceinline__
// Larger routines called from many places (the transcendentals, the 3x3
// inverse): one out-of-line copy per translation unit keeps the integrator
// kernels' instruction footprint small (city path pass 32.6 -> 26.2 ms).  A
// translation unit that defines ZGL_INLINE_MATH inlines them (the
// differentiable renderer, measured faster that way).
#if defined(__CUDACC__) && !defined(ZGL_INLINE_MATH)
#define ZHD_CALL static __host__ __device__ __noinline__
#else
#define ZHD_CALL static inline __host__ __device__
#endif

namespace zgl {

ZHD float zbits2f(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}
ZHD uint32_t zf2bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}
ZHD bool zisnan(float x) { return x != x; }
ZHD bool zisinf(float x) { return (zf2bits(x) & 0x7fffffffu) == 0x7f800000u; }
ZHD bool zsignbit(float x) { return (zf2bits(x) >> 31) != 0u; }
ZHD float zrint(float x) {
#ifdef __CUDA_ARCH__
    return rintf(x);
#else
    return std::nearbyint(x);
#endif
}
ZHD float zsqrt(float x) {
#ifdef __CUDA_ARCH__
    return __fsqrt_rn(x);
#else
    return std::sqrt(x);
#endif
}
ZHD float zdiv(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

ZHD float zmin(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    if (a == b) return zsignbit(a) ? a : b;
    return a < b ? a : b;
}
ZHD float zmax(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    if (a == b) return zsignbit(a) ? b : a;
    return a > b ? a : b;
}
// truncating, saturating float -> int / uint (NaN -> 0)
ZHD int32_t zf2i(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int32_t)(-2147483647 - 1);
    return (int32_t)x;
}
ZHD uint32_t zf2u(float x) {
    if (x != x) return 0u;
    if (x >= 4294967296.0f) return 4294967295u;
    if (x <= 0.0f) return 0u;
    return (uint32_t)x;
}

// ------------------------------------------------------------------ vectors
struct v2 {
    float x, y;
};
struct v3 {
    float x, y, z;
};
ZHD v2 mk2(float x, float y) { return v2{x, y}; }
ZHD v3 mk3(float x, float y, float z) { return v3{x, y, z}; }
ZHD v3 mk3(float s) { return v3{s, s, s}; }
ZHD v3 operator+(v3 a, v3 b) { return v3{a.x + b.x, a.y + b.y, a.z + b.z}; }
ZHD v3 operator-(v3 a, v3 b) { return v3{a.x - b.x, a.y - b.y, a.z - b.z}; }
ZHD v3 operator*(v3 a, v3 b) { return v3{a.x * b.x, a.y * b.y, a.z * b.z}; }
ZHD v3 operator/(v3 a, v3 b) { return v3{a.x / b.x, a.y / b.y, a.z / b.z}; }
ZHD v3 operator*(v3 a, float s) { return v3{a.x * s, a.y * s, a.z * s}; }
ZHD v3 operator*(float s, v3 a) { return v3{s * a.x, s * a.y, s * a.z}; }
ZHD v3 operator/(v3 a, float s) { return v3{a.x / s, a.y / s, a.z / s}; }
ZHD v3 operator-(v3 a) { return v3{-a.x, -a.y, -a.z}; }
ZHD v2 operator+(v2 a, v2 b) { return v2{a.x + b.x, a.y + b.y}; }
ZHD v2 operator*(v2 a, v2 b) { return v2{a.x * b.x, a.y * b.y}; }
ZHD v2 operator*(v2 a, float s) { return v2{a.x * s, a.y * s}; }
ZHD v2 operator/(v2 a, v2 b) { return v2{a.x / b.x, a.y / b.y}; }
ZHD float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
ZHD float dot(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
ZHD v3 cross(v3 a, v3 b) { return v3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
ZHD float length(v3 v) { return zsqrt(dot(v, v)); }
ZHD float length(v2 v) { return zsqrt(dot(v, v)); }
ZHD v3 normalize(v3 v) { return v / length(v); }
ZHD float distance(v3 a, v3 b) { return length(a - b); }
ZHD float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
ZHD v3 mix3(v3 x, v3 y, float a) { return x * (1.0f - a) + y * a; }
ZHD v3 reflect(v3 I, v3 N) { return I - (2.0f * dot(N, I)) * N; }
ZHD float satDot(v3 a, v3 b) { return zmax(dot(a, b), 0.0f); }
ZHD float absDot(v3 a, v3 b) { return fabsf(dot(a, b)); }
ZHD float sq(float x) { return x * x; }
ZHD float distSquare(v3 x, v3 y) { return dot(x - y, x - y); }
ZHD float luminance(v3 c) { return dot(c, mk3(0.299f, 0.587f, 0.114f)); }
ZHD bool isBlack(v3 c) { return luminance(c) < 1e-5f; }
ZHD bool hasNan(v3 c) { return zisnan(c.x) || zisnan(c.y) || zisnan(c.z); }
ZHD float maxComponent(v3 v) { return zmax(v.x, zmax(v.y, v.z)); }
ZHD float pow5(float x) {
    float x2 = x * x;
    return x2 * x2 * x;
}

// column-major 3x3
struct m3 {
    v3 c0, c1, c2;
};
ZHD v3 mul(const m3& m, v3 v) {
    return v3{m.c0.x * v.x + m.c1.x * v.y + m.c2.x * v.z, m.c0.y * v.x + m.c1.y * v.y + m.c2.y * v.z,
              m.c0.z * v.x + m.c1.z * v.y + m.c2.z * v.z};
}
// cofactor inverse, determinant expanded along the first column
ZHD_CALL m3 inverse(const m3& m) {
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
    return m3{v3{i00, i10, i20}, v3{i01, i11, i21}, v3{i02, i12, i22}};
}

// ---------------------------------------------------------- transcendentals
constexpr float kPi = 3.14159265358979323846f;
constexpr float kPiInv = 1.0f / kPi;
constexpr float kPio2 = 1.57079632679489661923f;
constexpr float kPio4 = 0.78539816339744830962f;
constexpr float kPio2_1 = 1.5703125f;
constexpr float kPio2_2 = 4.83751296997070312500e-4f;
constexpr float kPio2_3 = 7.54978995489188216e-8f;

ZHD float sin_poly(float r) {
    float r2 = r * r;
    float p = 1.6059043836821613e-10f;
    p = p * r2 - 2.5052108385441720e-08f;
    p = p * r2 + 2.7557319223985893e-06f;
    p = p * r2 - 1.9841269841269841e-04f;
    p = p * r2 + 8.3333333333333333e-03f;
    p = p * r2 - 1.6666666666666667e-01f;
    return r + r * (r2 * p);
}
ZHD float cos_poly(float r) {
    float r2 = r * r;
    float p = 1.1470745597729725e-11f;
    p = p * r2 - 2.0876756987868099e-09f;
    p = p * r2 + 2.7557319223985888e-07f;
    p = p * r2 - 2.4801587301587302e-05f;
    p = p * r2 + 1.3888888888888889e-03f;
    p = p * r2 - 4.1666666666666667e-02f;
    p = p * r2 + 0.5f;
    return 1.0f - r2 * p;
}
ZHD float trig_reduce(float x, int& q) {
    float k = zrint(x * 0.63661977236758134f);
    q = (int)k;
    float r = x - k * kPio2_1;
    r = r - k * kPio2_2;
    r = r - k * kPio2_3;
    return r;
}
ZHD float znan() { return zbits2f(0x7fc00000u); }
ZHD float zinf() { return zbits2f(0x7f800000u); }

ZHD_CALL float zsin(float x) {
    if (x != x || zisinf(x)) return znan();
    int q;
    float r = trig_reduce(x, q);
    switch (q & 3) {
        case 0: return sin_poly(r);
        case 1: return cos_poly(r);
        case 2: return -sin_poly(r);
        default: return -cos_poly(r);
    }
}
ZHD_CALL float zcos(float x) {
    if (x != x || zisinf(x)) return znan();
    int q;
    float r = trig_reduce(x, q);
    switch (q & 3) {
        case 0: return cos_poly(r);
        case 1: return -sin_poly(r);
        case 2: return -cos_poly(r);
        default: return sin_poly(r);
    }
}

ZHD float atan_poly(float x) {
    float x2 = x * x;
    float p = -1.0f / 23.0f;
    p = p * x2 + 1.0f / 21.0f;
    p = p * x2 - 1.0f / 19.0f;
    p = p * x2 + 1.0f / 17.0f;
    p = p * x2 - 1.0f / 15.0f;
    p = p * x2 + 1.0f / 13.0f;
    p = p * x2 - 1.0f / 11.0f;
    p = p * x2 + 1.0f / 9.0f;
    p = p * x2 - 1.0f / 7.0f;
    p = p * x2 + 1.0f / 5.0f;
    p = p * x2 - 1.0f / 3.0f;
    return x + x * (x2 * p);
}
ZHD float atan_pos(float x) {
    if (x > 2.41421356237309504880f) return kPio2 - atan_poly(1.0f / x);
    if (x > 0.41421356237309504880f) return kPio4 + atan_poly((x - 1.0f) / (x + 1.0f));
    return atan_poly(x);
}
// atan(y, x) with the C99 special cases
ZHD_CALL float zatan2(float y, float x) {
    if (x != x || y != y) return x + y;
    if (y == 0.0f) {
        if (zsignbit(x)) return zsignbit(y) ? -kPi : kPi;
        return y;
    }
    if (x == 0.0f) return y > 0.0f ? kPio2 : -kPio2;
    if (zisinf(x)) {
        if (zisinf(y)) {
            float a = x > 0.0f ? kPio4 : 3.0f * kPio4;
            return y > 0.0f ? a : -a;
        }
        if (x > 0.0f) return y > 0.0f ? 0.0f : -0.0f;
        return y > 0.0f ? kPi : -kPi;
    }
    if (zisinf(y)) return y > 0.0f ? kPio2 : -kPio2;
    float ay = fabsf(y), ax = fabsf(x);
    float a;
    if (ay <= ax) a = atan_pos(ay / ax);
    else a = kPio2 - atan_pos(ax / ay);
    if (x < 0.0f) a = kPi - a;
    return y < 0.0f ? -a : a;
}

constexpr float kLn2Hi = 0.693145751953125f;
constexpr float kLn2Lo = 1.428606820309417232e-6f;

ZHD_CALL float zlog(float x) {
    if (x != x || x < 0.0f) return znan();
    if (x == 0.0f) return -zinf();
    if (zisinf(x)) return x;
    uint32_t u = zf2bits(x);
    int e = 0;
    if ((u >> 23) == 0u) {
        x = x * 33554432.0f;
        u = zf2bits(x);
        e = -25;
    }
    e += (int)((u >> 23) & 0xffu) - 127;
    float m = zbits2f((u & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356237309504880f) {
        m = m * 0.5f;
        e += 1;
    }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = 1.0f / 15.0f;
    p = p * s2 + 1.0f / 13.0f;
    p = p * s2 + 1.0f / 11.0f;
    p = p * s2 + 1.0f / 9.0f;
    p = p * s2 + 1.0f / 7.0f;
    p = p * s2 + 1.0f / 5.0f;
    p = p * s2 + 1.0f / 3.0f;
    float lm = 2.0f * s + 2.0f * s * (s2 * p);
    float fe = (float)e;
    return (fe * kLn2Hi + lm) + fe * kLn2Lo;
}
ZHD float zlog2(float x) { return zlog(x) * 1.44269504088896340736f; }
ZHD_CALL float zexp2(float x) {
    if (x != x) return x;
    if (x >= 128.0f) return zinf();
    if (x < -150.0f) return 0.0f;
    float n = zrint(x);
    float f = (x - n) * 0.69314718055994530942f;
    float p = 2.7557319223985891e-07f;
    p = p * f + 2.7557319223985891e-06f;
    p = p * f + 2.4801587301587302e-05f;
    p = p * f + 1.9841269841269841e-04f;
    p = p * f + 1.3888888888888889e-03f;
    p = p * f + 8.3333333333333333e-03f;
    p = p * f + 4.1666666666666667e-02f;
    p = p * f + 1.6666666666666667e-01f;
    p = p * f + 0.5f;
    p = p * f + 1.0f;
    float r = 1.0f + f * p;
    int ni = (int)n;
    if (ni != 0) {
        int a = ni / 2, b = ni - a;
        r = r * zbits2f((uint32_t)(a + 127) << 23);
        r = r * zbits2f((uint32_t)(b + 127) << 23);
    }
    return r;
}
ZHD float zpow(float x, float y) { return zexp2(y * zlog2(x)); }

}  // namespace zgl
