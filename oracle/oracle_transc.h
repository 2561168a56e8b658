// oracle_transc.h — float32 transcendental functions of the oracle.
//
// TEST INFRASTRUCTURE ONLY.  GLSL leaves the accuracy of sin/cos/atan/log/pow
// to the driver, so the build defines them: the CUDA kernels evaluate exactly
// the same sequence of float32 operations (no fused multiply-add), which makes
// radiance bit-identical between the oracle and the GPU.  Methods (all
// textbook, written from the mathematics):
//   * sin/cos: Cody–Waite reduction by pi/2 with a three-part constant, then
//     Taylor series on [-pi/4, pi/4] (sin to x^13, cos to x^14);
//   * atan: reduction to |x| <= tan(pi/8) via atan(x) = pi/4 + atan((x-1)/(x+1))
//     and atan(x) = pi/2 - atan(1/x), then the Taylor series to x^23;
//   * log: x = m * 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s),
//     s = (m-1)/(m+1), series to s^15, e*ln2 with a two-part constant;
//   * exp2: 2^x = 2^n * exp(f*ln2), |f| <= 1/2, Taylor to degree 10;
//   * pow(x, y) = exp2(y * log2(x)) (the GLSL 4.50 definition).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

static inline float t_bits2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline uint32_t t_f2bits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// pi/2 = P1 + P2 + P3; P1 and P2 carry few significant bits so k*P1 and k*P2
// are exact for |k| < 2^11.
static const float kPio2_1 = 1.5703125f;                 // 0x3FC90000
static const float kPio2_2 = 4.83751296997070312500e-4f; // 0x39FDA000
static const float kPio2_3 = 7.54978995489188216e-8f;    // pi/2 - P1 - P2 (rounded)

static inline float t_sin_poly(float r) {
    float r2 = r * r;
    // r - r^3/3! + r^5/5! - ... + r^13/13!
    float p = 1.6059043836821613e-10f;          // 1/13!
    p = p * r2 - 2.5052108385441720e-08f;       // 1/11!
    p = p * r2 + 2.7557319223985893e-06f;       // 1/9!
    p = p * r2 - 1.9841269841269841e-04f;       // 1/7!
    p = p * r2 + 8.3333333333333333e-03f;       // 1/5!
    p = p * r2 - 1.6666666666666667e-01f;       // 1/3!
    return r + r * (r2 * p);
}

static inline float t_cos_poly(float r) {
    float r2 = r * r;
    float p = 1.1470745597729725e-11f;          // 1/14!
    p = p * r2 - 2.0876756987868099e-09f;       // 1/12!
    p = p * r2 + 2.7557319223985888e-07f;       // 1/10!
    p = p * r2 - 2.4801587301587302e-05f;       // 1/8!
    p = p * r2 + 1.3888888888888889e-03f;       // 1/6!
    p = p * r2 - 4.1666666666666667e-02f;       // 1/4!
    p = p * r2 + 0.5f;                          // 1/2!
    return 1.0f - r2 * p;
}

// reduce x to r in [-pi/4, pi/4] and quadrant q
static inline float t_reduce(float x, int& q) {
    float k = std::nearbyint(x * 0.63661977236758134f);  // 2/pi
    q = (int)k;
    float r = x - k * kPio2_1;
    r = r - k * kPio2_2;
    r = r - k * kPio2_3;
    return r;
}

static inline float zsin(float x) {
    if (x != x || std::isinf(x)) return NAN;
    int q;
    float r = t_reduce(x, q);
    float s;
    switch (q & 3) {
        case 0: s = t_sin_poly(r); break;
        case 1: s = t_cos_poly(r); break;
        case 2: s = -t_sin_poly(r); break;
        default: s = -t_cos_poly(r); break;
    }
    return s;
}

static inline float zcos(float x) {
    if (x != x || std::isinf(x)) return NAN;
    int q;
    float r = t_reduce(x, q);
    float c;
    switch (q & 3) {
        case 0: c = t_cos_poly(r); break;
        case 1: c = -t_sin_poly(r); break;
        case 2: c = -t_cos_poly(r); break;
        default: c = t_sin_poly(r); break;
    }
    return c;
}

// atan on |x| <= tan(pi/8)
static inline float t_atan_poly(float x) {
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

static const float kPi = 3.14159265358979323846f;
static const float kPio2 = 1.57079632679489661923f;
static const float kPio4 = 0.78539816339744830962f;

// atan(x) for x >= 0
static inline float t_atan_pos(float x) {
    if (x > 2.41421356237309504880f) {  // tan(3pi/8)
        return kPio2 - t_atan_poly(1.0f / x);
    }
    if (x > 0.41421356237309504880f) {  // tan(pi/8)
        return kPio4 + t_atan_poly((x - 1.0f) / (x + 1.0f));
    }
    return t_atan_poly(x);
}

static inline float zatan(float x) {
    if (x != x) return x;
    if (std::isinf(x)) return x > 0.0f ? kPio2 : -kPio2;
    return x < 0.0f ? -t_atan_pos(-x) : t_atan_pos(x);
}

// atan2 with the C99 special cases (GLSL atan(y, x) leaves x = y = 0 undefined)
static inline float zatan2(float y, float x) {
    if (x != x || y != y) return x + y;
    if (y == 0.0f) {
        if (std::signbit(x)) return std::signbit(y) ? -kPi : kPi;
        return y;  // +-0
    }
    if (x == 0.0f) return y > 0.0f ? kPio2 : -kPio2;
    if (std::isinf(x)) {
        if (std::isinf(y)) {
            float a = x > 0.0f ? kPio4 : 3.0f * kPio4;
            return y > 0.0f ? a : -a;
        }
        if (x > 0.0f) return y > 0.0f ? 0.0f : -0.0f;
        return y > 0.0f ? kPi : -kPi;
    }
    if (std::isinf(y)) return y > 0.0f ? kPio2 : -kPio2;
    float ay = std::fabs(y), ax = std::fabs(x);
    float a;
    if (ay <= ax) a = t_atan_pos(ay / ax);
    else a = kPio2 - t_atan_pos(ax / ay);
    if (x < 0.0f) a = kPi - a;
    return y < 0.0f ? -a : a;
}

static const float kLn2Hi = 0.693145751953125f;       // 0x3F317200
static const float kLn2Lo = 1.428606820309417232e-6f;  // ln2 - kLn2Hi

static inline float zlog(float x) {
    if (x != x || x < 0.0f) return NAN;
    if (x == 0.0f) return -INFINITY;
    if (std::isinf(x)) return x;
    uint32_t u = t_f2bits(x);
    int e = 0;
    if ((u >> 23) == 0) {  // subnormal: scale by 2^25
        x = x * 33554432.0f;
        u = t_f2bits(x);
        e = -25;
    }
    e += (int)((u >> 23) & 0xff) - 127;
    float m = t_bits2f((u & 0x007fffffu) | 0x3f800000u);  // [1, 2)
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

static inline float zlog2(float x) { return zlog(x) * 1.44269504088896340736f; }

static inline float zexp2(float x) {
    if (x != x) return x;
    if (x >= 128.0f) return INFINITY;
    if (x < -150.0f) return 0.0f;
    float n = std::nearbyint(x);
    float f = (x - n) * 0.69314718055994530942f;  // |f| <= ln2/2
    float p = 2.7557319223985891e-07f;            // 1/10!
    p = p * f + 2.7557319223985891e-06f;          // 1/9!
    p = p * f + 2.4801587301587302e-05f;          // 1/8!
    p = p * f + 1.9841269841269841e-04f;          // 1/7!
    p = p * f + 1.3888888888888889e-03f;          // 1/6!
    p = p * f + 8.3333333333333333e-03f;          // 1/5!
    p = p * f + 4.1666666666666667e-02f;          // 1/4!
    p = p * f + 1.6666666666666667e-01f;          // 1/3!
    p = p * f + 0.5f;
    p = p * f + 1.0f;
    float r = 1.0f + f * p;
    int ni = (int)n;
    // scale by 2^ni in two steps to stay in range
    if (ni > 0) {
        int a = ni / 2, b = ni - a;
        r = r * t_bits2f((uint32_t)(a + 127) << 23);
        r = r * t_bits2f((uint32_t)(b + 127) << 23);
    } else if (ni < 0) {
        int a = ni / 2, b = ni - a;  // both >= -75
        r = r * t_bits2f((uint32_t)(a + 127) << 23);
        r = r * t_bits2f((uint32_t)(b + 127) << 23);
    }
    return r;
}

// GLSL pow(x, y) = exp2(y * log2(x)); x < 0 is undefined in GLSL, NaN here.
static inline float zpow(float x, float y) { return zexp2(y * zlog2(x)); }

}  // namespace orc
