// dual.cuh — forward-mode derivatives of the principled and Lambertian BSDF
// values with respect to the six differentiable material parameters
// (baseColor r, g, b; roughness before the mix(0.0134, 1, r) remap;
// metallic; specular), by dual numbers.  The value part follows the float32
// operations of material.glsl:357-490 (principledBRDF); the tangent part is
// the exact derivative of those operations.
#pragma once

#include "shading.cuh"

namespace zgl {

constexpr int kDiffMatParams = 6;  // baseColor.rgb, roughness, metallic, specular

struct Dl {
    float v;
    float d[kDiffMatParams];
};

__device__ __forceinline__ Dl dconst(float v) {
    Dl r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < kDiffMatParams; i++) r.d[i] = 0.0f;
    return r;
}
__device__ __forceinline__ Dl dvar(float v, int slot) {
    Dl r = dconst(v);
    r.d[slot] = 1.0f;
    return r;
}
__device__ __forceinline__ Dl operator+(Dl a, Dl b) {
    Dl r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < kDiffMatParams; i++) r.d[i] = a.d[i] + b.d[i];
    return r;
}
__device__ __forceinline__ Dl operator-(Dl a, Dl b) {
    Dl r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < kDiffMatParams; i++) r.d[i] = a.d[i] - b.d[i];
    return r;
}
__device__ __forceinline__ Dl operator*(Dl a, Dl b) {
    Dl r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < kDiffMatParams; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
__device__ __forceinline__ Dl operator/(Dl a, Dl b) {
    Dl r;
    r.v = a.v / b.v;
    float ib2 = 1.0f / (b.v * b.v);
#pragma unroll
    for (int i = 0; i < kDiffMatParams; i++) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) * ib2;
    return r;
}
__device__ __forceinline__ Dl operator+(Dl a, float b) { return a + dconst(b); }
__device__ __forceinline__ Dl operator+(float a, Dl b) { return dconst(a) + b; }
__device__ __forceinline__ Dl operator-(Dl a, float b) { return a - dconst(b); }
__device__ __forceinline__ Dl operator-(float a, Dl b) { return dconst(a) - b; }
__device__ __forceinline__ Dl operator*(Dl a, float b) {
    Dl r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < kDiffMatParams; i++) r.d[i] = a.d[i] * b;
    return r;
}
__device__ __forceinline__ Dl operator*(float a, Dl b) { return b * a; }
__device__ __forceinline__ Dl operator/(Dl a, float b) {
    Dl r;
    r.v = a.v / b;
#pragma unroll
    for (int i = 0; i < kDiffMatParams; i++) r.d[i] = a.d[i] / b;
    return r;
}

struct Dv3 {
    Dl x, y, z;
};
__device__ __forceinline__ Dv3 dv3(Dl a) { return Dv3{a, a, a}; }
__device__ __forceinline__ Dv3 dv3c(v3 a) { return Dv3{dconst(a.x), dconst(a.y), dconst(a.z)}; }
__device__ __forceinline__ Dv3 operator+(Dv3 a, Dv3 b) { return Dv3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ Dv3 operator-(Dv3 a, Dv3 b) { return Dv3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ Dv3 operator*(Dv3 a, Dv3 b) { return Dv3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ Dv3 operator*(Dv3 a, Dl s) { return Dv3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ Dv3 operator*(Dv3 a, float s) { return Dv3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ Dv3 operator/(Dv3 a, Dl s) { return Dv3{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ Dv3 operator/(Dv3 a, float s) { return Dv3{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ Dv3 dmix(Dv3 x, Dv3 y, Dl a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ Dv3 dmix(Dv3 x, Dv3 y, float a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ Dl dlum(Dv3 c) { return c.x * 0.299f + c.y * 0.587f + c.z * 0.114f; }

struct DParam {
    Dv3 baseColor;
    Dl roughness;  // after the remap
    Dl metallic, specular;
    float subsurface, specularTint, sheen, sheenTint, clearcoat, clearcoatGloss;
};

// Material record -> dual parameters (loadPrincipledBRDF, material_loader.glsl:37-58).
__device__ __forceinline__ DParam loadDParam(const DeviceScene& sc, int matId) {
    const float4 m0 = __ldg(&sc.materials[4 * matId + 0]);
    const float4 m1 = __ldg(&sc.materials[4 * matId + 1]);
    const float4 m2 = __ldg(&sc.materials[4 * matId + 2]);
    DParam p;
    p.baseColor = Dv3{dvar(m0.x, 0), dvar(m0.y, 1), dvar(m0.z, 2)};
    Dl r = dvar(m0.w, 3);
    p.roughness = 0.0134f * (1.0f - r) + 1.0f * r;
    p.subsurface = m1.x;
    p.metallic = dvar(m1.y, 4);
    p.specular = dvar(m1.z, 5);
    p.specularTint = m1.w;
    p.sheen = m2.x;
    p.sheenTint = m2.y;
    p.clearcoat = m2.z;
    p.clearcoatGloss = m2.w;
    return p;
}

__device__ __forceinline__ Dl dschlickG(float c, Dl alpha) {
    Dl k = alpha * 0.5f;
    return dconst(c) / (c * (1.0f - k) + k);
}
__device__ __forceinline__ Dl dggx(float c, Dl alpha) {
    if (c < 1e-6f) return dconst(0.0f);
    Dl a2 = alpha * alpha;
    Dl denom = c * c * (a2 - 1.0f) + 1.0f;
    denom = denom * denom * kPi;
    return a2 / denom;
}

// principledBRDF (material.glsl:462-490) with dual parameters.
__device__ __forceinline__ Dv3 dprincipledBRDF(v3 wo, v3 wi, v3 n, const DParam& p) {
    Dl alpha = p.roughness * p.roughness;
    float ccAlpha = mixf(0.1f, 0.001f, p.clearcoatGloss);
    Dl lum = dlum(p.baseColor);
    Dv3 tint = lum.v > 0.0f ? p.baseColor / lum : dv3(dconst(1.0f));
    Dv3 one = dv3(dconst(1.0f));
    Dv3 fm0 = dmix(dmix(one, tint, p.specularTint) * (0.08f * p.specular), p.baseColor, p.metallic);
    float hCosWiAll = dot(normalize(wo + wi), wi);
    Dv3 res = dv3(dconst(0.0f));
    // principledDiffuse (:429-452) * (1 - metallic)
    {
        float cosWo = satDot(n, wo), cosWi = satDot(n, wi);
        if (!(cosWo < 1e-10f || cosWi < 1e-10f)) {
            v3 h = normalize(wo + wi);
            float hCosWi = dot(h, wi);
            float hCosWi2 = hCosWi * hCosWi;
            float fi = schlickW(cosWi), fo = schlickW(cosWo);
            Dv3 fd90 = dv3(0.5f + 2.0f * p.roughness * hCosWi2);
            Dv3 fd = dmix(one, fd90, fi) * dmix(one, fd90, fo);
            Dv3 baseDiffuse = p.baseColor * fd * kPiInv;
            Dv3 fss90 = dv3(p.roughness * hCosWi2);
            Dv3 fss = dmix(one, fss90, fi) * dmix(one, fss90, fo);
            Dv3 ss = p.baseColor * kPiInv * 1.25f * (fss * (1.0f / (cosWi + cosWo) - 0.5f) + dv3(dconst(0.5f)));
            res = res + dmix(baseDiffuse, ss, p.subsurface) * (1.0f - p.metallic);
        }
    }
    // principledMetal (:357-373)
    {
        float cosWo = satDot(n, wo), cosWi = satDot(n, wi);
        v3 h = normalize(wo + wi);
        if (!(cosWo < 1e-10f || cosWi < 1e-10f)) {
            float w5 = pow5(1.0f - absDot(h, wo));
            Dv3 fm = fm0 + (one - fm0) * w5;
            Dl dm = dggx(dot(n, h), alpha);
            Dl gm = dschlickG(absDot(n, wo), alpha) * dschlickG(absDot(n, wi), alpha);
            float denom = 4.0f * cosWi * cosWo;
            if (!(denom < 1e-7f)) res = res + fm * dm * gm / denom;
        }
    }
    // principledClearcoat (:393-409) * clearcoat * 0.25
    {
        float cosWo = satDot(n, wo), cosWi = satDot(n, wi);
        v3 h = normalize(wo + wi);
        if (!(cosWo < 1e-6f || cosWi < 1e-6f)) {
            float w5 = pow5(1.0f - absDot(h, wo));
            Dv3 fc = p.baseColor + (one - p.baseColor) * w5;
            float dc = gtr1(satDot(n, h), ccAlpha);
            float gc = smithG(n, wo, wi, 0.25f);
            float denom = 4.0f * cosWi * cosWo;
            if (!(denom < 1e-7f)) res = res + fc * (dc * gc / denom) * (p.clearcoat * 0.25f);
        }
    }
    // sheen
    float sheenScale = schlickW(hCosWiAll) * p.sheen * (dot(n, wi) < 0.0f ? 0.0f : 1.0f);
    res = res + dmix(one, tint, p.sheenTint) * sheenScale;
    return res;
}

// BSDF value and its derivatives for a material (Lambertian: baseColor / pi).
struct BsdfGrad {
    v3 f;
    v3 df[kDiffMatParams];
};
__device__ __forceinline__ BsdfGrad bsdfGrad(const DeviceScene& sc, uint32_t type, int matId, v3 wo, v3 wi, v3 n) {
    BsdfGrad g;
    if (type == kPrincipled) {
        DParam p = loadDParam(sc, matId);
        Dv3 r = dprincipledBRDF(wo, wi, n, p);
        g.f = mk3(r.x.v, r.y.v, r.z.v);
#pragma unroll
        for (int i = 0; i < kDiffMatParams; i++) g.df[i] = mk3(r.x.d[i], r.y.d[i], r.z.d[i]);
    } else {
        const float4 m0 = __ldg(&sc.materials[4 * matId + 0]);
        g.f = mk3(m0.x, m0.y, m0.z) * kPiInv;
#pragma unroll
        for (int i = 0; i < kDiffMatParams; i++) g.df[i] = mk3(0.0f);
        g.df[0].x = kPiInv;
        g.df[1].y = kPiInv;
        g.df[2].z = kPiInv;
    }
    return g;
}

}  // namespace zgl
