// shading.cuh — device side of the render hot path: samplers, BSDFs, area
// and environment lights, thin-lens camera.  Each function follows the GLSL
// function it names (src/shader/*.glsl) operation for operation in float32.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "accel.h"
#include "device_scene.h"
#include "traverse.cuh"
#include "zmath.cuh"

namespace zgl {

enum : uint32_t { kDiffuse = 1u, kGlosRefl = 2u, kGlosTrans = 4u, kSpecRefl = 8u, kSpecTrans = 16u, kInvalid = 1u << 16 };
enum : uint32_t { kLambertian = 0, kPrincipled = 1, kMetalWorkflow = 2, kDielectric = 3, kThinDielectric = 4 };

__device__ __forceinline__ v3 f3(float3 a) { return v3{a.x, a.y, a.z}; }

// ------------------------------------------------------------- random.glsl
__device__ __forceinline__ uint32_t zhash(uint32_t seed) {  // random.glsl:5-13
    seed = (seed ^ 61u) ^ (seed >> 16u);
    seed *= 9u;
    seed = seed ^ (seed >> 4u);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15u);
    return seed;
}

struct Sampler {
    uint32_t randSeed;
    uint32_t sampleSeed;
    uint32_t sampleOffset;  // spp * 256, wrapped like path_integ_naive.glsl:163-164
    int32_t dim;            // the Sampler counter `s`
    int32_t mode;           // 0 independent, 1 sobol
    const uint32_t* rowCache;  // shared-memory copy of the 256 values of row sampleOffset/256
    const uint32_t* mats;      // 256*32 generator matrices
};

__device__ __forceinline__ float rand01(Sampler& g) {  // random.glsl:15-19
    g.randSeed = zhash(g.randSeed);
    return (float)g.randSeed * (1.0f / 4294967296.0f);
}

__device__ __forceinline__ uint32_t sobol_value(const uint32_t* mats, uint32_t index, uint32_t dim) {
    uint32_t r = 0;
    const uint32_t* col = mats + dim * 32u;
    for (int i = 0; index != 0u; index >>= 1, i++)
        if (index & 1u) r ^= __ldg(col + i);
    return r;
}

__device__ __forceinline__ float sample1D(Sampler& g) {  // random.glsl:61-70
    if (g.mode == 0) return rand01(g);
    uint32_t r;
    if (g.dim < 256) {
        r = g.rowCache[g.dim];
    } else {
        uint32_t idx = g.sampleOffset + (uint32_t)g.dim;
        r = sobol_value(g.mats, idx >> 8, idx & 255u);
    }
    r ^= g.sampleSeed;
    g.sampleSeed = zhash(g.sampleSeed);
    g.dim++;
    return (float)r / 4294967296.0f;
}

// --------------------------------------------------------------- math.glsl
__device__ __forceinline__ v2 toConcentricDisk(v2 v) {  // math.glsl:25-41
    if (v.x == 0.0f && v.y == 0.0f) return mk2(0.0f, 0.0f);
    v = mk2(v.x * 2.0f - 1.0f, v.y * 2.0f - 1.0f);
    float phi, r;
    if (v.x * v.x > v.y * v.y) {
        r = v.x;
        phi = kPi * v.y / v.x * 0.25f;
    } else {
        r = v.y;
        phi = kPi * 0.5f - kPi * v.x / v.y * 0.25f;
    }
    return mk2(r * zcos(phi), r * zsin(phi));
}
__device__ __forceinline__ m3 tbnMatrix(v3 n) {  // math.glsl:78-84
    v3 t = (fabsf(n.z) > 0.999f) ? mk3(0.0f, 1.0f, 0.0f) : mk3(0.0f, 0.0f, 1.0f);
    v3 b = normalize(cross(n, t));
    t = cross(b, n);
    return m3{t, b, n};
}
__device__ __forceinline__ v3 normalToWorld(v3 n, v3 v) { return normalize(mul(tbnMatrix(n), v)); }
__device__ __forceinline__ v3 sampleCosineWeighted(v3 n, v2 u, float& pdf) {  // math.glsl:99-105
    v2 uv = toConcentricDisk(u);
    float z = zsqrt(1.0f - dot(uv, uv));
    pdf = kPiInv * z;
    return normalToWorld(n, mk3(uv.x, uv.y, z));
}
__device__ __forceinline__ bool sameHemisphere(v3 n, v3 a, v3 b) { return dot(n, a) * dot(n, b) > 0.0f; }
__device__ __forceinline__ v3 sampleTriangleUniform(v3 va, v3 vb, v3 vc, v2 uv) {  // math.glsl:139-145
    float r = zsqrt(uv.y);
    float u = 1.0f - r;
    float v = uv.x * r;
    return va * (1.0f - u - v) + vb * u + vc * v;
}
__device__ __forceinline__ float triangleArea(v3 va, v3 vb, v3 vc) {
    return 0.5f * length(cross(vc - va, vb - va));
}
__device__ __forceinline__ v3 rotateZ(v3 v, float angle) {  // math.glsl:180-185
    float c = zcos(angle), s = zsin(angle);
    return mk3(v.x * c - v.y * s, v.x * s + v.y * c, v.z);
}
__device__ __forceinline__ v2 sphereToPlane(v3 uv) {  // math.glsl:58-64
    float theta = zatan2(uv.y, uv.x);
    if (theta < 0.0f) theta += kPi * 2.0f;
    float phi = zatan2(length(mk2(uv.x, uv.y)), uv.z);
    return mk2(theta * kPiInv * 0.5f, phi * kPiInv);
}
__device__ __forceinline__ v3 planeToSphere(v2 uv) {  // math.glsl:66-71
    float theta = uv.x * kPi * 2.0f;
    float phi = uv.y * kPi;
    return mk3(zcos(theta) * zsin(phi), zsin(theta) * zsin(phi), zcos(phi));
}
__device__ __forceinline__ float biHeuristic(float f, float g) { return f * f / (f * f + g * g); }

// ---------------------------------------------------------- microfacet.glsl
__device__ __forceinline__ float schlickW(float c) { return pow5(1.0f - c); }
__device__ __forceinline__ v3 schlickF(float c, v3 F0) { return F0 + (mk3(1.0f) - F0) * pow5(1.0f - c); }
__device__ __forceinline__ float schlickG(float c, float alpha) {
    float k = alpha * 0.5f;
    return c / (c * (1.0f - k) + k);
}
__device__ __forceinline__ float smithG(v3 n, v3 wo, v3 wi, float alpha) {
    return schlickG(absDot(n, wo), alpha) * schlickG(absDot(n, wi), alpha);
}
__device__ __forceinline__ float ggx(float c, float alpha) {  // microfacet.glsl:30-40
    if (c < 1e-6f) return 0.0f;
    float a2 = alpha * alpha;
    float denom = c * c * (a2 - 1.0f) + 1.0f;
    denom = denom * denom * kPi;
    return a2 / denom;
}
__device__ __forceinline__ float ggxPdfVisibleWm(v3 n, v3 m, v3 wo, float alpha) {
    return ggx(dot(n, m), alpha) * schlickG(dot(n, wo), alpha) * absDot(m, wo) / absDot(n, wo);
}
__device__ __forceinline__ v3 ggxSampleVisibleWm(v3 n, v3 wo, float alpha, v2 u) {  // microfacet.glsl:74-92
    m3 tbn = tbnMatrix(n);
    m3 tbnInv = inverse(tbn);
    v3 vh = normalize(mul(tbnInv, wo) * mk3(alpha, alpha, 1.0f));
    float lensq = vh.x * vh.x + vh.y * vh.y;
    v3 t1 = lensq > 0.0f ? mk3(-vh.y, vh.x, 0.0f) / zsqrt(lensq) : mk3(1.0f, 0.0f, 0.0f);
    v3 t2 = cross(vh, t1);
    v2 xi = toConcentricDisk(u);
    float s = 0.5f * (1.0f + vh.z);
    xi.y = (1.0f - s) * zsqrt(1.0f - xi.x * xi.x) + s * xi.y;
    v3 h = t1 * xi.x + t2 * xi.y + vh * zsqrt(zmax(0.0f, 1.0f - xi.x * xi.x - xi.y * xi.y));
    h = normalize(mk3(h.x * alpha, h.y * alpha, zmax(0.0f, h.z)));
    return normalToWorld(n, h);
}
__device__ __forceinline__ float gtr1(float c, float alpha) {  // microfacet.glsl:94-98
    float a2 = alpha * alpha;
    return (a2 - 1.0f) / (2.0f * kPi * zlog(alpha) * (1.0f + (a2 - 1.0f) * c * c));
}
__device__ __forceinline__ v3 gtr1SampleWm(v3 n, v3 wo, float alpha, v2 u) {  // microfacet.glsl:105-115
    float cosTheta = zsqrt(zmax(0.0f, (1.0f - zpow(alpha, 1.0f - u.x)) / (1.0f - alpha)));
    float sinTheta = zsqrt(zmax(0.0f, 1.0f - cosTheta * cosTheta));
    float phi = 2.0f * u.y * kPi;
    v3 m = normalize(mk3(zcos(phi) * sinTheta, zsin(phi) * sinTheta, cosTheta));
    if (!sameHemisphere(n, wo, m)) m = -m;
    return normalize(normalToWorld(n, m));
}

// ------------------------------------------------------------ material.glsl
struct BSDFParam {
    v3 baseColor;
    float subsurface, metallic, roughness;
    union {
        float specular;  // principled
        float ior;       // dielectric and thin dielectric (they have no specular)
    };
    float specularTint;
    float sheen, sheenTint, clearcoat, clearcoatGloss;
};
// TransportMode (material.glsl:19-21): the dielectric's refraction scales
// radiance by 1/eta^2 but not importance.
enum : uint32_t { kRadiance = 0, kImportance = 1 };
struct BSDFSample {
    v3 wi;
    float pdf;
    v3 bsdf;
    uint32_t flag;
};

__device__ __forceinline__ v3 principledMetal(v3 wo, v3 wi, v3 n, v3 fm0, float alpha) {  // material.glsl:357-373
    float cosWo = satDot(n, wo);
    float cosWi = satDot(n, wi);
    v3 h = normalize(wo + wi);
    if (cosWo < 1e-10f || cosWi < 1e-10f) return mk3(0.0f);
    v3 fm = schlickF(absDot(h, wo), fm0);
    float dm = ggx(dot(n, h), alpha);
    float gm = smithG(n, wo, wi, alpha);
    float denom = 4.0f * cosWi * cosWo;
    if (denom < 1e-7f) return mk3(0.0f);
    return fm * dm * gm / denom;
}
__device__ __forceinline__ float principledMetalPdf(v3 wo, v3 wi, v3 n, float alpha) {
    v3 h = normalize(wo + wi);
    return ggxPdfVisibleWm(n, h, wo, alpha) / (4.0f * absDot(h, wo));
}
__device__ __forceinline__ v3 principledClearcoat(v3 wo, v3 wi, v3 n, v3 baseColor, float alpha) {  // :393-409
    float cosWo = satDot(n, wo);
    float cosWi = satDot(n, wi);
    v3 h = normalize(wo + wi);
    if (cosWo < 1e-6f || cosWi < 1e-6f) return mk3(0.0f);
    v3 fc = schlickF(absDot(h, wo), baseColor);
    float dc = gtr1(satDot(n, h), alpha);
    float gc = smithG(n, wo, wi, 0.25f);
    float denom = 4.0f * cosWi * cosWo;
    if (denom < 1e-7f) return mk3(0.0f);
    return fc * dc * gc / denom;
}
__device__ __forceinline__ float principledClearcoatPdf(v3 wo, v3 wi, v3 n, float alpha) {
    v3 h = normalize(wo + wi);
    return gtr1(satDot(n, h), alpha) * absDot(n, h) / (4.0f * absDot(h, wo));
}
__device__ __forceinline__ v3 principledDiffuse(v3 wo, v3 wi, v3 n, v3 baseColor, float subsurface,
                                                float roughness) {  // :429-452
    float cosWo = satDot(n, wo);
    float cosWi = satDot(n, wi);
    if (cosWo < 1e-10f || cosWi < 1e-10f) return mk3(0.0f);
    v3 h = normalize(wo + wi);
    float hCosWi = dot(h, wi);
    float hCosWi2 = hCosWi * hCosWi;
    float fi = schlickW(cosWi);
    float fo = schlickW(cosWo);
    v3 fd90 = mk3(0.5f + 2.0f * roughness * hCosWi2);
    v3 fd = mix3(mk3(1.0f), fd90, fi) * mix3(mk3(1.0f), fd90, fo);
    v3 baseDiffuse = baseColor * fd * kPiInv;
    v3 fss90 = mk3(roughness * hCosWi2);
    v3 fss = mix3(mk3(1.0f), fss90, fi) * mix3(mk3(1.0f), fss90, fo);
    v3 ss = baseColor * kPiInv * 1.25f * (fss * (1.0f / (cosWi + cosWo) - 0.5f) + mk3(0.5f));
    return mix3(baseDiffuse, ss, subsurface);
}
__device__ __forceinline__ v3 principledBRDF(v3 wo, v3 wi, v3 n, const BSDFParam& p) {  // :462-490
    float alpha = sq(p.roughness);
    float ccAlpha = mixf(0.1f, 0.001f, p.clearcoatGloss);
    float lum = luminance(p.baseColor);
    v3 tint = lum > 0.0f ? p.baseColor / lum : mk3(1.0f);
    v3 fm0 = mix3(0.08f * p.specular * mix3(mk3(1.0f), tint, p.specularTint), p.baseColor, p.metallic);
    float hCosWi = dot(normalize(wo + wi), wi);
    v3 res = mk3(0.0f);
    res = res + principledDiffuse(wo, wi, n, p.baseColor, p.subsurface, p.roughness) * (1.0f - p.metallic);
    res = res + principledMetal(wo, wi, n, fm0, alpha);
    res = res + principledClearcoat(wo, wi, n, p.baseColor, ccAlpha) * p.clearcoat * 0.25f;
    res = res + mix3(mk3(1.0f), tint, p.sheenTint) * schlickW(hCosWi) * p.sheen * (dot(n, wi) < 0.0f ? 0.0f : 1.0f);
    return res;
}
__device__ __forceinline__ float principledBRDFPdf(v3 wo, v3 wi, v3 n, const BSDFParam& p) {  // :492-514
    float pdf = 0.0f;
    float alpha = sq(p.roughness);
    float ccAlpha = mixf(0.1f, 0.001f, p.clearcoatGloss);
    float spec = 1.0f / (2.0f - p.metallic);
    float cosinePdf = absDot(n, wi) * kPiInv;
    pdf += cosinePdf * (1.0f - spec);
    pdf += principledMetalPdf(wo, wi, n, alpha) * spec;
    pdf += principledClearcoatPdf(wo, wi, n, ccAlpha) * 0.25f * p.clearcoat;
    return pdf / (1.0f + 0.25f * p.clearcoat);
}
// One out-of-line copy of the principled evaluation and pdf per translation
// unit, called from the sampling routine and the light-sample evaluation.
static __device__ __noinline__ v3 principledBRDFCall(v3 wo, v3 wi, v3 n, BSDFParam p) {
    return principledBRDF(wo, wi, n, p);
}
static __device__ __noinline__ float principledBRDFPdfCall(v3 wo, v3 wi, v3 n, BSDFParam p) {
    return principledBRDFPdf(wo, wi, n, p);
}
// `ur` is the lobe pick's draw from the rand() stream (material.glsl:539),
// taken by the caller.
__device__ __forceinline__ BSDFSample principledBRDFSample(v3 n, v3 wo, const BSDFParam& p, v3 u, float ur) {
    float alpha = sq(p.roughness);  // material.glsl:516-555
    float spec = 1.0f / (2.0f - p.metallic);
    float cdf0 = 1.0f - spec, cdf1 = 1.0f, cdf2 = 1.0f + p.clearcoat * 0.25f;
    float s = ur * cdf2;
    v3 wi;
    if (s <= cdf0) {
        float pdf;
        wi = sampleCosineWeighted(n, mk2(u.y, u.z), pdf);
    } else if (s <= cdf1) {
        v3 h = ggxSampleVisibleWm(n, wo, alpha, mk2(u.y, u.z));
        v3 w = reflect(-wo, h);
        wi = (dot(n, w) < 0.0f) ? mk3(0.0f) : w;
    } else {
        v3 h = gtr1SampleWm(n, wo, alpha, mk2(u.y, u.z));  // base alpha, as the reference
        v3 w = reflect(-wo, h);
        wi = (dot(n, w) < 0.0f) ? mk3(0.0f) : w;
    }
    BSDFSample r;
    r.wi = wi;
    r.bsdf = principledBRDFCall(wo, wi, n, p);
    r.pdf = principledBRDFPdfCall(wo, wi, n, p);
    r.flag = kDiffuse;
    return r;
}

// metalWorkflow, dielectric and thinDielectric (material.glsl:85-355).
__device__ __forceinline__ BSDFSample invalidSample() {
    BSDFSample r;
    r.wi = mk3(0.0f);
    r.pdf = 0.0f;
    r.bsdf = mk3(0.0f);
    r.flag = kInvalid;
    return r;
}
__device__ __forceinline__ BSDFSample makeSample(v3 wi, float pdf, v3 bsdf, uint32_t flag) {
    BSDFSample r;
    r.wi = wi;
    r.pdf = pdf;
    r.bsdf = bsdf;
    r.flag = flag;
    return r;
}
__device__ __forceinline__ bool approximateDelta(float roughness) { return roughness < 0.02f; }
__device__ __forceinline__ v3 schlickFR(float c, v3 F0, float roughness) {  // microfacet.glsl:14-17
    const float r1 = 1.0f - roughness;
    return F0 + (mk3(zmax(r1, F0.x), zmax(r1, F0.y), zmax(r1, F0.z)) - F0) * pow5(1.0f - c);
}
__device__ __forceinline__ v3 ggxSampleWm(v3 n, v3 wo, float alpha, v2 u) {  // microfacet.glsl:57-64
    v2 xi = toConcentricDisk(u);
    v3 h = mk3(xi.x, xi.y, zsqrt(zmax(0.0f, 1.0f - xi.x * xi.x - xi.y * xi.y)));
    h = normalize(h * mk3(alpha, alpha, 1.0f));
    return normalToWorld(n, h);
}
__device__ __forceinline__ v3 metalWorkflowBSDF(v3 wo, v3 wi, v3 n, BSDFParam p) {  // :85-113
    const float alpha = sq(p.roughness);
    const v3 h = normalize(wi + wo);
    if (!sameHemisphere(n, wo, wi)) return mk3(0.0f);
    const float cosWi = dot(n, wi), cosWo = dot(n, wo);
    const v3 f0 = mix3(mk3(0.04f), p.baseColor, p.metallic);
    const v3 f = schlickFR(satDot(h, wo), f0, p.roughness);
    const float d = ggx(dot(n, h), alpha);
    const float g = smithG(n, wo, wi, alpha);
    v3 kd = mk3(1.0f) - f;
    kd = kd * (1.0f - p.metallic);
    const float denom = 4.0f * cosWo * cosWi;
    if (denom < 1e-7f) return mk3(0.0f);
    return kd * p.baseColor * kPiInv + f * d * g / denom;
}
__device__ __forceinline__ float metalWorkflowPdf(v3 wo, v3 wi, v3 n, BSDFParam p) {  // :115-123
    const float alpha = sq(p.roughness);
    const v3 h = normalize(wo + wi);
    const float pdfDiff = satDot(n, wi) * kPiInv;
    const float pdfSpec = ggxPdfVisibleWm(n, h, wo, alpha) / (4.0f * absDot(h, wo));
    const float spec = 1.0f / (2.0f - p.metallic);
    return mixf(pdfDiff, pdfSpec, spec);
}
__device__ __forceinline__ BSDFSample metalWorkflowSample(v3 n, v3 wo, BSDFParam p, v3 u) {  // :125-145
    const float alpha = sq(p.roughness);
    const float spec = 1.0f / (2.0f - p.metallic);
    const uint32_t type = u.x > spec ? kDiffuse : kGlosRefl;
    v3 wi;
    if (type == kDiffuse) {
        float pdf;
        wi = sampleCosineWeighted(n, mk2(u.y, u.z), pdf);
    } else {
        wi = reflect(-wo, ggxSampleVisibleWm(n, wo, alpha, mk2(u.y, u.z)));
    }
    if (dot(n, wi) < 0.0f) return invalidSample();
    return makeSample(wi, metalWorkflowPdf(wo, wi, n, p), metalWorkflowBSDF(wo, wi, n, p), type);
}
__device__ __forceinline__ bool refractDir(v3& wt, v3 wi, v3 n, float eta) {  // :147-161
    const float cosTi = dot(n, wi);
    if (cosTi < 0.0f) eta = 1.0f / eta;
    const float sin2Ti = zmax(0.0f, 1.0f - cosTi * cosTi);
    const float sin2Tt = sin2Ti / (eta * eta);
    if (sin2Tt >= 1.0f) return false;
    float cosTt = zsqrt(1.0f - sin2Tt);
    if (cosTi < 0.0f) cosTt = -cosTt;
    wt = normalize(-wi / eta + n * (cosTi / eta - cosTt));
    return true;
}
__device__ __forceinline__ float fresnelDielectric(float cosTi, float eta) {  // :163-182
    cosTi = zmin(zmax(cosTi, -1.0f), 1.0f);
    if (cosTi < 0.0f) {
        eta = 1.0f / eta;
        cosTi = -cosTi;
    }
    const float sinTi = zsqrt(1.0f - cosTi * cosTi);
    const float sinTt = sinTi / eta;
    if (sinTt >= 1.0f) return 1.0f;
    const float cosTt = zsqrt(1.0f - sinTt * sinTt);
    const float rPa = (cosTi - eta * cosTt) / (cosTi + eta * cosTt);
    const float rPe = (eta * cosTi - cosTt) / (eta * cosTi + cosTt);
    return (rPa * rPa + rPe * rPe) * 0.5f;
}
__device__ __forceinline__ v3 dielectricBSDF(v3 wo, v3 wi, v3 n, BSDFParam p, uint32_t mode) {  // :184-217
    if (approximateDelta(p.roughness)) return mk3(0.0f);
    const v3 h = normalize(wo + wi);
    const float hCosWo = absDot(h, wo), hCosWi = absDot(h, wi);
    const float alpha = p.roughness * p.roughness;
    if (sameHemisphere(n, wo, wi)) {
        const float refl = fresnelDielectric(absDot(h, wi), p.ior);
        return (hCosWo * hCosWi < 1e-7f)
                   ? mk3(0.0f)
                   : p.baseColor * ggx(dot(n, h), alpha) * smithG(n, wo, wi, alpha) / (4.0f * hCosWo * hCosWi) * refl;
    }
    const float eta = dot(n, wi) > 0.0f ? p.ior : 1.0f / p.ior;
    const float sqrtDenom = dot(h, wo) + eta * dot(h, wi);
    float denom = sqrtDenom * sqrtDenom;
    denom *= absDot(n, wi) * absDot(n, wo);
    const float refl = fresnelDielectric(dot(h, wi), eta);
    const float factor = (mode == kRadiance) ? sq(1.0f / eta) : 1.0f;
    return (denom < 1e-7f) ? mk3(0.0f)
                           : p.baseColor * fabsf(ggx(dot(n, h), alpha) * smithG(n, wo, wi, alpha) * hCosWo * hCosWi) /
                                 denom * (1.0f - refl) * factor;
}
__device__ __forceinline__ float dielectricPdf(v3 wo, v3 wi, v3 n, BSDFParam p) {  // :219-243
    if (approximateDelta(p.roughness)) return 0.0f;
    const float alpha = p.roughness * p.roughness;
    if (sameHemisphere(n, wo, wi)) {
        const v3 h = normalize(wo + wi);
        if (dot(wo, h) < 0.0f) return 0.0f;
        const float refl = fresnelDielectric(absDot(h, wi), p.ior);
        return ggx(dot(n, h), alpha) / (4.0f * absDot(h, wo)) * refl;
    }
    const float eta = dot(n, wo) > 0.0f ? p.ior : 1.0f / p.ior;
    const v3 h = normalize(wo + wi * eta);
    if (sameHemisphere(h, wo, wi)) return 0.0f;
    const float trans = 1.0f - fresnelDielectric(absDot(h, wo), eta);
    const float dHdWi = absDot(h, wi) / sq(dot(h, wo) + eta * dot(h, wi));
    return ggx(dot(n, h), alpha) * dHdWi * trans;
}
__device__ __forceinline__ BSDFSample dielectricSample(v3 n, v3 wo, BSDFParam p, uint32_t mode, v3 u) {  // :245-325
    float ior = p.ior;
    if (approximateDelta(p.roughness)) {
        const float refl = fresnelDielectric(dot(n, wo), ior);
        if (u.x < refl) return makeSample(reflect(-wo, n), 1.0f, p.baseColor, kSpecRefl);
        v3 wi;
        if (!refractDir(wi, wo, n, ior)) return invalidSample();
        if (dot(n, wo) < 0.0f) ior = 1.0f / ior;
        const float factor = (mode == kRadiance) ? sq(1.0f / ior) : 1.0f;
        return makeSample(wi, 1.0f, p.baseColor * factor, kSpecTrans);
    }
    const float alpha = p.roughness * p.roughness;
    v3 h = ggxSampleWm(n, wo, alpha, mk2(u.y, u.z));
    if (dot(n, h) < 0.0f) h = -h;
    const float refl = fresnelDielectric(dot(h, wo), ior);
    if (u.x < refl) {
        const v3 wi = -reflect(wo, h);
        if (!sameHemisphere(n, wo, wi)) return invalidSample();
        float pdf = ggx(dot(n, h), alpha) / (4.0f * absDot(h, wo));
        const float hCosWo = absDot(h, wo), hCosWi = absDot(h, wi);
        const v3 r = (hCosWo * hCosWi < 1e-7f)
                         ? mk3(0.0f)
                         : p.baseColor * ggx(dot(n, h), alpha) * smithG(n, wo, wi, alpha) / (4.0f * hCosWo * hCosWi);
        if (zisnan(pdf)) pdf = 0.0f;
        return makeSample(wi, pdf, r, kGlosRefl);
    }
    v3 wi;
    if (!refractDir(wi, wo, h, ior)) return invalidSample();
    if (sameHemisphere(n, wo, wi)) return invalidSample();
    if (absDot(n, wi) < 1e-10f) return invalidSample();
    const float hCosWo = absDot(h, wo), hCosWi = absDot(h, wi);
    if (dot(h, wo) < 0.0f) ior = 1.0f / ior;
    const float sqrtDenom = dot(h, wo) + ior * dot(h, wi);
    float denom = sqrtDenom * sqrtDenom;
    const float dHdWi = hCosWi / denom;
    const float factor = (mode == kRadiance) ? sq(1.0f / ior) : 1.0f;
    denom *= absDot(n, wi) * absDot(n, wo);
    const v3 t = (denom < 1e-7f) ? mk3(0.0f)
                                 : p.baseColor *
                                       fabsf(ggx(dot(n, h), alpha) * smithG(n, wo, wi, alpha) * hCosWo * hCosWi) /
                                       denom;
    float pdf = ggx(dot(n, h), alpha) * dHdWi;
    if (zisnan(pdf)) pdf = 0.0f;
    return makeSample(wi, pdf, t * factor, kGlosTrans);
}
__device__ __forceinline__ BSDFSample thinDielectricSample(v3 n, v3 wo, BSDFParam p, v3 u) {  // :327-340
    if (dot(n, wo) < 0.0f) n = -n;
    float refl = fresnelDielectric(dot(n, wo), p.ior);
    float trans = 1.0f - refl;
    if (refl < 1.0f) {
        refl += trans * trans * refl / (1.0f - refl * refl);
        trans = 1.0f - refl;
    }
    return (u.x < refl) ? makeSample(reflect(-wo, n), 1.0f, p.baseColor, kSpecRefl)
                        : makeSample(-wo, 1.0f, p.baseColor, kSpecTrans);
}

// One out-of-line entry per query for every material type but Lambertian
// (principled, metal workflow, dielectric, thin dielectric): each integrator
// call site holds one call, which keeps the kernels' instruction footprint
// small.
static __device__ __noinline__ v3 bsdfCall(uint32_t type, v3 wo, v3 wi, v3 n, BSDFParam p, uint32_t mode) {
    if (type == kPrincipled) return principledBRDF(wo, wi, n, p);
    if (type == kMetalWorkflow) return metalWorkflowBSDF(wo, wi, n, p);
    if (type == kDielectric) return dielectricBSDF(wo, wi, n, p, mode);
    return mk3(0.0f);  // thin dielectric: delta lobes only
}
static __device__ __noinline__ float pdfCall(uint32_t type, v3 wo, v3 wi, v3 n, BSDFParam p) {
    if (type == kPrincipled) return principledBRDFPdf(wo, wi, n, p);
    if (type == kMetalWorkflow) return metalWorkflowPdf(wo, wi, n, p);
    if (type == kDielectric) return dielectricPdf(wo, wi, n, p);
    return 0.0f;
}
static __device__ __noinline__ BSDFSample sampleCall(uint32_t type, v3 n, v3 wo, BSDFParam p, uint32_t mode, v3 u,
                                                     float ur) {
    if (type == kPrincipled) return principledBRDFSample(n, wo, p, u, ur);
    if (type == kMetalWorkflow) return metalWorkflowSample(n, wo, p, u);
    if (type == kDielectric) return dielectricSample(n, wo, p, mode, u);
    return thinDielectricSample(n, wo, p, u);
}

// ----------------------------------------------------- material_loader.glsl
__device__ __forceinline__ uint32_t loadMaterialType(const DeviceScene& sc, int matId) {
    return (uint32_t)__float_as_int(__ldg(&sc.materials[4 * matId + 3]).y);
}
// FULL = false: the scene holds Lambertian and principled materials only (the
// integrator kernels are instantiated for both cases and the host picks the
// lean one when it can; the dispatch for the other three types costs the
// lean scenes 6-16% otherwise).
template <bool FULL>
__device__ __forceinline__ BSDFParam loadMaterialParams(const DeviceScene& sc, uint32_t type, int matId) {
    const float4 m0 = __ldg(&sc.materials[4 * matId + 0]);
    BSDFParam p;
    p.baseColor = mk3(m0.x, m0.y, m0.z);
    p.subsurface = p.metallic = p.roughness = p.specular = p.specularTint = 0.0f;
    p.sheen = p.sheenTint = p.clearcoat = p.clearcoatGloss = 0.0f;
    if (!FULL) {
        // (the principled branch below)
    } else if (type == kMetalWorkflow) {  // loadMetalWorkflow (material_loader.glsl:26-35)
        p.roughness = mixf(0.0134f, 1.0f, m0.w);
        p.metallic = __ldg(&sc.materials[4 * matId + 1]).y;
    } else if (type == kDielectric) {  // loadDielectric (:60-69): roughness not remapped
        p.roughness = m0.w;
        p.ior = __ldg(&sc.materials[4 * matId + 3]).x;
    } else if (type == kThinDielectric) {  // loadThinDielectric (:71-79)
        p.ior = __ldg(&sc.materials[4 * matId + 3]).x;
    }
    if (type == kPrincipled) {  // loadPrincipledBRDF (material_loader.glsl:37-58)
        const float4 m1 = __ldg(&sc.materials[4 * matId + 1]);
        const float4 m2 = __ldg(&sc.materials[4 * matId + 2]);
        p.roughness = mixf(0.0134f, 1.0f, m0.w);
        p.subsurface = m1.x;
        p.metallic = m1.y;
        p.specular = m1.z;
        p.specularTint = m1.w;
        p.sheen = m2.x;
        p.sheenTint = m2.y;
        p.clearcoat = m2.z;
        p.clearcoatGloss = m2.w;
    }
    return p;
}
// materialBSDF / materialPdf / materialSample (material_loader.glsl:97-170);
// `mode` is kRadiance for camera paths and kImportance for light paths.
template <bool FULL>
__device__ __forceinline__ v3 materialBSDF(uint32_t type, const BSDFParam& p, v3 wo, v3 wi, v3 n,
                                           uint32_t mode = kRadiance) {
    if (FULL) {
        if (type != kLambertian) return bsdfCall(type, wo, wi, n, p, mode);
    } else if (type == kPrincipled) {
        return principledBRDFCall(wo, wi, n, p);
    }
    return p.baseColor * kPiInv;
}
template <bool FULL>
__device__ __forceinline__ float materialPdf(uint32_t type, const BSDFParam& p, v3 wo, v3 wi, v3 n) {
    if (FULL) {
        if (type != kLambertian) return pdfCall(type, wo, wi, n, p);
    } else if (type == kPrincipled) {
        return principledBRDFPdfCall(wo, wi, n, p);
    }
    return satDot(wi, n) * kPiInv;
}
template <bool FULL>
__device__ __forceinline__ BSDFSample materialSample(uint32_t type, const BSDFParam& p, v3 n, v3 wo, v3 u,
                                                     Sampler& g, uint32_t mode = kRadiance) {
    if (FULL) {
        if (type != kLambertian) {
            // only the principled lobe pick draws from the rand() stream
            const float ur = (type == kPrincipled) ? rand01(g) : 0.0f;
            return sampleCall(type, n, wo, p, mode, u, ur);
        }
    } else if (type == kPrincipled) {
        return principledBRDFSample(n, wo, p, u, rand01(g));
    }
    BSDFSample r;  // lambertianSample (material.glsl:78-83)
    float pdf;
    r.wi = sampleCosineWeighted(n, mk2(u.y, u.z), pdf);
    r.pdf = satDot(n, r.wi) * kPiInv;
    r.bsdf = p.baseColor * kPiInv;
    r.flag = kDiffuse;
    return r;
}

// ------------------------------------------------------- intersection.glsl
struct TriShade {
    v3 a, b, c, na, nb, nc;
    int32_t matTex;
};
__device__ __forceinline__ TriShade loadTri(const DeviceScene& sc, int id) {
    const float4* p = sc.shade + 5 * (size_t)id;
    float4 s0 = __ldg(p), s1 = __ldg(p + 1), s2 = __ldg(p + 2), s3 = __ldg(p + 3), s4 = __ldg(p + 4);
    TriShade t;
    t.a = mk3(s0.x, s0.y, s0.z);
    t.b = mk3(s0.w, s1.x, s1.y);
    t.c = mk3(s1.z, s1.w, s2.x);
    t.na = mk3(s2.y, s2.z, s2.w);
    t.nb = mk3(s3.x, s3.y, s3.z);
    t.nc = mk3(s3.w, s4.x, s4.y);
    t.matTex = __float_as_int(s4.z);
    return t;
}
struct Surface {
    v3 ns, ng;
    float la, lb;  // barycentric weights of corners a and b (lc = 1 - la - lb)
};
__device__ __forceinline__ Surface surfaceInfo(const TriShade& t, v3 p) {  // intersection.glsl:188-224
    v3 pa = t.a - p, pb = t.b - p, pc = t.c - p;
    float areaInv = 1.0f / length(cross(t.b - t.a, t.c - t.a));
    float la = length(cross(pb, pc)) * areaInv;
    float lb = length(cross(pc, pa)) * areaInv;
    float lc = 1.0f - la - lb;
    Surface s;
    s.la = la;
    s.lb = lb;
    s.ns = normalize(t.na * la + t.nb * lb + t.nc * lc);
    s.ng = normalize(cross(pa, pb));
    if (dot(s.ns, s.ng) < 0.0f) s.ng = -s.ng;
    return s;
}
// texture2DArray(uTextures, vec3(fract(uv) * uvScale, texId)).rgb
// (material_loader.glsl:14-15) on the 8-bit sRGB texture array of
// Texture.cpp:146-161.  A compute shader samples level 0, i.e. with the
// magnification filter (GL_LINEAR), wrapping GL_REPEAT over the whole layer;
// texels are decoded sRGB -> linear before filtering.  The bilinear weights
// are float32 (hardware filtering rounds them to fixed point).
__device__ __forceinline__ v3 albedoTexture(const DeviceScene& sc, int texId, v2 uv) {
    const float2 scale = __ldg(&sc.texScale[texId]);
    const float s = (uv.x - floorf(uv.x)) * scale.x;
    const float t = (uv.y - floorf(uv.y)) * scale.y;
    const int W = sc.texW, H = sc.texH;
    const float u = s * (float)W - 0.5f, v = t * (float)H - 0.5f;
    const float fu = floorf(u), fv = floorf(v);
    const float a = u - fu, b = v - fv;
    int i0 = (int)fu, j0 = (int)fv;
    if (i0 < 0) i0 += W;
    if (j0 < 0) j0 += H;
    const int i1 = i0 + 1 == W ? 0 : i0 + 1, j1 = j0 + 1 == H ? 0 : j0 + 1;
    const uint32_t* layer = sc.texels + (size_t)texId * W * H;
    const uint32_t t00 = __ldg(&layer[(size_t)j0 * W + i0]), t10 = __ldg(&layer[(size_t)j0 * W + i1]);
    const uint32_t t01 = __ldg(&layer[(size_t)j1 * W + i0]), t11 = __ldg(&layer[(size_t)j1 * W + i1]);
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    float c[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int sh = 8 * k;
        c[k] = w00 * __ldg(&sc.srgb[(t00 >> sh) & 255u]) + w10 * __ldg(&sc.srgb[(t10 >> sh) & 255u]) +
               w01 * __ldg(&sc.srgb[(t01 >> sh) & 255u]) + w11 * __ldg(&sc.srgb[(t11 >> sh) & 255u]);
    }
    return mk3(c[0], c[1], c[2]);
}
// ret.uv = ta * la + tb * lb + tc * lc (intersection.glsl:218)
__device__ __forceinline__ v2 surfaceUV(const DeviceScene& sc, int triId, const Surface& surf) {
    const float2 ta = __ldg(&sc.uv[3 * (size_t)triId]), tb = __ldg(&sc.uv[3 * (size_t)triId + 1]);
    const float2 tc = __ldg(&sc.uv[3 * (size_t)triId + 2]);
    const float lc = 1.0f - surf.la - surf.lb;
    return mk2(ta.x * surf.la + tb.x * surf.lb + tc.x * lc, ta.y * surf.la + tb.y * surf.lb + tc.y * lc);
}
// loadMaterial (material_loader.glsl:81-95): the record's parameters, with
// the base colour from the albedo texture when the triangle has one
// (matTex >> 16 != -1; only scenes that run the full instantiation have
// textured triangles).
template <bool FULL>
__device__ __forceinline__ BSDFParam loadMaterial(const DeviceScene& sc, uint32_t type, int32_t matTex, int triId,
                                                  const Surface& surf) {
    BSDFParam p = loadMaterialParams<FULL>(sc, type, matTex & 0x0000ffff);
    if (FULL) {
        const int texId = matTex >> 16;
        if (texId != -1) p.baseColor = albedoTexture(sc, texId, surfaceUV(sc, triId, surf));
    }
    return p;
}
__device__ __forceinline__ v3 geomNormal(const DeviceScene& sc, int triId, v3 p) {
    return surfaceInfo(loadTri(sc, triId), p).ng;
}

struct Ray {
    v3 ori, dir;
};
__device__ __forceinline__ Ray rayOffseted(v3 o, v3 d) { return Ray{o + d * 1e-4f, d}; }
__device__ __forceinline__ v3 rayPoint(const Ray& r, float t) { return r.ori + r.dir * t; }

// The integrators call traversal from several places (camera ray, bounce,
// light and environment shadow rays); each call goes to one out-of-line copy
// of the closest-hit and any-hit loops (five ray-mode variants each), which
// keeps the integrator kernels' instruction footprint small.  A translation
// unit that defines ZGL_INLINE_TRACE before including this header inlines
// them instead (the batched renderer, whose one call site per kind is hot).
struct ClosestHit {
    int id;
    float dist;
};
#ifdef ZGL_INLINE_TRACE
#define ZGL_TRACE_CALL __device__ __forceinline__
#else
#define ZGL_TRACE_CALL __device__ __noinline__
#endif
// A ray with a near-zero direction component that outruns kLongRayBudget
// table entries is finished by the lanes that reach the end of their own
// traversal together (traverse.cuh: finish_long_rays_group), as the trace
// kernels do with whole warps.  The walk is a separate out-of-line call,
// taken only when some lane of the group has such a ray, so that the
// traversal loop keeps its registers.
struct LongRayState {
    float dist;
    int k, closest;
};
template <bool ANY>
static __device__ __noinline__ LongRayState finishLongRays(unsigned group, DeviceAccel a, float ox, float oy,
                                                             float oz, float dx, float dy, float dz,
                                                             LongRayState s, bool done) {
    const TraceRay tr = make_trace_ray(make_float3(ox, oy, oz), make_float3(dx, dy, dz));
    finish_long_rays_group<ANY>(group, a, tr, s.dist, s.k, s.closest, done);
    return s;
}
// Closest-hit / any-hit of one ray.  Rays of modes 0-3 run the plain loops;
// a MODE 4 ray (near-zero direction component) runs a loop that stops after
// kLongRayBudget entries, and only that branch keeps what the walk needs, so
// the common loops carry no extra live values.
template <bool ANY>
__device__ __forceinline__ LongRayState traceOne(const DeviceAccel& a, const TraceRay& tr, float dist) {
    LongRayState s{dist, 0, -1};
    bool done = true;
    DeviceAccel wa{nullptr, nullptr, 0};
    float3 wo = make_float3(0.0f, 0.0f, 0.0f), wd = make_float3(0.0f, 0.0f, 1.0f);
    if (tr.mode != 4) {
        int v = 0, t = 0;
        switch (tr.mode) {
            case 3: s.closest = traverse_m<ANY, false, 3>(a, tr, s.dist, v, t); break;
            case 0: s.closest = traverse_m<ANY, false, 0>(a, tr, s.dist, v, t); break;
            case 1: s.closest = traverse_m<ANY, false, 1>(a, tr, s.dist, v, t); break;
            default: s.closest = traverse_m<ANY, false, 2>(a, tr, s.dist, v, t); break;
        }
        if (ANY) s.closest = s.closest ? 0 : -1;  // traverse_m returns the any-hit flag
    } else {
        done = traverse_lane<ANY, 4, false, 0>(a, tr, s.dist, s.k, s.closest, kLongRayBudget);
        wa = a;
        wo = tr.o;
        wd = tr.d;
    }
    const unsigned group = __activemask();
    if (__any_sync(group, !done)) s = finishLongRays<ANY>(group, wa, wo.x, wo.y, wo.z, wd.x, wd.y, wd.z, s, done);
    return s;
}
static ZGL_TRACE_CALL ClosestHit traceClosestCall(DeviceAccel a, float ox, float oy, float oz, float dx, float dy,
                                                    float dz) {
    TraceRay tr = make_trace_ray(make_float3(ox, oy, oz), make_float3(dx, dy, dz));
    float dist = 1e8f;
    int v = 0, t = 0;
    int id = traverse<false, false>(a, tr, dist, v, t);
    return ClosestHit{id, dist};
}
static ZGL_TRACE_CALL bool traceAnyCall(DeviceAccel a, float ox, float oy, float oz, float dx, float dy, float dz,
                                          float dist) {
    TraceRay tr = make_trace_ray(make_float3(ox, oy, oz), make_float3(dx, dy, dz));
    int v = 0, t = 0;
    return traverse<true, false>(a, tr, dist, v, t) != 0;
}

// Long rays cost a tail only in large trees: with fewer entries a face's
// table stays in L2 and even a ray that visits all of them ends quickly.
// Translation units that define ZGL_LONG_RAYS (render_long.cu: the
// integrator kernels for trees of at least kLongRayMinEntries entries) trace
// through the calls below; every other unit keeps the plain calls above, so
// the kernels that never meet a long ray keep their register budget and code
// as they were (sharing one function between both paths made the
// small-scene, batch and adjoint kernels 2-25% slower).
constexpr int kLongRayMinEntries = 1 << 21;
static __device__ __noinline__ ClosestHit traceClosestLong(DeviceAccel a, float ox, float oy, float oz, float dx,
                                                           float dy, float dz) {
    const LongRayState s = traceOne<false>(a, make_trace_ray(make_float3(ox, oy, oz), make_float3(dx, dy, dz)), 1e8f);
    return ClosestHit{s.closest, s.dist};
}
static __device__ __noinline__ bool traceAnyLong(DeviceAccel a, float ox, float oy, float oz, float dx, float dy,
                                                 float dz, float dist) {
    return traceOne<true>(a, make_trace_ray(make_float3(ox, oy, oz), make_float3(dx, dy, dz)), dist).closest >= 0;
}
#if defined(ZGL_LONG_RAYS) && ZGL_LONG_RAYS
__device__ __forceinline__ int bvhHit(const DeviceScene& sc, const Ray& r, float& dist) {
    ClosestHit h = traceClosestLong(sc.accel, r.ori.x, r.ori.y, r.ori.z, r.dir.x, r.dir.y, r.dir.z);
    dist = h.dist;
    return h.id;
}
__device__ __forceinline__ bool bvhTest(const DeviceScene& sc, const Ray& r, float dist) {
    return traceAnyLong(sc.accel, r.ori.x, r.ori.y, r.ori.z, r.dir.x, r.dir.y, r.dir.z, dist);
}
#else
__device__ __forceinline__ int bvhHit(const DeviceScene& sc, const Ray& r, float& dist) {
    ClosestHit h = traceClosestCall(sc.accel, r.ori.x, r.ori.y, r.ori.z, r.dir.x, r.dir.y, r.dir.z);
    dist = h.dist;
    return h.id;
}
__device__ __forceinline__ bool bvhTest(const DeviceScene& sc, const Ray& r, float dist) {
    return traceAnyCall(sc.accel, r.ori.x, r.ori.y, r.ori.z, r.dir.x, r.dir.y, r.dir.z, dist);
}
#endif
__device__ __forceinline__ bool visible(const DeviceScene& sc, v3 x, v3 y) {  // intersection.glsl:429-433
    float dist = distance(x, y) - 2e-5f;
    v3 wi = normalize(y - x);
    return !bvhTest(sc, Ray{x + wi * 1e-5f, wi}, dist);
}

// ----------------------------------------------------------------- light.glsl
struct LiSample {
    v3 wi, coef;
    float pdf;
};
__device__ __forceinline__ LiSample invalidLi() { return LiSample{mk3(0.0f), mk3(0.0f), 0.0f}; }

__device__ __forceinline__ int lightSampleOne(const DeviceScene& sc, v2 u) {  // light.glsl:68-72
    int cx = min(zf2i((float)sc.nLight * u.x), sc.nLight - 1);  // u.x == 1.0 would read past the table
    return (u.y < __ldg(&sc.lightProb[cx])) ? cx : __ldg(&sc.lightAlias[cx]);
}
__device__ __forceinline__ v3 lightPowerOf(const DeviceScene& sc, int id, float& area) {
    float4 p = __ldg(&sc.lightPower[id]);
    area = p.w;
    return mk3(p.x, p.y, p.z);
}
__device__ __forceinline__ float lightPdfSampleOne(const DeviceScene& sc, int id) {
    float a;
    return luminance(lightPowerOf(sc, id, a)) / sc.lightSum;
}
__device__ __forceinline__ v3 lightLe(const DeviceScene& sc, int id, v3 x, v3 wo) {  // light.glsl:79-86
    int triId = id + sc.objPrimCount;
    v3 ng = geomNormal(sc, triId, x);
    if (dot(wo, ng) <= 0.0f) return mk3(0.0f);
    float area;
    v3 pw = lightPowerOf(sc, id, area);
    return pw / area * 0.5f * kPiInv;
}
__device__ __forceinline__ float lightPdfLi(const DeviceScene& sc, int id, v3 x, v3 y) {  // light.glsl:88-98
    int triId = id + sc.objPrimCount;
    v3 norm = geomNormal(sc, triId, y);
    v3 yx = normalize(x - y);
    float cosTheta = absDot(norm, yx);
    if (cosTheta < 1e-8f) return -1.0f;
    float area;
    lightPowerOf(sc, id, area);
    return distSquare(x, y) / (area * cosTheta);
}
// The light sample's occlusion test.  TraceVis traces the shadow ray; other
// visibility sources (the adjoint's replay) return a result recorded when the
// same sample was first traced.
struct TraceVis {
    __device__ __forceinline__ bool operator()(const DeviceScene& sc, const Ray& r, float dist) const {
        return bvhTest(sc, r, dist);
    }
};

template <class Vis>
__device__ __forceinline__ LiSample lightSampleLiV(const DeviceScene& sc, int id, v3 x, v2 u,
                                                   const Vis& vis) {  // light.glsl:122-155
    int triId = id + sc.objPrimCount;
    TriShade t = loadTri(sc, triId);
    v3 y = sampleTriangleUniform(t.a, t.b, t.c, u);
    v3 wi = normalize(y - x);
    v3 norm = surfaceInfo(t, y).ng;
    float cosTheta = dot(norm, -wi);
    if (cosTheta < 1e-6f) return invalidLi();
    Ray lightRay = rayOffseted(x, wi);
    float dist = distance(x, y);
    float area;
    v3 pw = lightPowerOf(sc, id, area);
    float pdf = dist * dist / (area * cosTheta);
    float testDist = dist - 1e-4f - 1e-6f;
    if (vis(sc, lightRay, testDist) || pdf < 1e-8f) return invalidLi();
    v3 weight = lightLe(sc, id, y, -wi);
    float pdfSample = luminance(pw) / sc.lightSum;
    pdf *= pdfSample;
    return LiSample{wi, weight / pdf, pdf};
}
__device__ __forceinline__ LiSample lightSampleLi(const DeviceScene& sc, int id, v3 x, v2 u) {
    return lightSampleLiV(sc, id, x, u, TraceVis{});
}

__device__ __forceinline__ v3 envTexel(const DeviceScene& sc, int x, int y) {
    int W = sc.envW, H = sc.envH;
    x %= W;
    if (x < 0) x += W;
    y %= H;
    if (y < 0) y += H;
    float4 t = __ldg(&sc.envTexels[(size_t)y * W + x]);
    return mk3(t.x, t.y, t.z);
}
__device__ __forceinline__ v3 envTexture(const DeviceScene& sc, v2 st) {  // bilinear, repeat, texel centres
    float u = st.x * (float)sc.envW - 0.5f;
    float v = st.y * (float)sc.envH - 0.5f;
    float fu = floorf(u), fv = floorf(v);
    float au = u - fu, av = v - fv;
    int x0 = zf2i(fu), y0 = zf2i(fv);
    v3 t00 = envTexel(sc, x0, y0), t10 = envTexel(sc, x0 + 1, y0);
    v3 t01 = envTexel(sc, x0, y0 + 1), t11 = envTexel(sc, x0 + 1, y0 + 1);
    return mix3(mix3(t00, t10, au), mix3(t01, t11, au), av);
}
__device__ __forceinline__ v3 envLe(const DeviceScene& sc, v3 wi) {  // light.glsl:163-167
    if (sc.envTexels == nullptr) return mk3(0.0f);
    wi = rotateZ(wi, -sc.envRotation);
    return envTexture(sc, sphereToPlane(wi));
}
__device__ __forceinline__ float envGetPortion(const DeviceScene& sc, v3 wi) { return luminance(envLe(sc, wi)) / sc.envSum; }
__device__ __forceinline__ float envPdfLi(const DeviceScene& sc, v3 wi) {  // light.glsl:174-179
    if (sc.envSum == 0.0f) return 0.0f;
    return envGetPortion(sc, wi) * (float)sc.envW * (float)sc.envH * 0.5f * sq(kPiInv);
}
template <class Vis>
__device__ __forceinline__ LiSample envSampleLiV(const DeviceScene& sc, v3 x, float ux, float uy, float uz, float uw,
                                                 const Vis& vis) {
    if (sc.envTexels == nullptr) return invalidLi();  // light.glsl:181-219
    int w = sc.envW, h = sc.envH;
    int rx = min(zf2i((float)h * ux), h - 1);
    int rIdx = rx * (w + 1) + w;
    int row = (uy < __ldg(&sc.envProb[rIdx])) ? rx : __ldg(&sc.envAlias[rIdx]);
    int cx = min(zf2i((float)w * uz), w - 1);
    int cIdx = row * (w + 1) + cx;
    int col = (uw < __ldg(&sc.envProb[cIdx])) ? cx : __ldg(&sc.envAlias[cIdx]);
    v2 uv = mk2((float)col + 0.5f, (float)row + 0.5f) / mk2((float)w, (float)h);
    v3 wi = planeToSphere(uv);
    wi = rotateZ(wi, sc.envRotation);
    float pdf = envGetPortion(sc, wi) * (float)w * (float)h * 0.5f * sq(kPiInv);
    Ray ray = rayOffseted(x, wi);
    if (vis(sc, ray, 1e8f) || pdf == 0.0f) return invalidLi();
    return LiSample{wi, envLe(sc, wi) / pdf, pdf};
}
__device__ __forceinline__ LiSample envSampleLi(const DeviceScene& sc, v3 x, float ux, float uy, float uz, float uw) {
    return envSampleLiV(sc, x, ux, uy, uz, uw, TraceVis{});
}
__device__ __forceinline__ float pdfSampleLightSel(const DeviceScene& sc, int uniform, float portion) {
    return uniform ? portion : sc.lightSum / (sc.lightSum + sc.envSum);
}

// ---------------------------------------------------------------- camera.glsl
__device__ __forceinline__ Ray thinLensCameraSampleRay(const DeviceScene& sc, v2 uv, float u0, float u1, float u2,
                                                       float u3) {  // camera.glsl:62-77
    v2 texel = mk2(1.0f / (float)sc.filmW, 1.0f / (float)sc.filmH);
    v2 biased = uv + texel * mk2(u0, u1);
    v2 ndc = mk2(biased.x * 2.0f - 1.0f, biased.y * 2.0f - 1.0f);
    v2 lens = toConcentricDisk(mk2(u2, u3)) * sc.lensRadius;
    v2 fp = ndc * mk2(sc.camAsp, 1.0f) * sc.focalDist * sc.tanFOV;
    v3 dir = mk3(fp.x, fp.y, sc.focalDist) - mk3(lens.x, lens.y, 0.0f);
    v3 R = f3(sc.camR), U = f3(sc.camU), F = f3(sc.camF);
    dir = normalize(R * dir.x + U * dir.y + F * dir.z);
    return Ray{f3(sc.camPos) + R * lens.x + U * lens.y, dir};
}

// ------------------------------------------------ camera importance (camera.glsl)
__device__ __forceinline__ bool inFilmBound(v2 uv) { return uv.x >= 0.0f && uv.x <= 1.0f && uv.y >= 0.0f && uv.y <= 1.0f; }
__device__ __forceinline__ bool thinLensCameraDelta(const DeviceScene& sc) { return sc.lensRadius <= 1e-6f; }
__device__ __forceinline__ v2 thinLensCameraRasterPos(const DeviceScene& sc, const Ray& ray) {  // camera.glsl:79-91
    float cosTheta = dot(ray.dir, f3(sc.camF));
    float dFocus = sc.focalDist / cosTheta;
    const float* mi = sc.camMatInv;
    m3 inv{mk3(mi[0], mi[1], mi[2]), mk3(mi[3], mi[4], mi[5]), mk3(mi[6], mi[7], mi[8])};
    v3 pFocus = mul(inv, rayPoint(ray, dFocus) - f3(sc.camPos));
    float aspect = (float)sc.filmW / (float)sc.filmH;
    v3 div = mk3(aspect * sc.tanFOV * sc.focalDist, 1.0f * sc.tanFOV * sc.focalDist, 1.0f * sc.focalDist);
    pFocus = pFocus / div;
    return mk2((pFocus.x + 1.0f) * 0.5f, (pFocus.y + 1.0f) * 0.5f);
}
__device__ __forceinline__ v3 thinLensCameraIe(const DeviceScene& sc, const Ray& ray) {  // camera.glsl:93-107
    float cosTheta = dot(ray.dir, f3(sc.camF));
    if (cosTheta < 1e-6f) return mk3(0.0f);
    v2 pRaster = thinLensCameraRasterPos(sc, ray);
    if (!inFilmBound(pRaster)) return mk3(0.0f);
    float tanFOVInv = 1.0f / sc.tanFOV;
    float cos2Theta = cosTheta * cosTheta;
    float lensArea = thinLensCameraDelta(sc) ? 1.0f : kPi * sc.lensRadius * sc.lensRadius;
    return mk3(0.25f) * sq(tanFOVInv / cos2Theta) / (lensArea * sc.camAsp);
}
struct CameraIiSample {
    v3 wi, Ii;
    float dist;
    v2 uv;
    float pdf;
};
__device__ __forceinline__ CameraIiSample thinLensCameraSampleIi(const DeviceScene& sc, v3 ref, v2 u) {  // :109-127
    v2 l = toConcentricDisk(u) * sc.lensRadius;
    v3 y = f3(sc.camPos) + f3(sc.camR) * l.x + f3(sc.camU) * l.y + f3(sc.camF) * 0.0f;
    float dist = distance(ref, y);
    v3 wi = normalize(y - ref);
    float cosTheta = satDot(f3(sc.camF), -wi);
    CameraIiSample r;
    if (cosTheta < 1e-6f) {
        r.wi = r.Ii = mk3(0.0f);
        r.dist = 0.0f;
        r.uv = mk2(0.0f, 0.0f);
        r.pdf = 0.0f;
        return r;
    }
    Ray ray{y, -wi};
    r.wi = wi;
    r.Ii = thinLensCameraIe(sc, ray);
    r.uv = thinLensCameraRasterPos(sc, ray);
    float lensArea = thinLensCameraDelta(sc) ? 1.0f : kPi * sc.lensRadius * sc.lensRadius;
    r.dist = dist;
    r.pdf = dist * dist / (cosTheta * lensArea);
    return r;
}
struct PdfPair {
    float pdfPos, pdfDir;
};
__device__ __forceinline__ PdfPair thinLensCameraPdfIe(const DeviceScene& sc, const Ray& ray) {  // :129-141
    float cosTheta = dot(f3(sc.camF), ray.dir);
    if (cosTheta < 1e-6f) return PdfPair{0.0f, 0.0f};
    v2 pRaster = thinLensCameraRasterPos(sc, ray);
    if (!inFilmBound(pRaster)) return PdfPair{0.0f, 0.0f};
    float pdfPos = thinLensCameraDelta(sc) ? 1.0f : 1.0f / (kPi * sc.lensRadius * sc.lensRadius);
    float pdfDir = 1.0f / (cosTheta * cosTheta * cosTheta);
    return PdfPair{pdfPos, pdfDir};
}

// ------------------------------------------------------- light emission (light.glsl)
struct LightLeSample {
    Ray ray;
    v3 Le;
    float pdfPos, pdfDir;
};
__device__ __forceinline__ LightLeSample lightSampleOneLe(const DeviceScene& sc, int id, float u0, float u1, float u2,
                                                          float u3) {  // light.glsl:111-120
    int triId = id + sc.objPrimCount;
    TriShade t = loadTri(sc, triId);
    v3 ori = sampleTriangleUniform(t.a, t.b, t.c, mk2(u0, u1));
    v3 norm = surfaceInfo(t, ori).ng;
    float pdfDir;
    v3 dir = sampleCosineWeighted(norm, mk2(u2, u3), pdfDir);
    float area;
    lightPowerOf(sc, id, area);
    LightLeSample r;
    r.ray = rayOffseted(ori, dir);
    r.Le = lightLe(sc, id, ori, dir);
    r.pdfPos = 1.0f / area;
    r.pdfDir = pdfDir;
    return r;
}
__device__ __forceinline__ PdfPair lightPdfLe(const DeviceScene& sc, int id, const Ray& ray) {  // light.glsl:100-109
    int triId = id + sc.objPrimCount;
    v3 norm = geomNormal(sc, triId, ray.ori);
    float area;
    lightPowerOf(sc, id, area);
    PdfPair r;
    r.pdfPos = 1.0f / area;
    r.pdfDir = (dot(norm, ray.dir) <= 0.0f) ? 0.0f : 0.5f * kPiInv;
    return r;
}
__device__ __forceinline__ v3 triangleNormalShad(const DeviceScene& sc, int id, v3 p) {  // intersection.glsl:149-173
    TriShade t = loadTri(sc, id);
    v3 pa = t.a - p, pb = t.b - p, pc = t.c - p;
    float areaInv = 1.0f / length(cross(t.b - t.a, t.c - t.a));
    float la = length(cross(pb, pc)) * areaInv;
    float lb = length(cross(pc, pa)) * areaInv;
    float lc = 1.0f - la - lb;
    return normalize(t.na * la + t.nb * lb + t.nc * lc);
}
__device__ __forceinline__ float remap(float p) { return p < 1e-8f ? 1.0f : p * p; }

}  // namespace zgl
