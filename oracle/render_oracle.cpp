// render_oracle.cpp — CPU oracle of the ZillumGL MIS path tracer and the
// sampling tables it reads.
//
// TEST INFRASTRUCTURE ONLY: the checker of the CUDA integrators.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
//
// Parity: the shaders restated here (src/shader/{math,random,microfacet,
// material,material_loader,intersection,light,camera,path_integ_naive}.glsl)
// need OpenGL 4.5, unavailable on this machine, so the oracle is a line-by-line
// float32 restatement — PARITY UNPINNED at the shader level.  The host tables
// follow src/core/{Scene,EnvironmentMap,Sampler,Camera}.cpp; the light alias
// table is pinned against src/math/AliasTable.h compiled from the reference
// tree (tests), the Sobol matrices against src/math/SobolMatrices256x32.h.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

#include "oracle_math.h"
#include "oracle_transc.h"

using namespace orc;

#include "orc_scene.h"

namespace {

const float Pi = 3.14159265358979323846f;
const float PiInv = 1.0f / Pi;

inline float satDot(vec3 a, vec3 b) { return fmax_(dot(a, b), 0.0f); }
inline float absDot(vec3 a, vec3 b) { return std::fabs(dot(a, b)); }
inline float square(float x) { return x * x; }
inline float distSquare(vec3 x, vec3 y) { return dot(x - y, x - y); }
inline float luminance(vec3 c) { return dot(c, vec3(0.299f, 0.587f, 0.114f)); }
inline bool isBlack(vec3 c) { return luminance(c) < 1e-5f; }
inline bool hasNan(vec3 c) { return std::isnan(c.x) || std::isnan(c.y) || std::isnan(c.z); }
inline float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix3(vec3 x, vec3 y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix3(vec3 x, vec3 y, vec3 a) { return x * (vec3(1.0f) - a) + y * a; }
inline float maxComponent(vec3 v) { return fmax_(v.x, fmax_(v.y, v.z)); }
inline float pow5(float x) {
    float x2 = x * x;
    return x2 * x2 * x;
}
inline vec3 reflect(vec3 I, vec3 N) { return I - (2.0f * dot(N, I)) * N; }

// ---------------------------------------------------------------- random.glsl
struct Rng {
    uint32_t randSeed;
    uint32_t sampleSeed;
    int sampleOffset;
};

inline uint32_t hash(uint32_t seed) {  // random.glsl:5-13
    seed = (seed ^ 61u) ^ (seed >> 16u);
    seed *= 9u;
    seed = seed ^ (seed >> 4u);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15u);
    return seed;
}

inline float rand01(Rng& g) {  // random.glsl:15-19
    g.randSeed = hash(g.randSeed);
    return (float)g.randSeed * (1.0f / 4294967296.0f);
}

// Sampler::sobolSample (Sampler.cpp:19-28): XOR of the generator-matrix
// columns selected by the bits of the sample index.
inline uint32_t sobolSample(const uint32_t* m, uint32_t index, int dim) {
    uint32_t r = 0;
    for (int i = dim * 32; index != 0; index >>= 1, i++)
        if (index & 1u) r ^= m[i];
    return r;
}

struct SamplerCtx {
    const OrcScene* sc;
};

inline float sample1D(const OrcScene& sc, Rng& g, int& s) {  // random.glsl:61-70
    if (sc.sampler == 0) return rand01(g);
    // texelFetch(uSobolSeq, sampleOffset + s): row = index / 256, dim = index % 256
    uint32_t idx = (uint32_t)g.sampleOffset + (uint32_t)s;
    uint32_t r = sobolSample(sc.sobolMatrices, idx / 256u, (int)(idx % 256u));
    r ^= g.sampleSeed;
    g.sampleSeed = hash(g.sampleSeed);
    s++;
    return (float)r / 4294967296.0f;
}

// --------------------------------------------------------------- math.glsl
inline vec2 toConcentricDisk(vec2 v) {  // math.glsl:25-41
    if (v.x == 0.0f && v.y == 0.0f) return vec2(0.0f, 0.0f);
    v = v * 2.0f - 1.0f;
    float phi, r;
    if (v.x * v.x > v.y * v.y) {
        r = v.x;
        phi = Pi * v.y / v.x * 0.25f;
    } else {
        r = v.y;
        phi = Pi * 0.5f - Pi * v.x / v.y * 0.25f;
    }
    return vec2(r * zcos(phi), r * zsin(phi));
}

struct mat3 {
    vec3 c0, c1, c2;  // columns
};
inline vec3 mul(const mat3& m, vec3 v) {
    return vec3(m.c0.x * v.x + m.c1.x * v.y + m.c2.x * v.z, m.c0.y * v.x + m.c1.y * v.y + m.c2.y * v.z,
                m.c0.z * v.x + m.c1.z * v.y + m.c2.z * v.z);
}
// inverse(mat3) by cofactors: inv = adj(m) / det(m), det expanded along the
// first column.
inline mat3 inverse(const mat3& m) {
    float a00 = m.c0.x, a01 = m.c1.x, a02 = m.c2.x;  // row 0
    float a10 = m.c0.y, a11 = m.c1.y, a12 = m.c2.y;  // row 1
    float a20 = m.c0.z, a21 = m.c1.z, a22 = m.c2.z;  // row 2
    float C00 = a11 * a22 - a12 * a21;
    float C10 = a02 * a21 - a01 * a22;
    float C20 = a01 * a12 - a02 * a11;
    float det = a00 * C00 + a10 * C10 + a20 * C20;
    float id = 1.0f / det;
    // rows of the inverse
    float i00 = C00 * id, i01 = C10 * id, i02 = C20 * id;
    float i10 = (a12 * a20 - a10 * a22) * id, i11 = (a00 * a22 - a02 * a20) * id, i12 = (a02 * a10 - a00 * a12) * id;
    float i20 = (a10 * a21 - a11 * a20) * id, i21 = (a01 * a20 - a00 * a21) * id, i22 = (a00 * a11 - a01 * a10) * id;
    return mat3{vec3(i00, i10, i20), vec3(i01, i11, i21), vec3(i02, i12, i22)};
}

inline vec3 getTangent(vec3 n) { return (std::fabs(n.z) > 0.999f) ? vec3(0.0f, 1.0f, 0.0f) : vec3(0.0f, 0.0f, 1.0f); }
inline mat3 tbnMatrix(vec3 n) {  // math.glsl:78-84
    vec3 t = getTangent(n);
    vec3 b = normalize(cross(n, t));
    t = cross(b, n);
    return mat3{t, b, n};
}
inline vec3 normalToWorld(vec3 n, vec3 v) { return normalize(mul(tbnMatrix(n), v)); }

struct vec4r {
    vec3 v;
    float w;
};
inline vec4r sampleCosineWeighted(vec3 n, vec2 u) {  // math.glsl:99-105
    vec2 uv = toConcentricDisk(u);
    float z = std::sqrt(1.0f - dot(uv, uv));
    vec3 v = normalToWorld(n, vec3(uv.x, uv.y, z));
    return vec4r{v, PiInv * z};
}
inline bool sameHemisphere(vec3 n, vec3 a, vec3 b) { return dot(n, a) * dot(n, b) > 0.0f; }

inline vec3 sampleTriangleUniform(vec3 va, vec3 vb, vec3 vc, vec2 uv) {  // math.glsl:139-145
    float r = std::sqrt(uv.y);
    float u = 1.0f - r;
    float v = uv.x * r;
    return va * (1.0f - u - v) + vb * u + vc * v;
}
inline float triangleArea(vec3 va, vec3 vb, vec3 vc) { return 0.5f * length(cross(vc - va, vb - va)); }
inline vec3 rotateZ(vec3 v, float angle) {
    float c = zcos(angle), s = zsin(angle);
    return vec3(v.x * c - v.y * s, v.x * s + v.y * c, v.z);
}
inline vec2 sphereToPlane(vec3 uv) {  // math.glsl:58-64
    float theta = zatan2(uv.y, uv.x);
    if (theta < 0.0f) theta += Pi * 2.0f;
    float phi = zatan2(length(vec2(uv.x, uv.y)), uv.z);
    return vec2(theta * PiInv * 0.5f, phi * PiInv);
}
inline vec3 planeToSphere(vec2 uv) {  // math.glsl:66-71
    float theta = uv.x * Pi * 2.0f;
    float phi = uv.y * Pi;
    return vec3(zcos(theta) * zsin(phi), zsin(theta) * zsin(phi), zcos(phi));
}
inline float biHeuristic(float f, float g) { return f * f / (f * f + g * g); }

// --------------------------------------------------------- microfacet.glsl
inline float schlickW(float c) { return pow5(1.0f - c); }
inline vec3 schlickF(float c, vec3 F0) { return F0 + (vec3(1.0f) - F0) * pow5(1.0f - c); }
inline float schlickG(float c, float alpha) {
    float k = alpha * 0.5f;
    return c / (c * (1.0f - k) + k);
}
inline float smithG(vec3 n, vec3 wo, vec3 wi, float alpha) {
    return schlickG(absDot(n, wo), alpha) * schlickG(absDot(n, wi), alpha);
}
inline float ggx(float c, float alpha) {  // microfacet.glsl:30-40
    if (c < 1e-6f) return 0.0f;
    float a2 = alpha * alpha;
    float nom = a2;
    float denom = c * c * (a2 - 1.0f) + 1.0f;
    denom = denom * denom * Pi;
    return nom / denom;
}
inline float ggxD(vec3 n, vec3 m, float alpha) { return ggx(dot(n, m), alpha); }
inline float ggxPdfVisibleWm(vec3 n, vec3 m, vec3 wo, float alpha) {
    return ggx(dot(n, m), alpha) * schlickG(dot(n, wo), alpha) * absDot(m, wo) / absDot(n, wo);
}
inline vec3 ggxSampleVisibleWm(vec3 n, vec3 wo, float alpha, vec2 u) {  // microfacet.glsl:74-92
    mat3 tbn = tbnMatrix(n);
    mat3 tbnInv = inverse(tbn);
    vec3 vh = normalize(mul(tbnInv, wo) * vec3(alpha, alpha, 1.0f));
    float lensq = vh.x * vh.x + vh.y * vh.y;
    vec3 t1 = lensq > 0.0f ? vec3(-vh.y, vh.x, 0.0f) / std::sqrt(lensq) : vec3(1.0f, 0.0f, 0.0f);
    vec3 t2 = cross(vh, t1);
    vec2 xi = toConcentricDisk(u);
    float s = 0.5f * (1.0f + vh.z);
    xi.y = (1.0f - s) * std::sqrt(1.0f - xi.x * xi.x) + s * xi.y;
    vec3 h = t1 * xi.x + t2 * xi.y + vh * std::sqrt(fmax_(0.0f, 1.0f - xi.x * xi.x - xi.y * xi.y));
    h = normalize(vec3(h.x * alpha, h.y * alpha, fmax_(0.0f, h.z)));
    return normalToWorld(n, h);
}
inline float gtr1(float c, float alpha) {  // microfacet.glsl:94-98
    float a2 = alpha * alpha;
    return (a2 - 1.0f) / (2.0f * Pi * zlog(alpha) * (1.0f + (a2 - 1.0f) * c * c));
}
inline float gtr1D(vec3 n, vec3 m, float alpha) { return gtr1(satDot(n, m), alpha); }
inline vec3 gtr1SampleWm(vec3 n, vec3 wo, float alpha, vec2 u) {  // microfacet.glsl:105-115
    float cosTheta = std::sqrt(fmax_(0.0f, (1.0f - zpow(alpha, 1.0f - u.x)) / (1.0f - alpha)));
    float sinTheta = std::sqrt(fmax_(0.0f, 1.0f - cosTheta * cosTheta));
    float phi = 2.0f * u.y * Pi;
    vec3 m = normalize(vec3(zcos(phi) * sinTheta, zsin(phi) * sinTheta, cosTheta));
    if (!sameHemisphere(n, wo, m)) m = -m;
    return normalize(normalToWorld(n, m));
}
inline float gtr1PdfWm(vec3 n, vec3 m, vec3 wo, float alpha) { return gtr1D(n, m, alpha) * absDot(n, m); }

// ----------------------------------------------------------- material.glsl
enum : uint32_t { Diffuse = 1u << 0, GlosRefl = 1u << 1, GlosTrans = 1u << 2, SpecRefl = 1u << 3,
                  SpecTrans = 1u << 4, Invalid = 1u << 16 };
enum : uint32_t { Lambertian = 0, PrincipledBRDF = 1, MetalWorkflow = 2, Dielectric = 3, ThinDielectric = 4 };

struct BSDFParam {
    vec3 baseColor;
    float subsurface = 0, metallic = 0, roughness = 0, specular = 0, specularTint = 0;
    float sheen = 0, sheenTint = 0, clearcoat = 0, clearcoatGloss = 0, ior = 0;
};
struct BSDFSample {
    vec3 wi;
    float pdf;
    vec3 bsdf;
    float eta;
    uint32_t flag;
};
inline BSDFSample invalidSample() { return BSDFSample{vec3(0.0f), 0.0f, vec3(0.0f), 0.0f, Invalid}; }

inline vec3 lambertian(const BSDFParam& p) { return p.baseColor * PiInv; }
inline float lambertianPdf(vec3 wi, vec3 n) { return satDot(wi, n) * PiInv; }
inline BSDFSample lambertianSample(vec3 n, const BSDFParam& p, vec3 u) {  // material.glsl:78-83
    vec3 wi = sampleCosineWeighted(n, vec2(u.y, u.z)).v;
    float pdf = satDot(n, wi) * PiInv;
    return BSDFSample{wi, pdf, p.baseColor * PiInv, 1.0f, Diffuse};
}

inline vec3 principledMetal(vec3 wo, vec3 wi, vec3 n, vec3 fm0, float alpha) {  // :357-373
    float cosWo = satDot(n, wo);
    float cosWi = satDot(n, wi);
    vec3 h = normalize(wo + wi);
    if (cosWo < 1e-10f || cosWi < 1e-10f) return vec3(0.0f);
    vec3 fm = schlickF(absDot(h, wo), fm0);
    float dm = ggxD(n, h, alpha);
    float gm = smithG(n, wo, wi, alpha);
    float denom = 4.0f * cosWi * cosWo;
    if (denom < 1e-7f) return vec3(0.0f);
    return fm * dm * gm / denom;
}
inline float principledMetalPdf(vec3 wo, vec3 wi, vec3 n, float alpha) {
    vec3 h = normalize(wo + wi);
    return ggxPdfVisibleWm(n, h, wo, alpha) / (4.0f * absDot(h, wo));
}
inline vec3 principledClearcoat(vec3 wo, vec3 wi, vec3 n, vec3 baseColor, float alpha) {  // :393-409
    float cosWo = satDot(n, wo);
    float cosWi = satDot(n, wi);
    vec3 h = normalize(wo + wi);
    if (cosWo < 1e-6f || cosWi < 1e-6f) return vec3(0.0f);
    vec3 fc = schlickF(absDot(h, wo), baseColor);
    float dc = gtr1D(n, h, alpha);
    float gc = smithG(n, wo, wi, 0.25f);
    float denom = 4.0f * cosWi * cosWo;
    if (denom < 1e-7f) return vec3(0.0f);
    return fc * dc * gc / denom;
}
inline float principledClearcoatPdf(vec3 wo, vec3 wi, vec3 n, float alpha) {
    vec3 h = normalize(wo + wi);
    return gtr1PdfWm(n, h, wo, alpha) / (4.0f * absDot(h, wo));
}
inline vec3 principledDiffuse(vec3 wo, vec3 wi, vec3 n, vec3 baseColor, float subsurface, float roughness) {
    float cosWo = satDot(n, wo);  // :429-452
    float cosWi = satDot(n, wi);
    if (cosWo < 1e-10f || cosWi < 1e-10f) return vec3(0.0f);
    vec3 h = normalize(wo + wi);
    float hCosWi = dot(h, wi);
    float hCosWi2 = hCosWi * hCosWi;
    float fi = schlickW(cosWi);
    float fo = schlickW(cosWo);
    vec3 fd90 = vec3(0.5f + 2.0f * roughness * hCosWi2);
    vec3 fd = mix3(vec3(1.0f), fd90, fi) * mix3(vec3(1.0f), fd90, fo);
    vec3 baseDiffuse = baseColor * fd * PiInv;
    vec3 fss90 = vec3(roughness * hCosWi2);
    vec3 fss = mix3(vec3(1.0f), fss90, fi) * mix3(vec3(1.0f), fss90, fo);
    vec3 ss = baseColor * PiInv * 1.25f * (fss * (1.0f / (cosWi + cosWo) - 0.5f) + vec3(0.5f));
    return mix3(baseDiffuse, ss, subsurface);
}

inline void principledCommon(const BSDFParam& p, float& alpha, float& clearcoatAlpha, vec3& tintColor, vec3& fm0) {
    alpha = square(p.roughness);
    clearcoatAlpha = mixf(0.1f, 0.001f, p.clearcoatGloss);
    float lum = luminance(p.baseColor);
    tintColor = lum > 0.0f ? p.baseColor / lum : vec3(1.0f);
    fm0 = mix3(0.08f * p.specular * mix3(vec3(1.0f), tintColor, p.specularTint), p.baseColor, p.metallic);
}

inline vec3 principledBRDF(vec3 wo, vec3 wi, vec3 n, const BSDFParam& p) {  // :462-490
    vec3 res(0.0f);
    float alpha, ccAlpha;
    vec3 tint, fm0;
    principledCommon(p, alpha, ccAlpha, tint, fm0);
    float hCosWi = dot(normalize(wo + wi), wi);
    res = res + principledDiffuse(wo, wi, n, p.baseColor, p.subsurface, p.roughness) * (1.0f - p.metallic);
    res = res + principledMetal(wo, wi, n, fm0, alpha);
    res = res + principledClearcoat(wo, wi, n, p.baseColor, ccAlpha) * p.clearcoat * 0.25f;
    res = res + mix3(vec3(1.0f), tint, p.sheenTint) * schlickW(hCosWi) * p.sheen * (dot(n, wi) < 0.0f ? 0.0f : 1.0f);
    return res;
}
inline float principledBRDFPdf(vec3 wo, vec3 wi, vec3 n, const BSDFParam& p) {  // :492-514
    float pdf = 0.0f;
    float alpha = square(p.roughness);
    float ccAlpha = mixf(0.1f, 0.001f, p.clearcoatGloss);
    float spec = 1.0f / (2.0f - p.metallic);
    float cosinePdf = absDot(n, wi) * PiInv;
    pdf += cosinePdf * (1.0f - spec);
    pdf += principledMetalPdf(wo, wi, n, alpha) * spec;
    pdf += principledClearcoatPdf(wo, wi, n, ccAlpha) * 0.25f * p.clearcoat;
    return pdf / (1.0f + 0.25f * p.clearcoat);
}
inline BSDFSample principledBRDFSample(vec3 n, vec3 wo, const BSDFParam& p, vec3 u, Rng& g) {  // :516-555
    float alpha = square(p.roughness);
    float spec = 1.0f / (2.0f - p.metallic);
    float cdf0 = 1.0f - spec, cdf1 = 1.0f, cdf2 = 1.0f + p.clearcoat * 0.25f;
    vec3 wi;
    float s = rand01(g) * cdf2;
    if (s <= cdf0) {
        wi = sampleCosineWeighted(n, vec2(u.y, u.z)).v;  // principledDiffuseSample: .wi only
    } else if (s <= cdf1) {
        float lum = luminance(p.baseColor);
        vec3 tint = lum > 0.0f ? p.baseColor / lum : vec3(1.0f);
        vec3 fm0 = mix3(0.08f * p.specular * mix3(vec3(1.0f), tint, p.specularTint), p.baseColor, p.metallic);
        (void)fm0;
        // principledMetalSample(...).wi: InvalidBSDFSample has wi = 0
        vec3 h = ggxSampleVisibleWm(n, wo, alpha, vec2(u.y, u.z));
        vec3 w = reflect(-wo, h);
        wi = (dot(n, w) < 0.0f) ? vec3(0.0f) : w;
    } else {
        vec3 h = gtr1SampleWm(n, wo, alpha, vec2(u.y, u.z));  // base alpha, as the reference does
        vec3 w = reflect(-wo, h);
        wi = (dot(n, w) < 0.0f) ? vec3(0.0f) : w;
    }
    vec3 bsdf = principledBRDF(wo, wi, n, p);
    float pdf = principledBRDFPdf(wo, wi, n, p);
    return BSDFSample{wi, pdf, bsdf, 1.0f, Diffuse};
}

// metalWorkflow / dielectric / thinDielectric (material.glsl:85-355)
enum : uint32_t { Radiance = 0, Importance = 1 };
inline bool approximateDelta(float r) { return r < 0.02f; }
inline vec3 schlickFRough(float c, vec3 F0, float r) {  // microfacet.glsl:14-17
    vec3 m(fmax_(1.0f - r, F0.x), fmax_(1.0f - r, F0.y), fmax_(1.0f - r, F0.z));
    return F0 + (m - F0) * pow5(1.0f - c);
}
inline vec3 ggxSampleWm(vec3 n, vec3 wo, float alpha, vec2 u) {  // microfacet.glsl:57-64
    (void)wo;
    vec2 xi = toConcentricDisk(u);
    vec3 h(xi.x, xi.y, std::sqrt(fmax_(0.0f, 1.0f - xi.x * xi.x - xi.y * xi.y)));
    h = normalize(h * vec3(alpha, alpha, 1.0f));
    return normalToWorld(n, h);
}
inline vec3 metalWorkflow(vec3 wo, vec3 wi, vec3 n, const BSDFParam& p) {
    float alpha = square(p.roughness);
    vec3 h = normalize(wi + wo);
    if (!sameHemisphere(n, wo, wi)) return vec3(0.0f);
    float cosWi = dot(n, wi), cosWo = dot(n, wo);
    vec3 f0 = mix3(vec3(0.04f), p.baseColor, p.metallic);
    vec3 f = schlickFRough(satDot(h, wo), f0, p.roughness);
    float d = ggxD(n, h, alpha);
    float g = smithG(n, wo, wi, alpha);
    vec3 kd = vec3(1.0f) - f;
    kd = kd * (1.0f - p.metallic);
    float denom = 4.0f * cosWo * cosWi;
    if (denom < 1e-7f) return vec3(0.0f);
    return kd * p.baseColor * PiInv + f * d * g / denom;
}
inline float metalWorkflowPdf(vec3 wo, vec3 wi, vec3 n, const BSDFParam& p) {
    float alpha = square(p.roughness);
    vec3 h = normalize(wo + wi);
    float pdfDiff = satDot(n, wi) * PiInv;
    float pdfSpec = ggxPdfVisibleWm(n, h, wo, alpha) / (4.0f * absDot(h, wo));
    float spec = 1.0f / (2.0f - p.metallic);
    return mixf(pdfDiff, pdfSpec, spec);
}
inline BSDFSample metalWorkflowSample(vec3 n, vec3 wo, const BSDFParam& p, vec3 u) {
    float alpha = square(p.roughness);
    float spec = 1.0f / (2.0f - p.metallic);
    uint32_t type = u.x > spec ? Diffuse : GlosRefl;
    vec3 wi = type == Diffuse ? sampleCosineWeighted(n, vec2(u.y, u.z)).v
                              : reflect(-wo, ggxSampleVisibleWm(n, wo, alpha, vec2(u.y, u.z)));
    if (dot(n, wi) < 0.0f) return invalidSample();
    return BSDFSample{wi, metalWorkflowPdf(wo, wi, n, p), metalWorkflow(wo, wi, n, p), 1.0f, type};
}
inline bool refractDir(vec3& wt, vec3 wi, vec3 n, float eta) {
    float cosTi = dot(n, wi);
    if (cosTi < 0.0f) eta = 1.0f / eta;
    float sin2Ti = fmax_(0.0f, 1.0f - cosTi * cosTi);
    float sin2Tt = sin2Ti / (eta * eta);
    if (sin2Tt >= 1.0f) return false;
    float cosTt = std::sqrt(1.0f - sin2Tt);
    if (cosTi < 0.0f) cosTt = -cosTt;
    wt = normalize(-wi / eta + n * (cosTi / eta - cosTt));
    return true;
}
inline float fresnelDielectric(float cosTi, float eta) {
    cosTi = fmin_(fmax_(cosTi, -1.0f), 1.0f);
    if (cosTi < 0.0f) {
        eta = 1.0f / eta;
        cosTi = -cosTi;
    }
    float sinTi = std::sqrt(1.0f - cosTi * cosTi);
    float sinTt = sinTi / eta;
    if (sinTt >= 1.0f) return 1.0f;
    float cosTt = std::sqrt(1.0f - sinTt * sinTt);
    float rPa = (cosTi - eta * cosTt) / (cosTi + eta * cosTt);
    float rPe = (eta * cosTi - cosTt) / (eta * cosTi + cosTt);
    return (rPa * rPa + rPe * rPe) * 0.5f;
}
inline vec3 dielectric(vec3 wo, vec3 wi, vec3 n, const BSDFParam& p, uint32_t mode) {
    if (approximateDelta(p.roughness)) return vec3(0.0f);
    vec3 h = normalize(wo + wi);
    float hCosWo = absDot(h, wo), hCosWi = absDot(h, wi);
    float alpha = p.roughness * p.roughness;
    if (sameHemisphere(n, wo, wi)) {
        float refl = fresnelDielectric(absDot(h, wi), p.ior);
        return (hCosWo * hCosWi < 1e-7f) ? vec3(0.0f)
                                         : p.baseColor * ggxD(n, h, alpha) * smithG(n, wo, wi, alpha) /
                                               (4.0f * hCosWo * hCosWi) * refl;
    }
    float eta = dot(n, wi) > 0.0f ? p.ior : 1.0f / p.ior;
    float sqrtDenom = dot(h, wo) + eta * dot(h, wi);
    float denom = sqrtDenom * sqrtDenom;
    denom *= absDot(n, wi) * absDot(n, wo);
    float refl = fresnelDielectric(dot(h, wi), eta);
    float factor = (mode == Radiance) ? square(1.0f / eta) : 1.0f;
    return (denom < 1e-7f) ? vec3(0.0f)
                           : p.baseColor * std::fabs(ggxD(n, h, alpha) * smithG(n, wo, wi, alpha) * hCosWo * hCosWi) /
                                 denom * (1.0f - refl) * factor;
}
inline float dielectricPdf(vec3 wo, vec3 wi, vec3 n, const BSDFParam& p) {
    if (approximateDelta(p.roughness)) return 0.0f;
    float alpha = p.roughness * p.roughness;
    if (sameHemisphere(n, wo, wi)) {
        vec3 h = normalize(wo + wi);
        if (dot(wo, h) < 0.0f) return 0.0f;
        float refl = fresnelDielectric(absDot(h, wi), p.ior);
        return ggxD(n, h, alpha) / (4.0f * absDot(h, wo)) * refl;
    }
    float eta = dot(n, wo) > 0.0f ? p.ior : 1.0f / p.ior;
    vec3 h = normalize(wo + wi * eta);
    if (sameHemisphere(h, wo, wi)) return 0.0f;
    float trans = 1.0f - fresnelDielectric(absDot(h, wo), eta);
    float dHdWi = absDot(h, wi) / square(dot(h, wo) + eta * dot(h, wi));
    return ggxD(n, h, alpha) * dHdWi * trans;
}
inline BSDFSample dielectricSample(vec3 n, vec3 wo, const BSDFParam& p, uint32_t mode, vec3 u) {
    float ior = p.ior;
    if (approximateDelta(p.roughness)) {
        float refl = fresnelDielectric(dot(n, wo), ior);
        if (u.x < refl) return BSDFSample{reflect(-wo, n), 1.0f, p.baseColor, 1.0f, SpecRefl};
        vec3 wi;
        if (!refractDir(wi, wo, n, ior)) return invalidSample();
        if (dot(n, wo) < 0.0f) ior = 1.0f / ior;
        float factor = (mode == Radiance) ? square(1.0f / ior) : 1.0f;
        return BSDFSample{wi, 1.0f, p.baseColor * factor, ior, SpecTrans};
    }
    float alpha = p.roughness * p.roughness;
    vec3 h = ggxSampleWm(n, wo, alpha, vec2(u.y, u.z));
    if (dot(n, h) < 0.0f) h = -h;
    float refl = fresnelDielectric(dot(h, wo), ior);
    if (u.x < refl) {
        vec3 wi = -reflect(wo, h);
        if (!sameHemisphere(n, wo, wi)) return invalidSample();
        float pdf = ggxD(n, h, alpha) / (4.0f * absDot(h, wo));
        float hCosWo = absDot(h, wo), hCosWi = absDot(h, wi);
        vec3 r = (hCosWo * hCosWi < 1e-7f) ? vec3(0.0f)
                                           : p.baseColor * ggxD(n, h, alpha) * smithG(n, wo, wi, alpha) /
                                                 (4.0f * hCosWo * hCosWi);
        if (std::isnan(pdf)) pdf = 0.0f;
        return BSDFSample{wi, pdf, r, 1.0f, GlosRefl};
    }
    vec3 wi;
    if (!refractDir(wi, wo, h, ior)) return invalidSample();
    if (sameHemisphere(n, wo, wi)) return invalidSample();
    if (absDot(n, wi) < 1e-10f) return invalidSample();
    float hCosWo = absDot(h, wo), hCosWi = absDot(h, wi);
    if (dot(h, wo) < 0.0f) ior = 1.0f / ior;
    float sqrtDenom = dot(h, wo) + ior * dot(h, wi);
    float denom = sqrtDenom * sqrtDenom;
    float dHdWi = hCosWi / denom;
    float factor = (mode == Radiance) ? square(1.0f / ior) : 1.0f;
    denom *= absDot(n, wi) * absDot(n, wo);
    vec3 t = (denom < 1e-7f) ? vec3(0.0f)
                             : p.baseColor * std::fabs(ggxD(n, h, alpha) * smithG(n, wo, wi, alpha) * hCosWo * hCosWi) /
                                   denom;
    float pdf = ggxD(n, h, alpha) * dHdWi;
    if (std::isnan(pdf)) pdf = 0.0f;
    return BSDFSample{wi, pdf, t * factor, ior, GlosTrans};
}
inline BSDFSample thinDielectricSample(vec3 n, vec3 wo, const BSDFParam& p, vec3 u) {
    if (dot(n, wo) < 0.0f) n = -n;
    float refl = fresnelDielectric(dot(n, wo), p.ior);
    float trans = 1.0f - refl;
    if (refl < 1.0f) {
        refl += trans * trans * refl / (1.0f - refl * refl);
        trans = 1.0f - refl;
    }
    return (u.x < refl) ? BSDFSample{reflect(-wo, n), 1.0f, p.baseColor, 1.0f, SpecRefl}
                        : BSDFSample{-wo, 1.0f, p.baseColor, 1.0f, SpecTrans};
}

// ---------------------------------------------------- material_loader.glsl
inline uint32_t loadMaterialType(const OrcScene& sc, int matId) {
    int32_t t;
    std::memcpy(&t, &sc.materials[16 * matId + 13], 4);
    return (uint32_t)t;
}
// sRGB code -> linear (GL_SRGB decode), in double, rounded once to float
const float* srgbTable() {
    static float lut[256];
    static bool init = false;
    if (!init) {
        for (int i = 0; i < 256; i++) {
            double c = i / 255.0;
            lut[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
        }
        init = true;
    }
    return lut;
}

// texture2DArray(uTextures, vec3(fract(uv) * uvScale, texId)).rgb
// (material_loader.glsl:14-15): level 0 with GL_LINEAR magnification,
// GL_REPEAT over the layer, sRGB decoded per texel, then the bilinear blend
// (1-a)(1-b) T00 + a(1-b) T10 + (1-a) b T01 + a b T11 in float32.
vec3 albedoTexture(const OrcScene& sc, int texId, vec2 uv) {
    const float* lut = srgbTable();
    const float s = (uv.x - std::floor(uv.x)) * sc.texScale[2 * texId];
    const float t = (uv.y - std::floor(uv.y)) * sc.texScale[2 * texId + 1];
    const int W = sc.texMaxW, H = sc.texMaxH;
    const float u = s * (float)W - 0.5f, v = t * (float)H - 0.5f;
    const float a = u - std::floor(u), b = v - std::floor(v);
    auto wrap = [](int i, int n) { return ((i % n) + n) % n; };
    const int i0 = wrap((int)std::floor(u), W), j0 = wrap((int)std::floor(v), H);
    const int i1 = wrap(i0 + 1, W), j1 = wrap(j0 + 1, H);
    auto T = [&](int i, int j, int c) {
        return lut[sc.texLayers[(((size_t)texId * H + j) * W + i) * 3 + c]];
    };
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    float c3[3];
    for (int c = 0; c < 3; c++)
        c3[c] = w00 * T(i0, j0, c) + w10 * T(i1, j0, c) + w01 * T(i0, j1, c) + w11 * T(i1, j1, c);
    return vec3(c3[0], c3[1], c3[2]);
}

inline BSDFParam loadMaterial(const OrcScene& sc, uint32_t type, int matId) {  // :81-97
    const float* m = sc.materials + 16 * matId;
    BSDFParam p;
    p.baseColor = vec3(m[0], m[1], m[2]);
    if (type == MetalWorkflow) {  // loadMetalWorkflow :26-35
        p.roughness = mixf(0.0134f, 1.0f, m[3]);
        p.metallic = m[5];
    } else if (type == Dielectric) {  // loadDielectric :60-69
        p.roughness = m[3];
        p.ior = m[12];
    } else if (type == ThinDielectric) {  // loadThinDielectric :71-79
        p.ior = m[12];
    } else if (type == PrincipledBRDF) {
        p.roughness = mixf(0.0134f, 1.0f, m[3]);
        p.subsurface = m[4];
        p.metallic = m[5];
        p.specular = m[6];
        p.specularTint = m[7];
        p.sheen = m[8];
        p.sheenTint = m[9];
        p.clearcoat = m[10];
        p.clearcoatGloss = m[11];
    }
    return p;
}
inline vec3 materialBSDF(uint32_t type, const BSDFParam& p, vec3 wo, vec3 wi, vec3 n, uint32_t mode = Radiance) {
    if (type == PrincipledBRDF) return principledBRDF(wo, wi, n, p);
    if (type == MetalWorkflow) return metalWorkflow(wo, wi, n, p);
    if (type == Dielectric) return dielectric(wo, wi, n, p, mode);
    if (type == ThinDielectric) return vec3(0.0f);
    return lambertian(p);
}
inline float materialPdf(uint32_t type, const BSDFParam& p, vec3 wo, vec3 wi, vec3 n) {
    if (type == PrincipledBRDF) return principledBRDFPdf(wo, wi, n, p);
    if (type == MetalWorkflow) return metalWorkflowPdf(wo, wi, n, p);
    if (type == Dielectric) return dielectricPdf(wo, wi, n, p);
    if (type == ThinDielectric) return 0.0f;
    return lambertianPdf(wi, n);
}
inline BSDFSample materialSample(uint32_t type, const BSDFParam& p, vec3 n, vec3 wo, vec3 u, Rng& g,
                                 uint32_t mode = Radiance) {
    if (type == PrincipledBRDF) return principledBRDFSample(n, wo, p, u, g);
    if (type == MetalWorkflow) return metalWorkflowSample(n, wo, p, u);
    if (type == Dielectric) return dielectricSample(n, wo, p, mode, u);
    if (type == ThinDielectric) return thinDielectricSample(n, wo, p, u);
    return lambertianSample(n, p, u);
}

// -------------------------------------------------------- intersection.glsl
struct Ray {
    vec3 ori, dir;
};
inline Ray rayOffseted(vec3 o, vec3 d) { return Ray{o + d * 1e-4f, d}; }
inline vec3 rayPoint(const Ray& r, float t) { return r.ori + r.dir * t; }

inline vec3 V(const OrcScene& sc, uint32_t i) { return vec3(sc.vertices[3 * i], sc.vertices[3 * i + 1], sc.vertices[3 * i + 2]); }
inline vec3 N(const OrcScene& sc, uint32_t i) { return vec3(sc.normals[3 * i], sc.normals[3 * i + 1], sc.normals[3 * i + 2]); }

struct SurfaceInfo {
    vec3 ns, ng;
    vec2 uv;
};
inline SurfaceInfo triangleSurfaceInfo(const OrcScene& sc, int id, vec3 p) {  // :188-224
    uint32_t ia = sc.indices[3 * id], ib = sc.indices[3 * id + 1], ic = sc.indices[3 * id + 2];
    vec3 a = V(sc, ia), b = V(sc, ib), c = V(sc, ic);
    vec3 na = N(sc, ia), nb = N(sc, ib), nc = N(sc, ic);
    vec3 pa = a - p, pb = b - p, pc = c - p;
    float areaInv = 1.0f / length(cross(b - a, c - a));
    float la = length(cross(pb, pc)) * areaInv;
    float lb = length(cross(pc, pa)) * areaInv;
    float lc = 1.0f - la - lb;
    SurfaceInfo s;
    s.ns = normalize(na * la + nb * lb + nc * lc);
    s.ng = normalize(cross(pa, pb));
    s.uv = vec2(0.0f, 0.0f);
    if (sc.texCoords && id < sc.objPrimCount) {
        const float* T = sc.texCoords;
        s.uv = vec2(T[2 * ia] * la + T[2 * ib] * lb + T[2 * ic] * lc,
                    T[2 * ia + 1] * la + T[2 * ib + 1] * lb + T[2 * ic + 1] * lc);
    }
    if (dot(s.ns, s.ng) < 0.0f) s.ng = -s.ng;
    return s;
}
// the base colour of a textured triangle (matTex >> 16 != -1)
inline void applyTexture(const OrcScene& sc, int matTexId, const SurfaceInfo& surf, BSDFParam& p) {
    const int texId = matTexId >> 16;
    if (texId != -1) p.baseColor = albedoTexture(sc, texId, surf.uv);
}
inline float triangleArea(const OrcScene& sc, int id) {
    return triangleArea(V(sc, sc.indices[3 * id]), V(sc, sc.indices[3 * id + 1]), V(sc, sc.indices[3 * id + 2]));
}
inline vec3 triangleSampleUniform(const OrcScene& sc, int id, vec2 u) {
    return sampleTriangleUniform(V(sc, sc.indices[3 * id]), V(sc, sc.indices[3 * id + 1]), V(sc, sc.indices[3 * id + 2]), u);
}

}  // namespace

// traversal from bvh_oracle.cpp
extern "C" void orc_trace(const float*, const int32_t*, int64_t, const float*, const uint32_t*, const float*,
                          const float*, const float*, int64_t, int32_t, int32_t*, float*, int32_t*, int32_t*, int32_t);

namespace {

inline int bvhHit(const OrcScene& sc, const Ray& r, float& dist) {
    float o[3] = {r.ori.x, r.ori.y, r.ori.z}, d[3] = {r.dir.x, r.dir.y, r.dir.z};
    int32_t id;
    float t;
    orc_trace(sc.bounds, sc.hitTable, sc.bvhSize, sc.vertices, sc.indices, o, d, nullptr, 1, 0, &id, &t, nullptr,
              nullptr, 1);
    dist = t;
    return id;
}
inline bool bvhTest(const OrcScene& sc, const Ray& r, float dist) {
    float o[3] = {r.ori.x, r.ori.y, r.ori.z}, d[3] = {r.dir.x, r.dir.y, r.dir.z};
    int32_t occ;
    orc_trace(sc.bounds, sc.hitTable, sc.bvhSize, sc.vertices, sc.indices, o, d, &dist, 1, 1, &occ, nullptr, nullptr,
              nullptr, 1);
    return occ != 0;
}

// ---------------------------------------------------------------- light.glsl
struct LightLiSample {
    vec3 wi, coef;
    float pdf;
};
inline LightLiSample invalidLi() { return LightLiSample{vec3(0.0f), vec3(0.0f), 0.0f}; }

inline vec3 lightPowerOf(const OrcScene& sc, int id) {
    return vec3(sc.lightPower[3 * id], sc.lightPower[3 * id + 1], sc.lightPower[3 * id + 2]);
}
inline int lightSampleOne(const OrcScene& sc, vec2 u) {  // light.glsl:68-72
    // u.x can round to exactly 1.0 (random.glsl:69); the reference then reads
    // one entry past the table, the build clamps to the last entry.
    int cx = std::min(f2i((float)sc.nLightTriangles * u.x), sc.nLightTriangles - 1);
    return (u.y < sc.lightProb[cx]) ? cx : sc.lightAlias[cx];
}
inline float lightPdfSampleOne(const OrcScene& sc, int id) { return luminance(lightPowerOf(sc, id)) / sc.lightSum; }
inline vec3 lightLe(const OrcScene& sc, int id, vec3 x, vec3 wo) {  // :79-86
    int triId = id + sc.objPrimCount;
    SurfaceInfo s = triangleSurfaceInfo(sc, triId, x);
    if (dot(wo, s.ng) <= 0.0f) return vec3(0.0f);
    return lightPowerOf(sc, id) / triangleArea(sc, triId) * 0.5f * PiInv;
}
inline float lightPdfLi(const OrcScene& sc, int id, vec3 x, vec3 y) {  // :88-98
    int triId = id + sc.objPrimCount;
    vec3 norm = triangleSurfaceInfo(sc, triId, y).ng;
    vec3 yx = normalize(x - y);
    float cosTheta = absDot(norm, yx);
    if (cosTheta < 1e-8f) return -1.0f;
    return distSquare(x, y) / (triangleArea(sc, triId) * cosTheta);
}
inline LightLiSample lightSampleLi(const OrcScene& sc, int id, vec3 x, vec2 u) {  // :122-155
    int triId = id + sc.objPrimCount;
    vec3 a = V(sc, sc.indices[3 * triId]), b = V(sc, sc.indices[3 * triId + 1]), c = V(sc, sc.indices[3 * triId + 2]);
    vec3 y = sampleTriangleUniform(a, b, c, u);
    vec3 wi = normalize(y - x);
    vec3 norm = triangleSurfaceInfo(sc, triId, y).ng;
    float cosTheta = dot(norm, -wi);
    if (cosTheta < 1e-6f) return invalidLi();
    Ray lightRay = rayOffseted(x, wi);
    float dist = distance(x, y);
    float pdf = dist * dist / (triangleArea(a, b, c) * cosTheta);
    float testDist = dist - 1e-4f - 1e-6f;
    if (bvhTest(sc, lightRay, testDist) || pdf < 1e-8f) return invalidLi();
    vec3 weight = lightLe(sc, id, y, -wi);
    float pdfSample = luminance(lightPowerOf(sc, id)) / sc.lightSum;
    pdf *= pdfSample;
    return LightLiSample{wi, weight / pdf, pdf};
}

// Env texture: RGB16F texels, bilinear with repeat wrap at GL texel centres.
inline vec3 envTexel(const OrcScene& sc, int x, int y) {
    int W = sc.envWidth, H = sc.envHeight;
    x %= W;
    if (x < 0) x += W;
    y %= H;
    if (y < 0) y += H;
    const float* t = sc.envTexels + 3 * ((size_t)y * W + x);
    return vec3(t[0], t[1], t[2]);
}
inline vec3 envTexture(const OrcScene& sc, vec2 st) {
    float u = st.x * (float)sc.envWidth - 0.5f;
    float v = st.y * (float)sc.envHeight - 0.5f;
    float fu = std::floor(u), fv = std::floor(v);
    float au = u - fu, av = v - fv;
    int x0 = f2i(fu), y0 = f2i(fv);
    vec3 t00 = envTexel(sc, x0, y0), t10 = envTexel(sc, x0 + 1, y0);
    vec3 t01 = envTexel(sc, x0, y0 + 1), t11 = envTexel(sc, x0 + 1, y0 + 1);
    return mix3(mix3(t00, t10, au), mix3(t01, t11, au), av);
}
inline vec3 envLe(const OrcScene& sc, vec3 wi) {  // light.glsl:163-167
    if (!sc.envTexels) return vec3(0.0f);
    wi = rotateZ(wi, -sc.envRotation);
    return envTexture(sc, sphereToPlane(wi));
}
inline float envGetPortion(const OrcScene& sc, vec3 wi) { return luminance(envLe(sc, wi)) / sc.envSum; }
inline float envPdfLi(const OrcScene& sc, vec3 wi) {  // :174-179
    if (sc.envSum == 0.0f) return 0.0f;
    return envGetPortion(sc, wi) * (float)sc.envWidth * (float)sc.envHeight * 0.5f * square(PiInv);
}
struct EnvWi {
    vec3 wi;
    float pdf;
};
inline EnvWi envSampleWi(const OrcScene& sc, float ux, float uy, float uz, float uw) {  // :181-205
    int w = sc.envWidth, h = sc.envHeight;
    int rx = std::min(f2i((float)h * ux), h - 1);  // clamped like lightSampleOne
    int rIdx = rx * (w + 1) + w;
    int row = (uy < sc.envProb[rIdx]) ? rx : sc.envAlias[rIdx];
    int cx = std::min(f2i((float)w * uz), w - 1);
    int cIdx = row * (w + 1) + cx;
    int col = (uw < sc.envProb[cIdx]) ? cx : sc.envAlias[cIdx];
    vec2 uv = vec2((float)col + 0.5f, (float)row + 0.5f) / vec2((float)w, (float)h);
    vec3 wi = planeToSphere(uv);
    wi = rotateZ(wi, sc.envRotation);
    float pdf = envGetPortion(sc, wi) * (float)w * (float)h * 0.5f * square(PiInv);
    return EnvWi{wi, pdf};
}
inline LightLiSample envSampleLi(const OrcScene& sc, vec3 x, float ux, float uy, float uz, float uw) {
    if (!sc.envTexels) return invalidLi();  // black environment: nothing to sample
    EnvWi sp = envSampleWi(sc, ux, uy, uz, uw);
    Ray ray = rayOffseted(x, sp.wi);
    if (bvhTest(sc, ray, 1e8f) || sp.pdf == 0.0f) return invalidLi();
    return LightLiSample{sp.wi, envLe(sc, sp.wi) / sp.pdf, sp.pdf};
}
inline LightLiSample sampleLightAndEnv(const OrcScene& sc, vec3 x, float ud, float u0, float u1, float u2, float u3) {
    float pdfSampleLight = 0.0f;  // light.glsl:221-235
    if (sc.nLightTriangles > 0)
        pdfSampleLight = sc.lightEnvUniformSample ? sc.lightPortion : sc.lightSum / (sc.lightSum + sc.envSum);
    bool sampleLight = ud < pdfSampleLight;
    float pdfSelect = sampleLight ? pdfSampleLight : 1.0f - pdfSampleLight;
    LightLiSample s;
    if (sampleLight) {
        int id = lightSampleOne(sc, vec2(u0, u1));
        s = lightSampleLi(sc, id, x, vec2(u2, u3));
    } else {
        s = envSampleLi(sc, x, u0, u1, u2, u3);
    }
    s.coef = s.coef / pdfSelect;
    s.pdf *= pdfSelect;
    return s;
}
inline float pdfSelectLight(const OrcScene& sc, int id) {
    float fst = luminance(lightPowerOf(sc, id)) / sc.lightSum;
    float snd = sc.lightEnvUniformSample ? sc.lightPortion : sc.lightSum / (sc.lightSum + sc.envSum);
    return fst * snd;
}
inline float pdfSelectEnv(const OrcScene& sc) {
    return sc.lightEnvUniformSample ? (1.0f - sc.lightPortion) : sc.envSum / (sc.lightSum + sc.envSum);
}

// --------------------------------------------------------------- camera.glsl
inline vec3 cv(const float* p) { return vec3(p[0], p[1], p[2]); }
inline Ray thinLensCameraSampleRay(const OrcScene& sc, vec2 uv, float u0, float u1, float u2, float u3) {
    vec2 texelSize = vec2(1.0f) / vec2((float)sc.filmW, (float)sc.filmH);  // camera.glsl:62-77
    vec2 biased = uv + texelSize * vec2(u0, u1);
    vec2 ndc = biased * 2.0f - 1.0f;
    vec2 lens = toConcentricDisk(vec2(u2, u3)) * sc.lensRadius;
    vec3 pLens(lens.x, lens.y, 0.0f);
    vec2 fp = ndc * vec2(sc.camAsp, 1.0f) * sc.focalDist * sc.tanFOV;
    vec3 pFocus(fp.x, fp.y, sc.focalDist);
    vec3 dir = pFocus - pLens;
    dir = normalize(cv(sc.camR) * dir.x + cv(sc.camU) * dir.y + cv(sc.camF) * dir.z);
    return Ray{cv(sc.camPos) + cv(sc.camR) * pLens.x + cv(sc.camU) * pLens.y, dir};
}

// ------------------------------------------------------ path_integ_naive.glsl
vec3 pathIntegTrace(const OrcScene& sc, Ray ray, int& s, Rng& g) {  // :35-143
    float primDist;
    int id = bvhHit(sc, ray, primDist);
    vec3 pos = rayPoint(ray, primDist);
    if (id == -1) return envLe(sc, ray.dir);
    if (id - sc.objPrimCount >= 0) return lightLe(sc, id - sc.objPrimCount, pos, -ray.dir);
    vec3 wo = -ray.dir;
    vec3 result(0.0f), throughput(1.0f);
    for (int bounce = 1; bounce <= sc.maxDepth; bounce++) {
        SurfaceInfo surf = triangleSurfaceInfo(sc, id, pos);
        int matTexId = sc.matTexIndex[id];
        int matId = matTexId & 0x0000ffff;
        uint32_t matType = loadMaterialType(sc, matId);
        if (matType != Dielectric && matType != ThinDielectric) {
            if (dot(surf.ns, wo) < 0.0f) {
                surf.ns = -surf.ns;
                surf.ng = -surf.ng;
            }
        }
        BSDFParam mp = loadMaterial(sc, matType, matId);
        applyTexture(sc, sc.matTexIndex[id], surf, mp);
        if (sc.sampleLight) {
            float ud = sample1D(sc, g, s);
            float u0 = sample1D(sc, g, s), u1 = sample1D(sc, g, s), u2 = sample1D(sc, g, s), u3 = sample1D(sc, g, s);
            LightLiSample ls = sampleLightAndEnv(sc, pos, ud, u0, u1, u2, u3);
            if (ls.pdf > 0.0f) {
                vec3 f = materialBSDF(matType, mp, wo, ls.wi, surf.ns);
                float fpdf = materialPdf(matType, mp, wo, ls.wi, surf.ns);
                float weight = biHeuristic(ls.pdf, fpdf);
                result = result + f * throughput * satDot(surf.ns, ls.wi) * ls.coef * weight;
            }
        }
        float b0 = sample1D(sc, g, s), b1 = sample1D(sc, g, s), b2 = sample1D(sc, g, s);
        BSDFSample bs = materialSample(matType, mp, surf.ns, wo, vec3(b0, b1, b2), g);
        vec3 wi = bs.wi;
        float bsdfPdf = bs.pdf;
        vec3 bsdf = bs.bsdf;
        uint32_t flag = bs.flag;
        bool deltaBsdf = (flag == SpecRefl || flag == SpecTrans);
        if (bsdfPdf < 1e-8f) break;
        throughput = throughput * (bsdf / bsdfPdf * (deltaBsdf ? 1.0f : absDot(surf.ns, wi)));
        ray = rayOffseted(pos, wi);
        float dist;
        int nextId = bvhHit(sc, ray, dist);
        int lightId = nextId - sc.objPrimCount;
        vec3 nextPos = rayPoint(ray, dist);
        if (nextId == -1) {
            vec3 radiance = envLe(sc, wi);
            float weight = 1.0f;
            if (sc.sampleLight && !deltaBsdf) {
                float envPdf = envPdfLi(sc, wi) * pdfSelectEnv(sc);
                weight = (envPdf <= 0.0f) ? 0.0f : biHeuristic(bsdfPdf, envPdf);
            }
            result = result + radiance * throughput * weight;
            break;
        } else if (lightId >= 0) {
            vec3 radiance = lightLe(sc, lightId, nextPos, -wi);
            float weight = 1.0f;
            if (sc.sampleLight && !deltaBsdf) {
                float lightPdf = lightPdfLi(sc, lightId, pos, nextPos) * pdfSelectLight(sc, lightId);
                weight = (lightPdf <= 0.0f) ? 0.0f : biHeuristic(bsdfPdf, lightPdf);
            }
            result = result + radiance * throughput * weight;
            break;
        }
        if (sc.russianRoulette && bounce >= sc.rrStartDepth) {
            float continueProb = fmin_(maxComponent(bsdf / bsdfPdf), 0.95f);
            if (sample1D(sc, g, s) >= continueProb) break;
            throughput = throughput / continueProb;
        }
        id = nextId;
        pos = nextPos;
        wo = -wi;
    }
    return result;
}

// The path of pathIntegTrace with every sampling decision of the scene `sc`
// (directions, lobe picks, pdfs, MIS weights, Russian roulette) but the BSDF
// values of the materials `mat1`: the estimator whose derivative in mat1 the
// path-replay adjoint computes (sampling detached).  Finite differences of it
// over mat1 check the adjoint's material gradients, roughness and metallic
// included, independently of its own formulation.
vec3 pathFrozen(const OrcScene& sc, const float* mat1, Ray ray, int& s, Rng& g) {
    OrcScene sc1 = sc;
    sc1.materials = mat1;
    float primDist;
    int id = bvhHit(sc, ray, primDist);
    vec3 pos = rayPoint(ray, primDist);
    if (id == -1) return envLe(sc, ray.dir);
    if (id - sc.objPrimCount >= 0) return lightLe(sc, id - sc.objPrimCount, pos, -ray.dir);
    vec3 wo = -ray.dir;
    vec3 result(0.0f), throughput(1.0f);
    for (int bounce = 1; bounce <= sc.maxDepth; bounce++) {
        SurfaceInfo surf = triangleSurfaceInfo(sc, id, pos);
        int matTexId = sc.matTexIndex[id];
        int matId = matTexId & 0x0000ffff;
        uint32_t matType = loadMaterialType(sc, matId);
        if (matType != Dielectric && matType != ThinDielectric) {
            if (dot(surf.ns, wo) < 0.0f) {
                surf.ns = -surf.ns;
                surf.ng = -surf.ng;
            }
        }
        BSDFParam mp = loadMaterial(sc, matType, matId);
        BSDFParam mp1 = loadMaterial(sc1, matType, matId);
        applyTexture(sc, sc.matTexIndex[id], surf, mp);
        applyTexture(sc, sc.matTexIndex[id], surf, mp1);
        if (sc.sampleLight) {
            float ud = sample1D(sc, g, s);
            float u0 = sample1D(sc, g, s), u1 = sample1D(sc, g, s), u2 = sample1D(sc, g, s), u3 = sample1D(sc, g, s);
            LightLiSample ls = sampleLightAndEnv(sc, pos, ud, u0, u1, u2, u3);
            if (ls.pdf > 0.0f) {
                vec3 f1 = materialBSDF(matType, mp1, wo, ls.wi, surf.ns);
                float fpdf = materialPdf(matType, mp, wo, ls.wi, surf.ns);
                float weight = biHeuristic(ls.pdf, fpdf);
                result = result + f1 * throughput * satDot(surf.ns, ls.wi) * ls.coef * weight;
            }
        }
        float b0 = sample1D(sc, g, s), b1 = sample1D(sc, g, s), b2 = sample1D(sc, g, s);
        BSDFSample bs = materialSample(matType, mp, surf.ns, wo, vec3(b0, b1, b2), g);
        vec3 wi = bs.wi;
        float bsdfPdf = bs.pdf;
        bool deltaBsdf = (bs.flag == SpecRefl || bs.flag == SpecTrans);
        if (bsdfPdf < 1e-8f) break;
        vec3 bsdf1 = deltaBsdf ? bs.bsdf : materialBSDF(matType, mp1, wo, wi, surf.ns);
        throughput = throughput * (bsdf1 / bsdfPdf * (deltaBsdf ? 1.0f : absDot(surf.ns, wi)));
        ray = rayOffseted(pos, wi);
        float dist;
        int nextId = bvhHit(sc, ray, dist);
        int lightId = nextId - sc.objPrimCount;
        vec3 nextPos = rayPoint(ray, dist);
        if (nextId == -1) {
            vec3 radiance = envLe(sc, wi);
            float weight = 1.0f;
            if (sc.sampleLight && !deltaBsdf) {
                float envPdf = envPdfLi(sc, wi) * pdfSelectEnv(sc);
                weight = (envPdf <= 0.0f) ? 0.0f : biHeuristic(bsdfPdf, envPdf);
            }
            result = result + radiance * throughput * weight;
            break;
        } else if (lightId >= 0) {
            vec3 radiance = lightLe(sc, lightId, nextPos, -wi);
            float weight = 1.0f;
            if (sc.sampleLight && !deltaBsdf) {
                float lightPdf = lightPdfLi(sc, lightId, pos, nextPos) * pdfSelectLight(sc, lightId);
                weight = (lightPdf <= 0.0f) ? 0.0f : biHeuristic(bsdfPdf, lightPdf);
            }
            result = result + radiance * throughput * weight;
            break;
        }
        if (sc.russianRoulette && bounce >= sc.rrStartDepth) {
            float continueProb = fmin_(maxComponent(bs.bsdf / bsdfPdf), 0.95f);
            if (sample1D(sc, g, s) >= continueProb) break;
            throughput = throughput / continueProb;
        }
        id = nextId;
        pos = nextPos;
        wo = -wi;
    }
    return result;
}

// ---------------------------------------------- camera importance (camera.glsl)
inline bool inFilmBound(vec2 uv) { return uv.x >= 0.0f && uv.x <= 1.0f && uv.y >= 0.0f && uv.y <= 1.0f; }
inline bool thinLensCameraDelta(const OrcScene& sc) { return sc.lensRadius <= 1e-6f; }
inline vec2 thinLensCameraRasterPos(const OrcScene& sc, const Ray& ray) {  // camera.glsl:79-91
    float cosTheta = dot(ray.dir, cv(sc.camF));
    float dFocus = sc.focalDist / cosTheta;
    mat3 inv{vec3(sc.camMatInv[0], sc.camMatInv[1], sc.camMatInv[2]),
             vec3(sc.camMatInv[3], sc.camMatInv[4], sc.camMatInv[5]),
             vec3(sc.camMatInv[6], sc.camMatInv[7], sc.camMatInv[8])};
    vec3 pFocus = mul(inv, rayPoint(ray, dFocus) - cv(sc.camPos));
    vec2 filmSize((float)sc.filmW, (float)sc.filmH);
    float aspect = filmSize.x / filmSize.y;
    vec3 div = vec3(aspect * sc.tanFOV * sc.focalDist, 1.0f * sc.tanFOV * sc.focalDist, 1.0f * sc.focalDist);
    pFocus = pFocus / div;
    return vec2((pFocus.x + 1.0f) * 0.5f, (pFocus.y + 1.0f) * 0.5f);
}
inline vec3 thinLensCameraIe(const OrcScene& sc, const Ray& ray) {  // camera.glsl:93-107
    float cosTheta = dot(ray.dir, cv(sc.camF));
    if (cosTheta < 1e-6f) return vec3(0.0f);
    vec2 pRaster = thinLensCameraRasterPos(sc, ray);
    if (!inFilmBound(pRaster)) return vec3(0.0f);
    float tanFOVInv = 1.0f / sc.tanFOV;
    float cos2Theta = cosTheta * cosTheta;
    float lensArea = thinLensCameraDelta(sc) ? 1.0f : Pi * sc.lensRadius * sc.lensRadius;
    return vec3(0.25f) * square(tanFOVInv / cos2Theta) / (lensArea * sc.camAsp);
}
struct CameraIiSample {
    vec3 wi, Ii;
    float dist;
    vec2 uv;
    float pdf;
};
inline CameraIiSample thinLensCameraSampleIi(const OrcScene& sc, vec3 ref, vec2 u) {  // camera.glsl:109-127
    vec2 l = toConcentricDisk(u) * sc.lensRadius;
    vec3 pLens(l.x, l.y, 0.0f);
    vec3 y = cv(sc.camPos) + cv(sc.camR) * pLens.x + cv(sc.camU) * pLens.y + cv(sc.camF) * pLens.z;
    float dist = distance(ref, y);
    vec3 wi = normalize(y - ref);
    float cosTheta = satDot(cv(sc.camF), -wi);
    if (cosTheta < 1e-6f) return CameraIiSample{vec3(0.0f), vec3(0.0f), 0.0f, vec2(0.0f), 0.0f};
    Ray ray{y, -wi};
    vec3 Ie = thinLensCameraIe(sc, ray);
    vec2 uv = thinLensCameraRasterPos(sc, ray);
    float lensArea = thinLensCameraDelta(sc) ? 1.0f : Pi * sc.lensRadius * sc.lensRadius;
    float pdf = dist * dist / (cosTheta * lensArea);
    return CameraIiSample{wi, Ie, dist, uv, pdf};
}
struct CamPdf {
    float pdfPos, pdfDir;
};
inline CamPdf thinLensCameraPdfIe(const OrcScene& sc, const Ray& ray) {  // camera.glsl:129-141
    float cosTheta = dot(cv(sc.camF), ray.dir);
    if (cosTheta < 1e-6f) return CamPdf{0.0f, 0.0f};
    vec2 pRaster = thinLensCameraRasterPos(sc, ray);
    if (!inFilmBound(pRaster)) return CamPdf{0.0f, 0.0f};
    float pdfPos = thinLensCameraDelta(sc) ? 1.0f : 1.0f / (Pi * sc.lensRadius * sc.lensRadius);
    float pdfDir = 1.0f / (cosTheta * cosTheta * cosTheta);
    return CamPdf{pdfPos, pdfDir};
}

// ------------------------------------------------------- light emission (light.glsl)
struct LightLeSample {
    Ray ray;
    vec3 Le;
    float pdfPos, pdfDir;
};
inline LightLeSample lightSampleOneLe(const OrcScene& sc, int id, float u0, float u1, float u2, float u3) {
    int triId = id + sc.objPrimCount;  // light.glsl:111-120
    vec3 ori = triangleSampleUniform(sc, triId, vec2(u0, u1));
    vec3 norm = triangleSurfaceInfo(sc, triId, ori).ng;
    vec4r samp = sampleCosineWeighted(norm, vec2(u2, u3));
    return LightLeSample{rayOffseted(ori, samp.v), lightLe(sc, id, ori, samp.v), 1.0f / triangleArea(sc, triId), samp.w};
}
inline CamPdf lightPdfLe(const OrcScene& sc, int id, const Ray& ray) {  // light.glsl:100-109
    int triId = id + sc.objPrimCount;
    vec3 norm = triangleSurfaceInfo(sc, triId, ray.ori).ng;
    CamPdf r;
    r.pdfPos = 1.0f / triangleArea(sc, triId);
    r.pdfDir = (dot(norm, ray.dir) <= 0.0f) ? 0.0f : 0.5f * PiInv;
    return r;
}
inline vec3 triangleNormalShad(const OrcScene& sc, int id, vec3 p) {  // intersection.glsl:149-173
    uint32_t ia = sc.indices[3 * id], ib = sc.indices[3 * id + 1], ic = sc.indices[3 * id + 2];
    vec3 a = V(sc, ia), b = V(sc, ib), c = V(sc, ic);
    vec3 pa = a - p, pb = b - p, pc = c - p;
    float areaInv = 1.0f / length(cross(b - a, c - a));
    float la = length(cross(pb, pc)) * areaInv;
    float lb = length(cross(pc, pa)) * areaInv;
    float lc = 1.0f - la - lb;
    return normalize(N(sc, ia) * la + N(sc, ib) * lb + N(sc, ic) * lc);
}
inline bool visibleOrc(const OrcScene& sc, vec3 x, vec3 y) {  // intersection.glsl:429-433
    float dist = distance(x, y) - 2e-5f;
    vec3 wi = normalize(y - x);
    return !bvhTest(sc, Ray{x + wi * 1e-5f, wi}, dist);
}
inline float remap(float p) { return p < 1e-8f ? 1.0f : p * p; }

// Film of the light-tracing passes: float[H][W][3]; samples outside the film
// (or on its far edge, where int(uv * size) == size) are dropped like an
// out-of-range imageAtomicAdd.
inline void accumulateFilm(const OrcScene& sc, float* film, vec2 uv, vec3 res) {
    if (!inFilmBound(uv)) return;
    int x = f2i(uv.x * (float)sc.filmW), y = f2i(uv.y * (float)sc.filmH);
    if (x >= sc.filmW || y >= sc.filmH) return;
    float* p = film + 3 * ((size_t)y * sc.filmW + x);
    p[0] += res.x;
    p[1] += res.y;
    p[2] += res.z;
}

inline void loadSurface(const OrcScene& sc, int id, vec3 pos, vec3 wo, SurfaceInfo& surf, uint32_t& matType,
                        BSDFParam& mp) {
    surf = triangleSurfaceInfo(sc, id, pos);
    int matId = sc.matTexIndex[id] & 0x0000ffff;
    matType = loadMaterialType(sc, matId);
    if (matType != Dielectric && matType != ThinDielectric && dot(surf.ns, wo) < 0.0f) {
        surf.ns = -surf.ns;
        surf.ng = -surf.ng;
    }
    mp = loadMaterial(sc, matType, matId);
    applyTexture(sc, sc.matTexIndex[id], surf, mp);
}

// lightIntegTrace (light_path_integ.glsl:45-146); rand() stream only.
void lightIntegTrace(const OrcScene& sc, Rng& g, float* film) {
    float a0 = rand01(g), a1 = rand01(g);
    int light = lightSampleOne(sc, vec2(a0, a1));
    float pdfSource = lightPdfSampleOne(sc, light);
    Ray ray;
    vec3 wo, throughput;
    {
        int triId = light + sc.objPrimCount;
        float b0 = rand01(g), b1 = rand01(g);
        vec3 pLit = triangleSampleUniform(sc, triId, vec2(b0, b1));
        float c0 = rand01(g), c1 = rand01(g);
        CameraIiSample ci = thinLensCameraSampleIi(sc, pLit, vec2(c0, c1));
        if (ci.pdf > 0.0f) {
            vec3 pCam = pLit + ci.wi * ci.dist;
            float pdfPos = 1.0f / triangleArea(sc, triId);
            if (visibleOrc(sc, pLit, pCam)) {
                vec3 Le = lightLe(sc, light, pLit, ci.wi);
                vec3 contrib = Le * ci.Ii / (ci.pdf * pdfPos * pdfSource);
                if (!isBlack(contrib)) accumulateFilm(sc, film, ci.uv, contrib);
            }
        }
        float d0 = rand01(g), d1 = rand01(g), d2 = rand01(g), d3 = rand01(g);
        LightLeSample le = lightSampleOneLe(sc, light, d0, d1, d2, d3);
        vec3 nl = triangleSurfaceInfo(sc, triId, le.ray.ori).ng;
        wo = -le.ray.dir;
        ray = rayOffseted(le.ray.ori, le.ray.dir);
        throughput = le.Le * absDot(nl, -wo) / (pdfSource * le.pdfPos * le.pdfDir);
    }
    for (int bounce = 1; bounce <= sc.maxDepth; bounce++) {
        float dist;
        int id = bvhHit(sc, ray, dist);
        if (id == -1) break;
        if (id - sc.objPrimCount >= 0) break;
        vec3 pos = rayPoint(ray, dist);
        SurfaceInfo surf;
        uint32_t matType;
        BSDFParam mp;
        loadSurface(sc, id, pos, wo, surf, matType, mp);
        {
            float c0 = rand01(g), c1 = rand01(g);
            CameraIiSample ci = thinLensCameraSampleIi(sc, pos, vec2(c0, c1));
            if (ci.pdf > 0.0f) {
                vec3 pCam = pos + ci.wi * ci.dist;
                if (visibleOrc(sc, pos, pCam)) {
                    vec3 bsdf = materialBSDF(matType, mp, wo, ci.wi, surf.ns, Importance);  // light_path_integ.glsl:113
                    float cosWi = satDot(surf.ng, ci.wi) * std::fabs(dot(surf.ns, wo) / dot(surf.ng, wo));
                    vec3 res = ci.Ii * bsdf * throughput * cosWi / ci.pdf;
                    if (!hasNan(res) && !std::isnan(ci.pdf) && ci.pdf > 1e-8f && !isBlack(res))
                        accumulateFilm(sc, film, ci.uv, res);
                }
            }
        }
        float b0 = rand01(g), b1 = rand01(g), b2 = rand01(g);
        BSDFSample bs = materialSample(matType, mp, surf.ns, wo, vec3(b0, b1, b2), g, Importance);
        vec3 wi = bs.wi;
        float bsdfPdf = bs.pdf;
        bool deltaBsdf = (bs.flag == SpecRefl || bs.flag == SpecTrans);
        if (bsdfPdf < 1e-8f || std::isnan(bsdfPdf)) break;
        if (sc.russianRoulette && bounce >= sc.rrStartDepth) {
            float continueProb = fmin_(maxComponent(bs.bsdf / bsdfPdf), 1.0f);
            if (rand01(g) >= continueProb) break;
            throughput = throughput / continueProb;
        }
        float cosWi = deltaBsdf ? 1.0f : std::fabs(dot(surf.ng, wi) * dot(surf.ns, wo) / dot(surf.ng, wo));
        throughput = throughput * (bs.bsdf * cosWi / bsdfPdf);
        ray = rayOffseted(pos, wi);
        wo = -wi;
    }
}

inline float weightS0(float s1s0, float t1s0) { return 1.0f / (1.0f + s1s0 + t1s0); }
inline float weightS1(float s1s0, float t1s1) { return s1s0 / (1.0f + s1s0 + s1s0 * t1s1); }
inline float weightT1(float s0t1, float s1t1) { return 1.0f / (s0t1 + s1t1 + 1.0f); }

// traceCameraPath (triple_path_pass_pt.glsl:59-195)
vec3 traceCameraPath(const OrcScene& sc, Ray ray, Rng& g, int& s) {
    float primDist;
    int id = bvhHit(sc, ray, primDist);
    vec3 pos = rayPoint(ray, primDist);
    if (id == -1) return envLe(sc, ray.dir);
    if (id - sc.objPrimCount >= 0) return lightLe(sc, id - sc.objPrimCount, pos, -ray.dir);
    SurfaceInfo surf = triangleSurfaceInfo(sc, id, pos);
    vec3 wo = -ray.dir;
    vec3 prevNorm = cv(sc.camF);
    vec3 result(0.0f), throughput(1.0f);
    CamPdf camPdf = thinLensCameraPdfIe(sc, ray);
    float primaryPdf = remap(camPdf.pdfPos) / remap(camPdf.pdfDir * absDot(surf.ns, ray.dir) / square(primDist));
    float t1s0 = primaryPdf, t1s1 = primaryPdf;
    for (int bounce = 1; bounce <= sc.maxDepth; bounce++) {
        if (bounce > 1) surf = triangleSurfaceInfo(sc, id, pos);
        int matId = sc.matTexIndex[id] & 0x0000ffff;
        uint32_t matType = loadMaterialType(sc, matId);
        if (matType != Dielectric && matType != ThinDielectric && dot(surf.ns, wo) < 0.0f) {
            surf.ns = -surf.ns;
            surf.ng = -surf.ng;
        }
        BSDFParam mp = loadMaterial(sc, matType, matId);
        applyTexture(sc, sc.matTexIndex[id], surf, mp);
        {
            float a0 = sample1D(sc, g, s), a1 = sample1D(sc, g, s);
            int light = lightSampleOne(sc, vec2(a0, a1));
            int triId = light + sc.objPrimCount;
            float pdfSource = lightPdfSampleOne(sc, light);
            float b0 = sample1D(sc, g, s), b1 = sample1D(sc, g, s);
            vec3 pLit = triangleSampleUniform(sc, triId, vec2(b0, b1));
            vec3 wi = normalize(pLit - pos);
            vec3 Le = lightLe(sc, light, pLit, -wi);
            if (!isBlack(Le) && visibleOrc(sc, pos, pLit)) {
                vec3 nLit = triangleSurfaceInfo(sc, triId, pLit).ng;
                float pA = pdfSource / triangleArea(sc, triId);
                float dist2 = distSquare(pos, pLit);
                float pS = pA * dist2 / absDot(nLit, wi);
                vec3 f = materialBSDF(matType, mp, wo, wi, surf.ns);
                float fpdf = materialPdf(matType, mp, wo, wi, surf.ns);
                float pdfRev = materialPdf(matType, mp, wi, wo, surf.ns);
                float pdfPLit = remap(pA);
                float coefToSurf = remap(0.5f * PiInv * absDot(surf.ns, wi));
                float coefToLight = remap(fpdf * satDot(nLit, -wi));
                float coefToPrev = (bounce == 1) ? 1.0f : remap(pdfRev * absDot(prevNorm, wo));
                float coefDist = remap(dist2);
                float weight = weightS1(pdfPLit * coefDist / coefToLight, t1s1 * coefToSurf * coefToPrev / coefDist);
                result = result + Le * f * throughput * absDot(surf.ns, wi) / pS * weight;
            }
        }
        float b0 = sample1D(sc, g, s), b1 = sample1D(sc, g, s), b2 = sample1D(sc, g, s);
        BSDFSample bs = materialSample(matType, mp, surf.ns, wo, vec3(b0, b1, b2), g);
        vec3 wi = bs.wi;
        float bsdfPdf = bs.pdf;
        bool deltaBsdf = (bs.flag == SpecRefl || bs.flag == SpecTrans);
        if (bsdfPdf < 1e-8f) break;
        throughput = throughput * (bs.bsdf / bsdfPdf * (deltaBsdf ? 1.0f : absDot(surf.ns, wi)));
        Ray nextRay = rayOffseted(pos, wi);
        float dist;
        int nextId = bvhHit(sc, nextRay, dist);
        int lightId = nextId - sc.objPrimCount;
        vec3 nextPos = rayPoint(nextRay, dist);
        float pdfDirToNext = materialPdf(matType, mp, wo, wi, surf.ns);
        float pdfDirToPrev = materialPdf(matType, mp, wi, wo, surf.ns);
        if (nextId == -1) break;
        if (lightId >= 0) {
            vec3 nLit = triangleSurfaceInfo(sc, nextId, nextPos).ng;
            CamPdf pdfLit = lightPdfLe(sc, lightId, Ray{nextPos, -wi});
            float pdfPLit = remap(pdfLit.pdfPos * lightPdfSampleOne(sc, lightId));
            float coefToLight = remap(pdfDirToNext * satDot(nLit, -wi));
            float coefToSurf = remap(pdfLit.pdfDir * absDot(surf.ns, wi));
            float coefToPrev = (bounce == 1) ? 1.0f : remap(pdfDirToPrev * absDot(prevNorm, wo));
            float coefDist = remap(dist * dist);
            float weight = std::isnan(t1s0) ? 0.0f
                                            : weightS0(pdfPLit * coefDist / coefToLight,
                                                       t1s0 * coefToSurf * pdfPLit * coefToPrev / coefToLight);
            result = result + lightLe(sc, lightId, nextPos, -wi) * throughput * weight;
            break;
        }
        if (sc.russianRoulette && bounce >= sc.rrStartDepth) {
            float continueProb = fmin_(maxComponent(bs.bsdf / bsdfPdf), 0.95f);
            if (sample1D(sc, g, s) >= continueProb) break;
            throughput = throughput / continueProb;
        }
        float coef = ((bounce == 1) ? 1.0f : remap(pdfDirToPrev * absDot(prevNorm, wo))) /
                     remap(pdfDirToNext * absDot(triangleNormalShad(sc, nextId, nextPos), wi));
        t1s0 *= coef;
        t1s1 *= coef;
        prevNorm = surf.ns;
        pos = nextPos;
        wo = -wi;
        id = nextId;
    }
    return result;
}

// traceLightPath (triple_path_pass_lpt.glsl:58-182); contributions scaled by uScale.
void traceLightPath(const OrcScene& sc, Rng& g, float* film, float uScale) {
    float a0 = rand01(g), a1 = rand01(g);
    int light = lightSampleOne(sc, vec2(a0, a1));
    float pdfSource = lightPdfSampleOne(sc, light);
    Ray ray;
    vec3 wo, throughput, prevNorm;
    float prevPdfDir, s0t1, s1t1;
    {
        int triId = light + sc.objPrimCount;
        float b0 = rand01(g), b1 = rand01(g);
        (void)triangleSampleUniform(sc, triId, vec2(b0, b1));  // computed and unused by the reference
        float d0 = rand01(g), d1 = rand01(g), d2 = rand01(g), d3 = rand01(g);
        LightLeSample le = lightSampleOneLe(sc, light, d0, d1, d2, d3);
        vec3 nl = triangleSurfaceInfo(sc, triId, le.ray.ori).ng;
        wo = -le.ray.dir;
        ray = rayOffseted(le.ray.ori, le.ray.dir);
        throughput = le.Le * absDot(nl, -wo) / (pdfSource * le.pdfPos * le.pdfDir);
        prevNorm = nl;
        prevPdfDir = le.pdfDir;
        s0t1 = 1.0f / remap(le.pdfPos * pdfSource);
        s1t1 = 1.0f;
    }
    for (int bounce = 1; bounce <= sc.maxDepth; bounce++) {
        float dist;
        int id = bvhHit(sc, ray, dist);
        if (id == -1) break;
        if (id - sc.objPrimCount >= 0) break;
        vec3 pos = rayPoint(ray, dist);
        SurfaceInfo surf = triangleSurfaceInfo(sc, id, pos);
        int matId = sc.matTexIndex[id] & 0x0000ffff;
        uint32_t matType = loadMaterialType(sc, matId);
        if (matType != Dielectric && matType != ThinDielectric && dot(surf.ns, wo) < 0.0f) {
            surf.ns = -surf.ns;
            surf.ng = -surf.ng;
        }
        float coefToPos = remap(prevPdfDir * absDot(surf.ns, wo));
        s0t1 /= coefToPos;
        s1t1 /= coefToPos / (bounce == 1 ? remap(dist * dist) : 1.0f);
        BSDFParam mp = loadMaterial(sc, matType, matId);
        applyTexture(sc, sc.matTexIndex[id], surf, mp);
        {
            float c0 = rand01(g), c1 = rand01(g);
            CameraIiSample ci = thinLensCameraSampleIi(sc, pos, vec2(c0, c1));
            if (ci.pdf > 0.0f) {
                vec3 pCam = pos + ci.wi * ci.dist;
                if (visibleOrc(sc, pos, pCam)) {
                    float cosWi = satDot(surf.ng, ci.wi) * std::fabs(dot(surf.ns, wo) / dot(surf.ng, wo));
                    vec3 bsdf = materialBSDF(matType, mp, wo, ci.wi, surf.ns, Importance);  // triple_path_pass_lpt.glsl:129
                    vec3 contrib = ci.Ii * bsdf * throughput * cosWi / ci.pdf;
                    float coefToSurf = remap(thinLensCameraPdfIe(sc, Ray{pCam, -ci.wi}).pdfDir * satDot(surf.ns, ci.wi));
                    float coefToPrev = remap(materialPdf(matType, mp, ci.wi, wo, surf.ns) * absDot(prevNorm, wo));
                    float coefDist = remap(ci.dist * ci.dist);
                    float coef0 = coefToSurf * coefToPrev / coefDist;
                    float coef1 = ((bounce == 1) ? 1.0f : coefToPrev) * coefToSurf / coefDist;
                    float weight = weightT1(s0t1 * coef0, s1t1 * coef1);
                    vec3 res = contrib * weight;
                    if (!hasNan(res) && !std::isnan(ci.pdf) && ci.pdf > 1e-8f && !isBlack(res))
                        accumulateFilm(sc, film, ci.uv, res * uScale);
                }
            }
        }
        float b0 = rand01(g), b1 = rand01(g), b2 = rand01(g);
        BSDFSample bs = materialSample(matType, mp, surf.ns, wo, vec3(b0, b1, b2), g, Importance);
        vec3 wi = bs.wi;
        float bsdfPdf = bs.pdf;
        bool deltaBsdf = (bs.flag == SpecRefl || bs.flag == SpecTrans);
        if (bsdfPdf < 1e-8f || std::isnan(bsdfPdf)) break;
        if (sc.russianRoulette && bounce >= sc.rrStartDepth) {
            float continueProb = fmin_(maxComponent(bs.bsdf / bsdfPdf), 1.0f);
            if (rand01(g) >= continueProb) break;
            throughput = throughput / continueProb;
        }
        float coefToPrev = remap(materialPdf(matType, mp, wi, wo, surf.ns) * absDot(prevNorm, wo));
        s0t1 *= coefToPrev;
        s1t1 *= (bounce == 1) ? 1.0f : coefToPrev;
        prevPdfDir = materialPdf(matType, mp, wo, wi, surf.ns);
        prevNorm = surf.ns;
        float cosWi = deltaBsdf ? 1.0f : std::fabs(dot(surf.ng, wi) * dot(surf.ns, wo) / dot(surf.ng, wo));
        throughput = throughput * (bs.bsdf * cosWi / bsdfPdf);
        ray = rayOffseted(pos, wi);
        wo = -wi;
    }
}

// Per-pixel seeds: noise = tex(noise, tex(noise, coord / size)) with bilinear
// filtering and repeat wrap at GL texel centres (path_integ_naive.glsl:156-160).
inline vec2 noiseTexel(const OrcScene& sc, int x, int y) {
    int W = sc.filmW, H = sc.filmH;
    x %= W;
    if (x < 0) x += W;
    y %= H;
    if (y < 0) y += H;
    const float* t = sc.noise + 2 * ((size_t)y * W + x);
    return vec2(t[0], t[1]);
}
inline vec2 mix2(vec2 a, vec2 b, float t) { return vec2(a.x * (1.0f - t) + b.x * t, a.y * (1.0f - t) + b.y * t); }
inline vec2 noiseTexture(const OrcScene& sc, vec2 st) {
    float u = st.x * (float)sc.filmW - 0.5f;
    float v = st.y * (float)sc.filmH - 0.5f;
    float fu = std::floor(u), fv = std::floor(v);
    float au = u - fu, av = v - fv;
    int x0 = f2i(fu), y0 = f2i(fv);
    vec2 t00 = noiseTexel(sc, x0, y0), t10 = noiseTexel(sc, x0 + 1, y0);
    vec2 t01 = noiseTexel(sc, x0, y0 + 1), t11 = noiseTexel(sc, x0 + 1, y0 + 1);
    return mix2(mix2(t00, t10, au), mix2(t01, t11, au), av);
}

// main() of path_integ_naive.glsl:145-174 for one pixel and one pass.
vec3 renderPixel(const OrcScene& sc, int px, int py, int spp, int freeCounter, bool& valid,
                 const float* frozenMat = nullptr) {
    vec2 texSize((float)sc.filmW, (float)sc.filmH);
    vec2 scr = vec2((float)px, (float)py) / texSize;
    vec2 nc = noiseTexture(sc, scr);
    nc = noiseTexture(sc, nc);
    vec2 tc = texSize * nc;
    Rng g;
    g.randSeed = f2u(tc.x) * (uint32_t)freeCounter + f2u(tc.y);
    g.sampleSeed = f2u(tc.x) * f2u(tc.y);
    const int sampleNum = 131072, sampleDim = 256;
    int off = (int)((uint32_t)spp * (uint32_t)sampleDim);
    if (off > sampleNum * sampleDim) off -= sampleNum * sampleDim;
    g.sampleOffset = off;
    int s = 0;
    float u0 = sample1D(sc, g, s), u1 = sample1D(sc, g, s), u2 = sample1D(sc, g, s), u3 = sample1D(sc, g, s);
    Ray ray = thinLensCameraSampleRay(sc, scr, u0, u1, u2, u3);
    vec3 r = frozenMat ? pathFrozen(sc, frozenMat, ray, s, g) : pathIntegTrace(sc, ray, s, g);
    valid = !hasNan(r);
    return r;
}

// ------------------------------------------------- adjoint of the path tracer
// The gradient oracle of the differentiable renderer.  Every contribution C
// of a path (light sample, emitter hit, environment) is a product of the
// sampled BSDF values along the path, the BSDF value of its own light
// sample, and emitted radiance (linear in its light instance's power), with
// pdfs, MIS weights and Russian roulette held fixed.  Its derivative is
// therefore C * (sum of dlog f over those BSDF values) plus C / P for the
// power P of its emitter, accumulated here in double precision per
// contribution.  BSDF log-derivatives are central differences of a double
// precision evaluation of the same BRDF formulas (material.glsl:357-490).

struct D3 {
    double x, y, z;
};
inline D3 d3(vec3 a) { return D3{a.x, a.y, a.z}; }
inline D3 operator+(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(D3 a, D3 b) { return D3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline D3 operator*(D3 a, double t) { return D3{a.x * t, a.y * t, a.z * t}; }
inline D3 operator/(D3 a, double t) { return D3{a.x / t, a.y / t, a.z / t}; }
inline double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 dnormalize(D3 a) { return a / std::sqrt(ddot(a, a)); }
inline D3 dmix(D3 a, D3 b, double t) { return a * (1.0 - t) + b * t; }
inline double dpow5(double x) { return x * x * x * x * x; }
inline double dschlickG(double c, double alpha) { return c / (c * (1.0 - alpha * 0.5) + alpha * 0.5); }

const double kPiD = 3.14159265358979323846;

// principledBRDF with the differentiable values q = (baseColor rgb, raw
// roughness, metallic, specular) and the rest of the record from m.
D3 principledD(const float* m, const double* q, D3 wo, D3 wi, D3 n) {
    const D3 base{q[0], q[1], q[2]}, one{1.0, 1.0, 1.0};
    const double rough = 0.0134 * (1.0 - q[3]) + q[3];
    const double subsurface = m[4], metallic = q[4], specular = q[5], specTint = m[7];
    const double sheen = m[8], sheenTint = m[9], clearcoat = m[10], ccGloss = m[11];
    const double alpha = rough * rough, a2 = alpha * alpha;
    const double ccAlpha = 0.1 * (1.0 - ccGloss) + 0.001 * ccGloss;
    const double lum = base.x * 0.299 + base.y * 0.587 + base.z * 0.114;
    const D3 tint = lum > 0.0 ? base / lum : one;
    const D3 fm0 = dmix(dmix(one, tint, specTint) * (0.08 * specular), base, metallic);
    const double cosWo = std::max(ddot(n, wo), 0.0), cosWi = std::max(ddot(n, wi), 0.0);
    const D3 h = dnormalize(wo + wi);
    const double hCosWi = ddot(h, wi);
    D3 res{0.0, 0.0, 0.0};
    if (!(cosWo < 1e-10 || cosWi < 1e-10)) {
        // diffuse with the subsurface mix, times (1 - metallic)
        const double hc2 = hCosWi * hCosWi;
        const double fi = dpow5(1.0 - cosWi), fo = dpow5(1.0 - cosWo);
        const double fd90 = 0.5 + 2.0 * rough * hc2;
        const double fd = ((1.0 - fi) + fd90 * fi) * ((1.0 - fo) + fd90 * fo);
        const double fss90 = rough * hc2;
        const double fss = ((1.0 - fi) + fss90 * fi) * ((1.0 - fo) + fss90 * fo);
        const double ss = 1.25 * (fss * (1.0 / (cosWi + cosWo) - 0.5) + 0.5);
        res = res + base * ((fd * (1.0 - subsurface) + ss * subsurface) / kPiD * (1.0 - metallic));
        // metal: Schlick Fresnel, GGX, Smith-Schlick G
        const double w5 = dpow5(1.0 - std::fabs(ddot(h, wo)));
        const D3 fm = fm0 + (one - fm0) * w5;
        const double c = ddot(n, h);
        double dm = 0.0;
        if (!(c < 1e-6)) {
            const double den = c * c * (a2 - 1.0) + 1.0;
            dm = a2 / (den * den * kPiD);
        }
        const double gm = dschlickG(std::fabs(ddot(n, wo)), alpha) * dschlickG(std::fabs(ddot(n, wi)), alpha);
        const double denom = 4.0 * cosWi * cosWo;
        if (!(denom < 1e-7)) res = res + fm * (dm * gm / denom);
    }
    if (!(cosWo < 1e-6 || cosWi < 1e-6)) {  // clearcoat
        const double w5 = dpow5(1.0 - std::fabs(ddot(h, wo)));
        const D3 fc = base + (one - base) * w5;
        const double c = std::max(ddot(n, h), 0.0), ca2 = ccAlpha * ccAlpha;
        const double dc = (ca2 - 1.0) / (2.0 * kPiD * std::log(ccAlpha) * (1.0 + (ca2 - 1.0) * c * c));
        const double gc = dschlickG(std::fabs(ddot(n, wo)), 0.25) * dschlickG(std::fabs(ddot(n, wi)), 0.25);
        const double denom = 4.0 * cosWi * cosWo;
        if (!(denom < 1e-7)) res = res + fc * (dc * gc / denom * clearcoat * 0.25);
    }
    const double sheenScale = dpow5(1.0 - hCosWi) * sheen * (ddot(n, wi) < 0.0 ? 0.0 : 1.0);
    res = res + dmix(one, tint, sheenTint) * sheenScale;
    return res;
}

// out[i][c] = (d f_c / d q_i) / f_c for the BSDF value of material matId.
// A textured triangle (tex != nullptr: its texture colour) has no base
// colour parameter: those entries stay zero and the others are taken at the
// texture colour.
void bsdfLogGrad(const OrcScene& sc, int matId, vec3 wo, vec3 wi, vec3 n, double out[6][3],
                 const vec3* tex = nullptr) {
    const float* m = sc.materials + 16 * matId;
    for (int i = 0; i < 6; i++) out[i][0] = out[i][1] = out[i][2] = 0.0;
    const uint32_t type = loadMaterialType(sc, matId);
    if (type != PrincipledBRDF && type != Lambertian) return;  // no differentiable parameters
    if (type == Lambertian) {
        if (!tex)
            for (int c = 0; c < 3; c++) out[c][c] = m[c] != 0.0f ? 1.0 / (double)m[c] : 0.0;
        return;
    }
    const D3 o = d3(wo), i3 = d3(wi), nn = d3(n);
    double q[6] = {m[0], m[1], m[2], m[3], m[5], m[6]};
    if (tex) {
        q[0] = tex->x;
        q[1] = tex->y;
        q[2] = tex->z;
    }
    const D3 f = principledD(m, q, o, i3, nn);
    const double fv[3] = {f.x, f.y, f.z};
    for (int i = 0; i < 6; i++) {
        const double q0 = q[i], h = 1e-6 * std::max(1.0, std::fabs(q0));
        q[i] = q0 + h;
        const D3 fp = principledD(m, q, o, i3, nn);
        q[i] = q0 - h;
        const D3 fmn = principledD(m, q, o, i3, nn);
        q[i] = q0;
        const double dv[3] = {(fp.x - fmn.x) / (2 * h), (fp.y - fmn.y) / (2 * h), (fp.z - fmn.z) / (2 * h)};
        for (int c = 0; c < 3; c++) out[i][c] = fv[c] != 0.0 ? dv[c] / fv[c] : 0.0;
    }
    if (tex)
        for (int i = 0; i < 3; i++) out[i][0] = out[i][1] = out[i][2] = 0.0;
}

struct AdjCtx {
    const int32_t* lightInst;  // per light triangle: its instance
    const float* instPower;    // 3 per instance
    int nmat;
    double delta[3];           // d loss / d sample radiance
    std::vector<double> A;     // nmat*6*3: sum of dlog f of the path's sampled BSDF values
    double* grad;              // nmat*6 + 3*ninst
};

void addContribution(AdjCtx& cx, vec3 C, const double (*local)[3], int localMat, int lightId) {
    const double Cc[3] = {C.x, C.y, C.z};
    for (int m = 0; m < cx.nmat; m++)
        for (int i = 0; i < 6; i++) {
            double g = 0.0;
            for (int c = 0; c < 3; c++) {
                double l = cx.A[(size_t)(6 * m + i) * 3 + c] + (local && m == localMat ? local[i][c] : 0.0);
                g += cx.delta[c] * Cc[c] * l;
            }
            cx.grad[6 * m + i] += g;
        }
    if (lightId >= 0) {
        const int k = cx.lightInst[lightId];
        for (int c = 0; c < 3; c++) {
            const double P = cx.instPower[3 * k + c];
            if (P != 0.0) cx.grad[6 * cx.nmat + 3 * k + c] += cx.delta[c] * Cc[c] / P;
        }
    }
}

// pathIntegTrace (path_integ_naive.glsl:35-143) with the same sample
// consumption, feeding every contribution to addContribution.
void pathAdjoint(const OrcScene& sc, Ray ray, int& s, Rng& g, AdjCtx& cx) {
    std::fill(cx.A.begin(), cx.A.end(), 0.0);
    float primDist;
    int id = bvhHit(sc, ray, primDist);
    vec3 pos = rayPoint(ray, primDist);
    if (id == -1) return;
    if (id - sc.objPrimCount >= 0) {
        addContribution(cx, lightLe(sc, id - sc.objPrimCount, pos, -ray.dir), nullptr, -1, id - sc.objPrimCount);
        return;
    }
    vec3 wo = -ray.dir;
    vec3 throughput(1.0f);
    double lg[6][3];
    for (int bounce = 1; bounce <= sc.maxDepth; bounce++) {
        SurfaceInfo surf = triangleSurfaceInfo(sc, id, pos);
        int matId = sc.matTexIndex[id] & 0x0000ffff;
        uint32_t matType = loadMaterialType(sc, matId);
        if (matType != Dielectric && matType != ThinDielectric && dot(surf.ns, wo) < 0.0f) {
            surf.ns = -surf.ns;
            surf.ng = -surf.ng;
        }
        BSDFParam mp = loadMaterial(sc, matType, matId);
        applyTexture(sc, sc.matTexIndex[id], surf, mp);
        vec3 texC = mp.baseColor;
        const vec3* texColor = (sc.matTexIndex[id] >> 16) != -1 ? &texC : nullptr;
        if (sc.sampleLight) {
            float ud = sample1D(sc, g, s);
            float u0 = sample1D(sc, g, s), u1 = sample1D(sc, g, s), u2 = sample1D(sc, g, s), u3 = sample1D(sc, g, s);
            float pdfSampleLight = 0.0f;
            if (sc.nLightTriangles > 0)
                pdfSampleLight = sc.lightEnvUniformSample ? sc.lightPortion : sc.lightSum / (sc.lightSum + sc.envSum);
            int lid = ud < pdfSampleLight ? lightSampleOne(sc, vec2(u0, u1)) : -1;
            LightLiSample ls = sampleLightAndEnv(sc, pos, ud, u0, u1, u2, u3);
            if (ls.pdf > 0.0f) {
                vec3 f = materialBSDF(matType, mp, wo, ls.wi, surf.ns);
                float fpdf = materialPdf(matType, mp, wo, ls.wi, surf.ns);
                float weight = biHeuristic(ls.pdf, fpdf);
                vec3 C = f * throughput * satDot(surf.ns, ls.wi) * ls.coef * weight;
                bsdfLogGrad(sc, matId, wo, ls.wi, surf.ns, lg, texColor);
                addContribution(cx, C, lg, matId, lid);
            }
        }
        float b0 = sample1D(sc, g, s), b1 = sample1D(sc, g, s), b2 = sample1D(sc, g, s);
        BSDFSample bs = materialSample(matType, mp, surf.ns, wo, vec3(b0, b1, b2), g);
        vec3 wi = bs.wi;
        float bsdfPdf = bs.pdf;
        bool deltaBsdf = (bs.flag == SpecRefl || bs.flag == SpecTrans);
        if (bsdfPdf < 1e-8f) break;
        bsdfLogGrad(sc, matId, wo, wi, surf.ns, lg, texColor);
        for (int i = 0; i < 6; i++)
            for (int c = 0; c < 3; c++) cx.A[(size_t)(6 * matId + i) * 3 + c] += lg[i][c];
        throughput = throughput * (bs.bsdf / bsdfPdf * (deltaBsdf ? 1.0f : absDot(surf.ns, wi)));
        ray = rayOffseted(pos, wi);
        float dist;
        int nextId = bvhHit(sc, ray, dist);
        int lightId = nextId - sc.objPrimCount;
        vec3 nextPos = rayPoint(ray, dist);
        if (nextId == -1) {
            vec3 radiance = envLe(sc, wi);
            float weight = 1.0f;
            if (sc.sampleLight && !deltaBsdf) {
                float envPdf = envPdfLi(sc, wi) * pdfSelectEnv(sc);
                weight = (envPdf <= 0.0f) ? 0.0f : biHeuristic(bsdfPdf, envPdf);
            }
            addContribution(cx, radiance * throughput * weight, nullptr, -1, -1);
            break;
        } else if (lightId >= 0) {
            vec3 radiance = lightLe(sc, lightId, nextPos, -wi);
            float weight = 1.0f;
            if (sc.sampleLight && !deltaBsdf) {
                float lightPdf = lightPdfLi(sc, lightId, pos, nextPos) * pdfSelectLight(sc, lightId);
                weight = (lightPdf <= 0.0f) ? 0.0f : biHeuristic(bsdfPdf, lightPdf);
            }
            addContribution(cx, radiance * throughput * weight, nullptr, -1, lightId);
            break;
        }
        if (sc.russianRoulette && bounce >= sc.rrStartDepth) {
            float continueProb = fmin_(maxComponent(bs.bsdf / bsdfPdf), 0.95f);
            if (sample1D(sc, g, s) >= continueProb) break;
            throughput = throughput / continueProb;
        }
        id = nextId;
        pos = nextPos;
        wo = -wi;
    }
}

// One sample of renderPixel replayed through pathAdjoint.
void pixelAdjoint(const OrcScene& sc, int px, int py, int spp, int freeCounter, AdjCtx& cx) {
    vec2 texSize((float)sc.filmW, (float)sc.filmH);
    vec2 scr = vec2((float)px, (float)py) / texSize;
    vec2 nc = noiseTexture(sc, scr);
    nc = noiseTexture(sc, nc);
    vec2 tc = texSize * nc;
    Rng g;
    g.randSeed = f2u(tc.x) * (uint32_t)freeCounter + f2u(tc.y);
    g.sampleSeed = f2u(tc.x) * f2u(tc.y);
    const int sampleNum = 131072, sampleDim = 256;
    int off = (int)((uint32_t)spp * (uint32_t)sampleDim);
    if (off > sampleNum * sampleDim) off -= sampleNum * sampleDim;
    g.sampleOffset = off;
    int s = 0;
    float u0 = sample1D(sc, g, s), u1 = sample1D(sc, g, s), u2 = sample1D(sc, g, s), u3 = sample1D(sc, g, s);
    Ray ray = thinLensCameraSampleRay(sc, scr, u0, u1, u2, u3);
    pathAdjoint(sc, ray, s, g, cx);
}

}  // namespace

extern "C" {

// Renders `passes` consecutive progressive passes (spp = spp0 + p,
// freeCounter = fc0 + p) of the MIS path tracer for the listed pixels and
// accumulates into out_rgb[npix*3] like imageStore(lastRes + result) does,
// skipping NaN samples.
static void render_pt_impl(const OrcScene* sc, int32_t spp0, int32_t passes, int32_t fc0, const int32_t* pixels,
                           int64_t npix, float* out_rgb, int32_t nthreads, const float* frozenMat) {
    std::atomic<int64_t> next{0};
    auto work = [&]() {
        for (;;) {
            int64_t i = next.fetch_add(16);
            if (i >= npix) break;
            int64_t e = std::min<int64_t>(npix, i + 16);
            for (; i < e; i++) {
                int p = pixels[i];
                int px = p % sc->filmW, py = p / sc->filmW;
                vec3 acc(out_rgb[3 * i], out_rgb[3 * i + 1], out_rgb[3 * i + 2]);
                for (int k = 0; k < passes; k++) {
                    bool ok;
                    vec3 r = renderPixel(*sc, px, py, spp0 + k, fc0 + k, ok, frozenMat);
                    if (ok) acc = acc + r;
                }
                out_rgb[3 * i] = acc.x;
                out_rgb[3 * i + 1] = acc.y;
                out_rgb[3 * i + 2] = acc.z;
            }
        }
    };
    if (nthreads <= 1) {
        work();
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) th.emplace_back(work);
    for (auto& t : th) t.join();
}

void orc_render_pt(const OrcScene* sc, int32_t spp0, int32_t passes, int32_t fc0, const int32_t* pixels, int64_t npix,
                   float* out_rgb, int32_t nthreads) {
    render_pt_impl(sc, spp0, passes, fc0, pixels, npix, out_rgb, nthreads, nullptr);
}

// render_pt with the sampling of `sc` and the BSDF values of materials mat1
// (pathFrozen).
void orc_render_pt_frozen(const OrcScene* sc, const float* mat1, int32_t spp0, int32_t passes, int32_t fc0,
                          const int32_t* pixels, int64_t npix, float* out_rgb, int32_t nthreads) {
    render_pt_impl(sc, spp0, passes, fc0, pixels, npix, out_rgb, nthreads, mat1);
}

// Light tracer passes (light_path_integ.glsl:148-158): `blocks` x 1536 light
// paths per pass, seeded spp * (1536 * blocks) + gid + freeCounter; film is
// float[H][W][3] and accumulates.
void orc_render_lt(const OrcScene* sc, int32_t spp0, int32_t passes, int32_t fc0, int32_t blocks, float* film) {
    const uint32_t group = 1536u * (uint32_t)blocks;
    for (int k = 0; k < passes; k++) {
        uint32_t spp = (uint32_t)(spp0 + k), fc = (uint32_t)(fc0 + k);
        for (uint32_t gid = 0; gid < group; gid++) {
            Rng g;
            g.randSeed = spp * group + gid + fc;
            g.sampleSeed = 0;
            g.sampleOffset = 0;
            lightIntegTrace(*sc, g, film);
        }
    }
}

// Triple-integrator passes (TriplePath.cpp:97-136): the camera pass of
// triple_path_pass_pt.glsl for every pixel, then `blocks` x 1536 x `loops`
// light paths of triple_path_pass_lpt.glsl scaled by W*H / (blocks*loops*1536).
void orc_render_triple(const OrcScene* sc, int32_t spp0, int32_t passes, int32_t fc0, int32_t blocks,
                       int32_t loops, float* film) {
    const uint32_t group = 1536u * (uint32_t)blocks * (uint32_t)loops;
    const float uScale = (float)(sc->filmW * sc->filmH) / (float)(blocks * loops * 1536);
    for (int k = 0; k < passes; k++) {
        int spp = spp0 + k, fc = fc0 + k;
        for (int py = 0; py < sc->filmH; py++)
            for (int px = 0; px < sc->filmW; px++) {
                vec2 texSize((float)sc->filmW, (float)sc->filmH);
                vec2 scr = vec2((float)px, (float)py) / texSize;
                vec2 nc = noiseTexture(*sc, scr);
                nc = noiseTexture(*sc, nc);
                vec2 tc = texSize * nc;
                Rng g;
                g.randSeed = f2u(tc.x) * (uint32_t)fc + f2u(tc.y);
                g.sampleSeed = f2u(tc.x) * f2u(tc.y);
                int off = (int)((uint32_t)spp * 256u);
                if (off > 131072 * 256) off -= 131072 * 256;
                g.sampleOffset = off;
                int s = 0;
                float u0 = sample1D(*sc, g, s), u1 = sample1D(*sc, g, s), u2 = sample1D(*sc, g, s), u3 = sample1D(*sc, g, s);
                Ray ray = thinLensCameraSampleRay(*sc, scr, u0, u1, u2, u3);
                vec3 r = traceCameraPath(*sc, ray, g, s);
                if (!hasNan(r)) {
                    float* p = film + 3 * ((size_t)py * sc->filmW + px);
                    p[0] += r.x;
                    p[1] += r.y;
                    p[2] += r.z;
                }
            }
        for (uint32_t gid = 0; gid < 1536u * (uint32_t)blocks; gid++) {
            Rng g;
            g.randSeed = (uint32_t)spp * group + gid + (uint32_t)fc;
            g.sampleSeed = 0;
            g.sampleOffset = 0;
            for (int i = 0; i < loops; i++) traceLightPath(*sc, g, film, uScale);
        }
    }
}

// The same passes on `nthreads` host threads, for timing the oracle as a CPU
// baseline: camera pixels by rows, light paths in contiguous ranges, each
// thread splatting into its own film; the films are summed at the end, so
// the result equals the sequential one up to the order of float additions.
static void camera_rows(const OrcScene* sc, int spp, int fc, int y0, int y1, float* film) {
    for (int py = y0; py < y1; py++)
        for (int px = 0; px < sc->filmW; px++) {
            vec2 texSize((float)sc->filmW, (float)sc->filmH);
            vec2 scr = vec2((float)px, (float)py) / texSize;
            vec2 nc = noiseTexture(*sc, scr);
            nc = noiseTexture(*sc, nc);
            vec2 tc = texSize * nc;
            Rng g;
            g.randSeed = f2u(tc.x) * (uint32_t)fc + f2u(tc.y);
            g.sampleSeed = f2u(tc.x) * f2u(tc.y);
            int off = (int)((uint32_t)spp * 256u);
            if (off > 131072 * 256) off -= 131072 * 256;
            g.sampleOffset = off;
            int s = 0;
            float u0 = sample1D(*sc, g, s), u1 = sample1D(*sc, g, s), u2 = sample1D(*sc, g, s), u3 = sample1D(*sc, g, s);
            Ray ray = thinLensCameraSampleRay(*sc, scr, u0, u1, u2, u3);
            vec3 r = traceCameraPath(*sc, ray, g, s);
            if (!hasNan(r)) {
                float* p = film + 3 * ((size_t)py * sc->filmW + px);
                p[0] += r.x;
                p[1] += r.y;
                p[2] += r.z;
            }
        }
}

void orc_render_mt(const OrcScene* sc, int32_t kind, int32_t spp0, int32_t passes, int32_t fc0, int32_t blocks,
                   int32_t loops, float* film, int32_t nthreads) {
    const int T = std::max(1, (int)nthreads);
    const size_t npix = (size_t)sc->filmW * sc->filmH * 3;
    std::vector<std::vector<float>> part((size_t)T, std::vector<float>(npix, 0.0f));
    const uint32_t paths = 1536u * (uint32_t)blocks;
    const uint32_t group = kind == 0 ? paths : paths * (uint32_t)loops;
    const float uScale = (float)(sc->filmW * sc->filmH) / (float)(blocks * loops * 1536);
    auto work = [&](int t) {
        float* f = part[(size_t)t].data();
        for (int k = 0; k < passes; k++) {
            const uint32_t spp = (uint32_t)(spp0 + k), fc = (uint32_t)(fc0 + k);
            if (kind == 1) {
                const int y0 = (int)((int64_t)sc->filmH * t / T), y1 = (int)((int64_t)sc->filmH * (t + 1) / T);
                camera_rows(sc, (int)spp, (int)fc, y0, y1, f);
            }
            const uint32_t g0 = (uint32_t)((uint64_t)paths * t / T), g1 = (uint32_t)((uint64_t)paths * (t + 1) / T);
            for (uint32_t gid = g0; gid < g1; gid++) {
                Rng g;
                g.randSeed = spp * group + gid + fc;
                g.sampleSeed = 0;
                g.sampleOffset = 0;
                if (kind == 0)
                    lightIntegTrace(*sc, g, f);
                else
                    for (int i = 0; i < loops; i++) traceLightPath(*sc, g, f, uScale);
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < T; t++) th.emplace_back(work, t);
    for (auto& x : th) x.join();
    for (int t = 0; t < T; t++)
        for (size_t i = 0; i < npix; i++) film[i] += part[(size_t)t][i];
}

// ----------------------------------------------------------- host tables

// Light power split and alias table (Scene.cpp:200-243, AliasTable.h:12-54).
// vertices are world-space light vertices, indices local to them; each
// instance k owns triangles [first[k], first[k+1]) and total power power[k].
float orc_light_tables(const float* vertices, const uint32_t* indices, const uint32_t* first, const float* power,
                       int32_t ninst, float* lightPower, int32_t* alias, float* prob) {
    std::vector<float> pdf;
    float lightSum = 0.0f;
    int out = 0;
    for (int k = 0; k < ninst; k++) {
        vec3 P(power[3 * k], power[3 * k + 1], power[3 * k + 2]);
        auto tri = [&](uint32_t t, vec3& a, vec3& b, vec3& c) {
            a = vec3(vertices[3 * indices[3 * t]], vertices[3 * indices[3 * t] + 1], vertices[3 * indices[3 * t] + 2]);
            b = vec3(vertices[3 * indices[3 * t + 1]], vertices[3 * indices[3 * t + 1] + 1], vertices[3 * indices[3 * t + 1] + 2]);
            c = vec3(vertices[3 * indices[3 * t + 2]], vertices[3 * indices[3 * t + 2] + 1], vertices[3 * indices[3 * t + 2] + 2]);
        };
        float sumArea = 0.0f;
        for (uint32_t t = first[k]; t < first[k + 1]; t++) {
            vec3 a, b, c;
            tri(t, a, b, c);
            sumArea += length(cross(c - a, b - a));
        }
        for (uint32_t t = first[k]; t < first[k + 1]; t++) {
            vec3 a, b, c;
            tri(t, a, b, c);
            float area = length(cross(c - a, b - a));
            vec3 pw = P * area / sumArea;
            lightPower[3 * out] = pw.x;
            lightPower[3 * out + 1] = pw.y;
            lightPower[3 * out + 2] = pw.z;
            out++;
            float l = dot(pw, vec3(0.299f, 0.587f, 0.114f));
            pdf.push_back(l);
            lightSum += l;
        }
    }
    // AliasTable::build
    int n = (int)pdf.size();
    std::vector<float> pr = pdf;
    float sumPdf = 0.0f;
    for (int i = 0; i < n; i++) sumPdf += pr[i];
    float sumInv = (float)n / sumPdf;
    std::vector<std::pair<int, float>> greater, lesser;
    for (int i = 0; i < n; i++) {
        pr[i] *= sumInv;
        (pr[i] < 1.0f ? lesser : greater).push_back({i, pr[i]});
    }
    std::vector<int> al(n, 0);
    while (!greater.empty() && !lesser.empty()) {
        auto [l, pl] = lesser.back();
        lesser.pop_back();
        auto [g, pg] = greater.back();
        greater.pop_back();
        al[l] = g;
        pr[l] = pl;
        pg += pl - 1.0f;
        (pg < 1.0f ? lesser : greater).push_back({g, pg});
    }
    while (!greater.empty()) {
        auto [g, pg] = greater.back();
        greater.pop_back();
        al[g] = g;
        pr[g] = pg;
    }
    while (!lesser.empty()) {
        auto [l, pl] = lesser.back();
        lesser.pop_back();
        al[l] = l;
        pr[l] = pl;
    }
    for (int i = 0; i < n; i++) {
        alias[i] = al[i];
        prob[i] = pr[i];
    }
    return lightSum;
}

// AliasTable::build alone, through the light-table routine: one instance per
// pdf entry would change the pdf, so the construction is repeated here.
void orc_alias_build(const float* pdf, int32_t n, int32_t* alias, float* prob) {
    std::vector<float> pr(pdf, pdf + n);
    float sumPdf = 0.0f;
    for (int i = 0; i < n; i++) sumPdf += pr[i];
    float sumInv = (float)n / sumPdf;
    std::vector<std::pair<int, float>> greater, lesser;
    for (int i = 0; i < n; i++) {
        pr[i] *= sumInv;
        (pr[i] < 1.0f ? lesser : greater).push_back({i, pr[i]});
    }
    std::vector<int> al(n, 0);
    while (!greater.empty() && !lesser.empty()) {
        auto [l, pl] = lesser.back();
        lesser.pop_back();
        auto [g, pg] = greater.back();
        greater.pop_back();
        al[l] = g;
        pr[l] = pl;
        pg += pl - 1.0f;
        (pg < 1.0f ? lesser : greater).push_back({g, pg});
    }
    while (!greater.empty()) {
        auto [g, pg] = greater.back();
        greater.pop_back();
        al[g] = g;
        pr[g] = pg;
    }
    while (!lesser.empty()) {
        auto [l, pl] = lesser.back();
        lesser.pop_back();
        al[l] = l;
        pr[l] = pl;
    }
    for (int i = 0; i < n; i++) {
        alias[i] = al[i];
        prob[i] = pr[i];
    }
}

// Env-map sampling tables (EnvironmentMap.cpp:8-59, setupAliasTable :66-114).
// rgb: float image W*H*3 (before the RGB16F upload).  alias/prob: (W+1)*H.
// Returns the pdf sum; the shader receives int(sum) (EnvironmentMap.h:22).
float orc_env_tables(const float* rgb, int32_t W, int32_t H, int32_t* alias, float* prob) {
    auto off = [W](int i, int j) { return (size_t)i * (W + 1) + j; };
    for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++) {
            const float* p = rgb + 3 * ((size_t)i * W + j);
            float lum = 0.2126f * p[0] + 0.7152f * p[1] + 0.0722f * p[2];
            prob[off(i, j)] = lum * std::sin((float)(i + 0.5f) / (float)H * 3.141592653589793f);
        }
    auto setup = [](int32_t* al, float* pdf, int n, int stride) -> float {
        float sum = 0.0f;
        for (int i = 0, o = 0; i < n; i++, o += stride) sum += pdf[o];
        float sumInv = (float)n / sum;
        std::vector<std::pair<int, float>> greater, lesser;
        for (int i = 0, o = 0; i < n; i++, o += stride) {
            pdf[o] *= sumInv;
            (pdf[o] < 1.0f ? lesser : greater).push_back({i, pdf[o]});
        }
        while (!greater.empty() && !lesser.empty()) {
            auto [l, pl] = lesser.back();
            lesser.pop_back();
            auto [g, pg] = greater.back();
            greater.pop_back();
            al[l * stride] = g;
            pdf[l * stride] = pl;
            pg += pl - 1.0f;
            (pg < 1.0f ? lesser : greater).push_back({g, pg});
        }
        while (!greater.empty()) {
            auto [g, pg] = greater.back();
            (void)pg;
            greater.pop_back();
            al[g * stride] = g;
            pdf[g * stride] = 1.0f;
        }
        while (!lesser.empty()) {
            auto [l, pl] = lesser.back();
            (void)pl;
            lesser.pop_back();
            al[l * stride] = l;
            pdf[l * stride] = 1.0f;
        }
        return sum;
    };
    for (int i = 0; i < H; i++) prob[off(i, W)] = setup(alias + off(i, 0), prob + off(i, 0), W, 1);
    return setup(alias + W, prob + W, H, W + 1);
}

// Noise texture of Sampler::genNoiseTexture (Sampler.cpp:66-80) with the
// libstdc++ engines: std::default_random_engine = minstd_rand0 (seed 1) and
// uniform_real_distribution<float>(0, 1) = generate_canonical<float, 24>.
void orc_noise(int32_t W, int32_t H, float* out) {
    uint64_t x = 1;
    size_t n = (size_t)W * H * 2;
    for (size_t i = 0; i < n; i++) {
        x = (x * 16807u) % 2147483647u;
        float v = (float)(x - 1) / 2147483646.0f;
        if (v >= 1.0f) v = std::nextafter(1.0f, 0.0f);
        out[i] = v * (1.0f - 0.0f) + 0.0f;
    }
}

// glm::normalize: x * inversesqrt(dot(x, x))
static vec3 glmNormalize(vec3 v) { return v * (1.0f / std::sqrt(dot(v, v))); }

// Camera::update (Camera.cpp:149-162) and the uniforms of NaivePath.cpp:49-60.
// out: F[3], R[3], U[3], camMatInv[9] (column-major), tanFOV
void orc_camera(const float* angle, float fov, float* out) {
    const float rad = 0.01745329251994329576923690768489f;
    float ax = angle[0] * rad, ay = angle[1] * rad;
    float x = std::sin(ax) * std::cos(ay);
    float y = std::cos(ax) * std::cos(ay);
    float z = std::sin(ay);
    vec3 front = glmNormalize(vec3(x, y, z));
    vec3 right = glmNormalize(cross(front, vec3(0.0f, 0.0f, 1.0f)));
    // glm::rotate(mat4(1), angle.z (radians), front) applied to (right, 1)
    float c = std::cos(angle[2]), s = std::sin(angle[2]);
    vec3 axis = glmNormalize(front);
    vec3 temp = axis * (1.0f - c);
    float R00 = c + temp.x * axis.x, R01 = temp.x * axis.y + s * axis.z, R02 = temp.x * axis.z - s * axis.y;
    float R10 = temp.y * axis.x - s * axis.z, R11 = c + temp.y * axis.y, R12 = temp.y * axis.z + s * axis.x;
    float R20 = temp.z * axis.x + s * axis.y, R21 = temp.z * axis.y - s * axis.x, R22 = c + temp.z * axis.z;
    // rotMatrix columns: col j = Rotate[j] (m = identity); result = M * (right, 1)
    vec3 rr((R00 * right.x + R10 * right.y) + R20 * right.z, (R01 * right.x + R11 * right.y) + R21 * right.z,
            (R02 * right.x + R12 * right.y) + R22 * right.z);
    right = glmNormalize(rr);
    vec3 up = glmNormalize(cross(right, front));
    mat3 m{right, up, front};
    mat3 inv = inverse(m);
    float* o = out;
    o[0] = front.x; o[1] = front.y; o[2] = front.z;
    o[3] = right.x; o[4] = right.y; o[5] = right.z;
    o[6] = up.x; o[7] = up.y; o[8] = up.z;
    o[9] = inv.c0.x; o[10] = inv.c0.y; o[11] = inv.c0.z;
    o[12] = inv.c1.x; o[13] = inv.c1.y; o[14] = inv.c1.z;
    o[15] = inv.c2.x; o[16] = inv.c2.y; o[17] = inv.c2.z;
    o[18] = std::tan(fov * 0.5f * rad);
}

// Gradient of sum(dimage * image) for the image = mean of samples 0..spp-1
// of the path tracer (sample k with freeCounter k + 1; NaN samples dropped),
// with respect to (per material: baseColor rgb, raw roughness, metallic,
// specular; per light instance: power rgb), into grad[nmat*6 + ninst*3].
void orc_diff_grad(const OrcScene* sc, int32_t spp, const float* dimage, const int32_t* lightInst,
                   const float* instPower, int32_t nmat, int32_t ninst, double* grad, int32_t nthreads) {
    const int64_t npix = (int64_t)sc->filmW * sc->filmH;
    const size_t np = (size_t)nmat * 6 + (size_t)ninst * 3;
    std::atomic<int64_t> next{0};
    std::vector<std::vector<double>> part((size_t)std::max(nthreads, 1), std::vector<double>(np, 0.0));
    auto work = [&](int t) {
        AdjCtx cx;
        cx.lightInst = lightInst;
        cx.instPower = instPower;
        cx.nmat = nmat;
        cx.A.assign((size_t)nmat * 18, 0.0);
        cx.grad = part[(size_t)t].data();
        for (;;) {
            int64_t i = next.fetch_add(8);
            if (i >= npix) break;
            int64_t e = std::min<int64_t>(npix, i + 8);
            for (; i < e; i++) {
                int px = (int)(i % sc->filmW), py = (int)(i / sc->filmW);
                for (int c = 0; c < 3; c++) cx.delta[c] = (double)dimage[3 * i + c] / spp;
                if (cx.delta[0] == 0.0 && cx.delta[1] == 0.0 && cx.delta[2] == 0.0) continue;
                for (int k = 0; k < spp; k++) {
                    bool ok;
                    renderPixel(*sc, px, py, k, k + 1, ok);
                    if (ok) pixelAdjoint(*sc, px, py, k, k + 1, cx);
                }
            }
        }
    };
    if (nthreads <= 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nthreads; t++) th.emplace_back(work, t);
        for (auto& t : th) t.join();
    }
    for (size_t j = 0; j < np; j++) {
        double acc = 0.0;
        for (auto& p : part) acc += p[j];
        grad[j] = acc;
    }
}

// The display pass of post_proc.glsl:11-59 (the tone mappers reinhard and CE
// are defined there but never selected): frame RGBA32F of (W/s) x (H/s)
// texels, out RGBA32F of W x H; texels past the film read as zero.
// albedoTexture of texture texId at n texcoords (uv float[n*2]) -> out float[n*3]
void orc_texture_sample(const OrcScene* sc, int32_t texId, const float* uv, int64_t n, float* out) {
    for (int64_t i = 0; i < n; i++) {
        vec3 c = albedoTexture(*sc, texId, vec2(uv[2 * i], uv[2 * i + 1]));
        out[3 * i] = c.x;
        out[3 * i + 1] = c.y;
        out[3 * i + 2] = c.z;
    }
}

void orc_postprocess(const float* frame, int32_t W, int32_t H, int32_t s, float scale, int32_t mapper, float* out) {
    const int inW = W / s, inH = H / s;
    auto calc = [](float x) {
        const float A = 0.22f, B = 0.3f, C = 0.1f, D = 0.2f, E = 0.01f, F = 0.3f;
        return (x * (x * A + B * C) + D * E) / (x * (x * A + B) + D * F) - E / F;
    };
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const int sx = x / s, sy = y / s;
            const float* c = (sx < inW && sy < inH) ? frame + 4 * ((size_t)sy * inW + sx) : nullptr;
            float* o = out + 4 * ((size_t)y * W + x);
            for (int k = 0; k < 3; k++) {
                float v = (c ? c[k] : 0.0f) * scale;
                v = fmin_(fmax_(v, 0.0f), 1e30f);
                if (mapper == 1) v = calc(v * 1.6f) / calc(11.2f);
                else if (mapper == 2) v = (v * (v * 2.51f + 0.03f)) / (v * (v * 2.43f + 0.59f) + 0.14f);
                o[k] = zpow(v, 1.0f / 2.2f);
            }
            o[3] = 1.0f;
        }
}

}  // extern "C"
