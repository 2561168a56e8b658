// bsdf_grad.cuh — the BSDF value and its partial derivatives with respect to
// the six differentiable material parameters: baseColor r, g, b; roughness
// before the load-time remap R = mix(0.0134, 1, r) (dR/dr = 0.9866);
// metallic; specular.  The value follows principledBRDF
// (material.glsl:462-490) and lambertian (:68-76); the derivatives are the
// analytic ones of those formulas, term by term:
//   diffuse   rho K(R) / pi (1 - metallic), K = fd (1 - sub) + ss sub
//   metal     (fm0 (1 - w5) + w5) D(alpha) G(alpha) / (4 cosI cosO),
//             fm0 = 0.08 spec mix(1, tint, specTint) (1 - metallic) + rho metallic,
//             alpha = R^2, tint = rho / luminance(rho)
//   clearcoat (rho (1 - w5) + w5) Dc Gc / (4 cosI cosO) clearcoat / 4
//   sheen     mix(1, tint, sheenTint) schlickW(h.wi) sheen
#pragma once

#include "shading.cuh"

namespace zgl {

constexpr int kDiffMatParams = 6;  // baseColor.rgb, raw roughness, metallic, specular

struct BsdfGrad {
    v3 f;
    v3 df[kDiffMatParams];  // df[i].c = d f_c / d theta_i
};

__device__ __forceinline__ v3 unit3(int k) { return mk3(k == 0 ? 1.0f : 0.0f, k == 1 ? 1.0f : 0.0f, k == 2 ? 1.0f : 0.0f); }

// d/dk of the Schlick-Smith factor c / (c (1 - k) + k)
__device__ __forceinline__ float dSchlickGdk(float c, float k) {
    float den = c * (1.0f - k) + k;
    return -c * (1.0f - c) / (den * den);
}

static __device__ __noinline__ BsdfGrad principledGrad(v3 wo, v3 wi, v3 n, BSDFParam p) {
    BsdfGrad g;
    g.f = mk3(0.0f);
#pragma unroll
    for (int i = 0; i < kDiffMatParams; i++) g.df[i] = mk3(0.0f);
    const v3 rho = p.baseColor;
    const float R = p.roughness, m = p.metallic, s = p.specular;
    const float alpha = R * R;
    const float ccAlpha = mixf(0.1f, 0.001f, p.clearcoatGloss);
    const float lum = luminance(rho);
    const v3 tint = lum > 0.0f ? rho / lum : mk3(1.0f);
    // dtint[k] = d tint / d rho_k = (e_k - tint w_k) / lum
    const float wl[3] = {0.299f, 0.587f, 0.114f};
    v3 dtint[3];
#pragma unroll
    for (int k = 0; k < 3; k++) dtint[k] = lum > 0.0f ? (unit3(k) - tint * wl[k]) / lum : mk3(0.0f);
    const v3 spTint = mix3(mk3(1.0f), tint, p.specularTint);
    const v3 fm0 = mix3(spTint * (0.08f * s), rho, m);
    const float cosWo = satDot(n, wo), cosWi = satDot(n, wi);
    const v3 h = normalize(wo + wi);
    const float hCosWi = dot(h, wi);
    if (!(cosWo < 1e-10f || cosWi < 1e-10f)) {
        // diffuse (principledDiffuse, material.glsl:429-452) times (1 - metallic)
        const float hc2 = hCosWi * hCosWi;
        const float fi = schlickW(cosWi), fo = schlickW(cosWo);
        const float fd90 = 0.5f + 2.0f * R * hc2;
        const float A = (1.0f - fi) + fd90 * fi, B = (1.0f - fo) + fd90 * fo;
        const float fd = A * B, dfd = 2.0f * hc2 * (fi * B + fo * A);
        const float fss90 = R * hc2;
        const float As = (1.0f - fi) + fss90 * fi, Bs = (1.0f - fo) + fss90 * fo;
        const float fss = As * Bs, dfss = hc2 * (fi * Bs + fo * As);
        const float q = 1.0f / (cosWi + cosWo) - 0.5f;
        const float ssf = 1.25f * (fss * q + 0.5f), dssf = 1.25f * q * dfss;
        const float sub = p.subsurface;
        const float K = fd * (1.0f - sub) + ssf * sub, dK = dfd * (1.0f - sub) + dssf * sub;
        const float om = 1.0f - m;
        const float kd = K * kPiInv;
        g.f = g.f + rho * (kd * om);
        g.df[0].x += kd * om;
        g.df[1].y += kd * om;
        g.df[2].z += kd * om;
        g.df[3] = g.df[3] + rho * (dK * kPiInv * om);
        g.df[4] = g.df[4] - rho * kd;
        // metal (principledMetal, :357-373)
        const float denom = 4.0f * cosWi * cosWo;
        if (!(denom < 1e-7f)) {
            const float w5 = pow5(1.0f - absDot(h, wo));
            const float c = dot(n, h);
            float Dm = 0.0f, dDm = 0.0f;  // dDm = dD / dalpha
            if (!(c < 1e-6f)) {
                const float a2 = alpha * alpha;
                const float t = c * c * (a2 - 1.0f) + 1.0f;
                Dm = a2 / (t * t * kPi);
                dDm = (t - 2.0f * a2 * c * c) / (kPi * t * t * t) * (2.0f * alpha);
            }
            const float k = alpha * 0.5f;
            const float co = absDot(n, wo), ci = absDot(n, wi);
            const float g1 = schlickG(co, alpha), g2 = schlickG(ci, alpha);
            const float dG = 0.5f * (dSchlickGdk(co, k) * g2 + g1 * dSchlickGdk(ci, k));
            const float G = g1 * g2;
            const float DG = Dm * G / denom, dDG = (dDm * G + Dm * dG) / denom;
            const v3 fm = fm0 * (1.0f - w5) + mk3(w5);
            g.f = g.f + fm * DG;
            const float a = (1.0f - w5) * DG;
            // d fm0 / d rho_k = 0.08 s specTint dtint_k (1 - m) + e_k m
#pragma unroll
            for (int kk = 0; kk < 3; kk++)
                g.df[kk] = g.df[kk] + (dtint[kk] * (0.08f * s * p.specularTint * (1.0f - m)) + unit3(kk) * m) * a;
            g.df[5] = g.df[5] + spTint * (0.08f * (1.0f - m) * a);
            g.df[4] = g.df[4] + (rho - spTint * (0.08f * s)) * a;
            g.df[3] = g.df[3] + fm * (dDG * 2.0f * R);
        }
    }
    if (!(cosWo < 1e-6f || cosWi < 1e-6f)) {  // clearcoat (:393-409) * clearcoat * 0.25
        const float denom = 4.0f * cosWi * cosWo;
        if (!(denom < 1e-7f)) {
            const float w5 = pow5(1.0f - absDot(h, wo));
            const float X = gtr1(satDot(n, h), ccAlpha) * smithG(n, wo, wi, 0.25f) / denom * p.clearcoat * 0.25f;
            g.f = g.f + (rho * (1.0f - w5) + mk3(w5)) * X;
            const float d = (1.0f - w5) * X;
            g.df[0].x += d;
            g.df[1].y += d;
            g.df[2].z += d;
        }
    }
    // sheen
    const float W = schlickW(hCosWi) * p.sheen * (dot(n, wi) < 0.0f ? 0.0f : 1.0f);
    g.f = g.f + mix3(mk3(1.0f), tint, p.sheenTint) * W;
#pragma unroll
    for (int kk = 0; kk < 3; kk++) g.df[kk] = g.df[kk] + dtint[kk] * (p.sheenTint * W);
    g.df[3] = g.df[3] * 0.9866f;  // d R / d raw roughness
    return g;
}

__device__ __forceinline__ BsdfGrad bsdfGrad(uint32_t type, const BSDFParam& p, v3 wo, v3 wi, v3 n) {
    if (type == kPrincipled) return principledGrad(wo, wi, n, p);
    BsdfGrad g;
    g.f = p.baseColor * kPiInv;
#pragma unroll
    for (int i = 0; i < kDiffMatParams; i++) g.df[i] = mk3(0.0f);
    g.df[0].x = kPiInv;
    g.df[1].y = kPiInv;
    g.df[2].z = kPiInv;
    return g;
}

}  // namespace zgl
