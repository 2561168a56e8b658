// path_trace.cuh — the MIS path tracer's per-sample function (pathIntegTrace,
// path_integ_naive.glsl:35-143) and the per-block Sobol row, shared by the
// progressive integrator kernels (render.cu) and the differentiable renderer
// (render_diff.cu).
#pragma once

#include "shading.cuh"

namespace zgl {
namespace {

constexpr int kTileX = 16, kTileY = 8;

struct PathParams {
    int32_t maxDepth;
    int32_t rr;
    int32_t rrStart;
    int32_t sampleLight;
    int32_t uniformSel;
    float portion;
};

template <class Vis>
__device__ __forceinline__ LiSample sampleLightAndEnvV(const DeviceScene& sc, const PathParams& pp, v3 x, float ud,
                                                       float u0, float u1, float u2, float u3, const Vis& vis) {
    float pdfSampleLight = 0.0f;  // light.glsl:221-235
    if (sc.nLight > 0) pdfSampleLight = pdfSampleLightSel(sc, pp.uniformSel, pp.portion);
    bool sampleLight = ud < pdfSampleLight;
    float pdfSelect = sampleLight ? pdfSampleLight : 1.0f - pdfSampleLight;
    LiSample s;
    if (sampleLight) {
        int id = lightSampleOne(sc, mk2(u0, u1));
        s = lightSampleLiV(sc, id, x, mk2(u2, u3), vis);
    } else {
        s = envSampleLiV(sc, x, u0, u1, u2, u3, vis);
    }
    s.coef = s.coef / pdfSelect;
    s.pdf *= pdfSelect;
    return s;
}
__device__ __forceinline__ LiSample sampleLightAndEnv(const DeviceScene& sc, const PathParams& pp, v3 x, float ud,
                                                      float u0, float u1, float u2, float u3) {
    return sampleLightAndEnvV(sc, pp, x, ud, u0, u1, u2, u3, TraceVis{});
}

__device__ __forceinline__ float pdfSelectLight(const DeviceScene& sc, const PathParams& pp, int id) {
    float fst = lightPdfSampleOne(sc, id);
    float snd = pp.uniformSel ? pp.portion : sc.lightSum / (sc.lightSum + sc.envSum);
    return fst * snd;
}
__device__ __forceinline__ float pdfSelectEnv(const DeviceScene& sc, const PathParams& pp) {
    return pp.uniformSel ? (1.0f - pp.portion) : sc.envSum / (sc.lightSum + sc.envSum);
}

// Ray casts of a path: closest hits in path order (`hit`) and the light
// samples' occlusion tests (operator(), the TraceVis interface).  DirectCast
// traverses the accelerator for both.
struct DirectCast {
    __device__ __forceinline__ int hit(const DeviceScene& sc, const Ray& r, float& dist) const {
        return bvhHit(sc, r, dist);
    }
    __device__ __forceinline__ bool operator()(const DeviceScene& sc, const Ray& r, float dist) const {
        return bvhTest(sc, r, dist);
    }
};

// pathIntegTrace (path_integ_naive.glsl:35-143) with the ray casts of `rc`
template <bool FULL, class RC>
__device__ __forceinline__ v3 pathTraceRC(const DeviceScene& sc, const PathParams& pp, Ray ray, Sampler& g,
                                          const RC& rc) {
    float primDist;
    int id = rc.hit(sc, ray, primDist);
    v3 pos = rayPoint(ray, primDist);
    if (id == -1) return envLe(sc, ray.dir);
    if (id - sc.objPrimCount >= 0) return lightLe(sc, id - sc.objPrimCount, pos, -ray.dir);
    v3 wo = -ray.dir;
    v3 result = mk3(0.0f), throughput = mk3(1.0f);
    for (int bounce = 1; bounce <= pp.maxDepth; bounce++) {
        TriShade tri = loadTri(sc, id);
        Surface surf = surfaceInfo(tri, pos);
        int matId = tri.matTex & 0x0000ffff;
        uint32_t matType = loadMaterialType(sc, matId);
        if (matType != kDielectric && matType != kThinDielectric) {
            if (dot(surf.ns, wo) < 0.0f) {
                surf.ns = -surf.ns;
                surf.ng = -surf.ng;
            }
        }
        BSDFParam mp = loadMaterial<FULL>(sc, matType, tri.matTex, id, surf);
        if (pp.sampleLight) {
            float ud = sample1D(g);
            float u0 = sample1D(g), u1 = sample1D(g), u2 = sample1D(g), u3 = sample1D(g);
            LiSample ls = sampleLightAndEnvV(sc, pp, pos, ud, u0, u1, u2, u3, rc);
            if (ls.pdf > 0.0f) {
                v3 f = materialBSDF<FULL>(matType, mp, wo, ls.wi, surf.ns);
                float fpdf = materialPdf<FULL>(matType, mp, wo, ls.wi, surf.ns);
                float weight = biHeuristic(ls.pdf, fpdf);
                result = result + f * throughput * satDot(surf.ns, ls.wi) * ls.coef * weight;
            }
        }
        float b0 = sample1D(g), b1 = sample1D(g), b2 = sample1D(g);
        BSDFSample bs = materialSample<FULL>(matType, mp, surf.ns, wo, mk3(b0, b1, b2), g);
        v3 wi = bs.wi;
        float bsdfPdf = bs.pdf;
        bool deltaBsdf = (bs.flag == kSpecRefl || bs.flag == kSpecTrans);
        if (bsdfPdf < 1e-8f) break;
        throughput = throughput * (bs.bsdf / bsdfPdf * (deltaBsdf ? 1.0f : absDot(surf.ns, wi)));
        ray = rayOffseted(pos, wi);
        float dist;
        int nextId = rc.hit(sc, ray, dist);
        int lightId = nextId - sc.objPrimCount;
        v3 nextPos = rayPoint(ray, dist);
        if (nextId == -1) {
            v3 radiance = envLe(sc, wi);
            float weight = 1.0f;
            if (pp.sampleLight && !deltaBsdf) {
                float envPdf = envPdfLi(sc, wi) * pdfSelectEnv(sc, pp);
                weight = (envPdf <= 0.0f) ? 0.0f : biHeuristic(bsdfPdf, envPdf);
            }
            result = result + radiance * throughput * weight;
            break;
        } else if (lightId >= 0) {
            v3 radiance = lightLe(sc, lightId, nextPos, -wi);
            float weight = 1.0f;
            if (pp.sampleLight && !deltaBsdf) {
                float lightPdf = lightPdfLi(sc, lightId, pos, nextPos) * pdfSelectLight(sc, pp, lightId);
                weight = (lightPdf <= 0.0f) ? 0.0f : biHeuristic(bsdfPdf, lightPdf);
            }
            result = result + radiance * throughput * weight;
            break;
        }
        if (pp.rr && bounce >= pp.rrStart) {
            float continueProb = zmin(maxComponent(bs.bsdf / bsdfPdf), 0.95f);
            if (sample1D(g) >= continueProb) break;
            throughput = throughput / continueProb;
        }
        id = nextId;
        pos = nextPos;
        wo = -wi;
    }
    return result;
}

template <bool FULL>
__device__ v3 pathTrace(const DeviceScene& sc, const PathParams& pp, Ray ray, Sampler& g) {
    return pathTraceRC<FULL>(sc, pp, ray, g, DirectCast{});
}

__device__ __forceinline__ void load_sobol_row(const DeviceScene& sc, uint32_t sampleOffset, uint32_t* row) {
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nthr = blockDim.x * blockDim.y;
    if (sc.sampler == 1)
        for (int i = tid; i < 256; i += nthr) row[i] = sobol_value(sc.sobol, sampleOffset >> 8, (uint32_t)i);
    __syncthreads();
}

// sampleOffset = uSpp * uSampleDim, minus the table size once when beyond it
// (path_integ_naive.glsl:163-164), in 32-bit arithmetic.
__host__ __device__ inline uint32_t sample_offset(int32_t spp) {
    const int32_t sampleNum = 131072, sampleDim = 256;
    int32_t off = (int32_t)((uint32_t)spp * (uint32_t)sampleDim);
    if (off > sampleNum * sampleDim) off -= sampleNum * sampleDim;
    return (uint32_t)off;
}

}  // namespace
}  // namespace zgl
