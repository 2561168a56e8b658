// render.cu — progressive MIS path tracer (one path per pixel per pass) and
// the zgl_integrator_* entry points.
//
// The kernel restates path_integ_naive.glsl (pathIntegTrace :35-143, main
// :145-174).  Pixels are mapped to 16x8 tiles so that a warp's camera rays are
// neighbours.  The 256 Sobol values of the pass's sample row are computed
// once per block into shared memory.
#include <cstring>
#include <new>

#include "scene.h"
#include "shading.cuh"
#include "zgl_internal.h"

struct zgl_integrator {
    zgl_scene* scene = nullptr;
    int32_t kind = 0;
    zgl_integrator_params params{};
    int32_t curSample = 0;    // mCurSample
    int32_t freeCounter = 0;  // mFreeCounter
    bool finished = false;
    float4* d_frame = nullptr;  // RGBA sum, filmW * filmH
};

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

__device__ __forceinline__ LiSample sampleLightAndEnv(const DeviceScene& sc, const PathParams& pp, v3 x, float ud,
                                                      float u0, float u1, float u2, float u3) {
    float pdfSampleLight = 0.0f;  // light.glsl:221-235
    if (sc.nLight > 0) pdfSampleLight = pdfSampleLightSel(sc, pp.uniformSel, pp.portion);
    bool sampleLight = ud < pdfSampleLight;
    float pdfSelect = sampleLight ? pdfSampleLight : 1.0f - pdfSampleLight;
    LiSample s;
    if (sampleLight) {
        int id = lightSampleOne(sc, mk2(u0, u1));
        s = lightSampleLi(sc, id, x, mk2(u2, u3));
    } else {
        s = envSampleLi(sc, x, u0, u1, u2, u3);
    }
    s.coef = s.coef / pdfSelect;
    s.pdf *= pdfSelect;
    return s;
}

__device__ __forceinline__ float pdfSelectLight(const DeviceScene& sc, const PathParams& pp, int id) {
    float fst = lightPdfSampleOne(sc, id);
    float snd = pp.uniformSel ? pp.portion : sc.lightSum / (sc.lightSum + sc.envSum);
    return fst * snd;
}
__device__ __forceinline__ float pdfSelectEnv(const DeviceScene& sc, const PathParams& pp) {
    return pp.uniformSel ? (1.0f - pp.portion) : sc.envSum / (sc.lightSum + sc.envSum);
}

// pathIntegTrace (path_integ_naive.glsl:35-143)
__device__ v3 pathTrace(const DeviceScene& sc, const PathParams& pp, Ray ray, Sampler& g) {
    float primDist;
    int id = bvhHit(sc, ray, primDist);
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
        BSDFParam mp = loadMaterial(sc, matType, matId);
        if (pp.sampleLight) {
            float ud = sample1D(g);
            float u0 = sample1D(g), u1 = sample1D(g), u2 = sample1D(g), u3 = sample1D(g);
            LiSample ls = sampleLightAndEnv(sc, pp, pos, ud, u0, u1, u2, u3);
            if (ls.pdf > 0.0f) {
                v3 f = materialBSDF(matType, mp, wo, ls.wi, surf.ns);
                float fpdf = materialPdf(matType, mp, wo, ls.wi, surf.ns);
                float weight = biHeuristic(ls.pdf, fpdf);
                result = result + f * throughput * satDot(surf.ns, ls.wi) * ls.coef * weight;
            }
        }
        float b0 = sample1D(g), b1 = sample1D(g), b2 = sample1D(g);
        BSDFSample bs = materialSample(matType, mp, surf.ns, wo, mk3(b0, b1, b2), g);
        v3 wi = bs.wi;
        float bsdfPdf = bs.pdf;
        bool deltaBsdf = (bs.flag == kSpecRefl || bs.flag == kSpecTrans);
        if (bsdfPdf < 1e-8f) break;
        throughput = throughput * (bs.bsdf / bsdfPdf * (deltaBsdf ? 1.0f : absDot(surf.ns, wi)));
        ray = rayOffseted(pos, wi);
        float dist;
        int nextId = bvhHit(sc, ray, dist);
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

__device__ __forceinline__ void load_sobol_row(const DeviceScene& sc, uint32_t sampleOffset, uint32_t* row) {
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nthr = blockDim.x * blockDim.y;
    if (sc.sampler == 1)
        for (int i = tid; i < 256; i += nthr) row[i] = sobol_value(sc.sobol, sampleOffset >> 8, (uint32_t)i);
    __syncthreads();
}

// main() of path_integ_naive.glsl:145-174
__global__ void __launch_bounds__(kTileX* kTileY)
path_kernel(DeviceScene sc, PathParams pp, int32_t spp, int32_t freeCounter, uint32_t sampleOffset,
            float4* __restrict__ frame) {
    __shared__ uint32_t row[256];
    load_sobol_row(sc, sampleOffset, row);
    const int px = blockIdx.x * kTileX + threadIdx.x;
    const int py = blockIdx.y * kTileY + threadIdx.y;
    if (px >= sc.filmW || py >= sc.filmH) return;
    const size_t pix = (size_t)py * sc.filmW + px;
    const uint2 seed = __ldg(&sc.pixelSeeds[pix]);
    Sampler g;
    g.randSeed = seed.x * (uint32_t)freeCounter + seed.y;
    g.sampleSeed = seed.x * seed.y;
    g.sampleOffset = sampleOffset;
    g.dim = 0;
    g.mode = sc.sampler;
    g.rowCache = row;
    g.mats = sc.sobol;
    v2 scr = mk2((float)px, (float)py) / mk2((float)sc.filmW, (float)sc.filmH);
    float u0 = sample1D(g), u1 = sample1D(g), u2 = sample1D(g), u3 = sample1D(g);
    Ray ray = thinLensCameraSampleRay(sc, scr, u0, u1, u2, u3);
    v3 result = pathTrace(sc, pp, ray, g);
    v3 last = mk3(0.0f);
    if (spp != 0) {
        float4 f = frame[pix];
        last = mk3(f.x, f.y, f.z);
    }
    if (!hasNan(result)) {
        v3 r = last + result;
        frame[pix] = make_float4(r.x, r.y, r.z, 1.0f);
    }
}

// sampleOffset = uSpp * uSampleDim, minus the table size once when beyond it
// (path_integ_naive.glsl:163-164), in 32-bit arithmetic.
uint32_t sample_offset(int32_t spp) {
    const int32_t sampleNum = 131072, sampleDim = 256;
    int32_t off = (int32_t)((uint32_t)spp * (uint32_t)sampleDim);
    if (off > sampleNum * sampleDim) off -= sampleNum * sampleDim;
    return (uint32_t)off;
}

}  // namespace

cudaError_t launch_path_pass(const zgl_scene* s, const zgl_integrator_params& p, int32_t spp, int32_t freeCounter,
                             float4* frame, cudaStream_t st) {
    PathParams pp{p.max_depth, p.russian_roulette, p.rr_start_depth, p.sample_light, p.light_env_uniform_sample,
                  p.light_portion};
    dim3 block(kTileX, kTileY);
    dim3 grid((unsigned)((s->filmW + kTileX - 1) / kTileX), (unsigned)((s->filmH + kTileY - 1) / kTileY));
    path_kernel<<<grid, block, 0, st>>>(s->view(), pp, spp, freeCounter, sample_offset(spp), frame);
    return cudaGetLastError();
}

}  // namespace zgl

using namespace zgl;

namespace {

void check_params(const zgl_integrator_params& p) {
    if (p.max_depth < 0 || p.max_depth > 1024) fail(ZGL_ERR_INVALID_ARG, "integrator: max_depth %d out of range", p.max_depth);
    if (p.rr_start_depth < 1) fail(ZGL_ERR_INVALID_ARG, "integrator: rr_start_depth must be >= 1");
    if (!(p.light_portion >= 0.0f && p.light_portion <= 1.0f))
        fail(ZGL_ERR_INVALID_ARG, "integrator: light_portion must lie in [0, 1]");
}

bool is_device_memory(const void* p) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" {

zgl_status zgl_integrator_params_default(zgl_integrator_params* p) {
    ZGL_API_BEGIN
    if (!p) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_params_default: NULL");
    p->max_depth = 4;
    p->russian_roulette = 0;
    p->rr_start_depth = 1;
    p->sample_light = 1;
    p->light_env_uniform_sample = 0;
    p->light_portion = 0.5f;
    p->finite_sample = 0;
    p->max_sample = 64;
    ZGL_API_END
}

zgl_status zgl_integrator_create(zgl_scene* scene, int32_t kind, const zgl_integrator_params* params,
                                 zgl_integrator** out) {
    ZGL_API_BEGIN
    if (!scene || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_create: NULL argument");
    *out = nullptr;
    if (scene->host_only) fail(ZGL_ERR_STATE, "zgl_integrator_create: scene was created host-only");
    if (kind != ZGL_INTEGRATOR_PATH) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_create: unknown kind %d", kind);
    zgl_integrator_params p;
    zgl_integrator_params_default(&p);
    if (params) p = *params;
    check_params(p);
    auto* it = new zgl_integrator();
    it->scene = scene;
    it->kind = kind;
    it->params = p;
    cudaError_t e = cudaMalloc(&it->d_frame, sizeof(float4) * (size_t)scene->filmW * scene->filmH);
    if (e == cudaSuccess) e = cudaMemset(it->d_frame, 0, sizeof(float4) * (size_t)scene->filmW * scene->filmH);
    if (e != cudaSuccess) {
        if (it->d_frame) cudaFree(it->d_frame);
        delete it;
        cuda_check(e, "zgl_integrator_create");
    }
    *out = it;
    ZGL_API_END
}

zgl_status zgl_integrator_render_pass(zgl_integrator* it, void* stream) {
    ZGL_API_BEGIN
    if (!it) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_render_pass: NULL");
    it->freeCounter++;  // NaivePath.cpp:79: counts every call
    if (it->params.finite_sample && it->curSample > it->params.max_sample) {
        it->finished = true;
        return ZGL_OK;
    }
    ZGL_CUDA(launch_path_pass(it->scene, it->params, it->curSample, it->freeCounter, it->d_frame,
                              (cudaStream_t)stream));
    it->curSample++;
    ZGL_API_END
}

zgl_status zgl_integrator_reset(zgl_integrator* it) {
    ZGL_API_BEGIN
    if (!it) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_reset: NULL");
    it->curSample = 0;
    it->finished = false;
    ZGL_API_END
}

zgl_status zgl_integrator_frame(zgl_integrator* it, float* out, int32_t* spp, void* stream) {
    ZGL_API_BEGIN
    if (!it || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_frame: NULL");
    size_t bytes = sizeof(float4) * (size_t)it->scene->filmW * it->scene->filmH;
    cudaStream_t st = (cudaStream_t)stream;
    if (is_device_memory(out)) {
        ZGL_CUDA(cudaMemcpyAsync(out, it->d_frame, bytes, cudaMemcpyDeviceToDevice, st));
    } else {
        ZGL_CUDA(cudaMemcpyAsync(out, it->d_frame, bytes, cudaMemcpyDeviceToHost, st));
        ZGL_CUDA(cudaStreamSynchronize(st));
    }
    if (spp) *spp = it->curSample;
    ZGL_API_END
}

zgl_status zgl_integrator_result_scale(const zgl_integrator* it, float* out) {
    ZGL_API_BEGIN
    if (!it || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_result_scale: NULL");
    *out = 1.0f / (float)(it->curSample + 1);
    ZGL_API_END
}

zgl_status zgl_integrator_destroy(zgl_integrator* it) {
    ZGL_API_BEGIN
    if (!it) return ZGL_OK;
    if (it->d_frame) cudaFree(it->d_frame);
    delete it;
    ZGL_API_END
}

}  // extern "C"
