// render_kernels.cuh — the integrator kernels (path tracer, light tracer,
// triple integrator) and their launchers, compiled twice: by render.cu into
// zgl::plain with the plain traversal calls, and by render_long.cu into
// zgl::long_rays with long rays finished by the lanes that trace together
// (shading.cuh, ZGL_LONG_RAYS).  The integrator entry points pick the
// long-ray kernels for trees of at least kLongRayMinEntries table entries.
//
// The path tracer restates path_integ_naive.glsl (pathIntegTrace :35-143,
// main :145-174).  Pixels are mapped to 16x8 tiles so that a warp's camera
// rays are neighbours.  The 256 Sobol values of the pass's sample row are
// computed once per block into shared memory.
#pragma once

#ifndef ZGL_RENDER_NS
#error "define ZGL_RENDER_NS (plain or long_rays) before including render_kernels.cuh"
#endif
#ifndef ZGL_LONG_RAYS
#define ZGL_LONG_RAYS 0
#endif

#include <algorithm>
#include <atomic>
#include <cmath>

#include "batch_flat.h"
#include "path_trace.cuh"
#include "scene.h"
#include "shading.cuh"
#include "zgl_internal.h"

namespace zgl {
namespace ZGL_RENDER_NS {
namespace {

// main() of path_integ_naive.glsl:145-174; MINB = minimum resident blocks
// per SM (1: uncapped registers, kOccupied: full occupancy)
template <bool FULL, int MINB>
__global__ void __launch_bounds__(kTileX* kTileY, MINB)
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
    v3 result = pathTrace<FULL>(sc, pp, ray, g);
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

constexpr int kOccupied = 16;  // blocks of 128 threads per SM: 2048 threads

// SM count of the current device (cached per device)
int sm_count() {
    static std::atomic<int> cache[64];
    int dev = 0;
    cudaGetDevice(&dev);
    const bool cached = dev >= 0 && dev < 64;
    int n = cached ? cache[dev].load(std::memory_order_relaxed) : 0;
    if (n == 0) {
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
        if (cached) cache[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

// Occupancy: the integrator kernels are bound by instruction fetch and
// latency, not by registers.  Full occupancy (kOccupied blocks of 128 threads
// per SM, at most 32 registers a thread, the rest spilled to L1) is measured
// fastest whenever the grid fills the GPU: the 16-pass Cornell launch 4.85 ->
// 3.11 ms, the 1080p city pass 26.2 -> 22.7 ms, the batch 3.12 -> 1.99 s.
// A single pass of a small film (fewer than eight blocks per SM) keeps the
// uncapped instantiation of path_kernel (0.41 vs 0.49 ms for 256x256), and
// the light tracer stays uncapped (4.45 vs 4.63 ms).
// Several consecutive passes in one launch: pass j = blockIdx.z renders
// sample c0 + j with freeCounter f0 + j, exactly as path_kernel would, into
// out[j][pix] (NaN samples kept, the accumulation drops them).
template <bool FULL>
__global__ void __launch_bounds__(kTileX* kTileY, kOccupied)
path_passes_kernel(DeviceScene sc, PathParams pp, int32_t c0, int32_t f0, float* __restrict__ out) {
    __shared__ uint32_t row[256];
    const int32_t j = blockIdx.z;
    const uint32_t off = sample_offset(c0 + j);
    load_sobol_row(sc, off, row);
    const int px = blockIdx.x * kTileX + threadIdx.x;
    const int py = blockIdx.y * kTileY + threadIdx.y;
    if (px >= sc.filmW || py >= sc.filmH) return;
    const size_t npix = (size_t)sc.filmW * sc.filmH;
    const size_t pix = (size_t)py * sc.filmW + px;
    const uint2 seed = __ldg(&sc.pixelSeeds[pix]);
    Sampler g;
    g.randSeed = seed.x * (uint32_t)(f0 + j) + seed.y;
    g.sampleSeed = seed.x * seed.y;
    g.sampleOffset = off;
    g.dim = 0;
    g.mode = sc.sampler;
    g.rowCache = row;
    g.mats = sc.sobol;
    v2 scr = mk2((float)px, (float)py) / mk2((float)sc.filmW, (float)sc.filmH);
    float u0 = sample1D(g), u1 = sample1D(g), u2 = sample1D(g), u3 = sample1D(g);
    Ray ray = thinLensCameraSampleRay(sc, scr, u0, u1, u2, u3);
    v3 r = pathTrace<FULL>(sc, pp, ray, g);
    float* o = out + 3 * ((size_t)j * npix + pix);
    o[0] = r.x;
    o[1] = r.y;
    o[2] = r.z;
}

// The frame updates of those passes in pass order, as consecutive
// path_kernel launches make them (main(), path_integ_naive.glsl:166-173):
// a pass with sample index 0 starts from zero, a NaN sample leaves the pixel
// as it was.
__global__ void accumulate_passes_kernel(const float* __restrict__ in, int64_t npix, int32_t c0, int32_t n,
                                         float4* __restrict__ frame) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const float4 f = frame[p];
    v3 acc = mk3(f.x, f.y, f.z);
    bool written = false;
    for (int j = 0; j < n; j++) {
        const float* x = in + 3 * ((size_t)j * npix + p);
        const v3 r = mk3(x[0], x[1], x[2]);
        const v3 last = (c0 + j != 0) ? acc : mk3(0.0f);
        if (!hasNan(r)) {
            acc = last + r;
            written = true;
        }
    }
    if (written) frame[p] = make_float4(acc.x, acc.y, acc.z, 1.0f);
}

#if !ZGL_LONG_RAYS
// Flat schedule of the batched renderer (batch_flat.h): block b is a 16x8
// tile of one sample of one request.
template <bool FULL>
__global__ void __launch_bounds__(kTileX* kTileY, kOccupied) batch_flat_kernel(const __grid_constant__ FlatLaunch L) {
    const int64_t blk = blockIdx.x;
    int lo = 0, hi = L.nreq - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (L.req[mid].blockBase <= blk) lo = mid;
        else hi = mid - 1;
    }
    const FlatRequest& rq = L.req[lo];
    const int64_t local = blk - rq.blockBase;
    const int64_t perSample = (int64_t)rq.tilesX * rq.tilesY;
    const int j = L.j0 + (int)(local / perSample);
    const int64_t tile = local % perSample;
    const DeviceScene& sc = rq.sc;
    // the block's sample row, staged in shared memory
    __shared__ uint32_t row[256];
    for (int i = threadIdx.y * kTileX + threadIdx.x; i < 256; i += kTileX * kTileY)
        row[i] = __ldg(&L.rows[256 * (size_t)j + i]);
    __syncthreads();
    const int px = (int)(tile % rq.tilesX) * kTileX + threadIdx.x;
    const int py = (int)(tile / rq.tilesX) * kTileY + threadIdx.y;
    if (px >= sc.filmW || py >= sc.filmH) return;
    const size_t pix = (size_t)py * sc.filmW + px;
    const uint2 seed = __ldg(&sc.pixelSeeds[pix]);
    Sampler g;
    g.randSeed = seed.x * (uint32_t)(j + 1) + seed.y;
    g.sampleSeed = seed.x * seed.y;
    g.sampleOffset = sample_offset(j);
    g.dim = 0;
    g.mode = sc.sampler;
    g.rowCache = row;
    g.mats = L.mats;
    const PathParams pp{rq.maxDepth, rq.rr, rq.rrStart, rq.sampleLight, rq.uniformSel, rq.portion};
    v2 scr = mk2((float)px, (float)py) / mk2((float)sc.filmW, (float)sc.filmH);
    float u0 = sample1D(g), u1 = sample1D(g), u2 = sample1D(g), u3 = sample1D(g);
    Ray ray = thinLensCameraSampleRay(sc, scr, u0, u1, u2, u3);
    v3 r = pathTrace<FULL>(sc, pp, ray, g);
    float* o = rq.scratch + 3 * ((size_t)(j - L.j0) * ((size_t)sc.filmW * sc.filmH) + pix);
    o[0] = r.x;
    o[1] = r.y;
    o[2] = r.z;
}
#endif

// Film of the light-tracing passes, float[H][W][3].  int(uv * size) == size
// (uv on the far edge) falls outside the image and is dropped, as an
// out-of-range imageAtomicAdd is.
__device__ __forceinline__ void accumulateFilm(const DeviceScene& sc, float* film, v2 uv, v3 res) {
    if (!inFilmBound(uv)) return;
    int x = zf2i(uv.x * (float)sc.filmW), y = zf2i(uv.y * (float)sc.filmH);
    if (x >= sc.filmW || y >= sc.filmH) return;
    float* p = film + 3 * ((size_t)y * sc.filmW + x);
    atomicAdd(p, res.x);
    atomicAdd(p + 1, res.y);
    atomicAdd(p + 2, res.z);
}

template <bool FULL>
__device__ __forceinline__ void shadeSurface(const DeviceScene& sc, int id, v3 pos, v3 wo, Surface& surf,
                                             uint32_t& matType, BSDFParam& mp) {
    TriShade tri = loadTri(sc, id);
    surf = surfaceInfo(tri, pos);
    int matId = tri.matTex & 0x0000ffff;
    matType = loadMaterialType(sc, matId);
    if (matType != kDielectric && matType != kThinDielectric && dot(surf.ns, wo) < 0.0f) {
        surf.ns = -surf.ns;
        surf.ng = -surf.ng;
    }
    mp = loadMaterial<FULL>(sc, matType, tri.matTex, id, surf);
}

// lightIntegTrace (light_path_integ.glsl:45-146); the light tracer forces the
// independent sampler (LightPath.cpp:49), so every dimension is rand().
template <bool FULL>
__device__ void lightTrace(const DeviceScene& sc, const PathParams& pp, Sampler& g, float* film) {
    float a0 = rand01(g), a1 = rand01(g);
    int light = lightSampleOne(sc, mk2(a0, a1));
    float pdfSource = lightPdfSampleOne(sc, light);
    Ray ray;
    v3 wo, throughput;
    {
        int triId = light + sc.objPrimCount;
        float b0 = rand01(g), b1 = rand01(g);
        TriShade t = loadTri(sc, triId);
        v3 pLit = sampleTriangleUniform(t.a, t.b, t.c, mk2(b0, b1));
        float c0 = rand01(g), c1 = rand01(g);
        CameraIiSample ci = thinLensCameraSampleIi(sc, pLit, mk2(c0, c1));
        if (ci.pdf > 0.0f) {
            v3 pCam = pLit + ci.wi * ci.dist;
            float area;
            lightPowerOf(sc, light, area);
            float pdfPos = 1.0f / area;
            if (visible(sc, pLit, pCam)) {
                v3 Le = lightLe(sc, light, pLit, ci.wi);
                v3 contrib = Le * ci.Ii / (ci.pdf * pdfPos * pdfSource);
                if (!isBlack(contrib)) accumulateFilm(sc, film, ci.uv, contrib);
            }
        }
        float d0 = rand01(g), d1 = rand01(g), d2 = rand01(g), d3 = rand01(g);
        LightLeSample le = lightSampleOneLe(sc, light, d0, d1, d2, d3);
        v3 nl = geomNormal(sc, triId, le.ray.ori);
        wo = -le.ray.dir;
        ray = rayOffseted(le.ray.ori, le.ray.dir);
        throughput = le.Le * absDot(nl, -wo) / (pdfSource * le.pdfPos * le.pdfDir);
    }
    for (int bounce = 1; bounce <= pp.maxDepth; bounce++) {
        float dist;
        int id = bvhHit(sc, ray, dist);
        if (id == -1) break;
        if (id - sc.objPrimCount >= 0) break;
        v3 pos = rayPoint(ray, dist);
        Surface surf;
        uint32_t matType;
        BSDFParam mp;
        shadeSurface<FULL>(sc, id, pos, wo, surf, matType, mp);
        {
            float c0 = rand01(g), c1 = rand01(g);
            CameraIiSample ci = thinLensCameraSampleIi(sc, pos, mk2(c0, c1));
            if (ci.pdf > 0.0f) {
                v3 pCam = pos + ci.wi * ci.dist;
                if (visible(sc, pos, pCam)) {
                    v3 bsdf = materialBSDF<FULL>(matType, mp, wo, ci.wi, surf.ns, kImportance);
                    float cosWi = satDot(surf.ng, ci.wi) * fabsf(dot(surf.ns, wo) / dot(surf.ng, wo));
                    v3 res = ci.Ii * bsdf * throughput * cosWi / ci.pdf;
                    if (!hasNan(res) && !zisnan(ci.pdf) && ci.pdf > 1e-8f && !isBlack(res))
                        accumulateFilm(sc, film, ci.uv, res);
                }
            }
        }
        float b0 = rand01(g), b1 = rand01(g), b2 = rand01(g);
        BSDFSample bs = materialSample<FULL>(matType, mp, surf.ns, wo, mk3(b0, b1, b2), g, kImportance);
        v3 wi = bs.wi;
        float bsdfPdf = bs.pdf;
        bool deltaBsdf = (bs.flag == kSpecRefl || bs.flag == kSpecTrans);
        if (bsdfPdf < 1e-8f || zisnan(bsdfPdf)) break;
        if (pp.rr && bounce >= pp.rrStart) {
            float continueProb = zmin(maxComponent(bs.bsdf / bsdfPdf), 1.0f);
            if (rand01(g) >= continueProb) break;
            throughput = throughput / continueProb;
        }
        float cosWi = deltaBsdf ? 1.0f : fabsf(dot(surf.ng, wi) * dot(surf.ns, wo) / dot(surf.ng, wo));
        throughput = throughput * (bs.bsdf * cosWi / bsdfPdf);
        ray = rayOffseted(pos, wi);
        wo = -wi;
    }
}

__device__ __forceinline__ float weightS0(float s1s0, float t1s0) { return 1.0f / (1.0f + s1s0 + t1s0); }
__device__ __forceinline__ float weightS1(float s1s0, float t1s1) { return s1s0 / (1.0f + s1s0 + s1s0 * t1s1); }
__device__ __forceinline__ float weightT1(float s0t1, float s1t1) { return 1.0f / (s0t1 + s1t1 + 1.0f); }

// traceCameraPath (triple_path_pass_pt.glsl:59-195)
template <bool FULL>
__device__ v3 tripleCameraTrace(const DeviceScene& sc, const PathParams& pp, Ray ray, Sampler& g) {
    float primDist;
    int id = bvhHit(sc, ray, primDist);
    v3 pos = rayPoint(ray, primDist);
    if (id == -1) return envLe(sc, ray.dir);
    if (id - sc.objPrimCount >= 0) return lightLe(sc, id - sc.objPrimCount, pos, -ray.dir);
    Surface surf = surfaceInfo(loadTri(sc, id), pos);
    v3 wo = -ray.dir;
    v3 prevNorm = f3(sc.camF);
    v3 result = mk3(0.0f), throughput = mk3(1.0f);
    PdfPair camPdf = thinLensCameraPdfIe(sc, ray);
    float primaryPdf = remap(camPdf.pdfPos) / remap(camPdf.pdfDir * absDot(surf.ns, ray.dir) / sq(primDist));
    float t1s0 = primaryPdf, t1s1 = primaryPdf;
    for (int bounce = 1; bounce <= pp.maxDepth; bounce++) {
        TriShade tri = loadTri(sc, id);
        if (bounce > 1) surf = surfaceInfo(tri, pos);
        int matId = tri.matTex & 0x0000ffff;
        uint32_t matType = loadMaterialType(sc, matId);
        if (matType != kDielectric && matType != kThinDielectric && dot(surf.ns, wo) < 0.0f) {
            surf.ns = -surf.ns;
            surf.ng = -surf.ng;
        }
        BSDFParam mp = loadMaterial<FULL>(sc, matType, tri.matTex, id, surf);
        {
            float a0 = sample1D(g), a1 = sample1D(g);
            int light = lightSampleOne(sc, mk2(a0, a1));
            int triId = light + sc.objPrimCount;
            float pdfSource = lightPdfSampleOne(sc, light);
            float b0 = sample1D(g), b1 = sample1D(g);
            TriShade lt = loadTri(sc, triId);
            v3 pLit = sampleTriangleUniform(lt.a, lt.b, lt.c, mk2(b0, b1));
            v3 wi = normalize(pLit - pos);
            v3 Le = lightLe(sc, light, pLit, -wi);
            if (!isBlack(Le) && visible(sc, pos, pLit)) {
                v3 nLit = surfaceInfo(lt, pLit).ng;
                float area;
                lightPowerOf(sc, light, area);
                float pA = pdfSource / area;
                float dist2 = distSquare(pos, pLit);
                float pS = pA * dist2 / absDot(nLit, wi);
                v3 f = materialBSDF<FULL>(matType, mp, wo, wi, surf.ns);
                float fpdf = materialPdf<FULL>(matType, mp, wo, wi, surf.ns);
                float pdfRev = materialPdf<FULL>(matType, mp, wi, wo, surf.ns);
                float pdfPLit = remap(pA);
                float coefToSurf = remap(0.5f * kPiInv * absDot(surf.ns, wi));
                float coefToLight = remap(fpdf * satDot(nLit, -wi));
                float coefToPrev = (bounce == 1) ? 1.0f : remap(pdfRev * absDot(prevNorm, wo));
                float coefDist = remap(dist2);
                float weight = weightS1(pdfPLit * coefDist / coefToLight, t1s1 * coefToSurf * coefToPrev / coefDist);
                result = result + Le * f * throughput * absDot(surf.ns, wi) / pS * weight;
            }
        }
        float b0 = sample1D(g), b1 = sample1D(g), b2 = sample1D(g);
        BSDFSample bs = materialSample<FULL>(matType, mp, surf.ns, wo, mk3(b0, b1, b2), g);
        v3 wi = bs.wi;
        float bsdfPdf = bs.pdf;
        bool deltaBsdf = (bs.flag == kSpecRefl || bs.flag == kSpecTrans);
        if (bsdfPdf < 1e-8f) break;
        throughput = throughput * (bs.bsdf / bsdfPdf * (deltaBsdf ? 1.0f : absDot(surf.ns, wi)));
        Ray nextRay = rayOffseted(pos, wi);
        float dist;
        int nextId = bvhHit(sc, nextRay, dist);
        int lightId = nextId - sc.objPrimCount;
        v3 nextPos = rayPoint(nextRay, dist);
        float pdfDirToNext = materialPdf<FULL>(matType, mp, wo, wi, surf.ns);
        float pdfDirToPrev = materialPdf<FULL>(matType, mp, wi, wo, surf.ns);
        if (nextId == -1) break;
        if (lightId >= 0) {
            v3 nLit = geomNormal(sc, nextId, nextPos);
            PdfPair pdfLit = lightPdfLe(sc, lightId, Ray{nextPos, -wi});
            float pdfPLit = remap(pdfLit.pdfPos * lightPdfSampleOne(sc, lightId));
            float coefToLight = remap(pdfDirToNext * satDot(nLit, -wi));
            float coefToSurf = remap(pdfLit.pdfDir * absDot(surf.ns, wi));
            float coefToPrev = (bounce == 1) ? 1.0f : remap(pdfDirToPrev * absDot(prevNorm, wo));
            float coefDist = remap(dist * dist);
            float weight = zisnan(t1s0) ? 0.0f
                                        : weightS0(pdfPLit * coefDist / coefToLight,
                                                   t1s0 * coefToSurf * pdfPLit * coefToPrev / coefToLight);
            result = result + lightLe(sc, lightId, nextPos, -wi) * throughput * weight;
            break;
        }
        if (pp.rr && bounce >= pp.rrStart) {
            float continueProb = zmin(maxComponent(bs.bsdf / bsdfPdf), 0.95f);
            if (sample1D(g) >= continueProb) break;
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

// traceLightPath (triple_path_pass_lpt.glsl:58-182)
template <bool FULL>
__device__ void tripleLightTrace(const DeviceScene& sc, const PathParams& pp, Sampler& g, float* film, float uScale) {
    float a0 = rand01(g), a1 = rand01(g);
    int light = lightSampleOne(sc, mk2(a0, a1));
    float pdfSource = lightPdfSampleOne(sc, light);
    Ray ray;
    v3 wo, throughput, prevNorm;
    float prevPdfDir, s0t1, s1t1;
    {
        int triId = light + sc.objPrimCount;
        rand01(g);  // the reference samples a point here and never uses it
        rand01(g);
        float d0 = rand01(g), d1 = rand01(g), d2 = rand01(g), d3 = rand01(g);
        LightLeSample le = lightSampleOneLe(sc, light, d0, d1, d2, d3);
        v3 nl = geomNormal(sc, triId, le.ray.ori);
        wo = -le.ray.dir;
        ray = rayOffseted(le.ray.ori, le.ray.dir);
        throughput = le.Le * absDot(nl, -wo) / (pdfSource * le.pdfPos * le.pdfDir);
        prevNorm = nl;
        prevPdfDir = le.pdfDir;
        s0t1 = 1.0f / remap(le.pdfPos * pdfSource);
        s1t1 = 1.0f;
    }
    for (int bounce = 1; bounce <= pp.maxDepth; bounce++) {
        float dist;
        int id = bvhHit(sc, ray, dist);
        if (id == -1) break;
        if (id - sc.objPrimCount >= 0) break;
        v3 pos = rayPoint(ray, dist);
        TriShade tri = loadTri(sc, id);
        Surface surf = surfaceInfo(tri, pos);
        int matId = tri.matTex & 0x0000ffff;
        uint32_t matType = loadMaterialType(sc, matId);
        if (matType != kDielectric && matType != kThinDielectric && dot(surf.ns, wo) < 0.0f) {
            surf.ns = -surf.ns;
            surf.ng = -surf.ng;
        }
        float coefToPos = remap(prevPdfDir * absDot(surf.ns, wo));
        s0t1 /= coefToPos;
        s1t1 /= coefToPos / (bounce == 1 ? remap(dist * dist) : 1.0f);
        BSDFParam mp = loadMaterial<FULL>(sc, matType, tri.matTex, id, surf);
        {
            float c0 = rand01(g), c1 = rand01(g);
            CameraIiSample ci = thinLensCameraSampleIi(sc, pos, mk2(c0, c1));
            if (ci.pdf > 0.0f) {
                v3 pCam = pos + ci.wi * ci.dist;
                if (visible(sc, pos, pCam)) {
                    float cosWi = satDot(surf.ng, ci.wi) * fabsf(dot(surf.ns, wo) / dot(surf.ng, wo));
                    v3 bsdf = materialBSDF<FULL>(matType, mp, wo, ci.wi, surf.ns, kImportance);
                    v3 contrib = ci.Ii * bsdf * throughput * cosWi / ci.pdf;
                    float coefToSurf = remap(thinLensCameraPdfIe(sc, Ray{pCam, -ci.wi}).pdfDir * satDot(surf.ns, ci.wi));
                    float coefToPrev = remap(materialPdf<FULL>(matType, mp, ci.wi, wo, surf.ns) * absDot(prevNorm, wo));
                    float coefDist = remap(ci.dist * ci.dist);
                    float coef0 = coefToSurf * coefToPrev / coefDist;
                    float coef1 = ((bounce == 1) ? 1.0f : coefToPrev) * coefToSurf / coefDist;
                    float weight = weightT1(s0t1 * coef0, s1t1 * coef1);
                    v3 res = contrib * weight;
                    if (!hasNan(res) && !zisnan(ci.pdf) && ci.pdf > 1e-8f && !isBlack(res))
                        accumulateFilm(sc, film, ci.uv, res * uScale);
                }
            }
        }
        float b0 = rand01(g), b1 = rand01(g), b2 = rand01(g);
        BSDFSample bs = materialSample<FULL>(matType, mp, surf.ns, wo, mk3(b0, b1, b2), g, kImportance);
        v3 wi = bs.wi;
        float bsdfPdf = bs.pdf;
        bool deltaBsdf = (bs.flag == kSpecRefl || bs.flag == kSpecTrans);
        if (bsdfPdf < 1e-8f || zisnan(bsdfPdf)) break;
        if (pp.rr && bounce >= pp.rrStart) {
            float continueProb = zmin(maxComponent(bs.bsdf / bsdfPdf), 1.0f);
            if (rand01(g) >= continueProb) break;
            throughput = throughput / continueProb;
        }
        float coefToPrev = remap(materialPdf<FULL>(matType, mp, wi, wo, surf.ns) * absDot(prevNorm, wo));
        s0t1 *= coefToPrev;
        s1t1 *= (bounce == 1) ? 1.0f : coefToPrev;
        prevPdfDir = materialPdf<FULL>(matType, mp, wo, wi, surf.ns);
        prevNorm = surf.ns;
        float cosWi = deltaBsdf ? 1.0f : fabsf(dot(surf.ng, wi) * dot(surf.ns, wo) / dot(surf.ng, wo));
        throughput = throughput * (bs.bsdf * cosWi / bsdfPdf);
        ray = rayOffseted(pos, wi);
        wo = -wi;
    }
}

constexpr int kLightBlock = 256;

// main() of light_path_integ.glsl:148-158: logical group 1536 x blocks
template <bool FULL>
__global__ void __launch_bounds__(kLightBlock)
light_kernel(DeviceScene sc, PathParams pp, uint32_t spp, uint32_t freeCounter, uint32_t nPaths, float* film) {
    uint32_t gid = blockIdx.x * kLightBlock + threadIdx.x;
    if (gid >= nPaths) return;
    Sampler g;
    g.randSeed = spp * nPaths + gid + freeCounter;
    g.sampleSeed = 0;
    g.sampleOffset = 0;
    g.dim = 0;
    g.mode = 0;
    g.rowCache = nullptr;
    g.mats = sc.sobol;
    lightTrace<FULL>(sc, pp, g, film);
}

// main() of triple_path_pass_pt.glsl:197-224 (addFilm: one owner per pixel)
template <bool FULL>
__global__ void __launch_bounds__(kTileX* kTileY, kOccupied)
triple_pt_kernel(DeviceScene sc, PathParams pp, int32_t spp, int32_t freeCounter, uint32_t sampleOffset,
                 float* __restrict__ film) {
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
    v3 r = tripleCameraTrace<FULL>(sc, pp, ray, g);
    if (!hasNan(r)) {
        float* p = film + 3 * pix;
        p[0] = p[0] + r.x;
        p[1] = p[1] + r.y;
        p[2] = p[2] + r.z;
    }
}

// main() of triple_path_pass_lpt.glsl:184-191
template <bool FULL>
__global__ void __launch_bounds__(kLightBlock, kOccupied / 2)
triple_lpt_kernel(DeviceScene sc, PathParams pp, uint32_t spp, uint32_t freeCounter, uint32_t nThreads,
                  uint32_t loops, float uScale, float* film) {
    uint32_t gid = blockIdx.x * kLightBlock + threadIdx.x;
    if (gid >= nThreads) return;
    Sampler g;
    g.randSeed = spp * (nThreads * loops) + gid + freeCounter;
    g.sampleSeed = 0;
    g.sampleOffset = 0;
    g.dim = 0;
    g.mode = 0;
    g.rowCache = nullptr;
    g.mats = sc.sobol;
    for (uint32_t i = 0; i < loops; i++) tripleLightTrace<FULL>(sc, pp, g, film, uScale);
}

#if !ZGL_LONG_RAYS
// img_copy_1x32f_4x32f.glsl: film (r, g, b) -> frame (r, g, b, 1)
__global__ void film_to_frame_kernel(const float* __restrict__ film, float4* __restrict__ out, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = make_float4(film[3 * i], film[3 * i + 1], film[3 * i + 2], 1.0f);
}
#endif

}  // namespace

cudaError_t launch_path_pass(const zgl_scene* s, const zgl_integrator_params& p, int32_t spp, int32_t freeCounter,
                             float4* frame, cudaStream_t st) {
    PathParams pp{p.max_depth, p.russian_roulette, p.rr_start_depth, p.sample_light, p.light_env_uniform_sample,
                  p.light_portion};
    dim3 block(kTileX, kTileY);
    dim3 grid((unsigned)((s->filmW + kTileX - 1) / kTileX), (unsigned)((s->filmH + kTileY - 1) / kTileY));
    const bool fills = (int64_t)grid.x * grid.y >= 8 * (int64_t)sm_count();
    const DeviceScene v = s->view();
    const uint32_t off = sample_offset(spp);
    if (s->fullMaterials) {
        if (fills) path_kernel<true, kOccupied><<<grid, block, 0, st>>>(v, pp, spp, freeCounter, off, frame);
        else path_kernel<true, 1><<<grid, block, 0, st>>>(v, pp, spp, freeCounter, off, frame);
    } else {
        if (fills) path_kernel<false, kOccupied><<<grid, block, 0, st>>>(v, pp, spp, freeCounter, off, frame);
        else path_kernel<false, 1><<<grid, block, 0, st>>>(v, pp, spp, freeCounter, off, frame);
    }
    return cudaGetLastError();
}

cudaError_t launch_path_passes(const zgl_scene* s, const zgl_integrator_params& p, int32_t c0, int32_t f0, int32_t n,
                               float* scratch, float4* frame, cudaStream_t st) {
    PathParams pp{p.max_depth, p.russian_roulette, p.rr_start_depth, p.sample_light, p.light_env_uniform_sample,
                  p.light_portion};
    dim3 block(kTileX, kTileY);
    dim3 grid((unsigned)((s->filmW + kTileX - 1) / kTileX), (unsigned)((s->filmH + kTileY - 1) / kTileY), (unsigned)n);
    if (s->fullMaterials)
        path_passes_kernel<true><<<grid, block, 0, st>>>(s->view(), pp, c0, f0, scratch);
    else
        path_passes_kernel<false><<<grid, block, 0, st>>>(s->view(), pp, c0, f0, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int64_t npix = (int64_t)s->filmW * s->filmH;
    accumulate_passes_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(scratch, npix, c0, n, frame);
    return cudaGetLastError();
}

#if !ZGL_LONG_RAYS
cudaError_t launch_batch_flat(const FlatLaunch& L, cudaStream_t st) {
    if (L.nblocks <= 0) return cudaSuccess;
    if (L.full)
        batch_flat_kernel<true><<<(unsigned)L.nblocks, dim3(kTileX, kTileY), 0, st>>>(L);
    else
        batch_flat_kernel<false><<<(unsigned)L.nblocks, dim3(kTileX, kTileY), 0, st>>>(L);
    return cudaGetLastError();
}
#endif

cudaError_t launch_light_pass(const zgl_scene* s, const zgl_integrator_params& p, int32_t blocks, int32_t spp,
                              int32_t freeCounter, float* film, cudaStream_t st) {
    PathParams pp{p.max_depth, p.russian_roulette, p.rr_start_depth, p.sample_light, p.light_env_uniform_sample,
                  p.light_portion};
    uint32_t n = 1536u * (uint32_t)blocks;
    if (s->fullMaterials)
        light_kernel<true><<<(n + kLightBlock - 1) / kLightBlock, kLightBlock, 0, st>>>(s->view(), pp, (uint32_t)spp,
                                                                             (uint32_t)freeCounter, n, film);
    else
        light_kernel<false><<<(n + kLightBlock - 1) / kLightBlock, kLightBlock, 0, st>>>(s->view(), pp, (uint32_t)spp,
                                                                             (uint32_t)freeCounter, n, film);
    return cudaGetLastError();
}

cudaError_t launch_triple_pass(const zgl_scene* s, const zgl_integrator_params& p, int32_t blocks, int32_t loops,
                               int32_t spp, int32_t freeCounter, float* film, cudaStream_t st) {
    PathParams pp{p.max_depth, p.russian_roulette, p.rr_start_depth, p.sample_light, p.light_env_uniform_sample,
                  p.light_portion};
    dim3 block(kTileX, kTileY);
    dim3 grid((unsigned)((s->filmW + kTileX - 1) / kTileX), (unsigned)((s->filmH + kTileY - 1) / kTileY));
    if (s->fullMaterials)
        triple_pt_kernel<true><<<grid, block, 0, st>>>(s->view(), pp, spp, freeCounter, sample_offset(spp), film);
    else
        triple_pt_kernel<false><<<grid, block, 0, st>>>(s->view(), pp, spp, freeCounter, sample_offset(spp), film);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    uint32_t n = 1536u * (uint32_t)blocks;
    float uScale = (float)(s->filmW * s->filmH) / (float)(blocks * loops * 1536);
    if (s->fullMaterials)
        triple_lpt_kernel<true><<<(n + kLightBlock - 1) / kLightBlock, kLightBlock, 0, st>>>(
        s->view(), pp, (uint32_t)spp, (uint32_t)freeCounter, n, (uint32_t)loops, uScale, film);
    else
        triple_lpt_kernel<false><<<(n + kLightBlock - 1) / kLightBlock, kLightBlock, 0, st>>>(
        s->view(), pp, (uint32_t)spp, (uint32_t)freeCounter, n, (uint32_t)loops, uScale, film);
    return cudaGetLastError();
}

#if !ZGL_LONG_RAYS
cudaError_t launch_film_to_frame(const float* film, float4* out, int64_t n, cudaStream_t st) {
    film_to_frame_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(film, out, n);
    return cudaGetLastError();
}
#endif

}  // namespace ZGL_RENDER_NS
}  // namespace zgl
