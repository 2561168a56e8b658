// render_diff.cu — differentiable path tracing by path replay.
//
// Forward: every (pixel, sample) path of the MIS path tracer
// (pathIntegTrace, path_integ_naive.glsl:35-143, with the plain integrator's
// seeds: sample s uses freeCounter = s + 1) is traced once; its radiance is
// kept per sample and the image is the per-pixel sum over samples in sample
// order divided by spp.
//
// Backward (Path Replay Backpropagation, Vicini, Speierer and Jakob 2021):
// each path is replayed from its seed (no path storage), with sampling
// decisions, pdfs, MIS weights and Russian roulette detached.  The replay
// carries the remaining radiance L_rem = L_total - (contributions already
// met); at a vertex whose sampled BSDF value f enters every later
// contribution, d/dtheta of those contributions is L_rem / f * df/dtheta per
// channel; a light sample at the vertex contributes C / f_light *
// df_light/dtheta; emission contributes C / P * dP for the emitting light
// instance's power P.  BSDF derivatives are analytic (bsdf_grad.cuh).
// Visibility discontinuities are not differentiated.  Gradients are summed
// across each warp in registers, then per block in shared memory, then added
// to the output with one global atomic per parameter per block.
// No counterpart in the reference.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#define ZGL_INLINE_MATH 1
#include "bsdf_grad.cuh"
#include "path_trace.cuh"
#include "scene.h"
#include "zgl_internal.h"

struct zgl_diff {
    zgl_scene* scene = nullptr;
    zgl_integrator_params params{};
    int32_t spp = 0;
    int32_t nmat = 0, ninst = 0, nparams = 0;
    float* d_samples = nullptr;   // spp * npix * 3 per-sample radiance
    // ray casts of the last forward, kept for the replay (null when they
    // would exceed the budget; the replay then traverses again)
    int2* d_hits = nullptr;       // kCastDepth * spp * npix (primitive id, distance bits)
    uint32_t* d_vis = nullptr;    // spp * npix light-sample occlusion bits
    bool castsValid = false;
    float* d_dimage = nullptr;    // npix * 3, zgl_diff_step_l2's dloss/dimage
    int32_t* d_lightInst = nullptr;  // per light triangle: instance index
    float* d_values = nullptr;       // current parameter values
    std::vector<uint32_t> lightFirst;
    std::vector<float> instPower;  // 3 per instance (current)
    std::vector<float> params_host;
};

namespace zgl {
namespace {

constexpr int kMaxDiffParams = 1024;

struct DiffInfo {
    int32_t nmat;
    int32_t nparams;
    const int32_t* lightInst;
};

// ----------------------------------------------------------------------------
// Ray casts kept between the forward pass and the replay.  The forward
// records, per (sample, pixel) path, the closest hits of its camera ray and
// first kCastDepth - 1 extension rays (primitive id and distance) and the
// occlusion answers of its first 32 light samples; the replay takes them in
// the same order instead of traversing again (casts past the record are
// traced).  Layout: hits[(k * spp + s) * npix + pix], vis[s * npix + pix], so
// that a warp's lanes (neighbouring pixels of one sample) store and load
// consecutive words.  8 bytes per cast: 640 MB for 512^2 pixels x 32 spp.
// ----------------------------------------------------------------------------
constexpr int kCastDepth = 9;
constexpr size_t kCastBudget = (size_t)4 << 30;  // bytes of cast records a renderer may keep

struct CastCursor {
    int nhit, nvis;
    uint32_t vis;
};

struct RecordCast {
    int2* hits;   // this path's first record; record k at hits[k * stride]
    size_t stride;
    CastCursor* cur;
    __device__ __forceinline__ int hit(const DeviceScene& sc, const Ray& r, float& dist) const {
        const int id = bvhHit(sc, r, dist);
        if (cur->nhit < kCastDepth) hits[(size_t)cur->nhit * stride] = make_int2(id, __float_as_int(dist));
        cur->nhit++;
        return id;
    }
    __device__ __forceinline__ bool operator()(const DeviceScene& sc, const Ray& r, float dist) const {
        const bool occ = bvhTest(sc, r, dist);
        if (cur->nvis < 32 && occ) cur->vis |= 1u << cur->nvis;
        cur->nvis++;
        return occ;
    }
};

struct ReplayCast {
    const int2* hits;
    size_t stride;
    CastCursor* cur;
    __device__ __forceinline__ int hit(const DeviceScene& sc, const Ray& r, float& dist) const {
        const int k = cur->nhit++;
        if (k < kCastDepth) {
            const int2 h = __ldg(hits + (size_t)k * stride);
            dist = __int_as_float(h.y);
            return h.x;
        }
        return bvhHit(sc, r, dist);
    }
    __device__ __forceinline__ bool operator()(const DeviceScene& sc, const Ray& r, float dist) const {
        const int k = cur->nvis++;
        if (k < 32) return (cur->vis >> k) & 1u;
        return bvhTest(sc, r, dist);
    }
};

// forward: one thread per (pixel, sample); blockIdx.y = sample.  Both
// kernels run at full occupancy (16 blocks of 128 threads per SM, at most 32
// registers a thread, spills in L1): at 512x512 and 32 spp that measured
// 49.4 -> 28.1 ms for the forward and 91.2 -> 50.5 ms for the replay against
// three to four blocks per SM without spills.
template <bool FULL>
__global__ void __launch_bounds__(kTileX* kTileY, 16)
diff_forward_kernel(DeviceScene sc, PathParams pp, int32_t tilesX, int32_t spp, float* __restrict__ samples,
                    int2* __restrict__ hits, uint32_t* __restrict__ vis) {
    __shared__ uint32_t row[256];
    const int32_t s = blockIdx.y;
    const uint32_t off = sample_offset(s);
    load_sobol_row(sc, off, row);
    const int tile = blockIdx.x;
    const int px = (tile % tilesX) * kTileX + threadIdx.x;
    const int py = (tile / tilesX) * kTileY + threadIdx.y;
    if (px >= sc.filmW || py >= sc.filmH) return;
    const size_t pix = (size_t)py * sc.filmW + px;
    const uint2 seed = __ldg(&sc.pixelSeeds[pix]);
    Sampler g;
    g.randSeed = seed.x * (uint32_t)(s + 1) + seed.y;
    g.sampleSeed = seed.x * seed.y;
    g.sampleOffset = off;
    g.dim = 0;
    g.mode = sc.sampler;
    g.rowCache = row;
    g.mats = sc.sobol;
    v2 scr = mk2((float)px, (float)py) / mk2((float)sc.filmW, (float)sc.filmH);
    float u0 = sample1D(g), u1 = sample1D(g), u2 = sample1D(g), u3 = sample1D(g);
    Ray ray = thinLensCameraSampleRay(sc, scr, u0, u1, u2, u3);
    v3 r;
    if (hits) {
        const size_t npix = (size_t)sc.filmW * sc.filmH, path = (size_t)s * npix + pix;
        CastCursor cur{0, 0, 0u};
        r = pathTraceRC<FULL>(sc, pp, ray, g, RecordCast{hits + path, (size_t)spp * npix, &cur});
        vis[path] = cur.vis;
    } else {
        r = pathTrace<FULL>(sc, pp, ray, g);
    }
    float* o = samples + 3 * ((size_t)s * sc.filmW * sc.filmH + pix);
    o[0] = r.x;
    o[1] = r.y;
    o[2] = r.z;
}

// image = (sum over samples in order, NaN samples dropped) / spp
__global__ void diff_reduce_kernel(const float* __restrict__ samples, int64_t npix, int32_t spp,
                                   float* __restrict__ image) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float r = 0.0f, g = 0.0f, b = 0.0f;
    for (int s = 0; s < spp; s++) {
        const float* x = samples + 3 * ((size_t)s * npix + p);
        if (!(zisnan(x[0]) || zisnan(x[1]) || zisnan(x[2]))) {
            r = r + x[0];
            g = g + x[1];
            b = b + x[2];
        }
    }
    float inv = (float)spp;
    image[3 * p] = r / inv;
    image[3 * p + 1] = g / inv;
    image[3 * p + 2] = b / inv;
}

constexpr unsigned kFullMask = 0xffffffffu;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
    return v;
}

// Adds vals[0..K) of every lane to sg[key + j], summing lanes that share a key
// in registers first: one shared-memory atomic per (distinct key, j) per warp.
// key < 0: the lane adds nothing.  All 32 lanes must call it together.
template <int K>
__device__ __forceinline__ void warp_flush(float* sg, int key, const float* vals) {
    unsigned pending = __ballot_sync(kFullMask, key >= 0);
    unsigned lane;  // the hardware lane id (the block is two-dimensional)
    asm("mov.u32 %0, %%laneid;" : "=r"(lane));
    while (pending) {
        const int leader = __ffs(pending) - 1;
        const int k = __shfl_sync(kFullMask, key, leader);
        const bool mine = key == k;
#pragma unroll
        for (int j = 0; j < K; j++) {
            float v = warp_sum(mine ? vals[j] : 0.0f);
            if (lane == (unsigned)leader && v != 0.0f) atomicAdd(&sg[k + j], v);
        }
        pending &= ~__ballot_sync(kFullMask, mine);
    }
}

// sum_c w_c df[i]_c with w_c = delta_c scale_c / f_c (channels with f_c == 0
// carry no radiance), added to acc[i].
__device__ __forceinline__ float grad_weight(float delta, float scale, float f) {
    float w = f > 1e-30f ? delta * scale / f : 0.0f;
    return isfinite(w) ? w : 0.0f;
}
__device__ __forceinline__ void mat_grad(float* acc, const v3& delta, const v3& scale, const BsdfGrad& bg) {
    const v3 w = mk3(grad_weight(delta.x, scale.x, bg.f.x), grad_weight(delta.y, scale.y, bg.f.y),
                     grad_weight(delta.z, scale.z, bg.f.z));
#pragma unroll
    for (int i = 0; i < kDiffMatParams; i++) acc[i] += w.x * bg.df[i].x + w.y * bg.df[i].y + w.z * bg.df[i].z;
}

// delta_c C_c / P_c for the power P of light triangle lightId's instance;
// returns the slot of the instance's first channel.
__device__ __forceinline__ int power_grad(const DiffInfo& di, const float* params, int lightId, const v3& delta,
                                          const v3& C, float* out) {
    const int inst = __ldg(&di.lightInst[lightId]);
    const int base = kDiffMatParams * di.nmat + 3 * inst;
    const float P[3] = {__ldg(&params[base]), __ldg(&params[base + 1]), __ldg(&params[base + 2])};
    const float c[3] = {C.x, C.y, C.z}, d[3] = {delta.x, delta.y, delta.z};
#pragma unroll
    for (int k = 0; k < 3; k++) out[k] = (P[k] != 0.0f && c[k] != 0.0f) ? d[k] * c[k] / P[k] : 0.0f;
    return base;
}

// The replay of one path (pathIntegTrace, path_integ_naive.glsl:35-143) with
// its gradient contributions, in warp lockstep: one bounce per iteration of a
// warp-uniform loop, so that each iteration's gradients (one material, up to
// two light instances per lane) are reduced across the warp before the
// shared-memory atomics.  All 32 lanes of the warp call it together; a lane
// with alive == false only takes part in the reductions.  `g` is the sample's
// sampler right after its four camera dimensions, `ray` its camera ray, `L`
// its radiance and `delta` dL/d(radiance) of the sample.  The ray casts come
// from `rc` (traversal, or the results recorded by the forward pass).
template <bool FULL, class RC>
__device__ __forceinline__ void replayPath(const DeviceScene& sc, const PathParams& pp, const DiffInfo& di,
                                           const float* __restrict__ params, float* sg, bool alive, Sampler& g,
                                           Ray ray, v3 L, v3 delta, const RC& rc) {
    v3 Lrem = L, Ltot = L;
    int id = -1;
    v3 pos = mk3(0.0f), wo = mk3(0.0f), throughput = mk3(1.0f);
    float pw[3];
    int pkey = -1;
    if (alive) {
        float primDist;
        id = rc.hit(sc, ray, primDist);
        pos = rayPoint(ray, primDist);
        wo = -ray.dir;
        if (id == -1) {
            alive = false;  // environment: no differentiable parameter
        } else if (id - sc.objPrimCount >= 0) {
            const int lightId = id - sc.objPrimCount;
            pkey = power_grad(di, params, lightId, delta, lightLe(sc, lightId, pos, -ray.dir), pw);
            alive = false;
        }
    }
    warp_flush<3>(sg, pkey, pw);

    int bounce = 1;
    while (__any_sync(kFullMask, alive)) {
        int mkey = -1, nkey = -1, hkey = -1;
        bool textured = false;
        float mg[kDiffMatParams], npw[3], hpw[3];
#pragma unroll
        for (int i = 0; i < kDiffMatParams; i++) mg[i] = 0.0f;
        if (alive) {
            TriShade tri = loadTri(sc, id);
            Surface surf = surfaceInfo(tri, pos);
            const int matId = tri.matTex & 0x0000ffff;
            const uint32_t matType = loadMaterialType(sc, matId);
            if (matType != kDielectric && matType != kThinDielectric && dot(surf.ns, wo) < 0.0f) {
                surf.ns = -surf.ns;
                surf.ng = -surf.ng;
            }
            const BSDFParam mp = loadMaterial<FULL>(sc, matType, tri.matTex, id, surf);
            // metal-workflow and dielectric materials have no differentiable
            // parameters; their vertices only carry the paths
            const bool diffMat = !FULL || matType == kLambertian || matType == kPrincipled;
            mkey = diffMat ? kDiffMatParams * matId : -1;
            // a textured triangle's base colour is the texture's, not a parameter
            textured = FULL && (tri.matTex >> 16) != -1;
            if (pp.sampleLight) {
                const float ud = sample1D(g);
                const float u0 = sample1D(g), u1 = sample1D(g), u2 = sample1D(g), u3 = sample1D(g);
                float pdfSampleLight = 0.0f;  // the light pick of sampleLightAndEnv
                if (sc.nLight > 0) pdfSampleLight = pdfSampleLightSel(sc, pp.uniformSel, pp.portion);
                const int lid = ud < pdfSampleLight ? lightSampleOne(sc, mk2(u0, u1)) : -1;
                const LiSample ls = sampleLightAndEnvV(sc, pp, pos, ud, u0, u1, u2, u3, rc);
                if (ls.pdf > 0.0f) {
                    BsdfGrad bg;
                    if (diffMat) bg = bsdfGrad(matType, mp, wo, ls.wi, surf.ns);
                    const v3 f = diffMat ? bg.f : materialBSDF<FULL>(matType, mp, wo, ls.wi, surf.ns);
                    const float fpdf = materialPdf<FULL>(matType, mp, wo, ls.wi, surf.ns);
                    const float weight = biHeuristic(ls.pdf, fpdf);
                    const v3 C = f * throughput * satDot(surf.ns, ls.wi) * ls.coef * weight;
                    if (diffMat) mat_grad(mg, delta, C, bg);
                    if (lid >= 0) nkey = power_grad(di, params, lid, delta, C, npw);
                    // what is left below the rounding of the total is no radiance
                    Lrem = Lrem - C;
                    Lrem.x = Lrem.x > 1e-6f * Ltot.x ? Lrem.x : 0.0f;
                    Lrem.y = Lrem.y > 1e-6f * Ltot.y ? Lrem.y : 0.0f;
                    Lrem.z = Lrem.z > 1e-6f * Ltot.z ? Lrem.z : 0.0f;
                }
            }
            const float b0 = sample1D(g), b1 = sample1D(g), b2 = sample1D(g);
            const BSDFSample bs = materialSample<FULL>(matType, mp, surf.ns, wo, mk3(b0, b1, b2), g);
            const v3 wi = bs.wi;
            const float bsdfPdf = bs.pdf;
            const bool deltaBsdf = (bs.flag == kSpecRefl || bs.flag == kSpecTrans);
            if (bsdfPdf < 1e-8f) {
                alive = false;
            } else {
                // every later contribution carries this vertex's sampled BSDF value
                if (diffMat) mat_grad(mg, delta, Lrem, bsdfGrad(matType, mp, wo, wi, surf.ns));
                throughput = throughput * (bs.bsdf / bsdfPdf * (deltaBsdf ? 1.0f : absDot(surf.ns, wi)));
                ray = rayOffseted(pos, wi);
                float dist;
                const int nextId = rc.hit(sc, ray, dist);
                const int lightId = nextId - sc.objPrimCount;
                const v3 nextPos = rayPoint(ray, dist);
                if (nextId == -1) {
                    alive = false;  // environment emission: no parameter
                } else if (lightId >= 0) {
                    const v3 radiance = lightLe(sc, lightId, nextPos, -wi);
                    float weight = 1.0f;
                    if (pp.sampleLight && !deltaBsdf) {
                        const float lightPdf = lightPdfLi(sc, lightId, pos, nextPos) * pdfSelectLight(sc, pp, lightId);
                        weight = (lightPdf <= 0.0f) ? 0.0f : biHeuristic(bsdfPdf, lightPdf);
                    }
                    hkey = power_grad(di, params, lightId, delta, radiance * throughput * weight, hpw);
                    alive = false;
                } else {
                    if (pp.rr && bounce >= pp.rrStart) {
                        const float continueProb = zmin(maxComponent(bs.bsdf / bsdfPdf), 0.95f);
                        if (sample1D(g) >= continueProb) alive = false;
                        throughput = throughput / continueProb;
                    }
                    id = nextId;
                    pos = nextPos;
                    wo = -wi;
                }
            }
            if (++bounce > pp.maxDepth) alive = false;
        }
        if (textured) mg[0] = mg[1] = mg[2] = 0.0f;
        warp_flush<kDiffMatParams>(sg, mkey, mg);
        warp_flush<3>(sg, nkey, npw);
        warp_flush<3>(sg, hkey, hpw);
    }
}

// Backward: one thread per (pixel, sample), blockIdx.y = sample; the replay
// takes the ray casts the forward recorded (`hits` / `vis`), or traverses the
// accelerator again when there is no record.
template <bool FULL>
__global__ void __launch_bounds__(kTileX* kTileY, 16)
diff_backward_kernel(DeviceScene sc, PathParams pp, DiffInfo di, const float* __restrict__ params, int32_t tilesX,
                     int32_t spp, const float* __restrict__ samples, const float* __restrict__ dimage,
                     const int2* __restrict__ hits, const uint32_t* __restrict__ vis, float* __restrict__ grad) {
    __shared__ uint32_t row[256];
    __shared__ float sg[kMaxDiffParams];
    for (int i = threadIdx.y * kTileX + threadIdx.x; i < di.nparams; i += kTileX * kTileY) sg[i] = 0.0f;
    const int32_t s = blockIdx.y;
    const uint32_t off = sample_offset(s);
    load_sobol_row(sc, off, row);  // includes the barrier that publishes sg
    const int tile = blockIdx.x;
    const int px = (tile % tilesX) * kTileX + threadIdx.x;
    const int py = (tile / tilesX) * kTileY + threadIdx.y;

    bool alive = px < sc.filmW && py < sc.filmH;
    v3 L = mk3(0.0f), delta = mk3(0.0f);
    size_t pix = 0;
    if (alive) {
        const size_t npix = (size_t)sc.filmW * sc.filmH;
        pix = (size_t)py * sc.filmW + px;
        const float* Ls = samples + 3 * ((size_t)s * npix + pix);
        L = mk3(Ls[0], Ls[1], Ls[2]);
        const float inv = 1.0f / (float)spp;
        delta = mk3(dimage[3 * pix] * inv, dimage[3 * pix + 1] * inv, dimage[3 * pix + 2] * inv);
        // NaN samples are left out of the image; zero adjoints need no replay
        alive = !hasNan(L) && (delta.x != 0.0f || delta.y != 0.0f || delta.z != 0.0f);
    }
    Sampler g;
    Ray ray;
    if (alive) {
        const uint2 seed = __ldg(&sc.pixelSeeds[pix]);
        g.randSeed = seed.x * (uint32_t)(s + 1) + seed.y;
        g.sampleSeed = seed.x * seed.y;
        g.sampleOffset = off;
        g.dim = 0;
        g.mode = sc.sampler;
        g.rowCache = row;
        g.mats = sc.sobol;
        v2 scr = mk2((float)px, (float)py) / mk2((float)sc.filmW, (float)sc.filmH);
        float u0 = sample1D(g), u1 = sample1D(g), u2 = sample1D(g), u3 = sample1D(g);
        ray = thinLensCameraSampleRay(sc, scr, u0, u1, u2, u3);
    }
    if (hits) {
        const size_t npix = (size_t)sc.filmW * sc.filmH, path = (size_t)s * npix + pix;
        CastCursor cur{0, 0, alive ? __ldg(vis + path) : 0u};
        replayPath<FULL>(sc, pp, di, params, sg, alive, g, ray, L, delta,
                         ReplayCast{hits + path, (size_t)spp * npix, &cur});
    } else {
        replayPath<FULL>(sc, pp, di, params, sg, alive, g, ray, L, delta, DirectCast{});
    }
    __syncthreads();
    for (int i = threadIdx.y * kTileX + threadIdx.x; i < di.nparams; i += kTileX * kTileY)
        if (sg[i] != 0.0f) atomicAdd(&grad[i], sg[i]);
}

// dloss/dimage = 2 s (image - target) and the loss s * sum (image - target)^2
// of zgl_diff_step_l2; one atomic per block for the loss.
__global__ void diff_l2_kernel(const float* __restrict__ image, const float* __restrict__ target, int64_t n,
                               float scale, float* __restrict__ dimage, float* __restrict__ loss) {
    __shared__ float part[8];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (i < n) {
        const float diff = image[i] - target[i];
        dimage[i] = diff * (2.0f * scale);
        l = diff * diff * scale;
    }
    l = warp_sum(l);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += part[w];
        if (t != 0.0f) atomicAdd(loss, t);
    }
}

}  // namespace

}  // namespace zgl

using namespace zgl;

namespace {

PathParams path_params(const zgl_integrator_params& p) {
    return PathParams{p.max_depth, p.russian_roulette, p.rr_start_depth, p.sample_light, p.light_env_uniform_sample,
                      p.light_portion};
}

bool device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" {

zgl_status zgl_diff_create(zgl_scene* scene, const zgl_integrator_params* params, int32_t spp, zgl_diff** out) {
    ZGL_API_BEGIN
    if (!scene || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_create: NULL argument");
    *out = nullptr;
    if (scene->host_only) fail(ZGL_ERR_STATE, "zgl_diff_create: scene was created host-only");
    if (spp < 1 || spp > 4096) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_create: spp %d out of range", spp);
    auto* d = new zgl_diff();
    try {
        d->scene = scene;
        zgl_integrator_params_default(&d->params);
        if (params) d->params = *params;
        d->spp = spp;
        d->nmat = (int32_t)(scene->materials.size() / 16);
        d->lightFirst = scene->lightFirst;
        d->instPower = scene->lightInstPower;
        d->ninst = (int32_t)(d->instPower.size() / 3);
        d->nparams = kDiffMatParams * d->nmat + 3 * d->ninst;
        if (d->nparams > kMaxDiffParams) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_create: %d parameters exceed %d", d->nparams, kMaxDiffParams);
        size_t npix = (size_t)scene->filmW * scene->filmH;
        ZGL_CUDA(cudaMalloc(&d->d_samples, sizeof(float) * 3 * npix * (size_t)spp));
        const size_t paths = npix * (size_t)spp;
        if ((sizeof(int2) * kCastDepth + sizeof(uint32_t)) * paths <= kCastBudget) {
            ZGL_CUDA(cudaMalloc(&d->d_hits, sizeof(int2) * kCastDepth * paths));
            ZGL_CUDA(cudaMalloc(&d->d_vis, sizeof(uint32_t) * paths));
        }
        std::vector<int32_t> inst((size_t)std::max(scene->nLight, 1), 0);
        for (int k = 0; k < d->ninst; k++)
            for (uint32_t t = d->lightFirst[(size_t)k]; t < d->lightFirst[(size_t)k + 1]; t++) inst[t] = k;
        ZGL_CUDA(cudaMalloc(&d->d_lightInst, sizeof(int32_t) * inst.size()));
        ZGL_CUDA(cudaMemcpy(d->d_lightInst, inst.data(), sizeof(int32_t) * inst.size(), cudaMemcpyHostToDevice));
        // current parameter values
        d->params_host.assign((size_t)d->nparams, 0.0f);
        for (int m = 0; m < d->nmat; m++) {
            const float* r = &scene->materials[16 * (size_t)m];
            float v[6] = {r[0], r[1], r[2], r[3], r[5], r[6]};
            std::memcpy(&d->params_host[(size_t)kDiffMatParams * m], v, sizeof(v));
        }
        for (int k = 0; k < 3 * d->ninst; k++) d->params_host[(size_t)kDiffMatParams * d->nmat + k] = d->instPower[(size_t)k];
        ZGL_CUDA(cudaMalloc(&d->d_values, sizeof(float) * (size_t)std::max(d->nparams, 1)));
        ZGL_CUDA(cudaMemcpy(d->d_values, d->params_host.data(), sizeof(float) * (size_t)d->nparams, cudaMemcpyHostToDevice));
    } catch (...) {
        if (d->d_samples) cudaFree(d->d_samples);
        if (d->d_hits) cudaFree(d->d_hits);
        if (d->d_vis) cudaFree(d->d_vis);
        if (d->d_lightInst) cudaFree(d->d_lightInst);
        if (d->d_values) cudaFree(d->d_values);
        delete d;
        throw;
    }
    *out = d;
    ZGL_API_END
}

zgl_status zgl_diff_param_count(const zgl_diff* d, int32_t* n) {
    ZGL_API_BEGIN
    if (!d || !n) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_param_count: NULL");
    *n = d->nparams;
    ZGL_API_END
}

zgl_status zgl_diff_get_params(const zgl_diff* d, float* out) {
    ZGL_API_BEGIN
    if (!d || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_get_params: NULL");
    std::memcpy(out, d->params_host.data(), sizeof(float) * d->params_host.size());
    ZGL_API_END
}

zgl_status zgl_diff_set_params(zgl_diff* d, const float* params) {
    ZGL_API_BEGIN
    if (!d || !params) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_set_params: NULL");
    // work queued on any stream may still read the scene or write `params`
    ZGL_CUDA(cudaDeviceSynchronize());
    std::vector<float> p((size_t)d->nparams);
    if (device_ptr(params)) ZGL_CUDA(cudaMemcpy(p.data(), params, sizeof(float) * p.size(), cudaMemcpyDeviceToHost));
    else std::memcpy(p.data(), params, sizeof(float) * p.size());
    for (float v : p)
        if (!std::isfinite(v)) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_set_params: non-finite parameter");
    scene_set_diff_params(d->scene, p.data(), d->nmat, d->instPower);
    // new roughness or metallic values move the sampled directions: the kept casts no longer apply
    d->castsValid = false;
    d->params_host = p;
    ZGL_CUDA(cudaMemcpy(d->d_values, p.data(), sizeof(float) * p.size(), cudaMemcpyHostToDevice));
    ZGL_API_END
}

zgl_status zgl_diff_forward(zgl_diff* d, float* image, void* stream) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_diff_forward");
    if (!d || !image) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_forward: NULL");
    if (!device_ptr(image)) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_forward: image must be device memory");
    const zgl_scene* s = d->scene;
    cudaStream_t st = (cudaStream_t)stream;
    int tilesX = (s->filmW + kTileX - 1) / kTileX, tilesY = (s->filmH + kTileY - 1) / kTileY;
    dim3 grid((unsigned)(tilesX * tilesY), (unsigned)d->spp);
    if (s->fullMaterials)
        diff_forward_kernel<true><<<grid, dim3(kTileX, kTileY), 0, st>>>(s->view(), path_params(d->params), tilesX,
                                                                         d->spp, d->d_samples, d->d_hits, d->d_vis);
    else
        diff_forward_kernel<false><<<grid, dim3(kTileX, kTileY), 0, st>>>(s->view(), path_params(d->params), tilesX,
                                                                          d->spp, d->d_samples, d->d_hits, d->d_vis);
    d->castsValid = d->d_hits != nullptr;
    ZGL_CUDA(cudaGetLastError());
    int64_t npix = (int64_t)s->filmW * s->filmH;
    diff_reduce_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(d->d_samples, npix, d->spp, image);
    ZGL_CUDA(cudaGetLastError());
    ZGL_API_END
}

zgl_status zgl_diff_backward(zgl_diff* d, const float* d_image, float* d_params, void* stream) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_diff_backward");
    if (!d || !d_image || !d_params) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_backward: NULL");
    if (!device_ptr(d_image) || !device_ptr(d_params))
        fail(ZGL_ERR_INVALID_ARG, "zgl_diff_backward: arrays must be device memory");
    const zgl_scene* s = d->scene;
    cudaStream_t st = (cudaStream_t)stream;
    ZGL_CUDA(cudaMemsetAsync(d_params, 0, sizeof(float) * (size_t)d->nparams, st));
    DiffInfo di{d->nmat, d->nparams, d->d_lightInst};
    int tilesX = (s->filmW + kTileX - 1) / kTileX, tilesY = (s->filmH + kTileY - 1) / kTileY;
    dim3 grid((unsigned)(tilesX * tilesY), (unsigned)d->spp);
    const int2* hits = d->castsValid ? d->d_hits : nullptr;
    const uint32_t* vis = d->castsValid ? d->d_vis : nullptr;
    if (s->fullMaterials)
        diff_backward_kernel<true><<<grid, dim3(kTileX, kTileY), 0, st>>>(s->view(), path_params(d->params), di,
                                                                          d->d_values, tilesX, d->spp, d->d_samples,
                                                                          d_image, hits, vis, d_params);
    else
        diff_backward_kernel<false><<<grid, dim3(kTileX, kTileY), 0, st>>>(s->view(), path_params(d->params), di,
                                                                           d->d_values, tilesX, d->spp, d->d_samples,
                                                                           d_image, hits, vis, d_params);
    ZGL_CUDA(cudaGetLastError());
    ZGL_API_END
}

zgl_status zgl_diff_step_l2(zgl_diff* d, const float* target, float loss_scale, float* image, float* d_params,
                            float* loss, void* stream) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_diff_step_l2");
    if (!d || !target || !image || !d_params || !loss) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_step_l2: NULL");
    if (!device_ptr(target) || !device_ptr(image) || !device_ptr(d_params) || !device_ptr(loss))
        fail(ZGL_ERR_INVALID_ARG, "zgl_diff_step_l2: arrays must be device memory");
    if (!std::isfinite(loss_scale)) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_step_l2: non-finite loss scale");
    const zgl_scene* s = d->scene;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t n = (int64_t)s->filmW * s->filmH * 3;
    if (!d->d_dimage) ZGL_CUDA(cudaMalloc(&d->d_dimage, sizeof(float) * (size_t)n));
    zgl_status r = zgl_diff_forward(d, image, stream);
    if (r != ZGL_OK) return r;
    ZGL_CUDA(cudaMemsetAsync(loss, 0, sizeof(float), st));
    diff_l2_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(image, target, n, loss_scale, d->d_dimage, loss);
    ZGL_CUDA(cudaGetLastError());
    return zgl_diff_backward(d, d->d_dimage, d_params, stream);
    ZGL_API_END
}

zgl_status zgl_diff_destroy(zgl_diff* d) {
    ZGL_API_BEGIN
    if (!d) return ZGL_OK;
    if (d->d_samples) cudaFree(d->d_samples);
    if (d->d_hits) cudaFree(d->d_hits);
    if (d->d_vis) cudaFree(d->d_vis);
    if (d->d_dimage) cudaFree(d->d_dimage);
    if (d->d_lightInst) cudaFree(d->d_lightInst);
    if (d->d_values) cudaFree(d->d_values);
    delete d;
    ZGL_API_END
}

}  // extern "C"
