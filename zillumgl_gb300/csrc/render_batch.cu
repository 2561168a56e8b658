// render_batch.cu — batched wavefront path tracing: many render requests
// (each its own scene, film, samples per pixel and depth) rendered by one
// persistent launch over every (request, sample, pixel), captured in a CUDA
// graph with the frame updates.
//
// Work items are the pixels of every sample of every request, in 8x4 tiles
// per sample, so a warp's lanes hold neighbouring pixels of one sample.
// Persistent warps claim ranges of `queue_capacity` items with one atomicAdd
// on the launch's work counter and hand them to idle lanes with
// __ballot_sync/__popc once at least `regen_threshold` lanes are idle (or none
// is live).  Each lane runs its path as an explicit state machine whose step
// is one bounce (closest-hit trace, emission/MIS, Russian roulette, then
// next-event estimation and BSDF sampling at the new vertex); a lane whose
// path ends takes the next item at once (path regeneration), whatever its
// request or sample.  The Sobol rows of all sample indices sit in a small
// device table.  Each sample's radiance goes to a per-request scratch array;
// a second kernel then adds the samples to the frames in sample order
// (path_integ_naive.glsl main(), :166-173), so a request's frame is bit for
// bit the frame of the plain path integrator after `spp` passes from a fresh
// start (sample j uses freeCounter j + 1).  When the scratch of all samples
// would exceed a memory budget the samples are rendered in chunks of sample
// indices.  Request descriptors travel in the kernel parameter block (up to
// 64 per launch).  This schedule has no counterpart in the reference; its
// nearest relatives are the queue experiments pt_global_queue_*.glsl and
// pt_shared_queue.glsl.
#include <algorithm>
#include <cstring>
#include <vector>

#define ZGL_INLINE_TRACE 1
#include "batch_flat.h"
#include "scene.h"
#include "shading.cuh"
#include "zgl_internal.h"

namespace zgl {
namespace {

constexpr unsigned kFull = 0xffffffffu;

struct BatchPathParams {
    int32_t maxDepth, rr, rrStart, sampleLight, uniformSel;
    float portion;
};

struct BatchRequest {
    DeviceScene sc;
    BatchPathParams pp;
    int32_t spp;
    float4* frame;
    float* scratch;    // per-sample radiance of the current chunk, [sample - j0][npix][3]
    int64_t itemBase;  // first work item of this request in its launch
    int32_t npix;
    int32_t tilesX;    // 8x4 pixel tiles per film row
    int32_t perSample; // items per sample (whole tiles)
    int32_t j1;        // samples [j0, j1) of this request in the launch
};

constexpr int kMaxReqPerLaunch = 64;
constexpr size_t kScratchBudget = (size_t)8 << 30;  // default per-sample radiance of one launch chunk

struct BatchLaunch {
    BatchRequest req[kMaxReqPerLaunch];
    int32_t nreq;
    int64_t nitems;
    int32_t j0;             // first sample index of this launch
    unsigned long long* counter;
    int32_t queueCap;
    int32_t regenThreshold;
    const uint32_t* mats;   // Sobol generator matrices
    const uint32_t* rows;   // Sobol rows: 256 values per sample index
};
static_assert(sizeof(BatchLaunch) <= 32000, "kernel parameter block too large");

template <class Vis>
__device__ __forceinline__ LiSample sampleLightAndEnvB(const DeviceScene& sc, const BatchPathParams& pp, v3 x,
                                                       float ud, float u0, float u1, float u2, float u3,
                                                       const Vis& vis) {
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

struct PathState {
    Ray ray;        // pending ray
    v3 result, throughput;
    v3 wo, pos;     // vertex being left (valid after the first bounce)
    v3 bsdfOverPdf; // bsdf / pdf of the last sample (Russian roulette)
    float bsdfPdf;
    int32_t bounce; // 0 = camera ray pending
    bool delta;
};

__device__ __forceinline__ uint32_t sample_offset_dev(int32_t spp) {
    int32_t off = (int32_t)((uint32_t)spp * 256u);
    if (off > 131072 * 256) off -= 131072 * 256;
    return (uint32_t)off;
}

// Starts sample `j` of pixel (px, py): seeds and the camera ray (main(),
// path_integ_naive.glsl:145-166).
__device__ __forceinline__ void start_sample(const BatchRequest& rq, const BatchLaunch& L, int j, int px, int py,
                                             Sampler& g, PathState& st) {
    const DeviceScene& sc = rq.sc;
    const uint2 seed = __ldg(&sc.pixelSeeds[(size_t)py * sc.filmW + px]);
    const uint32_t freeCounter = (uint32_t)j + 1u;
    g.randSeed = seed.x * freeCounter + seed.y;
    g.sampleSeed = seed.x * seed.y;
    g.sampleOffset = sample_offset_dev(j);
    g.dim = 0;
    g.mode = sc.sampler;
    g.rowCache = L.rows + 256 * (size_t)j;
    g.mats = L.mats;
    v2 scr = mk2((float)px, (float)py) / mk2((float)sc.filmW, (float)sc.filmH);
    float u0 = sample1D(g), u1 = sample1D(g), u2 = sample1D(g), u3 = sample1D(g);
    st.ray = thinLensCameraSampleRay(sc, scr, u0, u1, u2, u3);
    st.result = mk3(0.0f);
    st.throughput = mk3(1.0f);
    st.bounce = 0;
}

// The light sample of a vertex whose occlusion test is left to a later
// trace: the shadow ray and the contribution the sample makes if nothing
// blocks it.
struct PendingShadow {
    v3 o, d, C;
    float tmax;
    bool pending;
};

// Visibility source that records the shadow ray instead of tracing it and
// answers "not occluded"; the contribution is added after the trace.
struct DeferVis {
    PendingShadow* ps;
    __device__ __forceinline__ bool operator()(const DeviceScene&, const Ray& r, float dist) const {
        ps->o = r.ori;
        ps->d = r.dir;
        ps->tmax = dist;
        return false;
    }
};

// One step of pathIntegTrace after the pending ray has been traced (closest
// hit `id` at `dist`): account for what it hits and, if the path continues,
// shade the new vertex (light sample + BSDF sample) to produce the next
// pending ray.  Returns false when the path ends.  DEFER: the light sample's
// occlusion test is recorded in `ps` for a later trace instead of run here.
template <bool FULL, bool DEFER>
__device__ __forceinline__ bool path_step_hit(const BatchRequest& rq, Sampler& g, PathState& st, int id, float dist,
                                              PendingShadow* ps) {
    const DeviceScene& sc = rq.sc;
    const BatchPathParams& pp = rq.pp;
    v3 hitPos = rayPoint(st.ray, dist);
    if (st.bounce == 0) {
        // primary hit (path_integ_naive.glsl:37-44)
        if (id == -1) {
            st.result = envLe(sc, st.ray.dir);
            return false;
        }
        if (id - sc.objPrimCount >= 0) {
            st.result = lightLe(sc, id - sc.objPrimCount, hitPos, -st.ray.dir);
            return false;
        }
        st.wo = -st.ray.dir;
    } else {
        // extension hit of bounce st.bounce (path_integ_naive.glsl:97-133)
        v3 wi = st.ray.dir;
        int lightId = id - sc.objPrimCount;
        if (id == -1) {
            v3 radiance = envLe(sc, wi);
            float weight = 1.0f;
            if (pp.sampleLight && !st.delta) {
                float envPdf = envPdfLi(sc, wi) * (pp.uniformSel ? (1.0f - pp.portion)
                                                                 : sc.envSum / (sc.lightSum + sc.envSum));
                weight = (envPdf <= 0.0f) ? 0.0f : biHeuristic(st.bsdfPdf, envPdf);
            }
            st.result = st.result + radiance * st.throughput * weight;
            return false;
        }
        if (lightId >= 0) {
            v3 radiance = lightLe(sc, lightId, hitPos, -wi);
            float weight = 1.0f;
            if (pp.sampleLight && !st.delta) {
                float snd = pp.uniformSel ? pp.portion : sc.lightSum / (sc.lightSum + sc.envSum);
                float lightPdf = lightPdfLi(sc, lightId, st.pos, hitPos) * (lightPdfSampleOne(sc, lightId) * snd);
                weight = (lightPdf <= 0.0f) ? 0.0f : biHeuristic(st.bsdfPdf, lightPdf);
            }
            st.result = st.result + radiance * st.throughput * weight;
            return false;
        }
        if (pp.rr && st.bounce >= pp.rrStart) {
            float continueProb = zmin(maxComponent(st.bsdfOverPdf), 0.95f);
            if (sample1D(g) >= continueProb) return false;
            st.throughput = st.throughput / continueProb;
        }
        st.wo = -wi;
    }
    // next bounce at the new vertex
    st.bounce++;
    if (st.bounce > pp.maxDepth) return false;
    st.pos = hitPos;
    TriShade tri = loadTri(sc, id);
    Surface surf = surfaceInfo(tri, hitPos);
    int matId = tri.matTex & 0x0000ffff;
    uint32_t matType = loadMaterialType(sc, matId);
    if (matType != kDielectric && matType != kThinDielectric && dot(surf.ns, st.wo) < 0.0f) {
        surf.ns = -surf.ns;
        surf.ng = -surf.ng;
    }
    BSDFParam mp = loadMaterial<FULL>(sc, matType, tri.matTex, id, surf);
    if (pp.sampleLight) {
        float ud = sample1D(g);
        float u0 = sample1D(g), u1 = sample1D(g), u2 = sample1D(g),
              u3 = sample1D(g);
        LiSample ls;
        if (DEFER) ls = sampleLightAndEnvB(sc, pp, hitPos, ud, u0, u1, u2, u3, DeferVis{ps});
        else ls = sampleLightAndEnvB(sc, pp, hitPos, ud, u0, u1, u2, u3, TraceVis{});
        if (ls.pdf > 0.0f) {
            v3 f = materialBSDF<FULL>(matType, mp, st.wo, ls.wi, surf.ns);
            float fpdf = materialPdf<FULL>(matType, mp, st.wo, ls.wi, surf.ns);
            float weight = biHeuristic(ls.pdf, fpdf);
            const v3 C = f * st.throughput * satDot(surf.ns, ls.wi) * ls.coef * weight;
            if (DEFER) {
                ps->C = C;
                ps->pending = true;
            } else {
                st.result = st.result + C;
            }
        }
    }
    float b0 = sample1D(g), b1 = sample1D(g), b2 = sample1D(g);
    BSDFSample bs = materialSample<FULL>(matType, mp, surf.ns, st.wo, mk3(b0, b1, b2), g);
    st.delta = (bs.flag == kSpecRefl || bs.flag == kSpecTrans);
    if (bs.pdf < 1e-8f) return false;
    st.throughput = st.throughput * (bs.bsdf / bs.pdf * (st.delta ? 1.0f : absDot(surf.ns, bs.wi)));
    st.bsdfPdf = bs.pdf;
    st.bsdfOverPdf = bs.bsdf / bs.pdf;
    st.ray = rayOffseted(hitPos, bs.wi);
    return true;
}

// One step with the pending ray traced here.
template <bool FULL>
__device__ __forceinline__ bool path_step(const BatchRequest& rq, Sampler& g, PathState& st) {
    float dist;
    const int id = bvhHit(rq.sc, st.ray, dist);
    return path_step_hit<FULL, false>(rq, g, st, id, dist, nullptr);
}

__device__ __forceinline__ int find_request(const BatchLaunch& L, int64_t item) {
    int lo = 0, hi = L.nreq - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (L.req[mid].itemBase <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int BLOCK, bool FULL>
__global__ void __launch_bounds__(BLOCK, 2048 / BLOCK) batch_kernel(const __grid_constant__ BatchLaunch L) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    // warp-uniform: claimed but not yet handed-out work items [qnext, qend)
    int64_t qnext = 0, qend = 0;
    bool exhausted = false;
    bool live = false;
    int rid = 0, px = 0, py = 0, js = 0;
    Sampler g;
    PathState st;
    for (;;) {
        const unsigned idle = __ballot_sync(kFull, !live);
        const int nidle = __popc(idle);
        const int64_t tail = qend - qnext;
        if (nidle != 0 && (nidle >= L.regenThreshold || nidle == 32) && (!exhausted || tail > 0)) {
            // idle lanes take the leftover of the claimed range first, then a
            // freshly claimed range of queueCap items (one atomic per claim)
            int64_t nb = 0, nlen = 0;
            if (!exhausted && tail < nidle) {
                unsigned long long b = 0;
                if (lane == 0) b = atomicAdd(L.counter, (unsigned long long)L.queueCap);
                b = __shfl_sync(kFull, b, 0);
                if ((int64_t)b >= L.nitems) {
                    exhausted = true;
                } else {
                    nb = (int64_t)b;
                    nlen = min((int64_t)L.queueCap, L.nitems - nb);
                }
            }
            if (!live) {
                const int r = __popc(idle & lt);
                int64_t item = -1;
                if (r < tail) item = qnext + r;
                else if (r - tail < nlen) item = nb + (r - tail);
                if (item >= 0) {
                    rid = find_request(L, item);
                    const BatchRequest& rq = L.req[rid];
                    const int64_t local = item - rq.itemBase;
                    js = (int)(local / rq.perSample);
                    const int64_t inSample = local - (int64_t)js * rq.perSample;
                    js += L.j0;
                    const int64_t tile = inSample >> 5;
                    const int w = (int)(inSample & 31);
                    px = (int)(tile % rq.tilesX) * 8 + (w & 7);
                    py = (int)(tile / rq.tilesX) * 4 + (w >> 3);
                    if (px < rq.sc.filmW && py < rq.sc.filmH) {
                        live = true;
                        start_sample(rq, L, js, px, py, g, st);
                    }
                }
            }
            const int64_t used = min((int64_t)nidle, tail + nlen);
            if (used <= tail) {
                qnext += used;
            } else {
                qnext = nb + (used - tail);
                qend = nb + nlen;
            }
        }
        if (__ballot_sync(kFull, live) == 0u) {
            if (exhausted && qnext >= qend) break;
            continue;
        }
        if (live) {
            const BatchRequest& rq = L.req[rid];
            if (!path_step<FULL>(rq, g, st)) {
                float* o = rq.scratch + 3 * ((size_t)(js - L.j0) * rq.npix + (size_t)py * rq.sc.filmW + px);
                o[0] = st.result.x;
                o[1] = st.result.y;
                o[2] = st.result.z;
                live = false;
            }
        }
    }
}

// ----------------------------------------------------------------------------
// Queue schedule: persistent blocks whose paths trade rays through queues
// staged in shared memory (the design of the reference's experiment
// src/shader/pt_shared_queue.glsl:45-50, 193-241, with each path's own
// sampler state kept, so the sample dimensions follow the naive schedule).
// Each thread owns a path slot.  One round of the block:
//   1. idle slots of a warp take new work items (one atomicAdd per warp,
//      handed out with __ballot_sync / __popc) and start their camera ray;
//   2. every live slot appends its pending ray to the closest-hit queue and,
//      when its last vertex left a light sample, that sample's shadow ray to
//      the occlusion queue (warp-aggregated shared-memory atomics, so both
//      queues are dense);
//   3. thread t traces closest-hit entry t and occlusion entry t;
//   4. every live slot adds its light sample if it was not occluded, then
//      takes its hit: emission and MIS, Russian roulette, and the next
//      vertex's light sample (shadow ray recorded, not traced) and BSDF
//      sample.
// The contributions are added in the order of the plain path tracer (a
// vertex's light sample before the emission its extension ray finds), so
// every sample equals the plain integrator's bit for bit.
// ----------------------------------------------------------------------------
constexpr int kQueueBlock = 256;

template <bool FULL>
__global__ void __launch_bounds__(kQueueBlock, 4) batch_queue_kernel(const __grid_constant__ BatchLaunch L) {
    __shared__ float4 cqO[kQueueBlock], cqD[kQueueBlock];  // closest-hit queue: origin + request, direction
    __shared__ float4 sqO[kQueueBlock], sqD[kQueueBlock];  // occlusion queue: origin + request, direction + tmax
    __shared__ int16_t cOwner[kQueueBlock], sOwner[kQueueBlock];
    __shared__ int cId[kQueueBlock];
    __shared__ float cT[kQueueBlock];
    __shared__ uint8_t sOcc[kQueueBlock];
    __shared__ int nc, ns;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const unsigned lt = (1u << lane) - 1u;
    if (tid == 0) nc = ns = 0;
    int64_t qnext = 0, qend = 0;  // warp-uniform: claimed items not yet handed out
    bool exhausted = false;       // warp-uniform
    bool live = false;
    int rid = 0, px = 0, py = 0, js = 0;
    Sampler g;
    PathState st;
    PendingShadow ps;
    ps.pending = false;
    for (;;) {
        // 1. refill idle slots
        const unsigned idle = __ballot_sync(kFull, !live);
        const int nidle = __popc(idle);
        const int64_t tail = qend - qnext;
        if (nidle != 0 && (nidle >= L.regenThreshold || nidle == 32) && (!exhausted || tail > 0)) {
            int64_t nb = 0, nlen = 0;
            if (!exhausted && tail < nidle) {
                unsigned long long b = 0;
                if (lane == 0) b = atomicAdd(L.counter, (unsigned long long)L.queueCap);
                b = __shfl_sync(kFull, b, 0);
                if ((int64_t)b >= L.nitems) {
                    exhausted = true;
                } else {
                    nb = (int64_t)b;
                    nlen = min((int64_t)L.queueCap, L.nitems - nb);
                }
            }
            if (!live) {
                const int r = __popc(idle & lt);
                int64_t item = -1;
                if (r < tail) item = qnext + r;
                else if (r - tail < nlen) item = nb + (r - tail);
                if (item >= 0) {
                    rid = find_request(L, item);
                    const BatchRequest& rq = L.req[rid];
                    const int64_t local = item - rq.itemBase;
                    js = (int)(local / rq.perSample);
                    const int64_t inSample = local - (int64_t)js * rq.perSample;
                    js += L.j0;
                    const int64_t tile = inSample >> 5;
                    const int w = (int)(inSample & 31);
                    px = (int)(tile % rq.tilesX) * 8 + (w & 7);
                    py = (int)(tile / rq.tilesX) * 4 + (w >> 3);
                    if (px < rq.sc.filmW && py < rq.sc.filmH) {
                        live = true;
                        ps.pending = false;
                        start_sample(rq, L, js, px, py, g, st);
                    }
                }
            }
            const int64_t used = min((int64_t)nidle, tail + nlen);
            if (used <= tail) {
                qnext += used;
            } else {
                qnext = nb + (used - tail);
                qend = nb + nlen;
            }
        }
        // the block ends when no slot is live and no warp can claim more
        if (!__syncthreads_or(live || !exhausted || qnext < qend)) break;
        // 2. queue the rays (dense, one shared atomic per warp and queue)
        {
            const unsigned m = __ballot_sync(kFull, live);
            int base = 0;
            if (lane == 0 && m) base = atomicAdd(&nc, __popc(m));
            base = __shfl_sync(kFull, base, 0);
            if (live) {
                const int e = base + __popc(m & lt);
                cqO[e] = make_float4(st.ray.ori.x, st.ray.ori.y, st.ray.ori.z, __int_as_float(rid));
                cqD[e] = make_float4(st.ray.dir.x, st.ray.dir.y, st.ray.dir.z, 0.0f);
                cOwner[e] = (int16_t)tid;
            }
            const bool shadow = live && ps.pending;
            const unsigned ms = __ballot_sync(kFull, shadow);
            int sbase = 0;
            if (lane == 0 && ms) sbase = atomicAdd(&ns, __popc(ms));
            sbase = __shfl_sync(kFull, sbase, 0);
            if (shadow) {
                const int e = sbase + __popc(ms & lt);
                sqO[e] = make_float4(ps.o.x, ps.o.y, ps.o.z, __int_as_float(rid));
                sqD[e] = make_float4(ps.d.x, ps.d.y, ps.d.z, ps.tmax);
                sOwner[e] = (int16_t)tid;
            }
        }
        __syncthreads();
        // 3. trace the queues
        {
            const int n1 = nc, n2 = ns;
            if (tid < n1) {
                const float4 o = cqO[tid], d = cqD[tid];
                const DeviceScene& sc = L.req[__float_as_int(o.w)].sc;
                float dist;
                const int id = bvhHit(sc, Ray{mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z)}, dist);
                const int own = cOwner[tid];
                cId[own] = id;
                cT[own] = dist;
            }
            if (tid < n2) {
                const float4 o = sqO[tid], d = sqD[tid];
                const DeviceScene& sc = L.req[__float_as_int(o.w)].sc;
                sOcc[sOwner[tid]] = bvhTest(sc, Ray{mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z)}, d.w) ? 1 : 0;
            }
        }
        __syncthreads();
        if (tid == 0) nc = ns = 0;
        // 4. take the results
        if (live) {
            const BatchRequest& rq = L.req[rid];
            if (ps.pending) {
                if (!sOcc[tid]) st.result = st.result + ps.C;
                ps.pending = false;
            }
            if (!path_step_hit<FULL, true>(rq, g, st, cId[tid], cT[tid], &ps)) {
                float* o = rq.scratch + 3 * ((size_t)(js - L.j0) * rq.npix + (size_t)py * rq.sc.filmW + px);
                o[0] = st.result.x;
                o[1] = st.result.y;
                o[2] = st.result.z;
                live = false;
                ps.pending = false;
            }
        }
        __syncthreads();
    }
}

// Adds the chunk's samples [j0, j1) of every request to its frame in sample
// order, as consecutive path-tracer passes do (main(),
// path_integ_naive.glsl:166-173): sample 0 starts from zero, a NaN sample
// leaves the pixel as it was.  One thread per pixel of the launch's requests.
__global__ void batch_accumulate_kernel(const __grid_constant__ BatchLaunch L) {
    const int64_t item = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (item >= L.nitems) return;
    int lo = 0, hi = L.nreq - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (L.req[mid].itemBase <= item) lo = mid;
        else hi = mid - 1;
    }
    const BatchRequest& rq = L.req[lo];
    const int64_t p = item - rq.itemBase;
    float4 f = rq.frame[p];
    v3 acc = mk3(f.x, f.y, f.z);
    bool written = false;
    for (int j = L.j0; j < rq.j1; j++) {
        const float* x = rq.scratch + 3 * ((size_t)(j - L.j0) * rq.npix + (size_t)p);
        const v3 r = mk3(x[0], x[1], x[2]);
        const v3 last = (j != 0) ? acc : mk3(0.0f);
        if (!hasNan(r)) {
            acc = last + r;
            written = true;
        }
    }
    if (written) rq.frame[p] = make_float4(acc.x, acc.y, acc.z, 1.0f);
}

int occupancy_grid(const void* kernel, int block) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
    return sms * std::max(per_sm, 1);
}

cudaError_t launch_accumulate(const BatchLaunch& a, cudaStream_t st) {
    batch_accumulate_kernel<<<(unsigned)((a.nitems + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

template <bool FULL>
void launch_batch_t(const BatchLaunch& a, int block, cudaStream_t st) {
    switch (block) {
        case 64:
            batch_kernel<64, FULL><<<occupancy_grid((const void*)batch_kernel<64, FULL>, 64), 64, 0, st>>>(a);
            break;
        case 256:
            batch_kernel<256, FULL><<<occupancy_grid((const void*)batch_kernel<256, FULL>, 256), 256, 0, st>>>(a);
            break;
        default:
            batch_kernel<128, FULL><<<occupancy_grid((const void*)batch_kernel<128, FULL>, 128), 128, 0, st>>>(a);
            break;
    }
}

cudaError_t launch_batch_queue(const BatchLaunch& a, bool full, cudaStream_t st) {
    if (full)
        batch_queue_kernel<true><<<occupancy_grid((const void*)batch_queue_kernel<true>, kQueueBlock), kQueueBlock, 0,
                                   st>>>(a);
    else
        batch_queue_kernel<false><<<occupancy_grid((const void*)batch_queue_kernel<false>, kQueueBlock), kQueueBlock,
                                    0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_batch(const BatchLaunch& a, int block, bool full, cudaStream_t st) {
    if (full) launch_batch_t<true>(a, block, st);
    else launch_batch_t<false>(a, block, st);
    return cudaGetLastError();
}

}  // namespace
}  // namespace zgl

struct zgl_batch {
    int device = 0;
    int32_t nreq = 0;
    int64_t nitems = 0;
    int32_t maxSpp = 0;
    int32_t chunkLen = 0;  // sample indices per launch (scratch budget)
    bool fullMaterials = false;  // some request's scene has metal-workflow or dielectric materials
    std::vector<zgl::BatchRequest> req;
    uint32_t* d_mats = nullptr;
    uint32_t* d_rows = nullptr;     // maxSpp x 256 Sobol values
    float* d_scratch = nullptr;     // per request: min(spp, chunkLen) x npix x 3
    unsigned long long* d_counters = nullptr;
    int32_t nchunks_cap = 0;
    zgl_batch_config cfg{};
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    zgl_batch_config graph_cfg{};
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
};

namespace zgl {
namespace {

void batch_free(zgl_batch* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->ev_in) cudaEventDestroy(b->ev_in);
    if (b->ev_out) cudaEventDestroy(b->ev_out);
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->d_mats) cudaFree(b->d_mats);
    if (b->d_rows) cudaFree(b->d_rows);
    if (b->d_scratch) cudaFree(b->d_scratch);
    if (b->d_counters) cudaFree(b->d_counters);
    delete b;
}

zgl_batch_config resolve(const zgl_batch_config& c) {
    zgl_batch_config r = c;
    if (r.block_size == 0) r.block_size = 128;
    if (r.queue_capacity == 0) r.queue_capacity = 32;
    if (r.regen_threshold == 0) r.regen_threshold = 16;
    if (r.schedule == ZGL_BATCH_DEFAULT) r.schedule = ZGL_BATCH_FLAT;
    return r;
}

void check_config(const zgl_batch_config& c) {
    if (c.block_size != 0 && c.block_size != 64 && c.block_size != 128 && c.block_size != 256)
        fail(ZGL_ERR_INVALID_ARG, "batch: block_size must be 64, 128 or 256");
    if (c.queue_capacity < 0 || c.queue_capacity > 4096) fail(ZGL_ERR_INVALID_ARG, "batch: queue_capacity out of range");
    if (c.regen_threshold < 0 || c.regen_threshold > 32) fail(ZGL_ERR_INVALID_ARG, "batch: regen_threshold out of range");
    if (c.scratch_mib < 0) fail(ZGL_ERR_INVALID_ARG, "batch: negative scratch budget");
    if (c.schedule != ZGL_BATCH_DEFAULT && c.schedule != ZGL_BATCH_FLAT && c.schedule != ZGL_BATCH_PERSISTENT &&
        c.schedule != ZGL_BATCH_QUEUE)
        fail(ZGL_ERR_INVALID_ARG, "batch: unknown schedule %d", c.schedule);
}

// Enqueues the whole render on `st`: frame clears, then per chunk of sample
// indices one persistent launch per group of up to 64 requests that need
// samples of the chunk (each with its own counter reset) and the in-order
// frame updates of that group.  `first_samples` > 0 renders only that many
// sample indices (autotuning).
void enqueue_render(zgl_batch* b, const zgl_batch_config& c, cudaStream_t st, int first_samples) {
    for (const auto& r : b->req)
        ZGL_CUDA(cudaMemsetAsync(r.frame, 0, sizeof(float4) * (size_t)r.npix, st));
    const int nsamples = first_samples > 0 ? std::min(first_samples, b->maxSpp) : b->maxSpp;
    int k = 0;
    for (int j0 = 0; j0 < nsamples; j0 += b->chunkLen) {
        const int j1 = std::min(j0 + b->chunkLen, nsamples);
        std::vector<int> active;
        for (int i = 0; i < b->nreq; i++)
            if (b->req[(size_t)i].spp > j0) active.push_back(i);
        // largest work first, so that small requests fill the launch's tail
        auto work = [&](int i) {
            const BatchRequest& q = b->req[(size_t)i];
            return (double)q.npix * (double)(std::min(j1, q.spp) - j0) * (double)std::max(q.pp.maxDepth, 1);
        };
        std::stable_sort(active.begin(), active.end(), [&](int x, int y) { return work(x) > work(y); });
        for (size_t g0 = 0; g0 < active.size(); g0 += kMaxReqPerLaunch) {
            if (k >= b->nchunks_cap) fail(ZGL_ERR_STATE, "batch: launch count exceeds the counter array");
            BatchLaunch L, A;
            std::memset(&L, 0, sizeof(L));
            int64_t base = 0, pbase = 0;
            for (size_t j = g0; j < active.size() && (int)(j - g0) < kMaxReqPerLaunch; j++) {
                BatchRequest q = b->req[(size_t)active[j]];
                q.j1 = std::min(j1, q.spp);
                q.itemBase = base;
                base += (int64_t)(q.j1 - j0) * q.perSample;
                L.req[L.nreq++] = q;
            }
            L.nitems = base;
            L.j0 = j0;
            L.counter = b->d_counters + k;
            L.queueCap = c.queue_capacity;
            L.regenThreshold = c.regen_threshold;
            L.mats = b->d_mats;
            L.rows = b->d_rows;
            A = L;
            for (int i = 0; i < A.nreq; i++) {
                A.req[i].itemBase = pbase;
                pbase += A.req[i].npix;
            }
            A.nitems = pbase;
            if (c.schedule == ZGL_BATCH_PERSISTENT) {
                ZGL_CUDA(cudaMemsetAsync(L.counter, 0, sizeof(unsigned long long), st));
                ZGL_CUDA(launch_batch(L, c.block_size, b->fullMaterials, st));
            } else if (c.schedule == ZGL_BATCH_QUEUE) {
                ZGL_CUDA(cudaMemsetAsync(L.counter, 0, sizeof(unsigned long long), st));
                ZGL_CUDA(launch_batch_queue(L, b->fullMaterials, st));
            } else {
                FlatLaunch F;
                std::memset(&F, 0, sizeof(F));
                int64_t bb = 0;
                for (int i = 0; i < L.nreq; i++) {
                    const BatchRequest& q = L.req[i];
                    FlatRequest& f = F.req[F.nreq++];
                    f.sc = q.sc;
                    f.maxDepth = q.pp.maxDepth;
                    f.rr = q.pp.rr;
                    f.rrStart = q.pp.rrStart;
                    f.sampleLight = q.pp.sampleLight;
                    f.uniformSel = q.pp.uniformSel;
                    f.portion = q.pp.portion;
                    f.scratch = q.scratch;
                    f.tilesX = (q.sc.filmW + 15) / 16;
                    f.tilesY = (q.sc.filmH + 7) / 8;
                    f.j1 = q.j1;
                    f.blockBase = bb;
                    bb += (int64_t)f.tilesX * f.tilesY * (q.j1 - j0);
                }
                F.nblocks = bb;
                F.j0 = j0;
                F.rows = b->d_rows;
                F.mats = b->d_mats;
                F.full = b->fullMaterials;
                if (bb > 0x7fffffff) fail(ZGL_ERR_INVALID_ARG, "batch: too many tiles in one launch");
                ZGL_CUDA(launch_batch_flat(F, st));
            }
            ZGL_CUDA(launch_accumulate(A, st));
            k++;
        }
    }
}

bool same_cfg(const zgl_batch_config& x, const zgl_batch_config& y) {
    return x.block_size == y.block_size && x.queue_capacity == y.queue_capacity &&
           x.regen_threshold == y.regen_threshold && x.schedule == y.schedule;
}

}  // namespace
}  // namespace zgl

using namespace zgl;

extern "C" {

zgl_status zgl_batch_config_default(zgl_batch_config* c) {
    ZGL_API_BEGIN
    if (!c) fail(ZGL_ERR_INVALID_ARG, "zgl_batch_config_default: NULL");
    std::memset(c, 0, sizeof(*c));
    ZGL_API_END
}

zgl_status zgl_batch_create(const zgl_render_request* requests, int32_t n, const zgl_batch_config* config,
                            zgl_batch** out) {
    ZGL_API_BEGIN
    if (!requests || !out || n <= 0) fail(ZGL_ERR_INVALID_ARG, "zgl_batch_create: empty request list");
    *out = nullptr;
    zgl_batch_config cfg{};
    if (config) cfg = *config;
    check_config(cfg);
    auto* b = new zgl_batch();
    try {
        ZGL_CUDA(cudaGetDevice(&b->device));
        b->nreq = n;
        int64_t base = 0;
        for (int i = 0; i < n; i++) {
            const zgl_render_request& r = requests[i];
            if (!r.scene || !r.frame) fail(ZGL_ERR_INVALID_ARG, "zgl_batch_create: request %d lacks scene or frame", i);
            if (r.scene->host_only) fail(ZGL_ERR_STATE, "zgl_batch_create: request %d scene is host-only", i);
            if (r.scene->device != b->device) fail(ZGL_ERR_INVALID_ARG, "zgl_batch_create: request %d on another device", i);
            if (r.spp < 1 || r.spp > 65536) fail(ZGL_ERR_INVALID_ARG, "zgl_batch_create: request %d spp %d out of range", i, r.spp);
            zgl_integrator_params p = r.params;
            if (p.max_depth < 0 || p.max_depth > 1024 || p.rr_start_depth < 1 || !(p.light_portion >= 0.0f && p.light_portion <= 1.0f))
                fail(ZGL_ERR_INVALID_ARG, "zgl_batch_create: request %d has invalid parameters", i);
            BatchRequest q{};
            q.sc = r.scene->view();
            q.pp = BatchPathParams{p.max_depth, p.russian_roulette, p.rr_start_depth, p.sample_light,
                                   p.light_env_uniform_sample, p.light_portion};
            q.spp = r.spp;
            q.frame = reinterpret_cast<float4*>(r.frame);
            q.npix = r.scene->filmW * r.scene->filmH;
            q.tilesX = (r.scene->filmW + 7) / 8;
            q.perSample = q.tilesX * ((r.scene->filmH + 3) / 4) * 32;
            q.itemBase = base;
            base += q.npix;
            b->maxSpp = std::max(b->maxSpp, r.spp);
            b->fullMaterials = b->fullMaterials || r.scene->fullMaterials;
            b->req.push_back(q);
        }
        b->nitems = base;
        std::vector<uint32_t> mats;
        sobol_matrices(mats);
        ZGL_CUDA(cudaMalloc(&b->d_mats, sizeof(uint32_t) * mats.size()));
        ZGL_CUDA(cudaMemcpy(b->d_mats, mats.data(), sizeof(uint32_t) * mats.size(), cudaMemcpyHostToDevice));
        // Sobol rows of every sample index (sampleOffset wrap of
        // path_integ_naive.glsl:163-164)
        std::vector<uint32_t> rows((size_t)b->maxSpp * 256);
        for (int j = 0; j < b->maxSpp; j++) {
            int32_t off = (int32_t)((uint32_t)j * 256u);
            if (off > 131072 * 256) off -= 131072 * 256;
            const uint32_t rowIndex = (uint32_t)off >> 8;
            for (uint32_t d = 0; d < 256; d++) {
                uint32_t v = 0, idx = rowIndex;
                for (int bit = 0; idx != 0u; idx >>= 1, bit++)
                    if (idx & 1u) v ^= mats[d * 32u + (uint32_t)bit];
                rows[(size_t)j * 256 + d] = v;
            }
        }
        ZGL_CUDA(cudaMalloc(&b->d_rows, sizeof(uint32_t) * rows.size()));
        ZGL_CUDA(cudaMemcpy(b->d_rows, rows.data(), sizeof(uint32_t) * rows.size(), cudaMemcpyHostToDevice));
        // sample indices per launch: the per-sample scratch of all requests
        // stays within kScratchBudget bytes
        auto scratch_floats = [&](int len) {
            size_t f = 0;
            for (const auto& q : b->req) f += (size_t)std::min(len, q.spp) * (size_t)q.npix * 3;
            return f;
        };
        const size_t budget = cfg.scratch_mib > 0 ? (size_t)cfg.scratch_mib << 20 : kScratchBudget;
        b->chunkLen = b->maxSpp;
        while (b->chunkLen > 1 && scratch_floats(b->chunkLen) * sizeof(float) > budget)
            b->chunkLen = (b->chunkLen + 1) / 2;
        ZGL_CUDA(cudaMalloc(&b->d_scratch, sizeof(float) * scratch_floats(b->chunkLen)));
        size_t off = 0;
        for (auto& q : b->req) {
            q.scratch = b->d_scratch + off;
            off += (size_t)std::min(b->chunkLen, q.spp) * (size_t)q.npix * 3;
        }
        const int nChunks = (b->maxSpp + b->chunkLen - 1) / b->chunkLen;
        b->nchunks_cap = nChunks * ((n + kMaxReqPerLaunch - 1) / kMaxReqPerLaunch);
        ZGL_CUDA(cudaMalloc(&b->d_counters, sizeof(unsigned long long) * (size_t)b->nchunks_cap));
        ZGL_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
        ZGL_CUDA(cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming));
        ZGL_CUDA(cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming));
        b->cfg = resolve(cfg);
    } catch (...) {
        batch_free(b);
        throw;
    }
    *out = b;
    ZGL_API_END
}

zgl_status zgl_batch_set_config(zgl_batch* b, const zgl_batch_config* config) {
    ZGL_API_BEGIN
    if (!b || !config) fail(ZGL_ERR_INVALID_ARG, "zgl_batch_set_config: NULL");
    check_config(*config);
    b->cfg = resolve(*config);
    ZGL_API_END
}

zgl_status zgl_batch_get_config(const zgl_batch* b, zgl_batch_config* out) {
    ZGL_API_BEGIN
    if (!b || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_batch_get_config: NULL");
    *out = b->cfg;
    ZGL_API_END
}

zgl_status zgl_batch_render(zgl_batch* b, void* stream) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_batch_render");
    if (!b) fail(ZGL_ERR_INVALID_ARG, "zgl_batch_render: NULL");
    cudaStream_t user = (cudaStream_t)stream;
    if (!b->exec || !same_cfg(b->graph_cfg, b->cfg)) {
        if (b->exec) {
            ZGL_CUDA(cudaGraphExecDestroy(b->exec));
            b->exec = nullptr;
        }
        cudaGraph_t graph = nullptr;
        ZGL_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue_render(b, b->cfg, b->stream, 0);
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(b->stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        ZGL_CUDA(cudaStreamEndCapture(b->stream, &graph));
        cudaError_t e = cudaGraphInstantiate(&b->exec, graph, 0);
        cudaGraphDestroy(graph);
        ZGL_CUDA(e);
        b->graph_cfg = b->cfg;
    }
    // order the graph after the caller's stream and the caller's stream after it
    ZGL_CUDA(cudaEventRecord(b->ev_in, user));
    ZGL_CUDA(cudaStreamWaitEvent(b->stream, b->ev_in, 0));
    ZGL_CUDA(cudaGraphLaunch(b->exec, b->stream));
    ZGL_CUDA(cudaEventRecord(b->ev_out, b->stream));
    ZGL_CUDA(cudaStreamWaitEvent(user, b->ev_out, 0));
    ZGL_API_END
}

zgl_status zgl_batch_autotune(zgl_batch* b, void* stream, zgl_batch_config* chosen) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_batch_autotune");
    if (!b) fail(ZGL_ERR_INVALID_ARG, "zgl_batch_autotune: NULL");
    cudaStream_t st = b->stream;
    ZGL_CUDA(cudaEventRecord(b->ev_in, (cudaStream_t)stream));
    ZGL_CUDA(cudaStreamWaitEvent(st, b->ev_in, 0));
    cudaEvent_t e0, e1;
    ZGL_CUDA(cudaEventCreate(&e0));
    ZGL_CUDA(cudaEventCreate(&e1));
    const int blocks[] = {64, 128, 256};
    const int caps[] = {8, 32, 128};
    const int thresholds[] = {4, 16, 32};
    zgl_batch_config best = b->cfg;
    float bestMs = 1e30f;
    auto trial = [&](const zgl_batch_config& c) {
        ZGL_CUDA(cudaEventRecord(e0, st));
        enqueue_render(b, c, st, 2);
        ZGL_CUDA(cudaEventRecord(e1, st));
        ZGL_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        ZGL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < bestMs) {
            bestMs = ms;
            best = c;
        }
    };
    try {
        zgl_batch_config flat = b->cfg;
        flat.schedule = ZGL_BATCH_FLAT;
        trial(flat);
        for (int bs : blocks)
            for (int cap : caps)
                for (int th : thresholds) {
                    zgl_batch_config c = b->cfg;
                    c.schedule = ZGL_BATCH_PERSISTENT;
                    c.block_size = bs;
                    c.queue_capacity = cap;
                    c.regen_threshold = th;
                    trial(c);
                }
        for (int cap : caps)
            for (int th : thresholds) {
                zgl_batch_config c = b->cfg;
                c.schedule = ZGL_BATCH_QUEUE;
                c.block_size = kQueueBlock;
                c.queue_capacity = cap;
                c.regen_threshold = th;
                trial(c);
            }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->cfg = best;
    if (chosen) *chosen = best;
    ZGL_API_END
}

zgl_status zgl_batch_destroy(zgl_batch* b) {
    ZGL_API_BEGIN
    if (b) cudaStreamSynchronize(b->stream);
    batch_free(b);
    ZGL_API_END
}

}  // extern "C"
