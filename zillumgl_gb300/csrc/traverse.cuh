// traverse.cuh — device-side MTBVH traversal shared by the trace kernels and
// the integrators.
//
// Arithmetic follows src/shader/intersection.glsl exactly in float32 with no
// fused multiply-add (the library is compiled with -fmad=false): slab test
// boxHit (:226-329) with its axis-dominant and near-zero-component branches,
// the double-sided ray–triangle test with the unscaled |det| < 1e-6 rejection
// (:63-109), and the stackless threaded loop of bvhHit / bvhTest
// (:367-427) with the `boxDist > dist` prune and strict `t < dist` closest
// update, so that hit ids and distances are bit-identical.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "accel.h"

namespace zgl {

struct TraceRay {
    float3 o, d, dinv;
    // 0/1/2: |d.axis| > 1 - 1e-6 (axis-dominant branch of boxHit)
    // 3: general slab test, no component below 1e-6 in magnitude
    // 4: general slab test with near-zero-component branches
    int mode;
    bool sx, sy, sz;  // |d.axis| < 1e-6
    int face;         // cubemapFace(-dir) (math.glsl:112-131)
};

__device__ __forceinline__ TraceRay make_trace_ray(float3 o, float3 d) {
    TraceRay r;
    r.o = o;
    r.d = d;
    r.dinv = make_float3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    const float eps = 1e-6f;
    const float big = 1.0f - eps;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    r.sx = ax < eps;
    r.sy = ay < eps;
    r.sz = az < eps;
    r.mode = (ax > big) ? 0 : (ay > big) ? 1 : (az > big) ? 2 : ((r.sx || r.sy || r.sz) ? 4 : 3);
    // cubemapFace(-d): maxExtent(|-d|) with strict '>', sign of -d
    float nx = -d.x, ny = -d.y, nz = -d.z;
    int m = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
    r.face = (m == 0) ? (nx > 0.0f ? 0 : 1) : (m == 1) ? (ny > 0.0f ? 2 : 3) : (nz > 0.0f ? 4 : 5);
    return r;
}

// boxHit specialised by ray mode.  fminf/fmaxf return the non-NaN operand
// like GPU GLSL min/max; the returned tMin only takes part in comparisons, so
// the sign of a zero result never matters.
template <int MODE>
__device__ __forceinline__ bool box_hit_m(const float4 lo, const float4 hi, const TraceRay& r, float& tmin) {
    const float3 o = r.o;
    if (MODE == 0 || MODE == 1 || MODE == 2) {
        // slab along the dominant axis, strict inside test on the other two
        const float oa = MODE == 0 ? o.x : MODE == 1 ? o.y : o.z;
        const float ia = MODE == 0 ? r.dinv.x : MODE == 1 ? r.dinv.y : r.dinv.z;
        const float la = MODE == 0 ? lo.x : MODE == 1 ? lo.y : lo.z;
        const float ha = MODE == 0 ? hi.x : MODE == 1 ? hi.y : hi.z;
        const float ob = MODE == 0 ? o.y : o.x, lb = MODE == 0 ? lo.y : lo.x, hb = MODE == 0 ? hi.y : hi.x;
        const float oc = MODE == 2 ? o.y : o.z, lc = MODE == 2 ? lo.y : lo.z, hc = MODE == 2 ? hi.y : hi.z;
        if (ob > lb && ob < hb && oc > lc && oc < hc) {
            float ta = (la - oa) * ia, tb = (ha - oa) * ia;
            tmin = fminf(ta, tb);
            float tmax = fmaxf(ta, tb);
            return tmax >= 0.0f && tmax >= tmin;
        }
        return false;
    }
    float ax = (lo.x - o.x) * r.dinv.x, ay = (lo.y - o.y) * r.dinv.y, az = (lo.z - o.z) * r.dinv.z;
    float bx = (hi.x - o.x) * r.dinv.x, by = (hi.y - o.y) * r.dinv.y, bz = (hi.z - o.z) * r.dinv.z;
    float nx = fminf(ax, bx), ny = fminf(ay, by), nz = fminf(az, bz);
    float fx = fmaxf(ax, bx), fy = fmaxf(ay, by), fz = fmaxf(az, bz);
    float dx = fx - nx, dy = fy - ny, dz = fz - nz;
    float tyz = fz - ny, tzx = fx - nz, txy = fy - nx;
    float tmax;
    if (MODE == 4) {
        if (r.sx && dy + dz > tyz) {
            tmin = fmaxf(ny, nz);
            tmax = fminf(fy, fz);
            return tmax >= 0.0f && tmax >= tmin;
        }
        if (r.sy && dz + dx > tzx) {
            tmin = fmaxf(nz, nx);
            tmax = fminf(fz, fx);
            return tmax >= 0.0f && tmax >= tmin;
        }
        if (r.sz && dx + dy > txy) {
            tmin = fmaxf(nx, ny);
            tmax = fminf(fx, fy);
            return tmax >= 0.0f && tmax >= tmin;
        }
    }
    tmin = fmaxf(fmaxf(nx, ny), nz);
    tmax = fminf(fminf(fx, fy), fz);
    return (dy + dz > tyz) && (dz + dx > tzx) && (dx + dy > txy) && tmax >= 0.0f && tmax >= tmin;
}

__device__ __forceinline__ bool box_hit(const float4 lo, const float4 hi, const TraceRay& r, float& tmin) {
    switch (r.mode) {
        case 0: return box_hit_m<0>(lo, hi, r, tmin);
        case 1: return box_hit_m<1>(lo, hi, r, tmin);
        case 2: return box_hit_m<2>(lo, hi, r, tmin);
        case 3: return box_hit_m<3>(lo, hi, r, tmin);
        default: return box_hit_m<4>(lo, hi, r, tmin);
    }
}

// intersectTriangle with precomputed a, ab = b - a, ac = c - a.
__device__ __forceinline__ bool tri_hit(const float4* __restrict__ tris, int prim,
                                        const TraceRay& r, float& t) {
    const float4 t0 = __ldg(tris + 3 * (size_t)prim);
    const float4 t1 = __ldg(tris + 3 * (size_t)prim + 1);
    const float4 t2 = __ldg(tris + 3 * (size_t)prim + 2);
    const float abx = t0.w, aby = t1.x, abz = t1.y;
    const float acx = t1.z, acy = t1.w, acz = t2.x;
    const float3 d = r.d;
    // p = cross(d, ac); det = dot(ab, p)
    float px = d.y * acz - d.z * acy;
    float py = d.z * acx - d.x * acz;
    float pz = d.x * acy - d.y * acx;
    float det = abx * px + aby * py + abz * pz;
    if (fabsf(det) < 1e-6f) return false;
    float aox = r.o.x - t0.x, aoy = r.o.y - t0.y, aoz = r.o.z - t0.z;
    if (det < 0.0f) {
        aox = -aox;
        aoy = -aoy;
        aoz = -aoz;
        det = -det;
    }
    float u = aox * px + aoy * py + aoz * pz;
    if (u < 0.0f || u > det) return false;
    // q = cross(ao, ab)
    float qx = aoy * abz - aoz * aby;
    float qy = aoz * abx - aox * abz;
    float qz = aox * aby - aoy * abx;
    float v = d.x * qx + d.y * qy + d.z * qz;
    if (v < 0.0f || u + v > det) return false;
    t = (acx * qx + acy * qy + acz * qz) / det;
    return t > 0.0f;
}

// bvhHit (ANY = false): returns the closest primitive or -1 and lowers `dist`.
// bvhTest (ANY = true): returns 1 at the first t < dist, else 0.
// The loop index only grows (k = max(miss, k + 1)), so it ends within M steps
// even on a corrupted table.  The loop is instantiated per ray mode so that
// the common general case carries no per-visit mode tests.
template <bool ANY, bool COUNT, int MODE>
__device__ __forceinline__ int traverse_m(const DeviceAccel& a, const TraceRay& r, float& dist, int& visits,
                                          int& tests) {
    const float4* __restrict__ base = a.nodes + (size_t)r.face * (size_t)a.M * 2;
    int closest = -1;
    int k = 0;
    const int M = a.M;
    while (k < M) {
        const float4 lo = __ldg(base + 2 * k);
        const float4 hi = __ldg(base + 2 * k + 1);
        if (COUNT) visits++;
        float tmin;
        const bool h = box_hit_m<MODE>(lo, hi, r, tmin) && !(tmin > dist);
        const int prim = __float_as_int(lo.w);
        int next = h ? k + 1 : max(__float_as_int(hi.w), k + 1);
        if (h && prim >= 0) {
            if (COUNT) tests++;
            float t;
            if (tri_hit(a.tris, prim, r, t) && t < dist) {
                closest = prim;
                if (ANY) break;
                dist = t;
            }
        }
        k = next;
    }
    return ANY ? (closest >= 0 ? 1 : 0) : closest;
}

// A node-record load, optionally with an L2 prefetch-size hint (the L2 then
// fetches the aligned 128 or 256 bytes around the record from DRAM: the
// next entries of a descent are the next records of the table).
template <int HINT>
__device__ __forceinline__ float4 load_node(const float4* p) {
    if (HINT == 0) return __ldg(p);
    float4 v;
    if (HINT == 256)
        asm("ld.global.nc.L2::256B.v4.f32 {%0, %1, %2, %3}, [%4];"
            : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
            : "l"(p));
    else
        asm("ld.global.nc.L2::128B.v4.f32 {%0, %1, %2, %3}, [%4];"
            : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
            : "l"(p));
    return v;
}

// bvhHit / bvhTest (ANY) in the reference's visiting order with the node
// loads arranged for memory-level parallelism.  PF: both possible
// successors of entry k (k + 1 after a box hit, the miss link after a box
// miss) are requested before the box and triangle tests of k, so their
// latency overlaps that work; the test result then picks one.  HINT: L2
// prefetch size of the node loads (0: none).  Results are those of
// traverse_m.
template <bool ANY, int MODE, bool PF, int HINT>
__device__ __forceinline__ int traverse_v(const DeviceAccel& a, const TraceRay& r, float& dist) {
    const float4* __restrict__ base = a.nodes + (size_t)r.face * (size_t)a.M * 2;
    const int M = a.M;
    int closest = -1;
    if (M <= 0) return ANY ? 0 : -1;
    int k = 0;
    float4 lo = load_node<HINT>(base), hi = load_node<HINT>(base + 1);
    for (;;) {
        const int prim = __float_as_int(lo.w);
        const int skip = max(__float_as_int(hi.w), k + 1);
        float4 alo, ahi, blo, bhi;
        if (PF) {
            const int ka = min(k + 1, M - 1), kb = min(skip, M - 1);
            alo = load_node<HINT>(base + 2 * ka);
            ahi = load_node<HINT>(base + 2 * ka + 1);
            blo = load_node<HINT>(base + 2 * kb);
            bhi = load_node<HINT>(base + 2 * kb + 1);
        }
        float tmin;
        const bool h = box_hit_m<MODE>(lo, hi, r, tmin) && !(tmin > dist);
        const int next = h ? k + 1 : skip;
        if (h && prim >= 0) {
            float t;
            if (tri_hit(a.tris, prim, r, t) && t < dist) {
                closest = prim;
                if (ANY) break;
                dist = t;
            }
        }
        if (next >= M) break;
        if (PF) {
            lo = h ? alo : blo;
            hi = h ? ahi : bhi;
        } else {
            lo = load_node<HINT>(base + 2 * next);
            hi = load_node<HINT>(base + 2 * next + 1);
        }
        k = next;
    }
    return ANY ? (closest >= 0 ? 1 : 0) : closest;
}

template <bool ANY, bool PF, int HINT>
__device__ __forceinline__ int traverse_vm(const DeviceAccel& a, const TraceRay& r, float& dist) {
    switch (r.mode) {
        case 3: return traverse_v<ANY, 3, PF, HINT>(a, r, dist);
        case 4: return traverse_v<ANY, 4, PF, HINT>(a, r, dist);
        case 0: return traverse_v<ANY, 0, PF, HINT>(a, r, dist);
        case 1: return traverse_v<ANY, 1, PF, HINT>(a, r, dist);
        default: return traverse_v<ANY, 2, PF, HINT>(a, r, dist);
    }
}

// ---------------------------------------------------------------------------
// Long rays.  A few rays visit tens of thousands of table entries: a
// direction component below 1e-6 takes boxHit's near-zero-component branch,
// which accepts every box whose slab holds the origin on that axis (on the
// 4M-triangle soup with 2^24 incoherent rays, 55 such rays visit up to
// 58,981 entries; the median ray visits 99 and no other ray more than
// 1,581).  Traversed by one lane, such a ray is a chain of dependent loads
// that outlasts the rest of its launch.  So a lane
// traverses alone for a budget of entries (traverse_lane), and a ray still
// unfinished then is walked by its whole warp (traverse_warp): each lane
// loads one entry of a window of 32 consecutive entries and evaluates its
// slab test and, for a leaf, its triangle test, neither of which depends on
// the running distance; the warp then follows the reference's path through
// the window in order, applying `!(tmin > dist)` and `t < dist` with the
// distance as it stands at each step.  Entries visited, tests taken and
// results are those of traverse_m.
// ---------------------------------------------------------------------------

// traverse_v from entry k with the running `closest`.  Only rays with a
// near-zero direction component (MODE 4) get long: on the soups every other
// ray visits at most about 1,600 entries.  So only their loop counts steps,
// and stops after `budget` entries; the other modes run to the end without
// the count.  Returns true when the ray is finished (k >= M, or an any-hit
// found); otherwise k is the next entry to visit.
template <bool ANY, int MODE, bool PF, int HINT>
__device__ __forceinline__ bool traverse_lane(const DeviceAccel& a, const TraceRay& r, float& dist, int& k,
                                              int& closest, int budget) {
    const float4* __restrict__ base = a.nodes + (size_t)r.face * (size_t)a.M * 2;
    const int M = a.M;
    if (MODE != 4) budget = 0x7fffffff;
    if (!PF) {  // the loop of traverse_m, with a step count in MODE 4
        for (int step = 0; k < M; step++) {
            if (MODE == 4 && step == budget) return false;
            const float4 lo = load_node<HINT>(base + 2 * k);
            const float4 hi = load_node<HINT>(base + 2 * k + 1);
            float tmin;
            const bool h = box_hit_m<MODE>(lo, hi, r, tmin) && !(tmin > dist);
            const int prim = __float_as_int(lo.w);
            const int next = h ? k + 1 : max(__float_as_int(hi.w), k + 1);
            if (h && prim >= 0) {
                float t;
                if (tri_hit(a.tris, prim, r, t) && t < dist) {
                    closest = prim;
                    if (ANY) return true;
                    dist = t;
                }
            }
            k = next;
        }
        return true;
    }
    if (k >= M) return true;
    float4 lo = load_node<HINT>(base + 2 * k), hi = load_node<HINT>(base + 2 * k + 1);
    for (int step = 0; MODE != 4 || step < budget; step++) {
        const int prim = __float_as_int(lo.w);
        const int skip = max(__float_as_int(hi.w), k + 1);
        float4 alo, ahi, blo, bhi;
        if (PF) {
            const int ka = min(k + 1, M - 1), kb = min(skip, M - 1);
            alo = load_node<HINT>(base + 2 * ka);
            ahi = load_node<HINT>(base + 2 * ka + 1);
            blo = load_node<HINT>(base + 2 * kb);
            bhi = load_node<HINT>(base + 2 * kb + 1);
        }
        float tmin;
        const bool h = box_hit_m<MODE>(lo, hi, r, tmin) && !(tmin > dist);
        const int next = h ? k + 1 : skip;
        if (h && prim >= 0) {
            float t;
            if (tri_hit(a.tris, prim, r, t) && t < dist) {
                closest = prim;
                if (ANY) return true;
                dist = t;
            }
        }
        k = next;
        if (next >= M) return true;
        if (PF) {
            lo = h ? alo : blo;
            hi = h ? ahi : bhi;
        } else {
            lo = load_node<HINT>(base + 2 * next);
            hi = load_node<HINT>(base + 2 * next + 1);
        }
    }
    return false;
}

template <bool ANY, bool PF, int HINT>
__device__ __forceinline__ bool traverse_lane_m(const DeviceAccel& a, const TraceRay& r, float& dist, int& k,
                                                int& closest, int budget) {
    switch (r.mode) {
        case 3: return traverse_lane<ANY, 3, PF, HINT>(a, r, dist, k, closest, budget);
        case 4: return traverse_lane<ANY, 4, PF, HINT>(a, r, dist, k, closest, budget);
        case 0: return traverse_lane<ANY, 0, PF, HINT>(a, r, dist, k, closest, budget);
        case 1: return traverse_lane<ANY, 1, PF, HINT>(a, r, dist, k, closest, budget);
        default: return traverse_lane<ANY, 2, PF, HINT>(a, r, dist, k, closest, budget);
    }
}

// The rest of one ray from entry k, walked by all 32 lanes of the warp (ray
// and state warp-uniform; every lane calls).
template <bool ANY, int MODE>
__device__ __forceinline__ void traverse_warp(const DeviceAccel& a, const TraceRay& r, float& dist, int& k,
                                              int& closest) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const float4* __restrict__ base = a.nodes + (size_t)r.face * (size_t)a.M * 2;
    const int M = a.M;
    while (k < M) {
        const int j = k + lane;
        float4 lo = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1)), hi = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (j < M) {
            lo = __ldg(base + 2 * (size_t)j);
            hi = __ldg(base + 2 * (size_t)j + 1);
        }
        float tmin = 0.0f, t = 0.0f;
        const bool geom = j < M && box_hit_m<MODE>(lo, hi, r, tmin);
        const int prim = __float_as_int(lo.w);
        const bool tri = geom && prim >= 0 && tri_hit(a.tris, prim, r, t);
        const int skip = max(__float_as_int(hi.w), j + 1);
        const unsigned G = __ballot_sync(full, geom), T = __ballot_sync(full, tri);
        // the path through the window: p only grows, so at most 32 steps
        int p = 0;
        for (;;) {
            const float tm = __shfl_sync(full, tmin, p);
            const float tt = __shfl_sync(full, t, p);
            const int pr = __shfl_sync(full, prim, p);
            const int sk = __shfl_sync(full, skip, p);
            const bool h = ((G >> p) & 1u) && !(tm > dist);
            if (h && ((T >> p) & 1u) && tt < dist) {
                closest = pr;
                if (ANY) {
                    k = M;
                    return;
                }
                dist = tt;
            }
            const int next = h ? k + p + 1 : max(sk, k + p + 1);  // the max holds by construction
            if (next >= M || next - k >= 32) {
                k = next;
                break;
            }
            p = next - k;
        }
    }
}

// The accelerator of lane `src` of `group`: lanes of one warp may trace in
// different scenes (the batched renderer's persistent and queue schedules),
// and a walk reads the tables of the ray it serves.
__device__ __forceinline__ DeviceAccel group_accel(unsigned group, const DeviceAccel& a, int src) {
    DeviceAccel w;
    w.nodes = reinterpret_cast<const float4*>(
        __shfl_sync(group, reinterpret_cast<unsigned long long>(a.nodes), src));
    w.tris = reinterpret_cast<const float4*>(
        __shfl_sync(group, reinterpret_cast<unsigned long long>(a.tris), src));
    w.M = __shfl_sync(group, a.M, src);
    return w;
}

// Finishes, one at a time with the whole warp, the rays of the warp's lanes
// that traverse_lane left unfinished (`done` false).  Every lane calls; a
// lane without a ray passes done = true.
template <bool ANY>
__device__ __forceinline__ void finish_long_rays(const DeviceAccel& a, const TraceRay& r, float& dist, int& k,
                                                 int& closest, bool done) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    unsigned pending = __ballot_sync(full, !done);
    while (pending) {
        const int src = __ffs(pending) - 1;
        pending &= pending - 1;
        const float3 o = make_float3(__shfl_sync(full, r.o.x, src), __shfl_sync(full, r.o.y, src),
                                     __shfl_sync(full, r.o.z, src));
        const float3 d = make_float3(__shfl_sync(full, r.d.x, src), __shfl_sync(full, r.d.y, src),
                                     __shfl_sync(full, r.d.z, src));
        float wd = __shfl_sync(full, dist, src);
        int wk = __shfl_sync(full, k, src), wc = __shfl_sync(full, closest, src);
        const TraceRay w = make_trace_ray(o, d);
        const DeviceAccel wa = group_accel(full, a, src);
        switch (w.mode) {
            case 3: traverse_warp<ANY, 3>(wa, w, wd, wk, wc); break;
            case 4: traverse_warp<ANY, 4>(wa, w, wd, wk, wc); break;
            case 0: traverse_warp<ANY, 0>(wa, w, wd, wk, wc); break;
            case 1: traverse_warp<ANY, 1>(wa, w, wd, wk, wc); break;
            default: traverse_warp<ANY, 2>(wa, w, wd, wk, wc); break;
        }
        if (lane == src) {
            dist = wd;
            k = wk;
            closest = wc;
        }
    }
}

// Entries a ray with a near-zero direction component traverses on its lane
// before its warp (or the group of lanes that called together) takes it
// over.
constexpr int kLongRayBudget = 256;

// traverse_warp for a group of lanes `group` (the lanes of the warp that
// called together; a window is as wide as the group, entry k + rank on the
// lane of that rank).  Only MODE 4 rays are handed over, so only that mode
// is instantiated.
template <bool ANY>
__device__ __forceinline__ void traverse_group(unsigned group, const DeviceAccel& a, const TraceRay& r,
                                               float& dist, int& k, int& closest) {
    const int lane = threadIdx.x & 31;
    const int width = __popc(group);
    const int rank = __popc(group & ((1u << lane) - 1u));
    const float4* __restrict__ base = a.nodes + (size_t)r.face * (size_t)a.M * 2;
    const int M = a.M;
    while (k < M) {
        const int j = k + rank;
        float4 lo = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1)), hi = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (j < M) {
            lo = __ldg(base + 2 * (size_t)j);
            hi = __ldg(base + 2 * (size_t)j + 1);
        }
        float tmin = 0.0f, t = 0.0f;
        const bool geom = j < M && box_hit_m<4>(lo, hi, r, tmin);
        const int prim = __float_as_int(lo.w);
        const bool tri = geom && prim >= 0 && tri_hit(a.tris, prim, r, t);
        const int skip = max(__float_as_int(hi.w), j + 1);
        const unsigned G = __ballot_sync(group, geom), T = __ballot_sync(group, tri);  // lane bits
        int p = 0;
        for (;;) {
            const int src = __ffs(__ballot_sync(group, rank == p)) - 1;  // lane holding window position p
            const float tm = __shfl_sync(group, tmin, src);
            const float tt = __shfl_sync(group, t, src);
            const int pr = __shfl_sync(group, prim, src);
            const int sk = __shfl_sync(group, skip, src);
            const bool h = ((G >> src) & 1u) && !(tm > dist);
            if (h && ((T >> src) & 1u) && tt < dist) {
                closest = pr;
                if (ANY) {
                    k = M;
                    return;
                }
                dist = tt;
            }
            const int next = h ? k + p + 1 : max(sk, k + p + 1);  // the max holds by construction
            if (next >= M || next - k >= width) {
                k = next;
                break;
            }
            p = next - k;
        }
    }
}

// finish_long_rays for the lanes in `group`, which all call it.
template <bool ANY>
__device__ __forceinline__ void finish_long_rays_group(unsigned group, const DeviceAccel& a, const TraceRay& r,
                                                       float& dist, int& k, int& closest, bool done) {
    const int lane = threadIdx.x & 31;
    unsigned pending = __ballot_sync(group, !done);
    while (pending) {
        const int src = __ffs(pending) - 1;
        pending &= pending - 1;
        const float3 o = make_float3(__shfl_sync(group, r.o.x, src), __shfl_sync(group, r.o.y, src),
                                     __shfl_sync(group, r.o.z, src));
        const float3 d = make_float3(__shfl_sync(group, r.d.x, src), __shfl_sync(group, r.d.y, src),
                                     __shfl_sync(group, r.d.z, src));
        float wd = __shfl_sync(group, dist, src);
        int wk = __shfl_sync(group, k, src), wc = __shfl_sync(group, closest, src);
        traverse_group<ANY>(group, group_accel(group, a, src), make_trace_ray(o, d), wd, wk, wc);
        if (lane == src) {
            dist = wd;
            k = wk;
            closest = wc;
        }
    }
}

template <bool ANY, bool COUNT>
__device__ __forceinline__ int traverse(const DeviceAccel& a, const TraceRay& r, float& dist, int& visits,
                                        int& tests) {
    switch (r.mode) {
        case 3: return traverse_m<ANY, COUNT, 3>(a, r, dist, visits, tests);
        case 4: return traverse_m<ANY, COUNT, 4>(a, r, dist, visits, tests);
        case 0: return traverse_m<ANY, COUNT, 0>(a, r, dist, visits, tests);
        case 1: return traverse_m<ANY, COUNT, 1>(a, r, dist, visits, tests);
        default: return traverse_m<ANY, COUNT, 2>(a, r, dist, visits, tests);
    }
}

}  // namespace zgl
