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
    int mode;  // 0/1/2: |d.axis| > 1 - 1e-6 (axis-dominant branch), 3: general
    bool sx, sy, sz;  // |d.axis| < 1e-6 (near-zero-component branches)
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
    r.mode = (ax > big) ? 0 : (ay > big) ? 1 : (az > big) ? 2 : 3;
    r.sx = ax < eps;
    r.sy = ay < eps;
    r.sz = az < eps;
    // cubemapFace(-d): maxExtent(|-d|) with strict '>', sign of -d
    float nx = -d.x, ny = -d.y, nz = -d.z;
    int m = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
    r.face = (m == 0) ? (nx > 0.0f ? 0 : 1) : (m == 1) ? (ny > 0.0f ? 2 : 3) : (nz > 0.0f ? 4 : 5);
    return r;
}

// boxHit.  fminf/fmaxf return the non-NaN operand like GPU GLSL min/max; the
// returned tMin only takes part in comparisons, so the sign of a zero result
// never matters.
__device__ __forceinline__ bool box_hit(const float4 lo, const float4 hi, const TraceRay& r,
                                        float& tmin) {
    const float3 o = r.o;
    if (r.mode == 0) {
        if (o.y > lo.y && o.y < hi.y && o.z > lo.z && o.z < hi.z) {
            float ta = (lo.x - o.x) * r.dinv.x, tb = (hi.x - o.x) * r.dinv.x;
            tmin = fminf(ta, tb);
            float tmax = fmaxf(ta, tb);
            return tmax >= 0.0f && tmax >= tmin;
        }
        return false;
    }
    if (r.mode == 1) {
        if (o.x > lo.x && o.x < hi.x && o.z > lo.z && o.z < hi.z) {
            float ta = (lo.y - o.y) * r.dinv.y, tb = (hi.y - o.y) * r.dinv.y;
            tmin = fminf(ta, tb);
            float tmax = fmaxf(ta, tb);
            return tmax >= 0.0f && tmax >= tmin;
        }
        return false;
    }
    if (r.mode == 2) {
        if (o.x > lo.x && o.x < hi.x && o.y > lo.y && o.y < hi.y) {
            float ta = (lo.z - o.z) * r.dinv.z, tb = (hi.z - o.z) * r.dinv.z;
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
    if (dy + dz > tyz && dz + dx > tzx && dx + dy > txy) {
        tmin = fmaxf(fmaxf(nx, ny), nz);
        tmax = fminf(fminf(fx, fy), fz);
        return tmax >= 0.0f && tmax >= tmin;
    }
    return false;
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
// even on a corrupted table.
template <bool ANY, bool COUNT>
__device__ __forceinline__ int traverse(const DeviceAccel& a, const TraceRay& r, float& dist,
                                        int& visits, int& tests) {
    const float4* __restrict__ base = a.nodes + (size_t)r.face * (size_t)a.M * 2;
    int closest = -1;
    int k = 0;
    const int M = a.M;
    while (k < M) {
        const float4 lo = __ldg(base + 2 * (size_t)k);
        const float4 hi = __ldg(base + 2 * (size_t)k + 1);
        if (COUNT) visits++;
        float tmin;
        bool h = box_hit(lo, hi, r, tmin);
        if (!h || tmin > dist) {
            k = max(__float_as_int(hi.w), k + 1);
            continue;
        }
        int prim = __float_as_int(lo.w);
        if (prim >= 0) {
            if (COUNT) tests++;
            float t;
            if (tri_hit(a.tris, prim, r, t) && t < dist) {
                if (ANY) return 1;
                dist = t;
                closest = prim;
            }
        }
        k++;
    }
    return ANY ? 0 : closest;
}

}  // namespace zgl
