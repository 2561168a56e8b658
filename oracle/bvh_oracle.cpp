// bvh_oracle.cpp — CPU oracle of the ZillumGL MTBVH build and its stackless
// traversal.
//
// TEST INFRASTRUCTURE ONLY: this file is the checker of the CUDA path.  Only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load the
// library built from it; the product never does.
//
// Parity status: the host build (quickBuild, buildHitTable) is restated from
// src/accelerator/BVH.cpp and AABB.cpp; those files cannot be compiled here
// (BVH.h pulls in the OpenGL buffer and assimp model headers), so the build is
// pinned by restatement and by structural invariants checked in tests.  The
// traversal (src/shader/intersection.glsl) is GLSL and needs OpenGL, which is
// unavailable on this machine: parity unpinned at the shader level; the oracle
// defines the arithmetic (float32, no fused multiply-add, left-to-right dot).
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle_math.h"

using namespace orc;

namespace {

// glm::min / glm::max on floats: (y < x) ? y : x and (x < y) ? y : x.
inline float hmin(float x, float y) { return (y < x) ? y : x; }
inline float hmax(float x, float y) { return (x < y) ? y : x; }
inline vec3 hmin3(vec3 a, vec3 b) { return vec3(hmin(a.x, b.x), hmin(a.y, b.y), hmin(a.z, b.z)); }
inline vec3 hmax3(vec3 a, vec3 b) { return vec3(hmax(a.x, b.x), hmax(a.y, b.y), hmax(a.z, b.z)); }

// AABB (src/accelerator/AABB.h:10-38, AABB.cpp:3-37). Default box is
// (1e8, -1e8), AABB.h:13.
struct AABB {
    vec3 pMin{1e8f, 1e8f, 1e8f};
    vec3 pMax{-1e8f, -1e8f, -1e8f};
    AABB() {}
    explicit AABB(vec3 p) : pMin(p), pMax(p) {}
    AABB(vec3 a, vec3 b, vec3 c) : pMin(hmin3(hmin3(a, b), c)), pMax(hmax3(hmax3(a, b), c)) {}
    static AABB join(const AABB& a, const AABB& b) {
        AABB r;
        r.pMin = hmin3(a.pMin, b.pMin);
        r.pMax = hmax3(a.pMax, b.pMax);
        return r;
    }
    void expand(const AABB& o) {
        pMin = hmin3(pMin, o.pMin);
        pMax = hmax3(pMax, o.pMax);
    }
    vec3 centroid() const { return (pMin + pMax) * 0.5f; }
    float surfaceArea() const {
        vec3 v = pMax - pMin;
        return 2.0f * (v.x * v.y + v.y * v.z + v.z * v.x);
    }
    int maxExtent() const {
        vec3 v = pMax - pMin;
        if (v.x > v.y) return v.x > v.z ? 0 : 2;
        return v.y > v.z ? 1 : 2;
    }
};

struct PrimInfo {
    AABB bound;
    vec3 centroid;
    int index;
};

struct Bucket {
    int count = 0;
    AABB box;
};

struct BuildRec {
    int offset;
    AABB nodeExtent;
    int splitDim;
    int l, r;
};

constexpr int kBuckets = 16;
constexpr int32_t kLeafMask = (int32_t)0x80000000u;  // BVH.h:11

// int(16 * (c - min) / (max - min)) clamped to [0, 15] (BVH.cpp:106-107,
// :256-257).  The float->int conversion is the truncating, saturating one
// (NaN from a zero-width extent gives 0).
inline int bucketOf(float c, float axisMin, float axisMax) {
    int b = f2i(16.0f * (c - axisMin) / (axisMax - axisMin));
    return std::max(std::min(b, kBuckets - 1), 0);
}

// partition<16> (BVH.cpp:97-114): stable left fill, reversed right fill,
// returns the index of the last left element; never leaves the right empty.
int partitionPrims(PrimInfo* a, int size, float axisMin, float axisMax, int dim, int splitBucket) {
    std::vector<PrimInfo> tmp(a, a + size);
    int l = 0, r = size;
    for (int i = 0; i < size; i++) {
        int b = bucketOf(tmp[i].centroid[dim], axisMin, axisMax);
        if (b <= splitBucket) a[l++] = tmp[i];
        else a[--r] = tmp[i];
    }
    if (r == size) r--;
    return r - 1;
}

struct Packed {
    std::vector<AABB> bounds;
    std::vector<int32_t> sizeIndices;
    std::vector<int32_t> hitTable;
};

// BVH::build + quickBuild (BVH.cpp:116-144, :217-296).
void quickBuild(const float* verts, const uint32_t* idx, int64_t ntri, Packed& out) {
    std::vector<PrimInfo> prim((size_t)ntri);
    AABB rootCent;
    for (int64_t i = 0; i < ntri; i++) {
        auto V = [&](uint32_t k) { return vec3(verts[3 * k], verts[3 * k + 1], verts[3 * k + 2]); };
        PrimInfo p;
        p.bound = AABB(V(idx[3 * i]), V(idx[3 * i + 1]), V(idx[3 * i + 2]));
        p.centroid = p.bound.centroid();
        p.index = (int)i;
        rootCent.expand(AABB(p.centroid));
        prim[(size_t)i] = p;
    }
    size_t M = (size_t)(2 * ntri - 1);
    out.bounds.assign(M, AABB());
    out.sizeIndices.assign(M, 0);

    std::vector<BuildRec> stack;
    stack.push_back({0, rootCent, rootCent.maxExtent(), 0, (int)ntri - 1});
    while (!stack.empty()) {
        BuildRec rec = stack.back();
        stack.pop_back();
        int offset = rec.offset, l = rec.l, r = rec.r, dim = rec.splitDim;
        int size = (r - l) * 2 + 1;
        out.sizeIndices[offset] = (size == 1) ? (prim[l].index | kLeafMask) : size;
        if (l == r) {
            out.bounds[offset] = prim[l].bound;
            continue;
        }
        int nBoxes = r - l + 1;
        if (nBoxes == 2) {
            out.bounds[offset] = AABB::join(prim[l].bound, prim[r].bound);
            if (prim[l].centroid[dim] > prim[r].centroid[dim]) std::swap(prim[l], prim[r]);
            stack.push_back({offset + 2, AABB(prim[r].centroid), 0, r, r});
            stack.push_back({offset + 1, AABB(prim[l].centroid), 0, l, l});
            continue;
        }
        float axisMin = rec.nodeExtent.pMin[dim];
        float axisMax = rec.nodeExtent.pMax[dim];
        Bucket buckets[kBuckets], prefix[kBuckets], suffix[kBuckets];
        for (int i = l; i <= r; i++) {
            int b = bucketOf(prim[i].centroid[dim], axisMin, axisMax);
            buckets[b].count++;
            buckets[b].box.expand(prim[i].bound);
        }
        prefix[0] = buckets[0];
        suffix[kBuckets - 1] = buckets[kBuckets - 1];
        for (int i = 1; i < kBuckets; i++) {
            prefix[i].count = prefix[i - 1].count + buckets[i].count;
            prefix[i].box = AABB::join(prefix[i - 1].box, buckets[i].box);
            suffix[kBuckets - 1 - i].count = suffix[kBuckets - i].count + buckets[kBuckets - i - 1].count;
            suffix[kBuckets - 1 - i].box = AABB::join(suffix[kBuckets - i].box, buckets[kBuckets - i - 1].box);
        }
        out.bounds[offset] = prefix[kBuckets - 1].box;
        int splitBucket = 0;
        float minCost = (float)prefix[0].count * prefix[0].box.surfaceArea() +
                        (float)suffix[1].count * suffix[1].box.surfaceArea();
        for (int i = 1; i < kBuckets - 1; i++) {
            float cost = (float)prefix[i].count * prefix[i].box.surfaceArea() +
                         (float)suffix[i + 1].count * suffix[i + 1].box.surfaceArea();
            if (cost < minCost) {
                minCost = cost;
                splitBucket = i;
            }
        }
        int split = l + partitionPrims(&prim[l], nBoxes, axisMin, axisMax, dim, splitBucket);
        AABB lc, rc;
        for (int i = l; i <= split; i++) lc.expand(AABB(prim[i].centroid));
        for (int i = split + 1; i <= r; i++) rc.expand(AABB(prim[i].centroid));
        stack.push_back({offset + 2 * (split - l) + 2, rc, rc.maxExtent(), split + 1, r});
        stack.push_back({offset + 1, lc, lc.maxExtent(), l, split});
    }
}

// buildHitTable (BVH.cpp:298-345): six threaded orders; face i visits the
// child with the larger (+axis) / smaller (-axis) box centroid first.
void buildHitTable(Packed& p) {
    size_t M = p.bounds.size();
    p.hitTable.assign(M * 18, 0);
    std::vector<size_t> stack(M + 1);
    for (int face = 0; face < 6; face++) {
        int axis = face >> 1;
        bool greater = (face & 1) == 0;
        size_t tableOffset = M * 3 * (size_t)face;
        size_t top = 0, index = 0;
        stack[top++] = 0;
        while (top) {
            size_t k = stack[--top];
            bool isLeaf = (p.sizeIndices[k] & kLeafMask) != 0;
            int nodeSize = isLeaf ? 1 : p.sizeIndices[k];
            p.hitTable[tableOffset + index * 3 + 0] = (int32_t)k;
            p.hitTable[tableOffset + index * 3 + 1] = isLeaf ? (p.sizeIndices[k] ^ kLeafMask) : -1;
            p.hitTable[tableOffset + index * 3 + 2] = (int32_t)(index + nodeSize);
            index++;
            if (isLeaf) continue;
            int lSize = p.sizeIndices[k + 1];
            if (lSize & kLeafMask) lSize = 1;
            size_t lch = k + 1, rch = k + 1 + (size_t)lSize;
            float cl = p.bounds[lch].centroid()[axis];
            float cr = p.bounds[rch].centroid()[axis];
            bool first = greater ? (cl > cr) : (cl < cr);
            if (!first) std::swap(lch, rch);
            stack[top++] = rch;
            stack[top++] = lch;
        }
    }
}

// ---------------------------------------------------------------------------
// Traversal (src/shader/intersection.glsl)
// ---------------------------------------------------------------------------

struct Ray {
    vec3 ori, dir;
};

struct Scene {
    const float* bounds;   // M*6
    const int32_t* hit;    // 6*M*3
    int64_t M;
    const float* verts;
    const uint32_t* idx;
};

// maxExtent / cubemapFace (src/shader/math.glsl:112-131).
inline int maxExtent(vec3 v) {
    if (v.x > v.y) return v.x > v.z ? 0 : 2;
    return v.y > v.z ? 1 : 2;
}
inline int cubemapFace(vec3 dir) {
    int m = maxExtent(vabs(dir));
    if (m == 0) return dir.x > 0.0f ? 0 : 1;
    if (m == 1) return dir.y > 0.0f ? 2 : 3;
    return dir.z > 0.0f ? 4 : 5;
}

// boxHit (intersection.glsl:226-329).
bool boxHit(const Scene& s, int id, const Ray& ray, float& tMin) {
    float tMax;
    vec3 pMin(s.bounds[6 * id + 0], s.bounds[6 * id + 1], s.bounds[6 * id + 2]);
    vec3 pMax(s.bounds[6 * id + 3], s.bounds[6 * id + 4], s.bounds[6 * id + 5]);
    const float eps = 1e-6f;
    vec3 o = ray.ori, d = ray.dir;
    if (std::fabs(d.x) > 1.0f - eps) {
        if (o.y > pMin.y && o.y < pMax.y && o.z > pMin.z && o.z < pMax.z) {
            float inv = 1.0f / d.x;
            float ta = (pMin.x - o.x) * inv, tb = (pMax.x - o.x) * inv;
            tMin = fmin_(ta, tb);
            tMax = fmax_(ta, tb);
            return tMax >= 0.0f && tMax >= tMin;
        }
        return false;
    }
    if (std::fabs(d.y) > 1.0f - eps) {
        if (o.x > pMin.x && o.x < pMax.x && o.z > pMin.z && o.z < pMax.z) {
            float inv = 1.0f / d.y;
            float ta = (pMin.y - o.y) * inv, tb = (pMax.y - o.y) * inv;
            tMin = fmin_(ta, tb);
            tMax = fmax_(ta, tb);
            return tMax >= 0.0f && tMax >= tMin;
        }
        return false;
    }
    if (std::fabs(d.z) > 1.0f - eps) {
        if (o.x > pMin.x && o.x < pMax.x && o.y > pMin.y && o.y < pMax.y) {
            float inv = 1.0f / d.z;
            float ta = (pMin.z - o.z) * inv, tb = (pMax.z - o.z) * inv;
            tMin = fmin_(ta, tb);
            tMax = fmax_(ta, tb);
            return tMax >= 0.0f && tMax >= tMin;
        }
        return false;
    }
    vec3 dInv = 1.0f / d;
    vec3 vta = (pMin - o) * dInv;
    vec3 vtb = (pMax - o) * dInv;
    vec3 vtMin = vmin(vta, vtb);
    vec3 vtMax = vmax(vta, vtb);
    vec3 dt = vtMax - vtMin;
    float tyz = vtMax.z - vtMin.y;
    float tzx = vtMax.x - vtMin.z;
    float txy = vtMax.y - vtMin.x;
    if (std::fabs(d.x) < eps) {
        if (dt.y + dt.z > tyz) {
            tMin = fmax_(vtMin.y, vtMin.z);
            tMax = fmin_(vtMax.y, vtMax.z);
            return tMax >= 0.0f && tMax >= tMin;
        }
    }
    if (std::fabs(d.y) < eps) {
        if (dt.z + dt.x > tzx) {
            tMin = fmax_(vtMin.z, vtMin.x);
            tMax = fmin_(vtMax.z, vtMax.x);
            return tMax >= 0.0f && tMax >= tMin;
        }
    }
    if (std::fabs(d.z) < eps) {
        if (dt.x + dt.y > txy) {
            tMin = fmax_(vtMin.x, vtMin.y);
            tMax = fmin_(vtMax.x, vtMax.y);
            return tMax >= 0.0f && tMax >= tMin;
        }
    }
    if (dt.y + dt.z > tyz && dt.z + dt.x > tzx && dt.x + dt.y > txy) {
        tMin = fmax_(fmax_(vtMin.x, vtMin.y), vtMin.z);
        tMax = fmin_(fmin_(vtMax.x, vtMax.y), vtMax.z);
        return tMax >= 0.0f && tMax >= tMin;
    }
    return false;
}

// intersectTriangle (intersection.glsl:63-121).
bool intersectTriangle(const Scene& s, int id, const Ray& ray, float& dist) {
    auto V = [&](uint32_t k) { return vec3(s.verts[3 * k], s.verts[3 * k + 1], s.verts[3 * k + 2]); };
    vec3 a = V(s.idx[3 * id]), b = V(s.idx[3 * id + 1]), c = V(s.idx[3 * id + 2]);
    const float eps = 1e-6f;
    vec3 ab = b - a, ac = c - a;
    vec3 o = ray.ori, d = ray.dir;
    vec3 p = cross(d, ac);
    float det = dot(ab, p);
    if (std::fabs(det) < eps) return false;
    vec3 ao = o - a;
    if (det < 0.0f) {
        ao = -ao;
        det = -det;
    }
    float u = dot(ao, p);
    if (u < 0.0f || u > det) return false;
    vec3 q = cross(ao, ab);
    float v = dot(d, q);
    if (v < 0.0f || u + v > det) return false;
    float t = dot(ac, q) / det;
    dist = t;
    return t > 0.0f;
}

// bvhHit (intersection.glsl:395-427) and bvhTest (:367-393) in one loop.
// Returns the closest primitive (or for any-hit, 1/0), counting entry visits
// and triangle tests.
int traverse(const Scene& s, const Ray& ray, float& dist, bool anyHit, int32_t& visits, int32_t& tests) {
    int closest = -1;
    visits = tests = 0;
    if (s.M == 0) return anyHit ? 0 : -1;
    int64_t tableOffset = (int64_t)cubemapFace(-ray.dir) * s.M;
    int64_t k = 0;
    while (k != s.M) {
        const int32_t* e = s.hit + 3 * (tableOffset + k);
        int nodeIndex = e[0], primIndex = e[1];
        float boxDist;
        visits++;
        bool bHit = boxHit(s, nodeIndex, ray, boxDist);
        if (!bHit || boxDist > dist) {
            k = e[2];
            continue;
        }
        if (primIndex >= 0) {
            float t;
            tests++;
            bool h = intersectTriangle(s, primIndex, ray, t);
            if (h && t < dist) {
                if (anyHit) return 1;
                dist = t;
                closest = primIndex;
            }
        }
        k++;
    }
    return anyHit ? 0 : closest;
}

template <class F>
void parallelFor(int64_t n, int nthreads, F&& f) {
    if (nthreads <= 1 || n < 256) {
        for (int64_t i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<int64_t> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([&]() {
            for (;;) {
                int64_t b = next.fetch_add(64);
                if (b >= n) break;
                int64_t e = std::min(n, b + 64);
                for (int64_t i = b; i < e; i++) f(i);
            }
        });
    for (auto& t : th) t.join();
}

}  // namespace

extern "C" {

// Build the PackedBVH.  bounds_out float[M*6], hit_out int32[6*M*3],
// size_out int32[M] (sizeIndices, may be NULL).  Returns M, or -1 on bad input.
int64_t orc_bvh_build(const float* verts, int64_t nverts, const uint32_t* idx, int64_t ntri,
                      float* bounds_out, int32_t* hit_out, int32_t* size_out) {
    if (ntri <= 0) return 0;
    for (int64_t i = 0; i < 3 * ntri; i++)
        if ((int64_t)idx[i] >= nverts) return -1;
    Packed p;
    quickBuild(verts, idx, ntri, p);
    buildHitTable(p);
    int64_t M = (int64_t)p.bounds.size();
    for (int64_t i = 0; i < M; i++) {
        const AABB& b = p.bounds[(size_t)i];
        float* o = bounds_out + 6 * i;
        o[0] = b.pMin.x; o[1] = b.pMin.y; o[2] = b.pMin.z;
        o[3] = b.pMax.x; o[4] = b.pMax.y; o[5] = b.pMax.z;
        if (size_out) size_out[i] = p.sizeIndices[(size_t)i];
    }
    std::memcpy(hit_out, p.hitTable.data(), sizeof(int32_t) * (size_t)M * 18);
    return M;
}

// Closest-hit (any_hit = 0) or any-hit (any_hit = 1) traversal of n rays over
// a PackedBVH in the reference layout.  hit_id: closest prim (-1) or occluded
// flag; hit_t: closest distance (1e8 on miss; unused for any-hit, may be NULL).
void orc_trace(const float* bounds, const int32_t* hit, int64_t M, const float* verts,
               const uint32_t* idx, const float* origins, const float* dirs, const float* tmax,
               int64_t n, int32_t any_hit, int32_t* hit_id, float* hit_t, int32_t* visits,
               int32_t* tests, int32_t nthreads) {
    Scene s{bounds, hit, M, verts, idx};
    parallelFor(n, nthreads, [&](int64_t i) {
        Ray r;
        r.ori = vec3(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]);
        r.dir = vec3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
        float dist = any_hit ? tmax[i] : 1e8f;
        int32_t v, t;
        int res = traverse(s, r, dist, any_hit != 0, v, t);
        hit_id[i] = res;
        if (hit_t) hit_t[i] = dist;
        if (visits) visits[i] = v;
        if (tests) tests[i] = t;
    });
}

}  // extern "C"
