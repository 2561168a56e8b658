// bvh_build.cpp — parallel host construction of the MTBVH.
//
// The tree is the one BVH::quickBuild produces (src/accelerator/BVH.cpp:217-296):
// 16-bucket SAH split on the node's centroid extent along its largest axis,
// single-triangle leaves, depth-first pre-order with the left child at
// offset+1 and the right child at offset + 2*(leftCount) .  Node arithmetic
// follows glm's host semantics (min(x,y) = y<x ? y : x) so that bounds are
// bit-identical.  Unlike the reference, independent subtrees are built
// concurrently from a shared task queue; every node is a pure function of
// its own primitive range, so the output is independent of scheduling.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <thread>

namespace zgl {
namespace {

inline float hmin(float x, float y) { return (y < x) ? y : x; }
inline float hmax(float x, float y) { return (x < y) ? y : x; }

struct Box {
    float lo[3] = {1e8f, 1e8f, 1e8f};  // AABB() default (AABB.h:13)
    float hi[3] = {-1e8f, -1e8f, -1e8f};
    void grow(const float* plo, const float* phi) {
        for (int a = 0; a < 3; a++) {
            lo[a] = hmin(lo[a], plo[a]);
            hi[a] = hmax(hi[a], phi[a]);
        }
    }
    void grow_point(const float* p) { grow(p, p); }
    static Box point(const float* p) {
        Box b;
        for (int a = 0; a < 3; a++) b.lo[a] = b.hi[a] = p[a];
        return b;
    }
    static Box join(const Box& a, const Box& b) {
        Box r;
        for (int k = 0; k < 3; k++) {
            r.lo[k] = hmin(a.lo[k], b.lo[k]);
            r.hi[k] = hmax(a.hi[k], b.hi[k]);
        }
        return r;
    }
    float area() const {
        float x = hi[0] - lo[0], y = hi[1] - lo[1], z = hi[2] - lo[2];
        return 2.0f * (x * y + y * z + z * x);
    }
    int max_extent() const {
        float x = hi[0] - lo[0], y = hi[1] - lo[1], z = hi[2] - lo[2];
        if (x > y) return x > z ? 0 : 2;
        return y > z ? 1 : 2;
    }
};

struct PrimRef {
    float lo[3], hi[3], c[3];
    int32_t index;
};

struct Task {
    int64_t offset;
    Box extent;
    int dim;
    int64_t l, r;
};

constexpr int kBuckets = 16;

inline int bucket_of(float c, float mn, float mx) {
    float f = 16.0f * (c - mn) / (mx - mn);
    // truncating, saturating conversion; NaN (zero-width extent) -> 0
    int b;
    if (f != f) b = 0;
    else if (f >= 2147483648.0f) b = INT32_MAX;
    else if (f <= -2147483648.0f) b = INT32_MIN;
    else b = (int)f;
    return std::max(std::min(b, kBuckets - 1), 0);
}

struct Builder {
    PrimRef* prims;
    float* bounds;
    int32_t* sizes;

    std::mutex mu;
    std::condition_variable cv;
    std::vector<Task> queue;
    int64_t pending = 0;
    int64_t serial_cutoff = 4096;

    void set_bounds(int64_t node, const Box& b) {
        float* o = bounds + 6 * node;
        o[0] = b.lo[0]; o[1] = b.lo[1]; o[2] = b.lo[2];
        o[3] = b.hi[0]; o[4] = b.hi[1]; o[5] = b.hi[2];
    }

    // One node of quickBuild; children go to `emit`.
    template <class Emit>
    void node(const Task& t, std::vector<PrimRef>& tmp, Emit&& emit) {
        int64_t l = t.l, r = t.r, offset = t.offset;
        int dim = t.dim;
        int64_t size = (r - l) * 2 + 1;
        sizes[offset] = (size == 1) ? (prims[l].index | kLeafMask) : (int32_t)size;
        if (l == r) {
            Box b;
            for (int a = 0; a < 3; a++) { b.lo[a] = prims[l].lo[a]; b.hi[a] = prims[l].hi[a]; }
            set_bounds(offset, b);
            return;
        }
        int64_t n = r - l + 1;
        if (n == 2) {
            Box b;
            for (int a = 0; a < 3; a++) {
                b.lo[a] = hmin(prims[l].lo[a], prims[r].lo[a]);
                b.hi[a] = hmax(prims[l].hi[a], prims[r].hi[a]);
            }
            set_bounds(offset, b);
            if (prims[l].c[dim] > prims[r].c[dim]) std::swap(prims[l], prims[r]);
            emit(Task{offset + 2, Box::point(prims[r].c), 0, r, r});
            emit(Task{offset + 1, Box::point(prims[l].c), 0, l, l});
            return;
        }
        float mn = t.extent.lo[dim], mx = t.extent.hi[dim];
        Box bbox[kBuckets];
        int64_t bcnt[kBuckets] = {0};
        for (int64_t i = l; i <= r; i++) {
            int b = bucket_of(prims[i].c[dim], mn, mx);
            bcnt[b]++;
            bbox[b].grow(prims[i].lo, prims[i].hi);
        }
        Box pbox[kBuckets], sbox[kBuckets];
        int64_t pcnt[kBuckets], scnt[kBuckets];
        pbox[0] = bbox[0]; pcnt[0] = bcnt[0];
        sbox[kBuckets - 1] = bbox[kBuckets - 1]; scnt[kBuckets - 1] = bcnt[kBuckets - 1];
        for (int i = 1; i < kBuckets; i++) {
            pbox[i] = Box::join(pbox[i - 1], bbox[i]);
            pcnt[i] = pcnt[i - 1] + bcnt[i];
            sbox[kBuckets - 1 - i] = Box::join(sbox[kBuckets - i], bbox[kBuckets - i - 1]);
            scnt[kBuckets - 1 - i] = scnt[kBuckets - i] + bcnt[kBuckets - i - 1];
        }
        set_bounds(offset, pbox[kBuckets - 1]);
        // counts enter the cost as float(int) like the reference's int*float
        int split_bucket = 0;
        float best = (float)(int)pcnt[0] * pbox[0].area() + (float)(int)scnt[1] * sbox[1].area();
        for (int i = 1; i < kBuckets - 1; i++) {
            float cost = (float)(int)pcnt[i] * pbox[i].area() + (float)(int)scnt[i + 1] * sbox[i + 1].area();
            if (cost < best) {
                best = cost;
                split_bucket = i;
            }
        }
        // partition<16> (BVH.cpp:97-114)
        tmp.assign(prims + l, prims + r + 1);
        int64_t lo = 0, hi = n;
        for (int64_t i = 0; i < n; i++) {
            int b = bucket_of(tmp[i].c[dim], mn, mx);
            if (b <= split_bucket) prims[l + lo++] = tmp[i];
            else prims[l + --hi] = tmp[i];
        }
        if (hi == n) hi--;
        int64_t split = l + hi - 1;
        Box lc, rc;
        for (int64_t i = l; i <= split; i++) lc.grow_point(prims[i].c);
        for (int64_t i = split + 1; i <= r; i++) rc.grow_point(prims[i].c);
        emit(Task{offset + 2 * (split - l) + 2, rc, rc.max_extent(), split + 1, r});
        emit(Task{offset + 1, lc, lc.max_extent(), l, split});
    }

    void subtree(const Task& root, std::vector<PrimRef>& tmp) {
        std::vector<Task> stack;
        stack.push_back(root);
        while (!stack.empty()) {
            Task t = stack.back();
            stack.pop_back();
            node(t, tmp, [&](const Task& c) { stack.push_back(c); });
        }
    }

    void push(const Task& t) {
        std::lock_guard<std::mutex> g(mu);
        queue.push_back(t);
        pending++;
        cv.notify_one();
    }

    void worker() {
        std::vector<PrimRef> tmp;
        for (;;) {
            Task t;
            {
                std::unique_lock<std::mutex> g(mu);
                cv.wait(g, [&] { return !queue.empty() || pending == 0; });
                if (queue.empty()) return;
                t = queue.back();
                queue.pop_back();
            }
            if (t.r - t.l + 1 <= serial_cutoff) subtree(t, tmp);
            else node(t, tmp, [&](const Task& c) { push(c); });
            {
                std::lock_guard<std::mutex> g(mu);
                if (--pending == 0) cv.notify_all();
            }
        }
    }
};

template <class F>
void parallel_range(int64_t n, int nthreads, F&& f) {
    if (nthreads <= 1 || n < 4096) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    int64_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        int64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        th.emplace_back([&f, b, e] { f(b, e); });
    }
    for (auto& x : th) x.join();
}

// buildHitTable (BVH.cpp:298-345) for one face.
void hit_table_face(const float* bounds, const int32_t* sizeIndices, int64_t M, int face, int32_t* table) {
    int axis = face >> 1;
    bool greater = (face & 1) == 0;
    std::vector<int64_t> stack;
    stack.reserve(64);
    stack.push_back(0);
    int64_t index = 0;
    while (!stack.empty()) {
        int64_t k = stack.back();
        stack.pop_back();
        int32_t s = sizeIndices[k];
        bool leaf = (s & kLeafMask) != 0;
        int64_t nsize = leaf ? 1 : s;
        table[index * 3 + 0] = (int32_t)k;
        table[index * 3 + 1] = leaf ? (s ^ kLeafMask) : -1;
        table[index * 3 + 2] = (int32_t)(index + nsize);
        index++;
        if (leaf) continue;
        int64_t lsize = sizeIndices[k + 1];
        if (lsize & kLeafMask) lsize = 1;
        int64_t lch = k + 1, rch = k + 1 + lsize;
        const float* bl = &bounds[6 * lch];
        const float* br = &bounds[6 * rch];
        float cl = (bl[axis] + bl[3 + axis]) * 0.5f;
        float cr = (br[axis] + br[3 + axis]) * 0.5f;
        bool first = greater ? (cl > cr) : (cl < cr);
        if (!first) std::swap(lch, rch);
        stack.push_back(rch);
        stack.push_back(lch);
    }
    (void)M;
}

}  // namespace

void build_bvh(const float* v, const uint32_t* idx, int64_t ntri, HostBVH& out, int nthreads) {
    out.ntri = ntri;
    out.M = ntri > 0 ? 2 * ntri - 1 : 0;
    out.bounds.resize((size_t)out.M * 6);
    out.sizeIndices.resize((size_t)out.M);
    out.hitTable.resize((size_t)out.M * 18);
    build_bvh_into(v, idx, ntri, out.bounds.data(), out.sizeIndices.data(), out.hitTable.data(), nthreads);
}

void build_bvh_into(const float* v, const uint32_t* idx, int64_t ntri, float* bounds, int32_t* sizeIndices,
                    int32_t* hitTable, int nthreads) {
    if (ntri <= 0) return;
    const int64_t M = 2 * ntri - 1;
    if (nthreads < 1) nthreads = 1;

    std::vector<PrimRef> prims((size_t)ntri);
    parallel_range(ntri, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            const float* a = v + 3 * (size_t)idx[3 * i];
            const float* bb = v + 3 * (size_t)idx[3 * i + 1];
            const float* c = v + 3 * (size_t)idx[3 * i + 2];
            PrimRef& p = prims[(size_t)i];
            for (int k = 0; k < 3; k++) {
                p.lo[k] = hmin(hmin(a[k], bb[k]), c[k]);
                p.hi[k] = hmax(hmax(a[k], bb[k]), c[k]);
                p.c[k] = (p.lo[k] + p.hi[k]) * 0.5f;
            }
            p.index = (int32_t)i;
        }
    });
    Box root;
    for (int64_t i = 0; i < ntri; i++) root.grow_point(prims[(size_t)i].c);

    Builder b;
    b.prims = prims.data();
    b.bounds = bounds;
    b.sizes = sizeIndices;
    b.serial_cutoff = std::max<int64_t>(1024, ntri / (16 * (int64_t)nthreads));
    b.push(Task{0, root, root.max_extent(), 0, ntri - 1});
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) th.emplace_back([&b] { b.worker(); });
    for (auto& x : th) x.join();

    std::vector<std::thread> faces;
    for (int f = 0; f < 6; f++)
        faces.emplace_back([=] { hit_table_face(bounds, sizeIndices, M, f, hitTable + (size_t)M * 3 * f); });
    for (auto& x : faces) x.join();
}

}  // namespace zgl
