// bvh_build_gpu.cu — MTBVH construction on the GPU.
//
// Produces the tree of BVH::quickBuild and the six threaded tables of
// BVH::buildHitTable (src/accelerator/BVH.cpp:217-296, :298-345) bit for bit,
// i.e. exactly what the host builder (bvh_build.cpp) produces:
//   * per node: 16-bucket binned SAH on the centroid extent along its largest
//     axis, float32 costs evaluated in the reference's order;
//   * partition<16> order (BVH.cpp:97-114): primitives of the left buckets keep
//     their order, those of the right buckets are stored in reverse order; an
//     empty right side takes the last primitive;
//   * node bounds equal the host's bucket-ordered fold, including which of
//     -0.0 / +0.0 a zero bound carries (the first zero in (bucket, position)
//     order, since glm's min/max keep the earlier operand on ties);
//   * node k's entry in face f's table is written when k is built: its index
//     is known top-down (first child at pos+1, second at pos+1+size(first),
//     child order by the centroid of the child boxes).
//
// Schedule (GB300-first):
//   level kernels   nodes with >= `small` primitives, all nodes of one tree
//                   level at once, split into tiles of 2048 primitives:
//                   bin (shared-memory histograms -> global atomics), split
//                   (one CTA per node: SAH, node record, tile offsets),
//                   scatter (stable block-wide partition into the other work
//                   buffer), finalize (one warp per node: child records);
//   subtree kernel  every node below `small` primitives: one warp builds the
//                   whole subtree depth-first (smaller child first, larger
//                   pushed), bins in shared memory, partitions with ballots.
// Primitive records (32 B: box and triangle id) ping-pong between two work
// buffers; a node's range lives in the buffer of its depth parity.
#include <algorithm>
#include <cstring>

#include "accel.h"
#include "zgl_internal.h"

namespace zgl {
namespace {

constexpr int kBuckets = 16;
constexpr int kTile = 2048;            // primitives per tile of the level kernels
constexpr int kLevelBlock = 256;       // threads of the level kernels
constexpr int kItems = kTile / kLevelBlock;
constexpr int kSubtreeBlock = 256;     // 8 warps, one subtree each
constexpr int kStack = 16;             // > log2(max small threshold) + 1
constexpr int kDefaultSmall = 512;
constexpr int kMaxSmall = 4096;

enum : uint32_t { kErrIndex = 1u, kErrVertex = 2u, kErrSplit = 4u, kErrStack = 8u };

struct __align__(16) PrimRec {
    float4 a;  // lo.x lo.y lo.z hi.x
    float4 b;  // hi.y hi.z id(bits) 0
};

// A node under construction: its primitives are rec[buf][l..r].
struct Seg {
    int32_t l, r;
    int32_t offset;  // node index, DFS pre-order
    int32_t dim;     // largest axis of the centroid extent
    float ext[6];    // centroid extent lo.xyz hi.xyz (default box 1e8 / -1e8)
    int32_t pos[6];  // entry index in each face's threaded table
    int32_t buf;
    int32_t pad;
};

struct Tile {
    int32_t seg;
    int32_t start;
};

// Per big node of one level: bins, first-zero keys, split, child boxes.
struct SegAcc {
    uint32_t cnt[kBuckets];
    uint32_t lo[kBuckets][3];
    uint32_t hi[kBuckets][3];
    unsigned long long zlo[3], zhi[3];
    uint32_t child[2][12];  // per child: centroid lo3 hi3, box lo3 hi3 (ordered keys)
    int32_t splitb, nleft;
};

struct Counters {
    uint32_t nbig, ntiles, nsmall, err;
    uint32_t next_small;  // work counter of the subtree kernel
    uint32_t pad[3];
};

struct Out {
    float4* nodes;     // [6][M][2]
    float* bounds;     // [M][6]
    int32_t* hit;      // [6][M][3]
    int64_t M;
};

// glm's host min/max: keep x unless y is strictly smaller / larger.
__device__ __forceinline__ float hmin(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float hmax(float x, float y) { return (x < y) ? y : x; }

// Order-preserving key of a (non-NaN) float; -0.0 and +0.0 share the key of +0.
__device__ __forceinline__ uint32_t fkey(float x) {
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7fffffffu) == 0u) u = 0u;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float funkey(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__device__ __forceinline__ int lane_id() {
    int l;
    asm("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}

__device__ __forceinline__ void rec_box(const PrimRec& p, float lo[3], float hi[3]) {
    lo[0] = p.a.x; lo[1] = p.a.y; lo[2] = p.a.z;
    hi[0] = p.a.w; hi[1] = p.b.x; hi[2] = p.b.y;
}
__device__ __forceinline__ int32_t rec_id(const PrimRec& p) { return __float_as_int(p.b.z); }

__device__ __forceinline__ float rec_centroid(const PrimRec& p, int dim) {
    float lo = dim == 0 ? p.a.x : (dim == 1 ? p.a.y : p.a.z);
    float hi = dim == 0 ? p.a.w : (dim == 1 ? p.b.x : p.b.y);
    return (lo + hi) * 0.5f;
}

// bucket of a centroid (BVH.cpp:74-77): truncating, saturating conversion,
// NaN (zero-width extent) -> 0, clamped to [0, 15]
__device__ __forceinline__ int bucket_of(float c, float mn, float mx) {
    float f = 16.0f * (c - mn) / (mx - mn);
    int b;
    if (f != f) b = 0;
    else if (f >= 2147483648.0f) b = 0x7fffffff;
    else if (f <= -2147483648.0f) b = (int)0x80000000;
    else b = (int)f;
    return max(min(b, kBuckets - 1), 0);
}

__device__ __forceinline__ int max_extent(const float e[6]) {
    float x = e[3] - e[0], y = e[4] - e[1], z = e[5] - e[2];
    if (x > y) return x > z ? 0 : 2;
    return y > z ? 1 : 2;
}

__device__ __forceinline__ float box_area(const float lo[3], const float hi[3]) {
    float x = hi[0] - lo[0], y = hi[1] - lo[1], z = hi[2] - lo[2];
    return 2.0f * (x * y + y * z + z * x);
}

// Writes node `offset` (bounds lo/hi, prim or -1, subtree size) into face
// f's table at index pos; lanes f = 0..5 of the caller each write one face.
__device__ __forceinline__ void write_entry(const Out& o, int f, int32_t pos, int32_t offset, int32_t prim,
                                            int32_t size, const float lo[3], const float hi[3]) {
    int64_t e = (int64_t)f * o.M + pos;
    o.nodes[2 * e + 0] = make_float4(lo[0], lo[1], lo[2], __int_as_float(prim));
    o.nodes[2 * e + 1] = make_float4(hi[0], hi[1], hi[2], __int_as_float(pos + size));
    o.hit[3 * e + 0] = offset;
    o.hit[3 * e + 1] = prim;
    o.hit[3 * e + 2] = pos + size;
    if (f == 0) {
        float* b = o.bounds + 6 * (int64_t)offset;
        b[0] = lo[0]; b[1] = lo[1]; b[2] = lo[2];
        b[3] = hi[0]; b[4] = hi[1]; b[5] = hi[2];
    }
}

// Bound value with the sign of zero resolved: `key` is the min/max over the
// node's primitives (default box included), `zkey` the smallest
// (bucket, position, sign) key among coordinates equal to zero.
__device__ __forceinline__ float resolve_zero(uint32_t key, unsigned long long zkey) {
    float v = funkey(key);
    if (v == 0.0f && zkey != ~0ull && (zkey & 1ull)) v = -0.0f;
    return v;
}

// Binned SAH over the 16 buckets held by lanes 0..15 of one warp (lane b:
// count, lo keys, hi keys of bucket b, default box included).  Every lane
// returns the split bucket (BVH.cpp:258-272: first strict minimum of the
// costs of splits 0..14, counts converted int -> float) and, via tot*, the
// node's bound keys; *nleft gets the count of buckets <= split.
__device__ int sah_split(uint32_t cnt, const uint32_t lk[3], const uint32_t hk[3], uint32_t* nleft,
                         uint32_t totlo[3], uint32_t tothi[3]) {
    const unsigned full = 0xffffffffu;
    const int lane = lane_id();
    const int b = lane & 15;
    uint32_t pc = cnt, pl[3] = {lk[0], lk[1], lk[2]}, ph[3] = {hk[0], hk[1], hk[2]};
    uint32_t sc = cnt, sl[3] = {lk[0], lk[1], lk[2]}, sh[3] = {hk[0], hk[1], hk[2]};
#pragma unroll
    for (int d = 1; d < 16; d <<= 1) {
        uint32_t tc = __shfl_up_sync(full, pc, d, 16);
        uint32_t uc = __shfl_down_sync(full, sc, d, 16);
        uint32_t tl[3], th[3], ul[3], uh[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            tl[k] = __shfl_up_sync(full, pl[k], d, 16);
            th[k] = __shfl_up_sync(full, ph[k], d, 16);
            ul[k] = __shfl_down_sync(full, sl[k], d, 16);
            uh[k] = __shfl_down_sync(full, sh[k], d, 16);
        }
        if (b >= d) {
            pc += tc;
#pragma unroll
            for (int k = 0; k < 3; k++) { pl[k] = min(pl[k], tl[k]); ph[k] = max(ph[k], th[k]); }
        }
        if (b + d < 16) {
            sc += uc;
#pragma unroll
            for (int k = 0; k < 3; k++) { sl[k] = min(sl[k], ul[k]); sh[k] = max(sh[k], uh[k]); }
        }
    }
    // cost of splitting after bucket b: prefix box b, suffix box b+1
    uint32_t nc = __shfl_down_sync(full, sc, 1, 16);
    uint32_t nl[3], nh[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        nl[k] = __shfl_down_sync(full, sl[k], 1, 16);
        nh[k] = __shfl_down_sync(full, sh[k], 1, 16);
    }
    float plo[3], phi[3], slo[3], shi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        plo[k] = funkey(pl[k]); phi[k] = funkey(ph[k]);
        slo[k] = funkey(nl[k]); shi[k] = funkey(nh[k]);
    }
    float cost = (float)(int)pc * box_area(plo, phi) + (float)(int)nc * box_area(slo, shi);
    float best = __shfl_sync(full, cost, 0);
    int split = 0;
    for (int i = 1; i < kBuckets - 1; i++) {
        float c = __shfl_sync(full, cost, i);
        if (c < best) {
            best = c;
            split = i;
        }
    }
    *nleft = __shfl_sync(full, pc, split);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        totlo[k] = __shfl_sync(full, pl[k], 15);
        tothi[k] = __shfl_sync(full, ph[k], 15);
    }
    return split;
}

// Child records of node p split after nleft primitives; ck = per child the
// centroid extent keys (default box included) and the box keys.
__device__ void make_children(const Seg& p, int32_t nleft, const uint32_t ck[2][12], Seg& L, Seg& R) {
    const int32_t n = p.r - p.l + 1;
    L.l = p.l; L.r = p.l + nleft - 1;
    R.l = L.r + 1; R.r = p.r;
    L.offset = p.offset + 1;
    R.offset = p.offset + 2 * nleft;
    L.buf = R.buf = 1 - p.buf;
    L.pad = R.pad = 0;
    int32_t cnt[2] = {nleft, n - nleft};
    float box[2][6];
    Seg* ch[2] = {&L, &R};
#pragma unroll
    for (int c = 0; c < 2; c++) {
#pragma unroll
        for (int k = 0; k < 6; k++) ch[c]->ext[k] = funkey(ck[c][k]);
        ch[c]->dim = max_extent(ch[c]->ext);
#pragma unroll
        for (int k = 0; k < 6; k++) box[c][k] = funkey(ck[c][6 + k]);
        if (cnt[c] >= 3) {  // stored bounds of such a node include the default box
#pragma unroll
            for (int k = 0; k < 3; k++) {
                box[c][k] = hmin(1e8f, box[c][k]);
                box[c][3 + k] = hmax(-1e8f, box[c][3 + k]);
            }
        }
    }
    const int32_t sL = 2 * cnt[0] - 1, sR = 2 * cnt[1] - 1;
#pragma unroll
    for (int f = 0; f < 6; f++) {
        int axis = f >> 1;
        bool greater = (f & 1) == 0;
        float cl = (box[0][axis] + box[0][3 + axis]) * 0.5f;
        float cr = (box[1][axis] + box[1][3 + axis]) * 0.5f;
        bool leftFirst = greater ? (cl > cr) : (cl < cr);
        L.pos[f] = p.pos[f] + 1 + (leftFirst ? 0 : sR);
        R.pos[f] = p.pos[f] + 1 + (leftFirst ? sL : 0);
    }
}

// ---------------------------------------------------------------------------
// set-up: primitive records, packed triangles, root centroid extent, checks
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) setup_kernel(const float* __restrict__ v, int64_t nv,
                                                    const uint32_t* __restrict__ idx, int64_t ntri,
                                                    PrimRec* __restrict__ rec, float4* __restrict__ tris,
                                                    uint32_t* __restrict__ rootExt, Counters* ctr) {
    uint32_t ek[6] = {fkey(1e8f), fkey(1e8f), fkey(1e8f), fkey(-1e8f), fkey(-1e8f), fkey(-1e8f)};
    uint32_t err = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntri; t += stride) {
        uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
        if (i0 >= nv || i1 >= nv || i2 >= nv) {
            err |= kErrIndex;
            continue;
        }
        float A[3], B[3], C[3], lo[3], hi[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            A[k] = v[3 * (int64_t)i0 + k];
            B[k] = v[3 * (int64_t)i1 + k];
            C[k] = v[3 * (int64_t)i2 + k];
            lo[k] = hmin(hmin(A[k], B[k]), C[k]);
            hi[k] = hmax(hmax(A[k], B[k]), C[k]);
        }
        PrimRec p;
        p.a = make_float4(lo[0], lo[1], lo[2], hi[0]);
        p.b = make_float4(hi[1], hi[2], __int_as_float((int32_t)t), 0.0f);
        rec[t] = p;
        // a, ab = b - a, ac = c - a (float32, intersection.glsl:68-69)
        tris[3 * t + 0] = make_float4(A[0], A[1], A[2], B[0] - A[0]);
        tris[3 * t + 1] = make_float4(B[1] - A[1], B[2] - A[2], C[0] - A[0], C[1] - A[1]);
        tris[3 * t + 2] = make_float4(C[2] - A[2], 0.0f, 0.0f, 0.0f);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            uint32_t c = fkey((lo[k] + hi[k]) * 0.5f);
            ek[k] = min(ek[k], c);
            ek[3 + k] = max(ek[3 + k], c);
        }
    }
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < 3 * nv; j += stride) {
        float x = v[j];
        if (!(fabsf(x) <= 1e8f)) err |= kErrVertex;  // NaN, inf or beyond the default box
    }
    const unsigned full = 0xffffffffu;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        ek[k] = __reduce_min_sync(full, ek[k]);
        ek[3 + k] = __reduce_max_sync(full, ek[3 + k]);
    }
    err = __reduce_or_sync(full, err);
    if (lane_id() == 0) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            atomicMin(&rootExt[k], ek[k]);
            atomicMax(&rootExt[3 + k], ek[3 + k]);
        }
        if (err) atomicOr(&ctr->err, err);
    }
}

// Root record; the level list when the mesh has >= `small` triangles, else
// the subtree list.
__global__ void root_kernel(const uint32_t* rootExt, int32_t ntri, int32_t small, Seg* big, Tile* tiles,
                            Seg* smallList, Counters* ctr) {
    Seg s;
    s.l = 0;
    s.r = ntri - 1;
    s.offset = 0;
    for (int k = 0; k < 6; k++) s.ext[k] = funkey(rootExt[k]);
    s.dim = max_extent(s.ext);
    for (int f = 0; f < 6; f++) s.pos[f] = 0;
    s.buf = 0;
    s.pad = 0;
    if (ntri >= small) {
        int32_t nt = (ntri + kTile - 1) / kTile;
        if (threadIdx.x == 0) {
            big[0] = s;
            ctr->nbig = 1;
            ctr->ntiles = nt;
            ctr->nsmall = 0;
        }
        for (int32_t t = threadIdx.x; t < nt; t += blockDim.x) tiles[t] = Tile{0, t * kTile};
    } else if (threadIdx.x == 0) {
        smallList[0] = s;
        ctr->nbig = 0;
        ctr->ntiles = 0;
        ctr->nsmall = 1;
    }
}

// ---------------------------------------------------------------------------
// level kernels (nodes with >= `small` primitives)
// ---------------------------------------------------------------------------

__global__ void acc_init_kernel(SegAcc* acc, int32_t nseg) {
    int32_t s = blockIdx.x;
    if (s >= nseg) return;
    SegAcc& A = acc[s];
    for (int i = threadIdx.x; i < kBuckets; i += blockDim.x) {
        A.cnt[i] = 0;
        for (int k = 0; k < 3; k++) {
            A.lo[i][k] = fkey(1e8f);
            A.hi[i][k] = fkey(-1e8f);
        }
    }
    if (threadIdx.x < 3) {
        A.zlo[threadIdx.x] = ~0ull;
        A.zhi[threadIdx.x] = ~0ull;
    }
    if (threadIdx.x < 2) {
        uint32_t* c = A.child[threadIdx.x];
        for (int k = 0; k < 3; k++) {
            c[k] = fkey(1e8f);
            c[3 + k] = fkey(-1e8f);
            c[6 + k] = 0xffffffffu;
            c[9 + k] = 0u;
        }
    }
}

__global__ void __launch_bounds__(kLevelBlock) level_bin_kernel(const Seg* __restrict__ segs,
                                                               const Tile* __restrict__ tiles,
                                                               const PrimRec* __restrict__ in,
                                                               SegAcc* acc, uint32_t* __restrict__ tileHist) {
    __shared__ uint32_t scnt[kBuckets], slo[kBuckets][3], shi[kBuckets][3];
    __shared__ unsigned long long szlo[3], szhi[3];
    const Tile tile = tiles[blockIdx.x];
    const Seg S = segs[tile.seg];
    if (threadIdx.x < kBuckets) {
        scnt[threadIdx.x] = 0;
        for (int k = 0; k < 3; k++) {
            slo[threadIdx.x][k] = fkey(1e8f);
            shi[threadIdx.x][k] = fkey(-1e8f);
        }
    }
    if (threadIdx.x < 3) {
        szlo[threadIdx.x] = ~0ull;
        szhi[threadIdx.x] = ~0ull;
    }
    __syncthreads();
    const float mn = S.ext[S.dim], mx = S.ext[3 + S.dim];
    const int32_t end = min(S.r, tile.start + kTile - 1);
    for (int32_t i = tile.start + threadIdx.x; i <= end; i += kLevelBlock) {
        PrimRec p = in[i];
        float lo[3], hi[3];
        rec_box(p, lo, hi);
        int b = bucket_of(rec_centroid(p, S.dim), mn, mx);
        atomicAdd(&scnt[b], 1u);
        unsigned long long rel = (unsigned long long)(i - S.l);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            atomicMin(&slo[b][k], fkey(lo[k]));
            atomicMax(&shi[b][k], fkey(hi[k]));
            if (lo[k] == 0.0f)
                atomicMin(&szlo[k], ((unsigned long long)b << 40) | (rel << 1) | (__float_as_uint(lo[k]) >> 31));
            if (hi[k] == 0.0f)
                atomicMin(&szhi[k], ((unsigned long long)b << 40) | (rel << 1) | (__float_as_uint(hi[k]) >> 31));
        }
    }
    __syncthreads();
    SegAcc& A = acc[tile.seg];
    if (threadIdx.x < kBuckets) {
        uint32_t c = scnt[threadIdx.x];
        tileHist[(int64_t)blockIdx.x * kBuckets + threadIdx.x] = c;
        if (c) {
            atomicAdd(&A.cnt[threadIdx.x], c);
            for (int k = 0; k < 3; k++) {
                atomicMin(&A.lo[threadIdx.x][k], slo[threadIdx.x][k]);
                atomicMax(&A.hi[threadIdx.x][k], shi[threadIdx.x][k]);
            }
        }
    } else if (threadIdx.x >= 32 && threadIdx.x < 35) {
        int k = threadIdx.x - 32;
        if (szlo[k] != ~0ull) atomicMin(&A.zlo[k], szlo[k]);
        if (szhi[k] != ~0ull) atomicMin(&A.zhi[k], szhi[k]);
    }
}

// One CTA per big node: SAH split, node record and table entries, and the
// left/right offsets of each of its tiles.
__global__ void __launch_bounds__(kLevelBlock) level_split_kernel(const Seg* __restrict__ segs, SegAcc* acc,
                                                                 const Tile* __restrict__ tiles,
                                                                 const uint32_t* __restrict__ tileHist,
                                                                 int2* __restrict__ tileOff,
                                                                 const int32_t* __restrict__ segTile0, Out o,
                                                                 Counters* ctr) {
    __shared__ int32_t sSplit, sNleft;
    __shared__ int32_t wsum[kLevelBlock / 32];
    const int32_t s = blockIdx.x;
    const Seg S = segs[s];
    SegAcc& A = acc[s];
    const int32_t n = S.r - S.l + 1;
    if (threadIdx.x < 32) {
        int b = threadIdx.x & 15;
        uint32_t lk[3], hk[3], tl[3], th[3], nleft;
        for (int k = 0; k < 3; k++) {
            lk[k] = A.lo[b][k];
            hk[k] = A.hi[b][k];
        }
        int split = sah_split(A.cnt[b], lk, hk, &nleft, tl, th);
        int32_t nl = (int32_t)nleft;
        if (nl == n) nl = n - 1;
        if (nl < 1) {  // cannot happen for coordinates inside the default box
            nl = 1;
            if (threadIdx.x == 0) atomicOr(&ctr->err, kErrSplit);
        }
        float lo[3], hi[3];
        for (int k = 0; k < 3; k++) {
            lo[k] = resolve_zero(tl[k], A.zlo[k]);
            hi[k] = resolve_zero(th[k], A.zhi[k]);
        }
        if (threadIdx.x < 6) write_entry(o, threadIdx.x, S.pos[threadIdx.x], S.offset, -1, 2 * n - 1, lo, hi);
        if (threadIdx.x == 0) {
            sSplit = split;
            sNleft = nl;
            A.splitb = split;
            A.nleft = nl;
        }
    }
    __syncthreads();
    const int split = sSplit;
    // exclusive prefix of the tiles' left counts, in tile order
    const int32_t t0 = segTile0[s];
    const int32_t nt = (n + kTile - 1) / kTile;
    int32_t running = 0;
    for (int32_t base = 0; base < nt; base += kLevelBlock) {
        int32_t t = base + threadIdx.x;
        int32_t lc = 0;
        if (t < nt) {
            const uint32_t* h = tileHist + (int64_t)(t0 + t) * kBuckets;
            for (int b = 0; b <= split; b++) lc += (int32_t)h[b];
        }
        // block exclusive scan of lc
        int32_t x = lc;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) wsum[w] = x;
        __syncthreads();
        int32_t wbase = 0, total = 0;
        for (int i = 0; i < kLevelBlock / 32; i++) {
            if (i < w) wbase += wsum[i];
            total += wsum[i];
        }
        int32_t excl = running + wbase + x - lc;
        if (t < nt) {
            int32_t startRel = tiles[t0 + t].start - S.l;
            tileOff[t0 + t] = make_int2(excl, startRel - excl);
        }
        running += total;
        __syncthreads();
    }
}

// Stable partition of one tile into the other work buffer, plus the child
// boxes and centroid extents.
__global__ void __launch_bounds__(kLevelBlock) level_scatter_kernel(const Seg* __restrict__ segs,
                                                                   SegAcc* acc, const Tile* __restrict__ tiles,
                                                                   const int2* __restrict__ tileOff,
                                                                   const PrimRec* __restrict__ in,
                                                                   PrimRec* __restrict__ out) {
    __shared__ int32_t wl[kLevelBlock / 32], wr[kLevelBlock / 32];
    __shared__ uint32_t sch[2][12];
    const Tile tile = tiles[blockIdx.x];
    const Seg S = segs[tile.seg];
    SegAcc& A = acc[tile.seg];
    const int split = A.splitb;
    const int32_t nleft = A.nleft;
    const int2 off = tileOff[blockIdx.x];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned full = 0xffffffffu, lt = (1u << lane) - 1u;
    const float mn = S.ext[S.dim], mx = S.ext[3 + S.dim];
    if (threadIdx.x < 24) {
        int c = threadIdx.x / 12, k = threadIdx.x % 12;
        sch[c][k] = k < 3 ? fkey(1e8f) : (k < 6 ? fkey(-1e8f) : (k < 9 ? 0xffffffffu : 0u));
    }
    PrimRec p[kItems];
    unsigned bl[kItems], br[kItems];
    int32_t cl = 0, cr = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        int32_t i = tile.start + w * (kItems * 32) + k * 32 + lane;
        bool valid = i <= S.r && i < tile.start + kTile;
        bool left = false;
        if (valid) {
            p[k] = in[i];
            left = bucket_of(rec_centroid(p[k], S.dim), mn, mx) <= split;
        }
        bl[k] = __ballot_sync(full, valid && left);
        br[k] = __ballot_sync(full, valid && !left);
        cl += __popc(bl[k]);
        cr += __popc(br[k]);
    }
    if (lane == 0) {
        wl[w] = cl;
        wr[w] = cr;
    }
    __syncthreads();
    int32_t lbase = off.x, rbase = off.y;
    for (int i = 0; i < w; i++) {
        lbase += wl[i];
        rbase += wr[i];
    }
    uint32_t ck[2][12];
#pragma unroll
    for (int c = 0; c < 2; c++)
#pragma unroll
        for (int k = 0; k < 12; k++) ck[c][k] = k < 3 ? 0xffffffffu : (k < 6 ? 0u : (k < 9 ? 0xffffffffu : 0u));
    const int32_t lastLeft = S.l + nleft - 1;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        bool isl = (bl[k] >> lane) & 1u, isr = (br[k] >> lane) & 1u;
        if (isl || isr) {
            int32_t dest = isl ? S.l + lbase + __popc(bl[k] & lt) : S.r - (rbase + __popc(br[k] & lt));
            out[dest] = p[k];
            int c = dest <= lastLeft ? 0 : 1;
            float lo[3], hi[3];
            rec_box(p[k], lo, hi);
#pragma unroll
            for (int a = 0; a < 3; a++) {
                uint32_t cc = fkey((lo[a] + hi[a]) * 0.5f);
                uint32_t kl = fkey(lo[a]), kh = fkey(hi[a]);
                if (c == 0) {
                    ck[0][a] = min(ck[0][a], cc); ck[0][3 + a] = max(ck[0][3 + a], cc);
                    ck[0][6 + a] = min(ck[0][6 + a], kl); ck[0][9 + a] = max(ck[0][9 + a], kh);
                } else {
                    ck[1][a] = min(ck[1][a], cc); ck[1][3 + a] = max(ck[1][3 + a], cc);
                    ck[1][6 + a] = min(ck[1][6 + a], kl); ck[1][9 + a] = max(ck[1][9 + a], kh);
                }
            }
        }
        lbase += __popc(bl[k]);
        rbase += __popc(br[k]);
    }
#pragma unroll
    for (int c = 0; c < 2; c++)
#pragma unroll
        for (int k = 0; k < 12; k++) {
            bool isMin = k < 3 || (k >= 6 && k < 9);
            ck[c][k] = isMin ? __reduce_min_sync(full, ck[c][k]) : __reduce_max_sync(full, ck[c][k]);
        }
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < 2; c++)
#pragma unroll
            for (int k = 0; k < 12; k++) {
                bool isMin = k < 3 || (k >= 6 && k < 9);
                if (isMin) atomicMin(&sch[c][k], ck[c][k]);
                else atomicMax(&sch[c][k], ck[c][k]);
            }
    }
    __syncthreads();
    if (threadIdx.x < 24) {
        int c = threadIdx.x / 12, k = threadIdx.x % 12;
        bool isMin = k < 3 || (k >= 6 && k < 9);
        if (isMin) atomicMin(&A.child[c][k], sch[c][k]);
        else atomicMax(&A.child[c][k], sch[c][k]);
    }
}

// One warp per big node: child records to the next level or the subtree list.
__global__ void level_finalize_kernel(const Seg* __restrict__ segs, const SegAcc* __restrict__ acc,
                                      int32_t nseg, int32_t small, Seg* __restrict__ nextBig,
                                      Tile* __restrict__ nextTiles, int32_t* __restrict__ nextTile0,
                                      Seg* __restrict__ smallList, Counters* ctr) {
    const int32_t s = blockIdx.x;
    if (s >= nseg) return;
    const Seg S = segs[s];
    const SegAcc& A = acc[s];
    uint32_t ck[2][12];
    for (int c = 0; c < 2; c++)
        for (int k = 0; k < 12; k++) ck[c][k] = A.child[c][k];
    Seg ch[2];
    make_children(S, A.nleft, ck, ch[0], ch[1]);
    for (int c = 0; c < 2; c++) {
        const Seg& C = ch[c];
        int32_t n = C.r - C.l + 1;
        if (n >= small) {
            int32_t nt = (n + kTile - 1) / kTile;
            int32_t slot = 0, t0 = 0;
            if (threadIdx.x == 0) {
                slot = (int32_t)atomicAdd(&ctr->nbig, 1u);
                t0 = (int32_t)atomicAdd(&ctr->ntiles, (uint32_t)nt);
                nextBig[slot] = C;
                nextTile0[slot] = t0;
            }
            slot = __shfl_sync(0xffffffffu, slot, 0);
            t0 = __shfl_sync(0xffffffffu, t0, 0);
            for (int32_t t = threadIdx.x; t < nt; t += 32) nextTiles[t0 + t] = Tile{slot, C.l + t * kTile};
        } else if (threadIdx.x == 0) {
            smallList[atomicAdd(&ctr->nsmall, 1u)] = C;
        }
    }
}

// ---------------------------------------------------------------------------
// subtree kernel (nodes with < `small` primitives): one warp per subtree
// ---------------------------------------------------------------------------

struct WarpScratch {
    uint32_t cnt[kBuckets];
    uint32_t lo[kBuckets][3];
    uint32_t hi[kBuckets][3];
    uint32_t zlo[3], zhi[3];
    Seg stack[kStack];
};

// Leaf (one primitive) or a node of two leaves, written by lanes 0..5.
__device__ void emit_tiny(const Seg& S, PrimRec* const bufs[2], const Out& o) {
    const int lane = lane_id();
    const PrimRec* in = bufs[S.buf];
    if (S.l == S.r) {
        if (lane < 6) {
            PrimRec p = in[S.l];
            float lo[3], hi[3];
            rec_box(p, lo, hi);
            write_entry(o, lane, S.pos[lane], S.offset, rec_id(p), 1, lo, hi);
        }
        return;
    }
    if (lane >= 6) return;
    PrimRec A = in[S.l], B = in[S.l + 1];
    float alo[3], ahi[3], blo[3], bhi[3], lo[3], hi[3];
    rec_box(A, alo, ahi);
    rec_box(B, blo, bhi);
    for (int k = 0; k < 3; k++) {
        lo[k] = hmin(alo[k], blo[k]);
        hi[k] = hmax(ahi[k], bhi[k]);
    }
    if (rec_centroid(A, S.dim) > rec_centroid(B, S.dim)) {  // BVH.cpp:239-242
        PrimRec t = A; A = B; B = t;
        rec_box(A, alo, ahi);
        rec_box(B, blo, bhi);
    }
    const int f = lane;
    write_entry(o, f, S.pos[f], S.offset, -1, 3, lo, hi);
    int axis = f >> 1;
    bool greater = (f & 1) == 0;
    float cl = (alo[axis] + ahi[axis]) * 0.5f, cr = (blo[axis] + bhi[axis]) * 0.5f;
    bool aFirst = greater ? (cl > cr) : (cl < cr);
    int32_t pa = S.pos[f] + (aFirst ? 1 : 2), pb = S.pos[f] + (aFirst ? 2 : 1);
    // the two leaves' bounds are written by face 0's lane, like every node's
    write_entry(o, f, pa, S.offset + 1, rec_id(A), 1, alo, ahi);
    write_entry(o, f, pb, S.offset + 2, rec_id(B), 1, blo, bhi);
}

__global__ void __launch_bounds__(kSubtreeBlock) subtree_kernel(const Seg* __restrict__ list, PrimRec* buf0,
                                                               PrimRec* buf1, Out o, Counters* ctr) {
    __shared__ WarpScratch scratch[kSubtreeBlock / 32];
    WarpScratch& ws = scratch[threadIdx.x >> 5];
    const int lane = lane_id();
    const unsigned full = 0xffffffffu, lt = (1u << lane) - 1u;
    PrimRec* const bufs[2] = {buf0, buf1};
    const uint32_t nsmall = ctr->nsmall;
    for (;;) {
        uint32_t item = 0;
        if (lane == 0) item = atomicAdd(&ctr->next_small, 1u);
        item = __shfl_sync(full, item, 0);
        if (item >= nsmall) return;
        Seg S = list[item];
        int sp = 0;
        for (;;) {
            const int32_t n = S.r - S.l + 1;
            if (n <= 2) {
                emit_tiny(S, bufs, o);
                __syncwarp();
                if (sp == 0) break;
                S = ws.stack[--sp];
                __syncwarp();
                continue;
            }
            const PrimRec* in = bufs[S.buf];
            PrimRec* out = bufs[1 - S.buf];
            const float mn = S.ext[S.dim], mx = S.ext[3 + S.dim];
            // bins
            if (lane < kBuckets) {
                ws.cnt[lane] = 0;
                for (int k = 0; k < 3; k++) {
                    ws.lo[lane][k] = fkey(1e8f);
                    ws.hi[lane][k] = fkey(-1e8f);
                }
            } else if (lane < kBuckets + 3) {
                ws.zlo[lane - kBuckets] = 0xffffffffu;
                ws.zhi[lane - kBuckets] = 0xffffffffu;
            }
            __syncwarp();
            for (int32_t i = S.l + lane; i <= S.r; i += 32) {
                PrimRec p = in[i];
                float lo[3], hi[3];
                rec_box(p, lo, hi);
                int b = bucket_of(rec_centroid(p, S.dim), mn, mx);
                atomicAdd(&ws.cnt[b], 1u);
                uint32_t rel = (uint32_t)(i - S.l);
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    atomicMin(&ws.lo[b][k], fkey(lo[k]));
                    atomicMax(&ws.hi[b][k], fkey(hi[k]));
                    if (lo[k] == 0.0f) atomicMin(&ws.zlo[k], ((uint32_t)b << 13) | (rel << 1) | (__float_as_uint(lo[k]) >> 31));
                    if (hi[k] == 0.0f) atomicMin(&ws.zhi[k], ((uint32_t)b << 13) | (rel << 1) | (__float_as_uint(hi[k]) >> 31));
                }
            }
            __syncwarp();
            uint32_t lk[3], hk[3], tl[3], th[3], nleftU;
            const int bb = lane & 15;
            for (int k = 0; k < 3; k++) {
                lk[k] = ws.lo[bb][k];
                hk[k] = ws.hi[bb][k];
            }
            const int split = sah_split(ws.cnt[bb], lk, hk, &nleftU, tl, th);
            int32_t nleft = (int32_t)nleftU;
            if (nleft == n) nleft = n - 1;
            if (nleft < 1) {
                nleft = 1;
                if (lane == 0) atomicOr(&ctr->err, kErrSplit);
            }
            if (lane < 6) {
                float lo[3], hi[3];
                for (int k = 0; k < 3; k++) {
                    uint32_t zl = ws.zlo[k], zh = ws.zhi[k];
                    lo[k] = resolve_zero(tl[k], zl == 0xffffffffu ? ~0ull : (unsigned long long)zl);
                    hi[k] = resolve_zero(th[k], zh == 0xffffffffu ? ~0ull : (unsigned long long)zh);
                }
                write_entry(o, lane, S.pos[lane], S.offset, -1, 2 * n - 1, lo, hi);
            }
            // stable partition: left buckets in order, right buckets reversed
            uint32_t ck[2][12];
#pragma unroll
            for (int c = 0; c < 2; c++)
#pragma unroll
                for (int k = 0; k < 12; k++)
                    ck[c][k] = k < 3 ? fkey(1e8f) : (k < 6 ? fkey(-1e8f) : (k < 9 ? 0xffffffffu : 0u));
            const int32_t lastLeft = S.l + nleft - 1;
            int32_t lb = 0, rb = 0;
            for (int32_t base = S.l; base <= S.r; base += 32) {
                int32_t i = base + lane;
                bool valid = i <= S.r;
                PrimRec p;
                bool left = false;
                if (valid) {
                    p = in[i];
                    left = bucket_of(rec_centroid(p, S.dim), mn, mx) <= split;
                }
                unsigned bl = __ballot_sync(full, valid && left), br = __ballot_sync(full, valid && !left);
                if (valid) {
                    int32_t dest = left ? S.l + lb + __popc(bl & lt) : S.r - (rb + __popc(br & lt));
                    out[dest] = p;
                    int c = dest <= lastLeft ? 0 : 1;
                    float lo[3], hi[3];
                    rec_box(p, lo, hi);
#pragma unroll
                    for (int a = 0; a < 3; a++) {
                        uint32_t cc = fkey((lo[a] + hi[a]) * 0.5f), kl = fkey(lo[a]), kh = fkey(hi[a]);
                        if (c == 0) {
                            ck[0][a] = min(ck[0][a], cc); ck[0][3 + a] = max(ck[0][3 + a], cc);
                            ck[0][6 + a] = min(ck[0][6 + a], kl); ck[0][9 + a] = max(ck[0][9 + a], kh);
                        } else {
                            ck[1][a] = min(ck[1][a], cc); ck[1][3 + a] = max(ck[1][3 + a], cc);
                            ck[1][6 + a] = min(ck[1][6 + a], kl); ck[1][9 + a] = max(ck[1][9 + a], kh);
                        }
                    }
                }
                lb += __popc(bl);
                rb += __popc(br);
            }
#pragma unroll
            for (int c = 0; c < 2; c++)
#pragma unroll
                for (int k = 0; k < 12; k++) {
                    bool isMin = k < 3 || (k >= 6 && k < 9);
                    ck[c][k] = isMin ? __reduce_min_sync(full, ck[c][k]) : __reduce_max_sync(full, ck[c][k]);
                }
            Seg L, R;
            make_children(S, nleft, ck, L, R);
            // continue with the smaller child, push the larger one
            const bool leftSmaller = (L.r - L.l) <= (R.r - R.l);
            if (sp < kStack) {
                if (lane == 0) ws.stack[sp] = leftSmaller ? R : L;
                sp++;
            } else if (lane == 0) {
                atomicOr(&ctr->err, kErrStack);
            }
            S = leftSmaller ? L : R;
            __syncwarp();
        }
    }
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    void alloc(size_t n) { ZGL_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T))); }
};

}  // namespace

int gpu_build_default_small() { return kDefaultSmall; }
int gpu_build_max_small() { return kMaxSmall; }

// Builds the MTBVH of `ntri` triangles on the current device (vertices and
// indices are device-accessible).  Fills nodes (float4[6][M][2]), tris
// (float4[ntri][3]), bounds (float[M][6]) and hit (int32[6][M][3]).
// Synchronous on `s`; throws zgl::Error.
void build_bvh_device(const float* v, int64_t nv, const uint32_t* idx, int64_t ntri, int small,
                      float4* nodes, float4* tris, float* bounds, int32_t* hit, cudaStream_t s) {
    if (ntri <= 0) return;
    if (small <= 0) small = kDefaultSmall;
    small = std::max(8, std::min(small, kMaxSmall));
    const int64_t M = 2 * ntri - 1;
    Out o{nodes, bounds, hit, M};

    DevBuf<PrimRec> rec0, rec1;
    DevBuf<Counters> ctr;
    DevBuf<uint32_t> rootExt;
    rec0.alloc(ntri);
    rec1.alloc(ntri);
    ctr.alloc(1);
    rootExt.alloc(6);
    const int64_t maxBig = ntri / small + 2;
    const int64_t maxTiles = (ntri + kTile - 1) / kTile + maxBig;
    DevBuf<Seg> big[2], smallList;
    DevBuf<Tile> tiles[2];
    DevBuf<int32_t> tile0[2];
    DevBuf<SegAcc> acc;
    DevBuf<uint32_t> tileHist;
    DevBuf<int2> tileOff;
    for (int i = 0; i < 2; i++) {
        big[i].alloc(maxBig);
        tiles[i].alloc(maxTiles);
        tile0[i].alloc(maxBig);
    }
    smallList.alloc(ntri + 1);
    acc.alloc(maxBig);
    tileHist.alloc(maxTiles * kBuckets);
    tileOff.alloc(maxTiles);

    int dev = 0, sms = 1;
    ZGL_CUDA(cudaGetDevice(&dev));
    ZGL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));

    ZGL_CUDA(cudaMemsetAsync(ctr.p, 0, sizeof(Counters), s));
    {
        uint32_t init[6];
        float lo = 1e8f, hi = -1e8f;
        uint32_t ul, uh;
        std::memcpy(&ul, &lo, 4);
        std::memcpy(&uh, &hi, 4);
        // host copy of fkey for the default box
        auto hkey = [](uint32_t u) { return (u & 0x80000000u) ? ~u : (u | 0x80000000u); };
        for (int k = 0; k < 3; k++) {
            init[k] = hkey(ul);
            init[3 + k] = hkey(uh);
        }
        ZGL_CUDA(cudaMemcpyAsync(rootExt.p, init, sizeof(init), cudaMemcpyHostToDevice, s));
    }
    int64_t work = std::max<int64_t>(ntri, 3 * nv);
    int grid = (int)std::min<int64_t>((work + 255) / 256, (int64_t)sms * 16);
    setup_kernel<<<grid, 256, 0, s>>>(v, nv, idx, ntri, rec0.p, tris, rootExt.p, ctr.p);
    ZGL_CUDA(cudaGetLastError());
    Counters h{};
    ZGL_CUDA(cudaMemcpyAsync(&h, ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    ZGL_CUDA(cudaStreamSynchronize(s));
    if (h.err & kErrIndex) fail(ZGL_ERR_INVALID_ARG, "bvh build: triangle index out of range");
    if (h.err & kErrVertex)
        fail(ZGL_ERR_INVALID_ARG, "bvh build: vertex component NaN, infinite or beyond +-1e8");

    root_kernel<<<1, 256, 0, s>>>(rootExt.p, (int32_t)ntri, small, big[0].p, tiles[0].p, smallList.p, ctr.p);
    ZGL_CUDA(cudaGetLastError());
    ZGL_CUDA(cudaMemsetAsync(tile0[0].p, 0, sizeof(int32_t), s));
    ZGL_CUDA(cudaMemcpyAsync(&h, ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    ZGL_CUDA(cudaStreamSynchronize(s));

    PrimRec* bufs[2] = {rec0.p, rec1.p};
    int cur = 0, level = 0;
    while (h.nbig > 0) {
        const int32_t nbig = (int32_t)h.nbig, ntiles = (int32_t)h.ntiles;
        const PrimRec* in = bufs[level & 1];
        PrimRec* outb = bufs[(level + 1) & 1];
        acc_init_kernel<<<nbig, 32, 0, s>>>(acc.p, nbig);
        level_bin_kernel<<<ntiles, kLevelBlock, 0, s>>>(big[cur].p, tiles[cur].p, in, acc.p, tileHist.p);
        level_split_kernel<<<nbig, kLevelBlock, 0, s>>>(big[cur].p, acc.p, tiles[cur].p, tileHist.p, tileOff.p,
                                                        tile0[cur].p, o, ctr.p);
        level_scatter_kernel<<<ntiles, kLevelBlock, 0, s>>>(big[cur].p, acc.p, tiles[cur].p, tileOff.p, in, outb);
        // next level's counters start at zero (the subtree count accumulates)
        ZGL_CUDA(cudaMemsetAsync(ctr.p, 0, 2 * sizeof(uint32_t), s));
        level_finalize_kernel<<<nbig, 32, 0, s>>>(big[cur].p, acc.p, nbig, small, big[1 - cur].p,
                                                  tiles[1 - cur].p, tile0[1 - cur].p, smallList.p, ctr.p);
        ZGL_CUDA(cudaGetLastError());
        ZGL_CUDA(cudaMemcpyAsync(&h, ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
        ZGL_CUDA(cudaStreamSynchronize(s));
        if (h.err) break;
        cur = 1 - cur;
        level++;
    }
    if (h.err & kErrSplit) fail(ZGL_ERR_STATE, "bvh build: empty split (coordinates beyond the default box)");
    if (h.nsmall > 0) {
        int warps = (int)std::min<int64_t>(h.nsmall, (int64_t)sms * 64);
        int blocks = (warps + kSubtreeBlock / 32 - 1) / (kSubtreeBlock / 32);
        subtree_kernel<<<blocks, kSubtreeBlock, 0, s>>>(smallList.p, rec0.p, rec1.p, o, ctr.p);
        ZGL_CUDA(cudaGetLastError());
    }
    ZGL_CUDA(cudaMemcpyAsync(&h, ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    ZGL_CUDA(cudaStreamSynchronize(s));
    if (h.err & kErrSplit) fail(ZGL_ERR_STATE, "bvh build: empty split (coordinates beyond the default box)");
    if (h.err & kErrStack) fail(ZGL_ERR_STATE, "bvh build: subtree stack overflow");
}

}  // namespace zgl
