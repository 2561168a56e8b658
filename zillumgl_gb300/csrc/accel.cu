// accel.cu — MTBVH upload and the closest-hit / any-hit trace kernels, plus
// the zgl_accel_* and zgl_trace_* entry points.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "accel.h"
#include "traverse.cuh"
#include "zgl_internal.h"

namespace zgl {
namespace {

constexpr int kTraceBlock = 128;

__global__ void pack_nodes_kernel(const float* __restrict__ bounds, const int32_t* __restrict__ hit,
                                  int64_t M, float4* __restrict__ nodes) {
    int64_t total = 6 * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int32_t node = hit[3 * e + 0];
        int32_t prim = hit[3 * e + 1];
        int32_t miss = hit[3 * e + 2];
        const float* b = bounds + 6 * (int64_t)node;
        nodes[2 * e + 0] = make_float4(b[0], b[1], b[2], __int_as_float(prim));
        nodes[2 * e + 1] = make_float4(b[3], b[4], b[5], __int_as_float(miss));
    }
}

__device__ __forceinline__ float3 load3(const float* p, int64_t i) {
    return make_float3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}

// Table entries a ray with a near-zero direction component traverses on its
// lane before its warp takes it over (finish_long_rays); other rays stay on
// their lanes (traverse_lane).  The thread-per-ray schedule passes no limit
// (every ray stays on its lane, the reference's schedule).
constexpr int kLaneBudget = kLongRayBudget;
constexpr int kNoBudget = 0x7fffffff;

__device__ __forceinline__ TraceRay lane_ray(const float* org, const float* dir, int64_t i, bool valid) {
    return make_trace_ray(valid ? load3(org, i) : make_float3(0.0f, 0.0f, 0.0f),
                          valid ? load3(dir, i) : make_float3(0.0f, 0.0f, 1.0f));
}

// One thread per ray; a ray still unfinished after `budget` entries is walked
// by its warp.  Lanes past n stay until their warp's long rays are done (the
// warp walks need all 32 lanes); whole warps past n leave at once.
__global__ void __launch_bounds__(kTraceBlock)
trace_closest_kernel(DeviceAccel a, const float* __restrict__ org, const float* __restrict__ dir,
                     int64_t n, int budget, int32_t* __restrict__ hit_id, float* __restrict__ hit_t) {
    const int64_t i = blockIdx.x * (int64_t)kTraceBlock + threadIdx.x;
    const bool valid = i < n;
    if (__all_sync(0xffffffffu, !valid)) return;
    const TraceRay r = lane_ray(org, dir, i, valid);
    float dist = 1e8f;
    int k = 0, closest = -1;
    const bool done = !valid || traverse_lane_m<false, false, 0>(a, r, dist, k, closest, budget);
    finish_long_rays<false>(a, r, dist, k, closest, done);
    if (valid) {
        hit_id[i] = closest;
        hit_t[i] = dist;
    }
}

__global__ void __launch_bounds__(kTraceBlock)
trace_any_kernel(DeviceAccel a, const float* __restrict__ org, const float* __restrict__ dir,
                 const float* __restrict__ tmax, int64_t n, int budget, uint8_t* __restrict__ occ) {
    const int64_t i = blockIdx.x * (int64_t)kTraceBlock + threadIdx.x;
    const bool valid = i < n;
    if (__all_sync(0xffffffffu, !valid)) return;
    const TraceRay r = lane_ray(org, dir, i, valid);
    float dist = valid ? tmax[i] : 0.0f;
    int k = 0, closest = -1;
    const bool done = !valid || traverse_lane_m<true, false, 0>(a, r, dist, k, closest, budget);
    finish_long_rays<true>(a, r, dist, k, closest, done);
    if (valid) occ[i] = (uint8_t)(closest >= 0);
}

__global__ void __launch_bounds__(kTraceBlock)
trace_count_kernel(DeviceAccel a, const float* __restrict__ org, const float* __restrict__ dir,
                   const float* __restrict__ tmax, int64_t n, int any_hit,
                   int32_t* __restrict__ visits, int32_t* __restrict__ tests) {
    int64_t i = blockIdx.x * (int64_t)kTraceBlock + threadIdx.x;
    if (i >= n) return;
    TraceRay r = make_trace_ray(load3(org, i), load3(dir, i));
    int v = 0, t = 0;
    if (any_hit) {
        float dist = tmax[i];
        traverse<true, true>(a, r, dist, v, t);
    } else {
        float dist = 1e8f;
        traverse<false, true>(a, r, dist, v, t);
    }
    visits[i] = v;
    tests[i] = t;
}

// Prefetching schedule: one thread per ray with the node loads of
// traverse_v: each lane requests both possible successors of an entry ahead
// (k + 1 and the miss link) with a 256-byte L2 prefetch hint, so that their
// latency overlaps the tests of the entry; long rays are finished by the
// warp as in the one-thread-per-ray kernels.  Measured on the GB300 (2^24
// rays per launch): before long rays went to their warp, this loop took the
// 16M-triangle incoherent launches from 93.7 / 57.8 ms to 79.1 / 48.7 ms
// (closest / any), mostly by shortening the few longest rays; with them
// finished by their warps the plain loop is faster everywhere.
template <bool ANY>
__global__ void __launch_bounds__(kTraceBlock)
trace_prefetch_kernel(DeviceAccel a, const float* __restrict__ org, const float* __restrict__ dir,
                      const float* __restrict__ tmax, int64_t n, int32_t* __restrict__ hit_id,
                      float* __restrict__ hit_t, uint8_t* __restrict__ occ) {
    const int64_t i = blockIdx.x * (int64_t)kTraceBlock + threadIdx.x;
    const bool valid = i < n;
    if (__all_sync(0xffffffffu, !valid)) return;
    const TraceRay r = lane_ray(org, dir, i, valid);
    float dist = ANY ? (valid ? tmax[i] : 0.0f) : 1e8f;
    int k = 0, closest = -1;
    const bool done = !valid || traverse_lane_m<ANY, true, 256>(a, r, dist, k, closest, kLaneBudget);
    finish_long_rays<ANY>(a, r, dist, k, closest, done);
    if (!valid) return;
    if (ANY) {
        occ[i] = (uint8_t)(closest >= 0);
    } else {
        hit_id[i] = closest;
        hit_t[i] = dist;
    }
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

// ---------------------------------------------------------------------------
// Persistent traversal: each warp keeps its lanes busy by refilling a lane
// with the next ray once its traversal ends (ray trip counts differ by two
// orders of magnitude, so one-thread-per-ray warps run at a third of their
// lanes).  Lanes run up to kSteps table steps on their own between warp-level
// checks; then idle lanes are counted with __ballot_sync/__popc and, once at
// least kRefillIdle lanes (or all) are idle, one lane takes that many ray
// indices with a single atomicAdd on the work counter and each idle lane
// takes its rank.  Every ray is still traversed by one lane in exactly the
// reference order, so results are identical to the one-thread-per-ray
// kernels.
// ---------------------------------------------------------------------------
constexpr int kPersistBlock = 128;
constexpr int kRefillIdle = 8;
constexpr int kSteps = 8;
constexpr int kChunk = 256;  // consecutive rays a warp takes from the work counter at a time
constexpr unsigned kFull = 0xffffffffu;

// One table step of ray r at entry k (bvhHit / bvhTest loop body).
template <bool ANY, int MODE>
__device__ __forceinline__ void trace_step(const DeviceAccel& a, const float4* __restrict__ base,
                                           const TraceRay& r, int& k, float& dist, int& closest) {
    const float4 lo = __ldg(base + 2 * k);
    const float4 hi = __ldg(base + 2 * k + 1);
    float tmin;
    const bool h = (MODE < 0 ? box_hit(lo, hi, r, tmin) : box_hit_m<MODE>(lo, hi, r, tmin)) && !(tmin > dist);
    const int prim = __float_as_int(lo.w);
    int next = h ? k + 1 : max(__float_as_int(hi.w), k + 1);
    if (h && prim >= 0) {
        float t;
        if (tri_hit(a.tris, prim, r, t) && t < dist) {
            dist = t;
            closest = prim;
            if (ANY) next = a.M;
        }
    }
    k = next;
}

template <bool ANY>
__global__ void __launch_bounds__(kPersistBlock)
trace_persistent_kernel(DeviceAccel a, const float* __restrict__ org, const float* __restrict__ dir,
                        const float* __restrict__ tmax, int64_t n, int32_t* __restrict__ hit_id,
                        float* __restrict__ hit_t, uint8_t* __restrict__ occ,
                        unsigned long long* __restrict__ counter) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int M = a.M;
    bool active = false;
    bool exhausted = false;  // warp-uniform
    unsigned long long next = 0, end = 0;  // the warp's current chunk of ray indices (warp-uniform)
    int64_t ray = 0;
    TraceRay r;
    const float4* __restrict__ base = a.nodes;
    float dist = 0.0f;
    int k = 0, closest = -1;
    for (;;) {
        const unsigned idle = __ballot_sync(kFull, !active);
        const int nidle = __popc(idle);
        if (nidle == 32 && exhausted) break;
        if (!exhausted && (nidle >= kRefillIdle || nidle == 32)) {
            if (next >= end) {  // take the next chunk
                unsigned long long c = 0;
                if (lane == 0) c = atomicAdd(counter, (unsigned long long)kChunk);
                next = __shfl_sync(kFull, c, 0);
                end = next + kChunk < (unsigned long long)n ? next + kChunk : (unsigned long long)n;
                if (next >= end) exhausted = true;
            }
            const unsigned long long b = next;
            next = b + nidle < end ? b + nidle : end;
            if (!active) {
                const unsigned long long idx = b + __popc(idle & lt);
                if (idx < end) {
                    ray = (int64_t)idx;
                    r = make_trace_ray(load3(org, ray), load3(dir, ray));
                    base = a.nodes + (size_t)r.face * (size_t)M * 2;
                    dist = ANY ? tmax[ray] : 1e8f;
                    k = 0;
                    closest = -1;
                    active = true;
                }
            }
            if (__ballot_sync(kFull, active) == 0u) continue;
        }
        if (active) {
            if (r.mode == 3) {
#pragma unroll 1
                for (int s = 0; s < kSteps && k < M; s++) trace_step<ANY, 3>(a, base, r, k, dist, closest);
            } else {
#pragma unroll 1
                for (int s = 0; s < kSteps && k < M; s++) trace_step<ANY, -1>(a, base, r, k, dist, closest);
            }
            if (k >= M) {
                if (ANY) {
                    occ[ray] = (uint8_t)(closest >= 0);
                } else {
                    hit_id[ray] = closest;
                    hit_t[ray] = dist;
                }
                active = false;
            }
        }
    }
}

// SMs x resident blocks of `kernel` on the current device.
int persistent_grid(const void* kernel) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPersistBlock, 0);
    if (per_sm < 1) per_sm = 1;
    return sms * per_sm;
}

}  // namespace

cudaError_t launch_pack_nodes(const float* bounds, const int32_t* hit, int64_t M, float4* nodes,
                              cudaStream_t s) {
    if (M == 0) return cudaSuccess;
    int64_t total = 6 * M;
    unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, 152 * 64);
    pack_nodes_kernel<<<grid, 256, 0, s>>>(bounds, hit, M, nodes);
    return cudaGetLastError();
}

cudaError_t launch_trace_closest(DeviceAccel a, const float* org, const float* dir, int64_t n,
                                 int32_t* hit_id, float* hit_t, int schedule, unsigned long long* counter,
                                 cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const unsigned g = grid_for(n, kTraceBlock);
    if (a.M > 0 && schedule == ZGL_TRACE_PREFETCH) {
        trace_prefetch_kernel<false><<<g, kTraceBlock, 0, s>>>(a, org, dir, nullptr, n, hit_id, hit_t, nullptr);
        return cudaGetLastError();
    }
    if (a.M == 0 || schedule != ZGL_TRACE_PERSISTENT || counter == nullptr) {
        const int budget = schedule == ZGL_TRACE_THREAD_PER_RAY ? kNoBudget : kLaneBudget;
        trace_closest_kernel<<<g, kTraceBlock, 0, s>>>(a, org, dir, n, budget, hit_id, hit_t);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    int grid = persistent_grid((const void*)trace_persistent_kernel<false>);
    int64_t need = (n + 31) / 32 * 32 / kPersistBlock + 1;
    if (need < grid) grid = (int)need;
    trace_persistent_kernel<false><<<grid, kPersistBlock, 0, s>>>(a, org, dir, nullptr, n, hit_id, hit_t, nullptr,
                                                                  counter);
    return cudaGetLastError();
}

cudaError_t launch_trace_any(DeviceAccel a, const float* org, const float* dir, const float* tmax,
                             int64_t n, uint8_t* occ, int schedule, unsigned long long* counter, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const unsigned g = grid_for(n, kTraceBlock);
    if (a.M > 0 && schedule == ZGL_TRACE_PREFETCH) {
        trace_prefetch_kernel<true><<<g, kTraceBlock, 0, s>>>(a, org, dir, tmax, n, nullptr, nullptr, occ);
        return cudaGetLastError();
    }
    if (a.M == 0 || schedule != ZGL_TRACE_PERSISTENT || counter == nullptr) {
        const int budget = schedule == ZGL_TRACE_THREAD_PER_RAY ? kNoBudget : kLaneBudget;
        trace_any_kernel<<<g, kTraceBlock, 0, s>>>(a, org, dir, tmax, n, budget, occ);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    int grid = persistent_grid((const void*)trace_persistent_kernel<true>);
    int64_t need = (n + 31) / 32 * 32 / kPersistBlock + 1;
    if (need < grid) grid = (int)need;
    trace_persistent_kernel<true><<<grid, kPersistBlock, 0, s>>>(a, org, dir, tmax, n, nullptr, nullptr, occ,
                                                                 counter);
    return cudaGetLastError();
}

cudaError_t launch_trace_count(DeviceAccel a, const float* org, const float* dir, const float* tmax,
                               int64_t n, int any_hit, int32_t* visits, int32_t* tests,
                               cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    trace_count_kernel<<<grid_for(n, kTraceBlock), kTraceBlock, 0, s>>>(a, org, dir, tmax, n, any_hit,
                                                                       visits, tests);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Pointer staging: trace calls accept host or device arrays.
// ---------------------------------------------------------------------------

bool is_device_ptr(const void* p) {
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

// Where a kernel reaches p: device and managed memory in place; page-locked
// host memory through its mapping in the device address space (the kernel
// reads and writes it over the host link, so no staging copy is needed; on
// Grace-Blackwell that link is NVLink-C2C).  nullptr for pageable host
// memory, which has to be staged.  `host` tells whether p is host memory.
void* device_address(const void* p, bool& host) {
    host = false;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        host = true;
        return nullptr;
    }
    if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) return const_cast<void*>(p);
    host = true;
    if (attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr) return attr.devicePointer;
    return nullptr;
}

// Moves the arguments of one trace call to device memory when they are
// pageable host arrays and copies outputs back.  Device arrays and mapped
// page-locked host arrays are used in place; a call with any host array
// returns after its results are in host memory.
class Staging {
public:
    Staging(const zgl_accel* a, cudaStream_t s) : a_(a), s_(s) {}

    // Registers an argument and returns its slot.
    int add(const void* p, size_t bytes, bool in, bool out) {
        Slot sl;
        sl.user = const_cast<void*>(p);
        sl.bytes = bytes;
        sl.in = in;
        sl.out = out;
        if (p != nullptr && bytes > 0) {
            bool host = false;
            sl.direct = device_address(p, host);
            sl.staged = sl.direct == nullptr;
            anyHost_ = anyHost_ || host;
        }
        if (sl.staged) {
            sl.off = offset_;
            offset_ += (bytes + 255) & ~size_t(255);
        }
        slots_.push_back(sl);
        return (int)slots_.size() - 1;
    }

    // Allocates (or reuses) the staging area and copies inputs in.
    void commit() {
        if (offset_ == 0) return;
        if (a_->stage_bytes < offset_) {
            if (a_->d_stage) ZGL_CUDA(cudaFree(a_->d_stage));
            a_->d_stage = nullptr;
            a_->stage_bytes = 0;
            ZGL_CUDA(cudaMalloc(&a_->d_stage, offset_));
            a_->stage_bytes = offset_;
        }
        for (auto& sl : slots_)
            if (sl.staged && sl.in)
                ZGL_CUDA(cudaMemcpyAsync(dev(sl), sl.user, sl.bytes, cudaMemcpyHostToDevice, s_));
    }

    void* ptr(int slot) const {
        const Slot& sl = slots_[(size_t)slot];
        return sl.staged ? dev(sl) : (sl.direct ? sl.direct : sl.user);
    }

    // Copies staged outputs back and, when any array is host memory, waits
    // until the results are there.
    void finish() {
        for (auto& sl : slots_)
            if (sl.staged && sl.out)
                ZGL_CUDA(cudaMemcpyAsync(sl.user, dev(sl), sl.bytes, cudaMemcpyDeviceToHost, s_));
        if (anyHost_) ZGL_CUDA(cudaStreamSynchronize(s_));
    }

private:
    struct Slot {
        void* user = nullptr;
        void* direct = nullptr;  // device-visible address when used in place
        size_t bytes = 0;
        bool in = false, out = false, staged = false;
        size_t off = 0;
    };
    void* dev(const Slot& sl) const { return static_cast<char*>(a_->d_stage) + sl.off; }
    const zgl_accel* a_;
    cudaStream_t s_;
    std::vector<Slot> slots_;
    size_t offset_ = 0;
    bool anyHost_ = false;
};

class DeviceGuard {
public:
    explicit DeviceGuard(int dev) {
        ZGL_CUDA(cudaGetDevice(&prev_));
        if (prev_ != dev) ZGL_CUDA(cudaSetDevice(dev));
        dev_ = dev;
    }
    ~DeviceGuard() {
        if (prev_ != dev_) cudaSetDevice(prev_);
    }

private:
    int prev_ = 0, dev_ = 0;
};

// The schedule a trace call runs (ZGL_TRACE_AUTO: one thread per ray, long
// rays finished by their warps).
int trace_schedule(const zgl_accel* a) { return a->trace_schedule; }

int host_threads() {
    unsigned n = std::thread::hardware_concurrency();
    return n == 0 ? 1 : (int)n;
}

// Builds the MTBVH on the host and uploads node records and triangles to the
// current device.  Throws zgl::Error.
zgl_accel* accel_create(const float* vertices, const uint32_t* indices, int64_t ntri) {
    auto* a = new zgl_accel();
    try {
        ZGL_CUDA(cudaGetDevice(&a->device));
        ZGL_CUDA(cudaMalloc(&a->d_counter, 256));
        a->ntri = ntri;
        build_bvh(vertices, indices, a->ntri, a->host, host_threads());
        a->M = a->host.M;
        if (a->M > 0) {
            size_t nb = sizeof(float) * a->M * 6, nh = sizeof(int32_t) * a->M * 18;
            float* d_bounds = nullptr;
            int32_t* d_hit = nullptr;
            ZGL_CUDA(cudaMalloc(&a->d_nodes, sizeof(float4) * 12 * a->M));
            ZGL_CUDA(cudaMalloc(&a->d_tris, sizeof(float4) * 3 * a->ntri));
            ZGL_CUDA(cudaMalloc(&d_bounds, nb));
            ZGL_CUDA(cudaMalloc(&d_hit, nh));
            ZGL_CUDA(cudaMemcpy(d_bounds, a->host.bounds.data(), nb, cudaMemcpyHostToDevice));
            ZGL_CUDA(cudaMemcpy(d_hit, a->host.hitTable.data(), nh, cudaMemcpyHostToDevice));
            ZGL_CUDA(launch_pack_nodes(d_bounds, d_hit, a->M, a->d_nodes, 0));
            // triangles: a, ab = b - a, ac = c - a (float32, as intersection.glsl:68-69)
            std::vector<float4> tris((size_t)a->ntri * 3);
            for (int64_t t = 0; t < a->ntri; t++) {
                const float* A = vertices + 3 * (size_t)indices[3 * t];
                const float* B = vertices + 3 * (size_t)indices[3 * t + 1];
                const float* C = vertices + 3 * (size_t)indices[3 * t + 2];
                float abx = B[0] - A[0], aby = B[1] - A[1], abz = B[2] - A[2];
                float acx = C[0] - A[0], acy = C[1] - A[1], acz = C[2] - A[2];
                tris[3 * t + 0] = make_float4(A[0], A[1], A[2], abx);
                tris[3 * t + 1] = make_float4(aby, abz, acx, acy);
                tris[3 * t + 2] = make_float4(acz, 0.0f, 0.0f, 0.0f);
            }
            ZGL_CUDA(cudaMemcpy(a->d_tris, tris.data(), sizeof(float4) * tris.size(), cudaMemcpyHostToDevice));
            ZGL_CUDA(cudaDeviceSynchronize());
            ZGL_CUDA(cudaFree(d_bounds));
            ZGL_CUDA(cudaFree(d_hit));
        }
    } catch (...) {
        accel_free(a);
        throw;
    }
    return a;
}

zgl_accel* accel_create_device(const float* vertices, int64_t nv, const uint32_t* indices, int64_t ntri,
                               int small, cudaStream_t s) {
    auto* a = new zgl_accel();
    float* d_v = nullptr;
    uint32_t* d_i = nullptr;
    try {
        ZGL_CUDA(cudaGetDevice(&a->device));
        ZGL_CUDA(cudaMalloc(&a->d_counter, 256));
        a->ntri = ntri;
        a->M = ntri > 0 ? 2 * ntri - 1 : 0;
        a->device_built = true;
        if (ntri > 0) {
            bool host = false;
            const float* v = static_cast<const float*>(device_address(vertices, host));
            const uint32_t* idx = static_cast<const uint32_t*>(device_address(indices, host));
            if (!v) {
                ZGL_CUDA(cudaMalloc(&d_v, sizeof(float) * 3 * std::max<int64_t>(nv, 1)));
                ZGL_CUDA(cudaMemcpyAsync(d_v, vertices, sizeof(float) * 3 * nv, cudaMemcpyHostToDevice, s));
                v = d_v;
            }
            if (!idx) {
                ZGL_CUDA(cudaMalloc(&d_i, sizeof(uint32_t) * 3 * ntri));
                ZGL_CUDA(cudaMemcpyAsync(d_i, indices, sizeof(uint32_t) * 3 * ntri, cudaMemcpyHostToDevice, s));
                idx = d_i;
            }
            ZGL_CUDA(cudaMalloc(&a->d_nodes, sizeof(float4) * 12 * a->M));
            ZGL_CUDA(cudaMalloc(&a->d_tris, sizeof(float4) * 3 * a->ntri));
            ZGL_CUDA(cudaMalloc(&a->d_bounds, sizeof(float) * 6 * a->M));
            ZGL_CUDA(cudaMalloc(&a->d_hit, sizeof(int32_t) * 18 * a->M));
            build_bvh_device(v, nv, idx, ntri, small, a->d_nodes, a->d_tris, a->d_bounds, a->d_hit, s);
        }
    } catch (...) {
        cudaStreamSynchronize(s);
        if (d_v) cudaFree(d_v);
        if (d_i) cudaFree(d_i);
        accel_free(a);
        throw;
    }
    if (d_v) cudaFree(d_v);
    if (d_i) cudaFree(d_i);
    return a;
}

void accel_free(zgl_accel* a) {
    if (!a) return;
    if (a->d_bounds) cudaFree(a->d_bounds);
    if (a->d_hit) cudaFree(a->d_hit);
    if (a->d_counter) cudaFree(a->d_counter);
    if (a->d_nodes) cudaFree(a->d_nodes);
    if (a->d_tris) cudaFree(a->d_tris);
    if (a->d_stage) cudaFree(a->d_stage);
    delete a;
}

}  // namespace zgl

using namespace zgl;

extern "C" {

static void validate_mesh(const char* fn, const float* vertices, size_t n_vertices, const uint32_t* indices,
                          size_t n_triangles) {
    if (n_triangles > 0 && (!vertices || !indices))
        fail(ZGL_ERR_INVALID_ARG, "%s: NULL vertex or index array", fn);
    if (n_triangles > (size_t)0x3fffffff)
        fail(ZGL_ERR_INVALID_ARG, "%s: %zu triangles exceed the 2^30 limit", fn, n_triangles);
    for (size_t i = 0; i < 3 * n_triangles; i++)
        if (indices[i] >= n_vertices)
            fail(ZGL_ERR_INVALID_ARG, "%s: index %zu = %u out of range (%zu vertices)", fn, i, indices[i],
                 n_vertices);
    // NaN, infinite and |x| > 1e8 are rejected: quickBuild's default box is
    // +-1e8 (src/accelerator/AABB.h:13) and a centroid outside it can give an
    // empty split
    for (size_t i = 0; i < 3 * n_vertices; i++)
        if (!(std::fabs(vertices[i]) <= 1e8f))
            fail(ZGL_ERR_INVALID_ARG, "%s: vertex component %zu is NaN, infinite or beyond +-1e8", fn, i);
}

zgl_status zgl_bvh_build_host(const float* vertices, size_t n_vertices, const uint32_t* indices,
                              size_t n_triangles, float* bounds, int32_t* hit_table) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_bvh_build_host");
    validate_mesh("zgl_bvh_build_host", vertices, n_vertices, indices, n_triangles);
    if (n_triangles > 0 && (!bounds || !hit_table))
        fail(ZGL_ERR_INVALID_ARG, "zgl_bvh_build_host: NULL output array");
    if (n_triangles > 0) {  // straight into the caller's arrays
        std::vector<int32_t> sizes(2 * n_triangles - 1);
        build_bvh_into(vertices, indices, (int64_t)n_triangles, bounds, sizes.data(), hit_table, host_threads());
    }
    ZGL_API_END
}

zgl_status zgl_accel_build(const float* vertices, size_t n_vertices, const uint32_t* indices,
                           size_t n_triangles, zgl_accel** out) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_accel_build");
    if (!out) fail(ZGL_ERR_INVALID_ARG, "zgl_accel_build: out is NULL");
    *out = nullptr;
    validate_mesh("zgl_accel_build", vertices, n_vertices, indices, n_triangles);
    *out = accel_create(vertices, indices, (int64_t)n_triangles);
    ZGL_API_END
}

zgl_status zgl_accel_build_device(const float* vertices, size_t n_vertices, const uint32_t* indices,
                                  size_t n_triangles, int32_t small_threshold, void* stream, zgl_accel** out) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_accel_build_device");
    if (!out) fail(ZGL_ERR_INVALID_ARG, "zgl_accel_build_device: out is NULL");
    *out = nullptr;
    if (n_triangles > 0 && (!vertices || !indices))
        fail(ZGL_ERR_INVALID_ARG, "zgl_accel_build_device: NULL vertex or index array");
    if (n_triangles > (size_t)0x3fffffff)
        fail(ZGL_ERR_INVALID_ARG, "zgl_accel_build_device: %zu triangles exceed the 2^30 limit", n_triangles);
    if (n_vertices > (size_t)0x3fffffffffffll)
        fail(ZGL_ERR_INVALID_ARG, "zgl_accel_build_device: too many vertices");
    if (small_threshold < 0 || small_threshold > gpu_build_max_small())
        fail(ZGL_ERR_INVALID_ARG, "zgl_accel_build_device: small_threshold %d outside [0, %d]", small_threshold,
             gpu_build_max_small());
    *out = accel_create_device(vertices, (int64_t)n_vertices, indices, (int64_t)n_triangles, small_threshold,
                               static_cast<cudaStream_t>(stream));
    ZGL_API_END
}

zgl_status zgl_accel_node_count(const zgl_accel* accel, size_t* out) {
    ZGL_API_BEGIN
    if (!accel || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_accel_node_count: NULL argument");
    *out = (size_t)accel->M;
    ZGL_API_END
}

zgl_status zgl_accel_export(const zgl_accel* accel, float* bounds, int32_t* hit_table) {
    ZGL_API_BEGIN
    if (!accel) fail(ZGL_ERR_INVALID_ARG, "zgl_accel_export: NULL accel");
    if (accel->M > 0 && (!bounds || !hit_table))
        fail(ZGL_ERR_INVALID_ARG, "zgl_accel_export: NULL output array");
    if (accel->M > 0 && accel->device_built) {
        ZGL_CUDA(cudaMemcpy(bounds, accel->d_bounds, sizeof(float) * accel->M * 6, cudaMemcpyDeviceToHost));
        ZGL_CUDA(cudaMemcpy(hit_table, accel->d_hit, sizeof(int32_t) * accel->M * 18, cudaMemcpyDeviceToHost));
    } else if (accel->M > 0) {
        std::memcpy(bounds, accel->host.bounds.data(), sizeof(float) * accel->M * 6);
        std::memcpy(hit_table, accel->host.hitTable.data(), sizeof(int32_t) * accel->M * 18);
    }
    ZGL_API_END
}

zgl_status zgl_accel_destroy(zgl_accel* accel) {
    ZGL_API_BEGIN
    accel_free(accel);
    ZGL_API_END
}

zgl_status zgl_accel_set_trace_schedule(zgl_accel* accel, int32_t schedule) {
    ZGL_API_BEGIN
    if (!accel) fail(ZGL_ERR_INVALID_ARG, "zgl_accel_set_trace_schedule: NULL accel");
    if (schedule < ZGL_TRACE_AUTO || schedule > ZGL_TRACE_PREFETCH)
        fail(ZGL_ERR_INVALID_ARG, "zgl_accel_set_trace_schedule: unknown schedule %d", schedule);
    accel->trace_schedule = schedule;
    ZGL_API_END
}

zgl_status zgl_trace_closest(const zgl_accel* accel, const float* origins, const float* dirs, size_t n,
                             int32_t* hit_id, float* hit_t, void* stream) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_trace_closest");
    if (!accel) fail(ZGL_ERR_INVALID_ARG, "zgl_trace_closest: NULL accel");
    if (n == 0) return ZGL_OK;
    if (!origins || !dirs || !hit_id || !hit_t) fail(ZGL_ERR_INVALID_ARG, "zgl_trace_closest: NULL array");
    DeviceGuard dg(accel->device);
    cudaStream_t s = (cudaStream_t)stream;
    Staging st(accel, s);
    int so = st.add(origins, 12 * n, true, false), sd = st.add(dirs, 12 * n, true, false);
    int si = st.add(hit_id, 4 * n, false, true), sx = st.add(hit_t, 4 * n, false, true);
    st.commit();
    ZGL_CUDA(launch_trace_closest(device_view(accel), (const float*)st.ptr(so), (const float*)st.ptr(sd),
                                  (int64_t)n, (int32_t*)st.ptr(si), (float*)st.ptr(sx), trace_schedule(accel),
                                  accel->d_counter, s));
    st.finish();
    ZGL_API_END
}

zgl_status zgl_trace_any(const zgl_accel* accel, const float* origins, const float* dirs, const float* tmax,
                         size_t n, uint8_t* occluded, void* stream) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_trace_any");
    if (!accel) fail(ZGL_ERR_INVALID_ARG, "zgl_trace_any: NULL accel");
    if (n == 0) return ZGL_OK;
    if (!origins || !dirs || !tmax || !occluded) fail(ZGL_ERR_INVALID_ARG, "zgl_trace_any: NULL array");
    DeviceGuard dg(accel->device);
    cudaStream_t s = (cudaStream_t)stream;
    Staging st(accel, s);
    int so = st.add(origins, 12 * n, true, false), sd = st.add(dirs, 12 * n, true, false);
    int sm = st.add(tmax, 4 * n, true, false), sc = st.add(occluded, n, false, true);
    st.commit();
    ZGL_CUDA(launch_trace_any(device_view(accel), (const float*)st.ptr(so), (const float*)st.ptr(sd),
                              (const float*)st.ptr(sm), (int64_t)n, (uint8_t*)st.ptr(sc), trace_schedule(accel),
                              accel->d_counter, s));
    st.finish();
    ZGL_API_END
}

zgl_status zgl_trace_count(const zgl_accel* accel, const float* origins, const float* dirs, const float* tmax,
                           size_t n, int32_t any_hit, int32_t* visits, int32_t* tests, void* stream) {
    ZGL_API_BEGIN
    if (!accel) fail(ZGL_ERR_INVALID_ARG, "zgl_trace_count: NULL accel");
    if (n == 0) return ZGL_OK;
    if (!origins || !dirs || !visits || !tests || (any_hit && !tmax))
        fail(ZGL_ERR_INVALID_ARG, "zgl_trace_count: NULL array");
    DeviceGuard dg(accel->device);
    cudaStream_t s = (cudaStream_t)stream;
    Staging st(accel, s);
    int so = st.add(origins, 12 * n, true, false), sd = st.add(dirs, 12 * n, true, false);
    int sm = st.add(any_hit ? tmax : nullptr, 4 * n, true, false);
    int sv = st.add(visits, 4 * n, false, true), sx = st.add(tests, 4 * n, false, true);
    st.commit();
    ZGL_CUDA(launch_trace_count(device_view(accel), (const float*)st.ptr(so), (const float*)st.ptr(sd),
                                (const float*)st.ptr(sm), (int64_t)n, any_hit, (int32_t*)st.ptr(sv),
                                (int32_t*)st.ptr(sx), s));
    st.finish();
    ZGL_API_END
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free closest-hit tracing.
//
// Some callers cannot let a library call cudaMalloc: a renderer that runs a
// frame loop under a fixed device-memory budget, or that hands all device
// memory to its own pool allocator, cannot afford an allocation that may fail
// mid-frame or that synchronises the whole device.  zgl_trace_closest_noalloc
// serves them: the persistent trace kernel's scratch (its work counter) and
// the staging area for host arrays live in one file-scope device array.  With
// lazy module loading a device reserves it when the first call looks up its
// address; from then on the device holds it until the process exits.
// ---------------------------------------------------------------------------
namespace zgl {
namespace {

constexpr size_t kNoAllocMaxRays = size_t(1) << 18;  // 262144 rays per call
constexpr size_t kNoAllocHeader = 256;               // work counter
constexpr size_t kNoAllocOrigins = kNoAllocHeader;
constexpr size_t kNoAllocDirs = kNoAllocOrigins + 12 * kNoAllocMaxRays;
constexpr size_t kNoAllocIds = kNoAllocDirs + 12 * kNoAllocMaxRays;
constexpr size_t kNoAllocDist = kNoAllocIds + 4 * kNoAllocMaxRays;
constexpr size_t kNoAllocBytes = kNoAllocDist + 4 * kNoAllocMaxRays;  // 8 MiB + 256 B

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// The array's name in host code is only a host-side handle, not a device
// address: the device address is looked up once per device, with that device
// current, and cached.
std::mutex g_noalloc_mu;
void* g_noalloc_addr[256] = {};

unsigned char* noalloc_scratch(int device) {
    if (device < 0 || device >= 256) fail(ZGL_ERR_INVALID_ARG, "zgl_trace_closest_noalloc: device %d", device);
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            fail(ZGL_ERR_CUDA, "zgl_trace_closest_noalloc: cudaGetSymbolAddress failed: %s",
                 cudaGetErrorString(e));
        }
        g_noalloc_addr[device] = p;
    }
    return static_cast<unsigned char*>(g_noalloc_addr[device]);
}

}  // namespace
}  // namespace zgl

extern "C" {

zgl_status zgl_trace_closest_noalloc(const zgl_accel* accel, const float* origins, const float* dirs, size_t n,
                                     int32_t* hit_id, float* hit_t, void* stream) {
    ZGL_API_BEGIN
    if (!accel) fail(ZGL_ERR_INVALID_ARG, "zgl_trace_closest_noalloc: NULL accel");
    if (n == 0) return ZGL_OK;
    if (!origins || !dirs || !hit_id || !hit_t) fail(ZGL_ERR_INVALID_ARG, "zgl_trace_closest_noalloc: NULL array");
    if (n > kNoAllocMaxRays)
        fail(ZGL_ERR_INVALID_ARG,
             "zgl_trace_closest_noalloc: %zu rays exceed the allocation-free limit of %zu rays per call", n,
             kNoAllocMaxRays);
    DeviceGuard dg(accel->device);
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* base = noalloc_scratch(accel->device);
    unsigned long long* counter = reinterpret_cast<unsigned long long*>(base);
    const bool ho = !is_device_ptr(origins), hd = !is_device_ptr(dirs);
    const bool hi = !is_device_ptr(hit_id), ht = !is_device_ptr(hit_t);
    const float* d_org = ho ? reinterpret_cast<const float*>(base + kNoAllocOrigins) : origins;
    const float* d_dir = hd ? reinterpret_cast<const float*>(base + kNoAllocDirs) : dirs;
    int32_t* d_id = hi ? reinterpret_cast<int32_t*>(base + kNoAllocIds) : hit_id;
    float* d_t = ht ? reinterpret_cast<float*>(base + kNoAllocDist) : hit_t;
    if (ho) ZGL_CUDA(cudaMemcpyAsync(base + kNoAllocOrigins, origins, 12 * n, cudaMemcpyHostToDevice, s));
    if (hd) ZGL_CUDA(cudaMemcpyAsync(base + kNoAllocDirs, dirs, 12 * n, cudaMemcpyHostToDevice, s));
    // the accelerator's schedule; the persistent one keeps its work counter in
    // the static array (the launcher resets it on the stream, since the array
    // keeps the previous call's contents)
    ZGL_CUDA(launch_trace_closest(device_view(accel), d_org, d_dir, (int64_t)n, d_id, d_t, trace_schedule(accel),
                                  counter, s));
    if (hi) ZGL_CUDA(cudaMemcpyAsync(hit_id, d_id, 4 * n, cudaMemcpyDeviceToHost, s));
    if (ht) ZGL_CUDA(cudaMemcpyAsync(hit_t, d_t, 4 * n, cudaMemcpyDeviceToHost, s));
    if (ho || hd || hi || ht) ZGL_CUDA(cudaStreamSynchronize(s));
    ZGL_API_END
}

}  // extern "C"
