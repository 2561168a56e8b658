// Test kernel for the integrators' long-ray walk (traverse.cuh:
// traverse_lane_m + finish_long_rays_group): lanes of one warp split into
// divergent groups, and neighbouring lanes trace in different accelerators,
// as in the batched renderer's persistent and queue schedules.  Built and
// loaded by tests/test_group_walk_gpu.py only.
#include "traverse.cuh"

using namespace zgl;

namespace {

__device__ __forceinline__ void trace_one(const DeviceAccel& a, float3 o, float3 d, float tmax, int any,
                                          int budget, int32_t* out_id, float* out_t, int64_t i) {
    const unsigned group = __activemask();
    const TraceRay r = make_trace_ray(o, d);
    float dist = any ? tmax : 1e8f;
    int k = 0, closest = -1;
    if (any) {
        const bool done = traverse_lane_m<true, false, 0>(a, r, dist, k, closest, budget);
        finish_long_rays_group<true>(group, a, r, dist, k, closest, done);
        out_id[i] = closest >= 0 ? 1 : 0;
    } else {
        const bool done = traverse_lane_m<false, false, 0>(a, r, dist, k, closest, budget);
        finish_long_rays_group<false>(group, a, r, dist, k, closest, done);
        out_id[i] = closest;
        out_t[i] = dist;
    }
}

// Ray i uses accelerator (i & 1); lanes with lane % 3 == 0 take one branch
// and the others another (11 and 21 lanes), with different lane budgets so
// that the two branches are distinct code (the budget does not change
// results).
__global__ void group_walk_kernel(DeviceAccel A, DeviceAccel B, const float* __restrict__ org,
                                  const float* __restrict__ dir, const float* __restrict__ tmax, int64_t n,
                                  int any, int32_t* __restrict__ out_id, float* __restrict__ out_t) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DeviceAccel a = (i & 1) ? B : A;
    const float3 o = make_float3(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
    const float3 d = make_float3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
    const float tm = any ? tmax[i] : 0.0f;
    if ((threadIdx.x & 31) % 3 == 0)
        trace_one(a, o, d, tm, any, kLongRayBudget / 2, out_id, out_t, i);
    else
        trace_one(a, o, d, tm, any, kLongRayBudget, out_id, out_t, i);
}

}  // namespace

extern "C" int group_walk(const void* nodes_a, const void* tris_a, int32_t m_a, const void* nodes_b,
                          const void* tris_b, int32_t m_b, const float* org, const float* dir, const float* tmax,
                          int64_t n, int32_t any, int32_t* out_id, float* out_t) {
    const DeviceAccel A{static_cast<const float4*>(nodes_a), static_cast<const float4*>(tris_a), m_a};
    const DeviceAccel B{static_cast<const float4*>(nodes_b), static_cast<const float4*>(tris_b), m_b};
    const unsigned grid = (unsigned)((n + 127) / 128);
    group_walk_kernel<<<grid, 128>>>(A, B, org, dir, tmax, n, any, out_id, out_t);
    cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? 0 : (int)e;
}
