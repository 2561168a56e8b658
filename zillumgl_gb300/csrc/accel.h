// accel.h — device-resident MTBVH.
//
// HBM layout (GB300-first; the reference keeps bounds, hit table, indices and
// vertices as separate GL buffer textures, src/core/Scene.cpp:245-250):
//
//   node records  float4[6][M][2]   32-byte record per threaded-table entry,
//                                   in traversal order of its face:
//                                     [0] = pMin.xyz, prim (int bits, -1 = inner)
//                                     [1] = pMax.xyz, miss (int bits)
//                 Each face stores every node in its own visiting order, so the
//                 common step k -> k+1 reads the next 32 bytes (streaming,
//                 sector-aligned, two 16-byte read-only loads).
//   triangles     float4[ntri][3]   a.xyz ab.x | ab.yz ac.xy | ac.z, 0
//                                   (ab = b - a and ac = c - a evaluated on the
//                                   host in float32, exactly the values the
//                                   ray-triangle test forms, intersection.glsl:68-69)
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "bvh_build.h"

struct zgl_accel {
    int device = 0;
    int64_t ntri = 0;
    int64_t M = 0;
    zgl::HostBVH host;
    float4* d_nodes = nullptr;  // 6*M*2
    float4* d_tris = nullptr;   // ntri*3
    // set when the tree was built on the device: the PackedBVH arrays stay
    // in device memory (bounds float[M*6], hit table int32[6*M*3]) and
    // `host` is empty
    bool device_built = false;
    float* d_bounds = nullptr;
    int32_t* d_hit = nullptr;
    // work counter of the persistent trace kernels (reset before each launch;
    // launches of one handle are serialised on its caller's stream)
    unsigned long long* d_counter = nullptr;
    int trace_schedule = 0;  // ZGL_TRACE_*
    // staging for calls made with host arrays
    mutable void* d_stage = nullptr;
    mutable size_t stage_bytes = 0;
};

namespace zgl {

struct DeviceAccel {
    const float4* nodes;
    const float4* tris;
    int32_t M;
};

inline DeviceAccel device_view(const zgl_accel* a) {
    return DeviceAccel{a->d_nodes, a->d_tris, (int32_t)a->M};
}

// Kernel launchers (accel.cu).  All pointers are device pointers.
cudaError_t launch_pack_nodes(const float* bounds, const int32_t* hit, int64_t M, float4* nodes,
                              cudaStream_t s);
// `schedule` is a ZGL_TRACE_* value; ZGL_TRACE_PERSISTENT needs `counter`, a
// device word it resets on the stream.
cudaError_t launch_trace_closest(DeviceAccel a, const float* org, const float* dir, int64_t n,
                                 int32_t* hit_id, float* hit_t, int schedule, unsigned long long* counter,
                                 cudaStream_t s);
cudaError_t launch_trace_any(DeviceAccel a, const float* org, const float* dir, const float* tmax,
                             int64_t n, uint8_t* occluded, int schedule, unsigned long long* counter,
                             cudaStream_t s);
cudaError_t launch_trace_count(DeviceAccel a, const float* org, const float* dir, const float* tmax,
                               int64_t n, int any_hit, int32_t* visits, int32_t* tests,
                               cudaStream_t s);

// Host build + upload (throws zgl::Error) and release of an accelerator.
zgl_accel* accel_create(const float* vertices, const uint32_t* indices, int64_t ntri);
// Device build (bvh_build_gpu.cu); inputs may be device, page-locked or
// pageable host arrays.  `small` = 0 selects the default subtree threshold.
zgl_accel* accel_create_device(const float* vertices, int64_t nv, const uint32_t* indices, int64_t ntri,
                               int small, cudaStream_t s);
void build_bvh_device(const float* v, int64_t nv, const uint32_t* idx, int64_t ntri, int small, float4* nodes,
                      float4* tris, float* bounds, int32_t* hit, cudaStream_t s);
int gpu_build_default_small();
int gpu_build_max_small();
// Device address of p (itself for device/managed memory, the mapped address
// of page-locked host memory) or nullptr for pageable host memory; `host`
// tells whether p is host memory.
void* device_address(const void* p, bool& host);
void accel_free(zgl_accel* a);
int host_threads();

}  // namespace zgl
