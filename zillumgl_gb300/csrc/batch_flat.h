// batch_flat.h — the flat schedule of the batched renderer: one grid whose
// blocks are 16x8 pixel tiles of every sample of every request in a launch,
// each running the path tracer's straight-line per-sample code
// (pathIntegTrace, path_integ_naive.glsl:35-143) and writing the sample's
// radiance to the request's scratch array.  The kernel lives with the other
// integrator kernels (render.cu, out-of-line traversal and BSDF calls); the
// batched renderer (render_batch.cu) fills the launch descriptor.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "device_scene.h"

namespace zgl {

struct FlatRequest {
    DeviceScene sc;
    int32_t maxDepth, rr, rrStart, sampleLight, uniformSel;
    float portion;
    float* scratch;     // [sample - j0][npix][3]
    int64_t blockBase;  // first block of this request in the launch
    int32_t tilesX, tilesY;
    int32_t j1;         // samples [j0, j1)
};

constexpr int kFlatMaxReq = 64;

struct FlatLaunch {
    FlatRequest req[kFlatMaxReq];
    int32_t nreq;
    int64_t nblocks;
    int32_t j0;
    const uint32_t* rows;  // Sobol rows, 256 values per sample index
    const uint32_t* mats;  // Sobol generator matrices (dimensions past 256)
    bool full;             // some request uses metal-workflow or dielectric materials
};

cudaError_t launch_batch_flat(const FlatLaunch& L, cudaStream_t st);

}  // namespace zgl
