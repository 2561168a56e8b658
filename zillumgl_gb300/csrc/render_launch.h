// render_launch.h — the integrator kernel launchers of render_kernels.cuh,
// in both builds: zgl::plain (render.cu) and zgl::long_rays (render_long.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "zgl.h"

struct zgl_scene;

#define ZGL_RENDER_LAUNCHERS                                                                                         \
    cudaError_t launch_path_pass(const zgl_scene* s, const zgl_integrator_params& p, int32_t spp,                  \
                                 int32_t freeCounter, float4* frame, cudaStream_t st);                              \
    cudaError_t launch_path_passes(const zgl_scene* s, const zgl_integrator_params& p, int32_t c0, int32_t f0,     \
                                   int32_t n, float* scratch, float4* frame, cudaStream_t st);                      \
    cudaError_t launch_light_pass(const zgl_scene* s, const zgl_integrator_params& p, int32_t blocks, int32_t spp, \
                                  int32_t freeCounter, float* film, cudaStream_t st);                               \
    cudaError_t launch_triple_pass(const zgl_scene* s, const zgl_integrator_params& p, int32_t blocks,             \
                                   int32_t loops, int32_t spp, int32_t freeCounter, float* film, cudaStream_t st);

namespace zgl {
namespace plain {
ZGL_RENDER_LAUNCHERS
cudaError_t launch_film_to_frame(const float* film, float4* out, int64_t n, cudaStream_t st);
}  // namespace plain
namespace long_rays {
ZGL_RENDER_LAUNCHERS
}  // namespace long_rays
// Whether a scene's integrator passes run the long-ray kernels (render.cu).
bool long_ray_scene(const zgl_scene* s);
}  // namespace zgl

#undef ZGL_RENDER_LAUNCHERS
