// device_scene.h — device view of a scene, shared by the host scene builder
// (scene.cpp) and the integrator kernels (render.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "accel.h"

namespace zgl {

// Device buffers of a scene.  Triangle shading records are 5 float4 per
// triangle: a.xyz b.x | b.yz c.xy | c.z na.xyz | nb.xyz nc.x | nc.yz matTex 0
// (matTex = (tex << 16) | mat as int32 bits, -1 for light triangles).
struct DeviceScene {
    DeviceAccel accel;
    const float4* shade;      // 5 float4 per triangle (scene.h)
    const float4* materials;  // 4 float4 per material (Material.h:32-53 layout)
    int32_t objPrimCount;
    int32_t nLight;
    const float4* lightPower;  // rgb, area
    const int32_t* lightAlias;
    const float* lightProb;
    float lightSum;
    const float4* envTexels;  // RGB16F-quantized texels, NULL = black environment
    int32_t envW, envH;
    const int32_t* envAlias;  // (W+1)*H
    const float* envProb;
    float envSum;
    float envRotation;
    const uint32_t* sobol;   // 256*32 generator matrices
    const uint2* pixelSeeds; // per pixel (uint(W*n.x), uint(H*n.y))
    int32_t sampler;         // 0 independent, 1 sobol
    float3 camF, camR, camU, camPos;
    float camMatInv[9];
    float tanFOV, lensRadius, focalDist, camAsp;
    int32_t filmW, filmH;
    // albedo textures: per object triangle the three corner texcoords; RGBA8
    // layers of texW x texH; per texture the uv scale; sRGB -> linear table
    const float2* uv;
    const uint32_t* texels;
    const float2* texScale;
    const float* srgb;
    int32_t texW, texH;
};

}  // namespace zgl
