// scene.h — host scene: flattened arrays, sampling tables and device buffers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/zgl.h"
#include "accel.h"
#include "device_scene.h"

struct zgl_scene {
    int device = 0;
    bool host_only = false;

    // flattened geometry: objects then lights (Scene.cpp:148-195)
    std::vector<float> vertices, normals;
    std::vector<uint32_t> indices;
    std::vector<int32_t> matTex;  // per object triangle
    int64_t ntri = 0;
    int32_t objPrimCount = 0;
    int64_t nObjVertices = 0;
    int32_t nLight = 0;
    std::vector<float> materials;  // 16 per material
    // some material is metal workflow, dielectric or thin dielectric, or some
    // triangle is textured
    bool fullMaterials = false;

    // albedo textures (Texture.cpp:134-171): layers of texMaxW x texMaxH
    // RGBA8 texels (the image in the top-left corner, zero elsewhere), the
    // per-texture uv scale and the per-corner texcoords of object triangles
    std::vector<float> texcoords;    // 2 per object vertex
    int32_t nTextures = 0, texMaxW = 0, texMaxH = 0;
    std::vector<uint32_t> texels;    // nTextures * texMaxH * texMaxW
    std::vector<float> texScale;     // 2 per texture
    std::vector<float> srgbLut;      // 256

    // lights (Scene.cpp:200-243): instance ranges and powers, then per triangle
    std::vector<uint32_t> lightFirst;   // n_instances + 1
    std::vector<float> lightInstPower;  // 3 per instance
    std::vector<float> lightPower;  // 3 per light triangle
    std::vector<float> lightArea;   // triangleArea of each light triangle
    std::vector<int32_t> lightAlias;
    std::vector<float> lightProb;
    float lightSum = 0.0f;

    // environment (EnvironmentMap.cpp)
    int32_t envW = 0, envH = 0;
    std::vector<float> envTexels;  // W*H*3 after RGB16F rounding
    std::vector<int32_t> envAlias;
    std::vector<float> envProb;
    float envSum = 0.0f;  // float(int(sum)) (EnvironmentMap.h:22)
    float envRotation = 0.0f;

    // sampler (Sampler.cpp)
    int32_t sampler = 1;
    std::vector<uint32_t> sobol;   // 256*32
    std::vector<float> noise;      // filmW*filmH*2
    std::vector<uint32_t> seeds;   // filmW*filmH*2

    // camera (Camera.cpp, NaivePath.cpp:49-60)
    float camF[3], camR[3], camU[3], camPos[3];
    float camMatInv[9];
    float tanFOV = 0, lensRadius = 0, focalDist = 1, camAsp = 1;
    int32_t filmW = 0, filmH = 0;

    // device
    zgl_accel* accel = nullptr;
    float4* d_shade = nullptr;
    float4* d_materials = nullptr;
    float4* d_lightPower = nullptr;
    int32_t* d_lightAlias = nullptr;
    float* d_lightProb = nullptr;
    float4* d_env = nullptr;
    int32_t* d_envAlias = nullptr;
    float* d_envProb = nullptr;
    uint32_t* d_sobol = nullptr;
    uint2* d_seeds = nullptr;
    float2* d_uv = nullptr;          // 3 per object triangle
    uint32_t* d_texels = nullptr;
    float2* d_texScale = nullptr;
    float* d_srgb = nullptr;

    zgl::DeviceScene view() const;
    void free_device();
};

namespace zgl {

// Host table builders (scene.cpp); exposed for the integrators.
void sobol_matrices(std::vector<uint32_t>& out);
float half_round(float x);  // float -> IEEE binary16 (round to nearest even) -> float

// Writes the differentiable parameters into a scene (scene.cpp): per material
// baseColor rgb, raw roughness, metallic, specular (record slots 0-3, 5, 6),
// then per light instance power rgb; rebuilds the light tables that depend on
// the powers (Scene.cpp:200-243) and updates the device copies.  instPower
// receives the new instance powers.
void scene_set_diff_params(zgl_scene* s, const float* p, int nmat, std::vector<float>& instPower);

}  // namespace zgl
