// orc_scene.h — the flattened scene that the oracle's render entry points
// and the GLSL-as-C++ checker read (the reference's buffer layout,
// src/core/Scene.cpp:245-263).
//
// TEST INFRASTRUCTURE ONLY.
#pragma once

#include <cstdint>

extern "C" {

// Flattened scene in the reference's buffer layout (Scene.cpp:245-263).
struct OrcScene {
    // geometry: objects first, then light triangles (Scene.cpp:148-195)
    const float* vertices;      // nv*3
    const float* normals;       // nv*3
    const uint32_t* indices;    // ntri*3
    const int32_t* matTexIndex; // objPrimCount: (tex << 16) | mat
    int64_t nTriangles;
    int32_t objPrimCount;
    // BVH in PackedBVH layout
    const float* bounds;        // M*6
    const int32_t* hitTable;    // 6*M*3
    int64_t bvhSize;
    // materials: 16 floats each (Material.h:32-53), slot 13 = type (int bits)
    const float* materials;
    // lights
    int32_t nLightTriangles;
    const float* lightPower;    // nL*3
    const int32_t* lightAlias;
    const float* lightProb;
    float lightSum;
    // environment map (texels already RGB16F-quantized, row-major, 3 floats)
    const float* envTexels;     // may be NULL (black environment)
    int32_t envWidth, envHeight;
    const int32_t* envAlias;    // (W+1)*H
    const float* envProb;       // (W+1)*H
    float envSum;               // int-truncated (EnvironmentMap.h:22)
    float envRotation;
    // sampler
    const uint32_t* sobolMatrices;  // 256*32
    const float* noise;             // filmW*filmH*2
    int32_t sampler;                // 0 independent, 1 sobol
    // camera uniforms (NaivePath.cpp:49-60)
    float camF[3], camR[3], camU[3], camPos[3];
    float camMatInv[9];  // column-major mat3
    float tanFOV, lensRadius, focalDist, camAsp;
    int32_t filmW, filmH;
    // integrator parameters (PathIntegParam, Integrator.h:56-66)
    int32_t maxDepth;
    int32_t russianRoulette;
    int32_t sampleLight;
    int32_t lightEnvUniformSample;
    float lightPortion;
    int32_t rrStartDepth;  // Russian roulette from this bounce on (1 = the reference)
    // albedo textures (Texture.cpp:134-171): per object vertex texcoords;
    // nTextures layers of texMaxW x texMaxH 8-bit sRGB RGB texels (each image
    // in the top-left corner, zero elsewhere) and the uv scale of each
    const float* texCoords;     // objVertices*2, NULL when nTextures == 0
    int32_t nTextures, texMaxW, texMaxH;
    const uint8_t* texLayers;   // nTextures*texMaxH*texMaxW*3
    const float* texScale;      // nTextures*2
};

}  // extern "C"
