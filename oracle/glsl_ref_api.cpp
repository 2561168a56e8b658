// glsl_ref_api.cpp — C ABI over the reference's integrator compute shaders
// compiled as C++.
//
// TEST INFRASTRUCTURE ONLY.  oracle/glsl_to_cpp.py turns
// src/shader/{path_integ_naive, light_path_integ, triple_path_pass_pt,
// triple_path_pass_lpt}.glsl and the libraries they include (random, math,
// microfacet, material, intersection, light, camera, material_loader) into
// oracle/_ref/glsl/*.inc, one namespace each.  This file binds their uniforms
// to an OrcScene (the tables the reference uploads in
// Scene::createGLContext and the integrators' updateUniforms) and runs each
// main() once per invocation, pass by pass, as the reference's
// renderOnePass dispatches them.  The result is the reference shaders' own
// arithmetic on the oracle's tables, under the defined arithmetic of
// glsl_shim.h.  Invocations that add into a shared film (the light paths)
// run on one thread in invocation order.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "glsl_shim.h"
#include "orc_scene.h"

namespace glsl {
thread_local GlobalId gl_GlobalInvocationID;
uvec3 gl_WorkGroupSize;
namespace naive {
#include "path_integ_naive.inc"
}
namespace light {
#include "light_path_integ.inc"
}
namespace triple_pt {
#include "triple_path_pass_pt.inc"
}
namespace triple_lpt {
#include "triple_path_pass_lpt.inc"
}
}  // namespace glsl

namespace {

// Sampler::sobolSample (src/core/Sampler.cpp:19-28) with scramble 0: the XOR
// of the generator-matrix columns picked by the bits of the sample index.
uint32_t sobol_sample(const uint32_t* m, uint32_t index, int dim) {
    uint32_t r = 0;
    for (int i = dim * 32; index != 0; index >>= 1, i++)
        if (index & 1u) r ^= m[i];
    return r;
}

const float* srgb_lut() {
    static float lut[256];
    static bool init = false;
    if (!init) {
        for (int i = 0; i < 256; i++) {
            double c = i / 255.0;
            lut[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
        }
        init = true;
    }
    return lut;
}

// Every uniform any of the four programs declares, by name.
struct Bindings {
    std::vector<uint32_t> sobol;     // genSobolSeqTexture rows that the passes read
    std::vector<float> texcoords;    // object texcoords padded to every vertex
    std::vector<float> blackEnv;     // a missing environment map reads as black
    std::vector<int32_t> blackAlias;
    std::vector<float> blackProb;

    glsl::image2D uFrame;
    glsl::usamplerBuffer uSobolSeq;
    int uSampler = 1;
    glsl::samplerBuffer uVertices, uNormals, uTexCoords, uBounds, uLightPower, uLightProb, uMaterials, uTexUVScale;
    glsl::isamplerBuffer uIndices, uHitTable, uLightAlias, uMatTypes, uMatTexIndices;
    int uBvhSize = 0, uNumLightTriangles = 0, uObjPrimCount = 0, uNumTextures = 0;
    float uLightSum = 0.0f, uLightSamplePortion = 0.0f, uEnvSum = 0.0f, uEnvRotation = 0.0f;
    bool uLightEnvUniformSample = false;
    glsl::sampler2D uEnvMap, uEnvAliasProb, uNoiseTex;
    glsl::isampler2D uEnvAliasTable;
    glsl::vec3 uCamF, uCamR, uCamU, uCamPos;
    glsl::mat3 uCamMatInv;
    float uTanFOV = 0.0f, uLensRadius = 0.0f, uFocalDist = 0.0f, uCamAsp = 0.0f;
    glsl::ivec2 uFilmSize;
    glsl::sampler2DArray uTextures;
    int uSpp = 0, uFreeCounter = 0, uSampleDim = 256, uSampleNum = 131072, uMaxDepth = 0;
    bool uSampleLight = true, uRussianRoulette = false;
    int uBlocksOnePass = 0, uLoopsPerPass = 1;
    float uScale = 1.0f;
};

int64_t vertex_count(const OrcScene& sc) {
    uint32_t m = 0;
    for (int64_t i = 0; i < 3 * sc.nTriangles; i++) m = std::max(m, sc.indices[i]);
    return (int64_t)m + 1;
}

// Uniform and texture bindings of NaivePathIntegrator (src/integrator/NaivePath.cpp:41-75)
// and Scene::createGLContext (src/core/Scene.cpp:245-263).
void bind(const OrcScene& sc, int rows, Bindings& b) {
    using namespace glsl;
    b.sobol.resize((size_t)rows * 256);
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < 256; j++) b.sobol[(size_t)i * 256 + j] = sobol_sample(sc.sobolMatrices, (uint32_t)i, j);
    b.uSobolSeq = usamplerBuffer{b.sobol.data(), 1};
    b.uSampler = sc.sampler;

    const int64_t nv = vertex_count(sc);
    b.uVertices = samplerBuffer{sc.vertices, 3};
    b.uNormals = samplerBuffer{sc.normals, 3};
    b.texcoords.assign((size_t)nv * 2, 0.0f);
    if (sc.texCoords) {
        int64_t nobj = 0;
        for (int64_t i = 0; i < 3 * (int64_t)sc.objPrimCount; i++) nobj = std::max<int64_t>(nobj, sc.indices[i] + 1);
        std::memcpy(b.texcoords.data(), sc.texCoords, sizeof(float) * 2 * (size_t)nobj);
    }
    b.uTexCoords = samplerBuffer{b.texcoords.data(), 2};
    b.uIndices = isamplerBuffer{reinterpret_cast<const int32_t*>(sc.indices), 1};
    b.uBounds = samplerBuffer{sc.bounds, 3};
    b.uHitTable = isamplerBuffer{sc.hitTable, 3};
    b.uBvhSize = (int)sc.bvhSize;

    b.uLightPower = samplerBuffer{sc.lightPower, 3};
    b.uLightAlias = isamplerBuffer{sc.lightAlias, 1};
    b.uLightProb = samplerBuffer{sc.lightProb, 1};
    b.uNumLightTriangles = sc.nLightTriangles;
    b.uLightSum = sc.lightSum;
    b.uLightEnvUniformSample = sc.lightEnvUniformSample != 0;
    b.uLightSamplePortion = sc.lightPortion;
    b.uObjPrimCount = sc.objPrimCount;

    if (sc.envTexels) {
        b.uEnvMap = sampler2D{sc.envTexels, sc.envWidth, sc.envHeight, 3};
        b.uEnvAliasTable = isampler2D{sc.envAlias, sc.envWidth + 1, sc.envHeight};
        b.uEnvAliasProb = sampler2D{sc.envProb, sc.envWidth + 1, sc.envHeight, 1};
    } else {
        b.blackEnv.assign(3, 0.0f);
        b.blackAlias.assign(2, 0);
        b.blackProb.assign(2, 1.0f);
        b.uEnvMap = sampler2D{b.blackEnv.data(), 1, 1, 3};
        b.uEnvAliasTable = isampler2D{b.blackAlias.data(), 2, 1};
        b.uEnvAliasProb = sampler2D{b.blackProb.data(), 2, 1, 1};
    }
    b.uEnvSum = sc.envSum;
    b.uEnvRotation = sc.envRotation;

    b.uCamF = vec3{sc.camF[0], sc.camF[1], sc.camF[2]};
    b.uCamR = vec3{sc.camR[0], sc.camR[1], sc.camR[2]};
    b.uCamU = vec3{sc.camU[0], sc.camU[1], sc.camU[2]};
    b.uCamPos = vec3{sc.camPos[0], sc.camPos[1], sc.camPos[2]};
    const float* mi = sc.camMatInv;
    b.uCamMatInv = mat3(vec3{mi[0], mi[1], mi[2]}, vec3{mi[3], mi[4], mi[5]}, vec3{mi[6], mi[7], mi[8]});
    b.uTanFOV = sc.tanFOV;
    b.uLensRadius = sc.lensRadius;
    b.uFocalDist = sc.focalDist;
    b.uCamAsp = sc.camAsp;
    b.uFilmSize = ivec2{sc.filmW, sc.filmH};

    b.uMaterials = samplerBuffer{sc.materials, 4};
    b.uMatTypes = isamplerBuffer{reinterpret_cast<const int32_t*>(sc.materials), 4};
    b.uMatTexIndices = isamplerBuffer{sc.matTexIndex, 1};
    b.uNumTextures = sc.nTextures;
    b.uTextures = sampler2DArray{sc.texLayers, sc.texMaxW, sc.texMaxH, srgb_lut()};
    b.uTexUVScale = samplerBuffer{sc.texScale, 2};

    b.uSampleDim = 256;
    b.uSampleNum = 131072;
    b.uNoiseTex = sampler2D{sc.noise, sc.filmW, sc.filmH, 2};
    b.uSampleLight = sc.sampleLight != 0;
    b.uRussianRoulette = sc.russianRoulette != 0;
    b.uMaxDepth = sc.maxDepth;
}

template <class F>
void parallel_for(int64_t n, int nthreads, F&& f) {
    nthreads = std::max(1, nthreads);
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([&, t] {
            for (int64_t i = t; i < n; i += nthreads) f(i);
        });
    for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

// Sum of `passes` progressive passes of the reference shader for the listed
// pixels (y * W + x): pass k runs with uSpp = spp0 + k and
// uFreeCounter = fc0 + k (NaivePath.cpp:77-105).  Russian roulette, if on,
// follows the shader (every bounce).  out: n x 3 floats.
void glslref_render_pt(const OrcScene* sc, int32_t spp0, int32_t passes, int32_t fc0, const int32_t* pixels,
                       int64_t n, float* out, int32_t nthreads) {
    using namespace glsl;
    Bindings b;
    bind(*sc, spp0 + passes + 2, b);
    std::vector<float> frame((size_t)sc->filmW * sc->filmH * 4, 0.0f);
    b.uFrame = image2D{frame.data(), sc->filmW, sc->filmH, 4};
    naive::bind_uniforms(b);
    for (int k = 0; k < passes; k++) {
        naive::uSpp = spp0 + k;
        naive::uFreeCounter = fc0 + k;
        parallel_for(n, nthreads, [&](int64_t i) {
            const int p = pixels[i];
            gl_GlobalInvocationID = GlobalId{(uint)(p % sc->filmW), (uint)(p / sc->filmW), 0u};
            naive::glsl_main();
        });
    }
    for (int64_t i = 0; i < n; i++) {
        const float* f = frame.data() + 4 * (size_t)pixels[i];
        out[3 * i] = f[0];
        out[3 * i + 1] = f[1];
        out[3 * i + 2] = f[2];
    }
}

// Film sum (H x W x 3) of `passes` passes of the light tracer
// (LightPath.cpp:83-113): 1536 x blocks light paths per pass with uSpp =
// spp0 + k, uFreeCounter = fc0 + k and the independent sampler (uSampler = 0,
// LightPath.cpp:49); every path adds into the R32F film of 3W x H texels.
void glslref_render_lt(const OrcScene* sc, int32_t spp0, int32_t passes, int32_t fc0, int32_t blocks, float* film) {
    using namespace glsl;
    Bindings b;
    bind(*sc, spp0 + passes + 2, b);
    b.uSampler = 0;
    b.uBlocksOnePass = blocks;
    std::fill(film, film + (size_t)sc->filmW * sc->filmH * 3, 0.0f);
    b.uFrame = image2D{film, sc->filmW * 3, sc->filmH, 1};
    light::bind_uniforms(b);
    light::uBlocksOnePass = blocks;
    gl_WorkGroupSize = uvec3{1536u, 1u, 1u};
    for (int k = 0; k < passes; k++) {
        light::uSpp = spp0 + k;
        light::uFreeCounter = fc0 + k;
        for (int64_t i = 0; i < (int64_t)1536 * blocks; i++) {
            gl_GlobalInvocationID = GlobalId{(uint)i, 0u, 0u};
            light::glsl_main();
        }
    }
}

// Film sum (H x W x 3) of `passes` passes of the triple integrator
// (TriplePath.cpp:97-134): per pass the camera-path program over every
// pixel (the scene's sampler), then 1536 x blocks invocations of the
// light-path program with `loops` paths each (uSampler = 0, uScale =
// W H / (blocks loops 1536), TriplePath.cpp:71-77).
void glslref_render_triple(const OrcScene* sc, int32_t spp0, int32_t passes, int32_t fc0, int32_t blocks,
                           int32_t loops, float* film, int32_t nthreads) {
    using namespace glsl;
    const int W = sc->filmW, H = sc->filmH;
    Bindings b;
    bind(*sc, spp0 + passes + 2, b);
    std::fill(film, film + (size_t)W * H * 3, 0.0f);
    b.uFrame = image2D{film, W * 3, H, 1};
    triple_pt::bind_uniforms(b);
    b.uSampler = 0;
    b.uBlocksOnePass = blocks;
    b.uLoopsPerPass = loops;
    b.uScale = (float)(W * H) / (float)(blocks * loops * 1536);
    triple_lpt::bind_uniforms(b);
    gl_WorkGroupSize = uvec3{1536u, 1u, 1u};
    for (int k = 0; k < passes; k++) {
        triple_pt::uSpp = triple_lpt::uSpp = spp0 + k;
        triple_pt::uFreeCounter = triple_lpt::uFreeCounter = fc0 + k;
        parallel_for((int64_t)W * H, nthreads, [&](int64_t i) {
            gl_GlobalInvocationID = GlobalId{(uint)(i % W), (uint)(i / W), 0u};
            triple_pt::glsl_main();
        });
        for (int64_t i = 0; i < (int64_t)1536 * blocks; i++) {
            gl_GlobalInvocationID = GlobalId{(uint)i, 0u, 0u};
            triple_lpt::glsl_main();
        }
    }
}

// bvhHit / bvhTest (src/shader/intersection.glsl:367-427) of the reference
// shader on the scene's PackedBVH: closest id and distance, or the occlusion
// flag when tmax is given.
void glslref_trace(const OrcScene* sc, const float* org, const float* dir, const float* tmax, int64_t n,
                   int32_t* hit, float* dist, int32_t nthreads) {
    using namespace glsl;
    Bindings b;
    bind(*sc, 1, b);
    naive::bind_uniforms(b);
    parallel_for(n, nthreads, [&](int64_t i) {
        naive::Ray r = naive::makeRay(vec3{org[3 * i], org[3 * i + 1], org[3 * i + 2]},
                                      vec3{dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]});
        if (tmax) {
            hit[i] = naive::bvhTest(r, tmax[i]) ? 1 : 0;
        } else {
            float d = 0.0f;
            hit[i] = naive::bvhHit(r, d);
            dist[i] = d;
        }
    });
}

}  // extern "C"
