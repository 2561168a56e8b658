// render.cu — the zgl_integrator_* entry points (progressive MIS path
// tracer, light tracer, triple integrator) over the kernels of
// render_kernels.cuh (compiled here with the plain traversal calls, and in
// render_long.cu with long rays finished by their lane groups).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "batch_flat.h"
#include "path_trace.cuh"
#include "scene.h"
#include "shading.cuh"
#include "zgl_internal.h"

struct zgl_integrator {
    zgl_scene* scene = nullptr;
    int32_t kind = 0;
    zgl_integrator_params params{};
    int32_t curSample = 0;    // mCurSample
    int32_t freeCounter = 0;  // mFreeCounter
    bool finished = false;
    float4* d_frame = nullptr;  // path tracer: RGBA sum, filmW * filmH
    float* d_film = nullptr;    // light / triple: RGB sum, filmW * filmH * 3 (the r32f 3W x H film)
    float samplePerPixel = 0.0f;
    int32_t blocks = 0, loops = 1;
    float* d_passes = nullptr;  // path tracer, several passes per launch: per-pass radiance
    size_t passesCap = 0;       // floats allocated in d_passes
};

#define ZGL_RENDER_NS plain
#include "render_kernels.cuh"
#include "render_launch.h"

namespace zgl {

// The batched renderer's flat schedule (render_batch.cu) runs the plain
// traversal calls.
cudaError_t launch_batch_flat(const FlatLaunch& L, cudaStream_t st) { return plain::launch_batch_flat(L, st); }

// Whether a scene's integrator passes run the long-ray kernels.
bool long_ray_scene(const zgl_scene* s) { return s->accel && s->accel->M >= kLongRayMinEntries; }

}  // namespace zgl

using namespace zgl;

namespace {

void check_params(const zgl_integrator_params& p) {
    if (p.max_depth < 0 || p.max_depth > 1024) fail(ZGL_ERR_INVALID_ARG, "integrator: max_depth %d out of range", p.max_depth);
    if (p.rr_start_depth < 1) fail(ZGL_ERR_INVALID_ARG, "integrator: rr_start_depth must be >= 1");
    if (!(p.light_portion >= 0.0f && p.light_portion <= 1.0f))
        fail(ZGL_ERR_INVALID_ARG, "integrator: light_portion must lie in [0, 1]");
    if (p.blocks_per_pass < 0 || p.blocks_per_pass > 65536)
        fail(ZGL_ERR_INVALID_ARG, "integrator: blocks_per_pass %d out of range", p.blocks_per_pass);
    if (p.loops_per_pass < 1 || p.loops_per_pass > 4096)
        fail(ZGL_ERR_INVALID_ARG, "integrator: loops_per_pass %d out of range", p.loops_per_pass);
}

bool is_device_memory(const void* p) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" {

zgl_status zgl_integrator_params_default(zgl_integrator_params* p) {
    ZGL_API_BEGIN
    if (!p) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_params_default: NULL");
    p->max_depth = 4;
    p->russian_roulette = 0;
    p->rr_start_depth = 1;
    p->sample_light = 1;
    p->light_env_uniform_sample = 0;
    p->light_portion = 0.5f;
    p->finite_sample = 0;
    p->max_sample = 64;
    p->blocks_per_pass = 0;
    p->loops_per_pass = 1;
    ZGL_API_END
}

zgl_status zgl_integrator_create(zgl_scene* scene, int32_t kind, const zgl_integrator_params* params,
                                 zgl_integrator** out) {
    ZGL_API_BEGIN
    if (!scene || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_create: NULL argument");
    *out = nullptr;
    if (scene->host_only) fail(ZGL_ERR_STATE, "zgl_integrator_create: scene was created host-only");
    if (kind < ZGL_INTEGRATOR_PATH || kind > ZGL_INTEGRATOR_TRIPLE)
        fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_create: unknown kind %d", kind);
    if (kind != ZGL_INTEGRATOR_PATH && scene->nLight == 0)
        fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_create: the light and triple integrators sample light triangles "
                                  "and the scene has none");
    zgl_integrator_params p;
    zgl_integrator_params_default(&p);
    if (params) p = *params;
    check_params(p);
    auto* it = new zgl_integrator();
    it->scene = scene;
    it->kind = kind;
    it->params = p;
    it->blocks = p.blocks_per_pass ? p.blocks_per_pass : (kind == ZGL_INTEGRATOR_TRIPLE ? 64 : 32);
    it->loops = p.loops_per_pass;
    size_t npix = (size_t)scene->filmW * scene->filmH;
    cudaError_t e;
    if (kind == ZGL_INTEGRATOR_PATH) {
        e = cudaMalloc(&it->d_frame, sizeof(float4) * npix);
        if (e == cudaSuccess) e = cudaMemset(it->d_frame, 0, sizeof(float4) * npix);
    } else {
        e = cudaMalloc(&it->d_film, sizeof(float) * 3 * npix);
        if (e == cudaSuccess) e = cudaMemset(it->d_film, 0, sizeof(float) * 3 * npix);
    }
    if (e != cudaSuccess) {
        if (it->d_frame) cudaFree(it->d_frame);
        if (it->d_film) cudaFree(it->d_film);
        delete it;
        cuda_check(e, "zgl_integrator_create");
    }
    *out = it;
    ZGL_API_END
}

zgl_status zgl_integrator_render_pass(zgl_integrator* it, void* stream) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_integrator_render_pass");
    if (!it) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_render_pass: NULL");
    it->freeCounter++;  // counts every call (NaivePath.cpp:79, LightPath.cpp:85, TriplePath.cpp:268)
    const zgl_scene* sc = it->scene;
    cudaStream_t st = (cudaStream_t)stream;
    if (it->kind == ZGL_INTEGRATOR_PATH) {
        if (it->params.finite_sample && it->curSample > it->params.max_sample) {
            it->finished = true;
            return ZGL_OK;
        }
        const auto pass = long_ray_scene(sc) ? long_rays::launch_path_pass : plain::launch_path_pass;
        ZGL_CUDA(pass(sc, it->params, it->curSample, it->freeCounter, it->d_frame, st));
    } else if (it->kind == ZGL_INTEGRATOR_LIGHT) {
        if (it->params.finite_sample && it->samplePerPixel > (float)it->params.max_sample) {
            it->finished = true;
            return ZGL_OK;
        }
        const auto pass = long_ray_scene(sc) ? long_rays::launch_light_pass : plain::launch_light_pass;
        ZGL_CUDA(pass(sc, it->params, it->blocks, it->curSample, it->freeCounter, it->d_film, st));
        it->samplePerPixel += (float)it->blocks * 1536.0f / (float)(sc->filmW * sc->filmH);
    } else {
        if (it->params.finite_sample && it->curSample > it->params.max_sample) {
            it->finished = true;
            return ZGL_OK;
        }
        const auto pass = long_ray_scene(sc) ? long_rays::launch_triple_pass : plain::launch_triple_pass;
        ZGL_CUDA(pass(sc, it->params, it->blocks, it->loops, it->curSample, it->freeCounter, it->d_film, st));
        it->samplePerPixel += 1.0f;
    }
    it->curSample++;
    ZGL_API_END
}

zgl_status zgl_integrator_render_passes(zgl_integrator* it, int32_t passes, void* stream) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_integrator_render_passes");
    if (!it) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_render_passes: NULL");
    if (passes < 0 || passes > 4096) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_render_passes: %d passes", passes);
    if (it->kind != ZGL_INTEGRATOR_PATH) {
        // light and triple passes splat into one film: one launch per pass
        for (int32_t k = 0; k < passes; k++) {
            zgl_status st = zgl_integrator_render_pass(it, stream);
            if (st != ZGL_OK) return st;
        }
        return ZGL_OK;
    }
    // passes that render before a finite sample budget stops the integrator;
    // every call counts in freeCounter, as consecutive render_pass calls do
    int32_t n = passes;
    if (it->params.finite_sample) n = std::max(0, std::min(passes, it->params.max_sample + 1 - it->curSample));
    const int32_t f0 = it->freeCounter + 1;
    if (n > 0) {
        const zgl_scene* sc = it->scene;
        const size_t need = (size_t)3 * sc->filmW * sc->filmH * (size_t)n;
        if (need > it->passesCap) {
            if (it->d_passes) ZGL_CUDA(cudaFree(it->d_passes));
            it->d_passes = nullptr;
            it->passesCap = 0;
            ZGL_CUDA(cudaMalloc(&it->d_passes, sizeof(float) * need));
            it->passesCap = need;
        }
        const auto passes = long_ray_scene(sc) ? long_rays::launch_path_passes : plain::launch_path_passes;
        ZGL_CUDA(passes(sc, it->params, it->curSample, f0, n, it->d_passes, it->d_frame, (cudaStream_t)stream));
        it->curSample += n;
    }
    if (n < passes) it->finished = true;
    it->freeCounter += passes;
    ZGL_API_END
}

zgl_status zgl_integrator_reset(zgl_integrator* it) {
    ZGL_API_BEGIN
    if (!it) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_reset: NULL");
    const zgl_scene* sc = it->scene;
    it->curSample = 0;
    it->finished = false;
    if (it->kind != ZGL_INTEGRATOR_PATH) {
        // the film is cleared (img_clear_1x32f.glsl); samplePerPixel restarts
        // at one pass worth (LightPath.cpp:133, TriplePath.cpp:322)
        ZGL_CUDA(cudaMemset(it->d_film, 0, sizeof(float) * 3 * (size_t)sc->filmW * sc->filmH));
        it->samplePerPixel = it->kind == ZGL_INTEGRATOR_LIGHT
                                 ? (float)it->blocks * 1536.0f / (float)(sc->filmW * sc->filmH)
                                 : 1.0f;
    }
    ZGL_API_END
}

zgl_status zgl_integrator_frame(zgl_integrator* it, float* out, int32_t* spp, void* stream) {
    ZGL_API_BEGIN
    if (!it || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_frame: NULL");
    size_t npix = (size_t)it->scene->filmW * it->scene->filmH;
    size_t bytes = sizeof(float4) * npix;
    cudaStream_t st = (cudaStream_t)stream;
    bool dev = is_device_memory(out);
    if (it->kind == ZGL_INTEGRATOR_PATH) {
        if (dev) {
            ZGL_CUDA(cudaMemcpyAsync(out, it->d_frame, bytes, cudaMemcpyDeviceToDevice, st));
        } else {
            ZGL_CUDA(cudaMemcpyAsync(out, it->d_frame, bytes, cudaMemcpyDeviceToHost, st));
            ZGL_CUDA(cudaStreamSynchronize(st));
        }
    } else if (dev) {
        ZGL_CUDA(plain::launch_film_to_frame(it->d_film, reinterpret_cast<float4*>(out), (int64_t)npix, st));
    } else {
        std::vector<float> film(3 * npix);
        ZGL_CUDA(cudaMemcpyAsync(film.data(), it->d_film, sizeof(float) * 3 * npix, cudaMemcpyDeviceToHost, st));
        ZGL_CUDA(cudaStreamSynchronize(st));
        for (size_t i = 0; i < npix; i++) {
            out[4 * i] = film[3 * i];
            out[4 * i + 1] = film[3 * i + 1];
            out[4 * i + 2] = film[3 * i + 2];
            out[4 * i + 3] = 1.0f;
        }
    }
    if (spp) *spp = it->curSample;
    ZGL_API_END
}

zgl_status zgl_integrator_result_scale(const zgl_integrator* it, float* out) {
    ZGL_API_BEGIN
    if (!it || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_result_scale: NULL");
    *out = it->kind == ZGL_INTEGRATOR_PATH ? 1.0f / (float)(it->curSample + 1) : 1.0f / it->samplePerPixel;
    ZGL_API_END
}

zgl_status zgl_integrator_state_size(const zgl_integrator* it, size_t* floats) {
    ZGL_API_BEGIN
    if (!it || !floats) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_state_size: NULL");
    const size_t npix = (size_t)it->scene->filmW * it->scene->filmH;
    *floats = (it->kind == ZGL_INTEGRATOR_PATH ? 4 : 3) * npix;
    ZGL_API_END
}

zgl_status zgl_integrator_save(const zgl_integrator* it, zgl_integrator_state* state, float* sum, void* stream) {
    ZGL_API_BEGIN
    if (!it || !state || !sum) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_save: NULL");
    const size_t npix = (size_t)it->scene->filmW * it->scene->filmH;
    cudaStream_t st = (cudaStream_t)stream;
    if (it->kind == ZGL_INTEGRATOR_PATH)
        ZGL_CUDA(cudaMemcpyAsync(sum, it->d_frame, sizeof(float4) * npix, cudaMemcpyDefault, st));
    else
        ZGL_CUDA(cudaMemcpyAsync(sum, it->d_film, sizeof(float) * 3 * npix, cudaMemcpyDefault, st));
    ZGL_CUDA(cudaStreamSynchronize(st));
    state->kind = it->kind;
    state->cur_sample = it->curSample;
    state->free_counter = it->freeCounter;
    state->finished = it->finished ? 1 : 0;
    state->sample_per_pixel = it->samplePerPixel;
    ZGL_API_END
}

zgl_status zgl_integrator_restore(zgl_integrator* it, const zgl_integrator_state* state, const float* sum,
                                  void* stream) {
    ZGL_API_BEGIN
    if (!it || !state || !sum) fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_restore: NULL");
    if (state->kind != it->kind)
        fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_restore: checkpoint of integrator kind %d, this one is %d",
             state->kind, it->kind);
    if (state->cur_sample < 0 || state->free_counter < 0 || !(state->sample_per_pixel >= 0.0f) ||
        !std::isfinite(state->sample_per_pixel))
        fail(ZGL_ERR_INVALID_ARG, "zgl_integrator_restore: invalid counters");
    const size_t npix = (size_t)it->scene->filmW * it->scene->filmH;
    cudaStream_t st = (cudaStream_t)stream;
    if (it->kind == ZGL_INTEGRATOR_PATH)
        ZGL_CUDA(cudaMemcpyAsync(it->d_frame, sum, sizeof(float4) * npix, cudaMemcpyDefault, st));
    else
        ZGL_CUDA(cudaMemcpyAsync(it->d_film, sum, sizeof(float) * 3 * npix, cudaMemcpyDefault, st));
    ZGL_CUDA(cudaStreamSynchronize(st));
    it->curSample = state->cur_sample;
    it->freeCounter = state->free_counter;
    it->finished = state->finished != 0;
    it->samplePerPixel = state->sample_per_pixel;
    ZGL_API_END
}

zgl_status zgl_integrator_destroy(zgl_integrator* it) {
    ZGL_API_BEGIN
    if (!it) return ZGL_OK;
    if (it->d_frame) cudaFree(it->d_frame);
    if (it->d_film) cudaFree(it->d_film);
    if (it->d_passes) cudaFree(it->d_passes);
    delete it;
    ZGL_API_END
}

}  // extern "C"
