// postproc.cu — the display pass of the reference (post_proc.glsl:1-59): the
// accumulated RGBA sum times the integrator's result scale, clamped to
// [0, 1e30], tone-mapped (none, filmic, ACES) and gamma-encoded with
// pow(x, 1/2.2), written as RGBA32F with alpha 1.  With a preview scale s
// the input film is (W / s) x (H / s) (integer division, the preview frame of
// Application.cpp:139) and each output pixel reads texel coord / s
// (texelFetch); a texel past the film reads as zero, as GL's robust fetch
// does.  The arithmetic is float32 in the operation order of the
// shader, pow from zmath (exp2(y log2 x)), so results are reproducible bit for
// bit.  One thread per output pixel: 16 bytes in, 16 bytes out.
#define ZGL_INLINE_MATH 1  // one short kernel: the pow is inlined
#include "zgl_internal.h"
#include "zmath.cuh"

namespace zgl {
namespace {

// calc() and filmic() of post_proc.glsl:22-32
__device__ __forceinline__ float filmic_calc(float x) {
    const float A = 0.22f, B = 0.3f, C = 0.1f, D = 0.2f, E = 0.01f, F = 0.3f;
    return (x * (x * A + B * C) + D * E) / (x * (x * A + B) + D * F) - E / F;
}
__device__ __forceinline__ float filmic(float c) { return filmic_calc(c * 1.6f) / filmic_calc(11.2f); }
// ACES() of post_proc.glsl:34-37
__device__ __forceinline__ float aces(float c) { return (c * (c * 2.51f + 0.03f)) / (c * (c * 2.43f + 0.59f) + 0.14f); }

__device__ __forceinline__ float tone(float c, float scale, int mapper) {
    c = c * scale;
    c = zmin(zmax(c, 0.0f), 1e30f);  // clamp(color, 0.0, 1e30)
    if (mapper == 1) c = filmic(c);
    else if (mapper == 2) c = aces(c);
    return zpow(c, 1.0f / 2.2f);
}

__global__ void __launch_bounds__(256) postprocess_kernel(const float4* __restrict__ in, int inW, int inH, int W,
                                                          int H, int previewScale, float scale, int mapper,
                                                          float4* __restrict__ out) {
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    const int sx = x / previewScale, sy = y / previewScale;
    const float4 c = (sx < inW && sy < inH) ? __ldg(&in[(size_t)sy * inW + sx]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    out[(size_t)y * W + x] = make_float4(tone(c.x, scale, mapper), tone(c.y, scale, mapper),
                                         tone(c.z, scale, mapper), 1.0f);
}

}  // namespace
}  // namespace zgl

extern "C" {

zgl_status zgl_postprocess(const float* frame, int32_t width, int32_t height, int32_t preview_scale,
                           float result_scale, int32_t tone_mapper, float* out, void* stream) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_postprocess");
    if (!frame || !out) zgl::fail(ZGL_ERR_INVALID_ARG, "zgl_postprocess: NULL array");
    if (width <= 0 || height <= 0 || width > 65536 || height > 65536)
        zgl::fail(ZGL_ERR_INVALID_ARG, "zgl_postprocess: size %dx%d out of range", width, height);
    if (preview_scale < 1 || preview_scale > 64) zgl::fail(ZGL_ERR_INVALID_ARG, "zgl_postprocess: preview scale");
    if (tone_mapper < 0 || tone_mapper > 2) zgl::fail(ZGL_ERR_INVALID_ARG, "zgl_postprocess: unknown tone mapper");
    const int inW = width / preview_scale, inH = height / preview_scale;
    if (inW < 1 || inH < 1) zgl::fail(ZGL_ERR_INVALID_ARG, "zgl_postprocess: preview film would be empty");
    dim3 grid((unsigned)((width + 31) / 32), (unsigned)((height + 7) / 8));
    zgl::postprocess_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4*>(frame), inW, inH, width, height, preview_scale, result_scale, tone_mapper,
        reinterpret_cast<float4*>(out));
    ZGL_CUDA(cudaGetLastError());
    ZGL_API_END
}

}  // extern "C"
