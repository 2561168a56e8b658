/*
 * zgl.h — C ABI of the GB300 render hot path (MTBVH traversal, ray–triangle
 * test, BSDFs, environment/area-light sampling, MIS path tracer).
 *
 * Conventions
 *   - Every call returns a zgl_status; nothing aborts.  zgl_last_error()
 *     returns a thread-local message for the last failing call on that thread.
 *   - Handles are opaque and owned by the library; destroy them with the
 *     matching *_destroy call.  One handle is used by one host thread at a time.
 *   - Array arguments of trace calls may be host or device pointers (the
 *     library asks the driver which).  Device arrays are used in place and the
 *     call is asynchronous on `stream`; when any array is host memory the call
 *     stages through device memory and returns after the results are back.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *
 * Each entry point names the reference interface it replaces (paths are
 * relative to the ZillumGL source tree).
 */
#ifndef ZGL_H
#define ZGL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t zgl_status;
enum {
    ZGL_OK = 0,
    ZGL_ERR_INVALID_ARG = 1,
    ZGL_ERR_CUDA = 2,
    ZGL_ERR_OOM = 3,
    ZGL_ERR_TIMEOUT = 4,
    ZGL_ERR_PARSE = 5,
    ZGL_ERR_STATE = 6
};

/* Library version as major*10000 + minor*100 + patch. */
int32_t zgl_version(void);

/* Message of the last failing call on this thread ("" when none).
 * Replaces Error::check / Error::exit (src/util/Error.h:24-42), which abort. */
const char* zgl_last_error(void);

/* ------------------------------------------------------------------------ */
/* Accelerator: host MTBVH build + device threaded tables                    */
/* ------------------------------------------------------------------------ */

typedef struct zgl_accel zgl_accel;

/* Build the MTBVH over `n_triangles` triangles and upload it to the current
 * device.  `vertices` is float[n_vertices*3] (xyz), `indices` is
 * uint32[n_triangles*3].  Host pointers.  n_triangles may be 0 (every ray
 * misses).
 * Replaces BVH::BVH(vertices, indices) + BVH::build()
 * (src/accelerator/BVH.h:29-32, src/accelerator/BVH.cpp:116-144) and the
 * bounds/hit-table upload of Scene::createGLContext (src/core/Scene.cpp:197-198,
 * :249-250). */
zgl_status zgl_accel_build(const float* vertices, size_t n_vertices,
                           const uint32_t* indices, size_t n_triangles,
                           zgl_accel** out);

/* Number of BVH nodes M = 2*n_triangles - 1 (0 for an empty accelerator).
 * The reference keeps it as Scene::boxCount / uBvhSize
 * (src/core/Scene.cpp:267, src/integrator/NaivePath.cpp:43). */
zgl_status zgl_accel_node_count(const zgl_accel* accel, size_t* out);

/* Copy the PackedBVH to host arrays: bounds float[M*6] (pMin.xyz, pMax.xyz per
 * node) and hit_table int32[6*M*3] ({node, prim or -1, miss} per entry, face
 * major).  Same layout as PackedBVH{bounds, hitTable}
 * (src/accelerator/BVH.h:13-17, BVH.cpp:298-345). */
zgl_status zgl_accel_export(const zgl_accel* accel, float* bounds, int32_t* hit_table);

zgl_status zgl_accel_destroy(zgl_accel* accel);

/* Host-only MTBVH build into caller-allocated arrays (no device work):
 * bounds float[M*6], hit_table int32[6*M*3], M = 2*n_triangles - 1.  This is
 * BVH::build() returning PackedBVH (src/accelerator/BVH.cpp:116-144) without
 * the upload; zgl_accel_build runs the same builder. */
zgl_status zgl_bvh_build_host(const float* vertices, size_t n_vertices,
                              const uint32_t* indices, size_t n_triangles,
                              float* bounds, int32_t* hit_table);

/* Trace kernel schedule of an accelerator: ZGL_TRACE_AUTO (0, default),
 * ZGL_TRACE_THREAD_PER_RAY (1: one thread per ray, neighbouring rays share a
 * warp) or ZGL_TRACE_PERSISTENT (2: persistent warps that refill idle lanes
 * by atomic fetch).  Results are identical; only speed differs.  The
 * reference has one fixed schedule (one invocation per pixel or path,
 * src/integrator/NaivePath.cpp:94-100). */
enum { ZGL_TRACE_AUTO = 0, ZGL_TRACE_THREAD_PER_RAY = 1, ZGL_TRACE_PERSISTENT = 2 };
zgl_status zgl_accel_set_trace_schedule(zgl_accel* accel, int32_t schedule);

/* Closest hit of n rays (origins/dirs float[n*3]): hit_id int32[n] (primitive
 * id, -1 on miss) and hit_t float[n] (1e8 on miss).
 * Replaces bvhHit (src/shader/intersection.glsl:395-427). */
zgl_status zgl_trace_closest(const zgl_accel* accel, const float* origins, const float* dirs,
                             size_t n, int32_t* hit_id, float* hit_t, void* stream);

/* Any hit closer than tmax[i]: occluded uint8[n] (1 = some triangle at
 * 0 < t < tmax[i]).  Replaces bvhTest (src/shader/intersection.glsl:367-393). */
zgl_status zgl_trace_any(const zgl_accel* accel, const float* origins, const float* dirs,
                         const float* tmax, size_t n, uint8_t* occluded, void* stream);

/* Per-ray traversal work of a closest-hit (any_hit = 0) or any-hit (any_hit =
 * 1, tmax required) query: visits int32[n] = threaded-table entries whose box
 * was tested, tests int32[n] = triangle tests.  These counts fix the
 * algorithmic bytes of a traversal and equal the step count of bvhDebug
 * (src/shader/intersection.glsl:331-365) plus the box-rejected entries. */
zgl_status zgl_trace_count(const zgl_accel* accel, const float* origins, const float* dirs,
                           const float* tmax, size_t n, int32_t any_hit,
                           int32_t* visits, int32_t* tests, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ZGL_H */
