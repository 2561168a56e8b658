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
 *     call is asynchronous on `stream`.  Page-locked (pinned) host arrays are
 *     used in place too: the kernels read and write them over the host link
 *     (NVLink-C2C on Grace-Blackwell); pageable host arrays are staged through
 *     device memory.  A call with any host array returns after the results
 *     are in host memory.
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

/* The same accelerator built by CUDA kernels on the current device: tree,
 * threaded tables and triangle records are bit-identical to
 * zgl_accel_build's (BVH::quickBuild + BVH::buildHitTable,
 * src/accelerator/BVH.cpp:217-345).  `vertices` / `indices` may be device
 * pointers, page-locked host pointers (read in place) or pageable host
 * memory (copied first).  Nodes with fewer than `small_threshold` triangles
 * are built one warp per subtree (0 = default 512; valid 0..4096, values
 * below 8 act as 8); the result does not depend on it.  Synchronous; the
 * work is ordered on `stream`.  Out-of-range indices and vertex components
 * that are NaN, infinite or beyond +-1e8 give ZGL_ERR_INVALID_ARG (the same
 * checks as zgl_accel_build). */
zgl_status zgl_accel_build_device(const float* vertices, size_t n_vertices,
                                  const uint32_t* indices, size_t n_triangles,
                                  int32_t small_threshold, void* stream,
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

/* Trace kernel schedule of an accelerator.  All give identical results;
 * only speed differs.  The reference has one fixed schedule (one invocation
 * per pixel or path, src/integrator/NaivePath.cpp:94-100).
 *   ZGL_TRACE_AUTO (0, default): one thread per ray; a ray with a
 *     direction component below 1e-6 in magnitude (boxHit's near-zero
 *     branch can make it visit tens of thousands of table entries) that has
 *     not finished after 256 entries is finished by its whole warp, 32
 *     consecutive entries at a time.
 *   ZGL_TRACE_THREAD_PER_RAY (1): one thread per ray, every ray on its own
 *     lane to the end (the reference's schedule).
 *   ZGL_TRACE_PERSISTENT (2): persistent warps that refill idle lanes by
 *     atomic fetch.
 *   ZGL_TRACE_PREFETCH (3): as ZGL_TRACE_AUTO, with every lane requesting
 *     both possible successors of a node ahead. */
enum { ZGL_TRACE_AUTO = 0, ZGL_TRACE_THREAD_PER_RAY = 1, ZGL_TRACE_PERSISTENT = 2, ZGL_TRACE_PREFETCH = 3 };
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

/* Allocation-free variant of zgl_trace_closest, for callers that must not
 * let the library allocate device memory (a frame loop under a fixed memory
 * budget, or an application whose own pool allocator owns the device).  No
 * counterpart in the reference.  It runs the schedule set with
 * zgl_accel_set_trace_schedule, like zgl_trace_closest; the persistent
 * schedule's work counter and the staging area for host arrays live in one
 * static device array of 8 MiB + 256 B, and the call makes no cudaMalloc or
 * cudaFree.  n is limited to 262144 rays per call (larger n returns
 * ZGL_ERR_INVALID_ARG); arrays may be host or device memory, as for
 * zgl_trace_closest.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current.  Under CUDA's lazy
 * module loading that lookup is also when the device reserves the array, so
 * the first call can fail with ZGL_ERR_CUDA when the device is out of memory:
 * make one warm-up call (n = 1) on each device before a budgeted frame loop
 * and before any stream capture.  From then on every GPU that loaded the
 * library holds the array until the process exits.  All calls share the
 * array: calls whose GPU work overlaps (other streams, other host threads)
 * race on it and must be serialised by the caller. */
zgl_status zgl_trace_closest_noalloc(const zgl_accel* accel, const float* origins, const float* dirs,
                                     size_t n, int32_t* hit_id, float* hit_t, void* stream);

/* ------------------------------------------------------------------------ */
/* Scene: flattened geometry, materials, lights, environment, camera         */
/* ------------------------------------------------------------------------ */

typedef struct zgl_scene zgl_scene;

/* World-space scene arrays (host pointers, borrowed for the call).  Object
 * triangles come first and light triangles after them, exactly as
 * Scene::createGLContext flattens them (src/core/Scene.cpp:148-195): a light
 * triangle k gets primitive id obj_n_triangles + k.  Per-vertex normals are
 * required; texture coordinates are optional (textures are not supported yet,
 * every obj_mat_tex entry must have texture index -1, i.e. 0xffff in the upper
 * half).  Materials are 16 floats each in the layout of struct Material
 * (src/core/Material.h:32-53) with the type stored as int32 bits in float
 * slot 13.  Light instance k owns light triangles [light_first[k],
 * light_first[k+1]) and total power light_power[3k..3k+2], split over its
 * triangles by area (Scene.cpp:200-243).  env_rgb is an optional float RGB
 * image (env_width x env_height), uploaded as RGB16F like EnvironmentMap
 * (src/core/EnvironmentMap.cpp:8-59); NULL means a black environment.  The
 * camera follows Camera::update (src/core/Camera.cpp:149-162). */
typedef struct zgl_scene_desc {
    const float* obj_vertices;
    size_t obj_n_vertices;
    const float* obj_normals;
    const uint32_t* obj_indices;
    size_t obj_n_triangles;
    const int32_t* obj_mat_tex;     /* per object triangle: (tex << 16) | mat */
    const float* materials;         /* 16 floats per material */
    size_t n_materials;
    const float* light_vertices;
    size_t light_n_vertices;
    const float* light_normals;
    const uint32_t* light_indices;  /* local to the light vertex array */
    size_t light_n_triangles;
    const uint32_t* light_first;    /* n_light_instances + 1 offsets */
    const float* light_power;       /* rgb per instance */
    size_t n_light_instances;
    const float* env_rgb;
    int32_t env_width, env_height;
    float env_rotation;
    float cam_pos[3];
    float cam_angle[3];             /* degrees: yaw, pitch; roll as Camera.cpp uses it */
    float cam_fov;                  /* degrees, clamped to [0.1, 90] like Camera::setFOV */
    float cam_lens_radius;
    float cam_focal_dist;
    int32_t film_width, film_height;
    int32_t sampler;                /* 0 independent (rand), 1 sobol */
    /* Albedo textures (material_loader.glsl:8-17, Texture.cpp:134-171): a
     * triangle whose obj_mat_tex has tex = mat_tex >> 16 != -1 takes its
     * base colour from texture `tex` at the interpolated texcoord instead of
     * from its material.  obj_texcoords: float[obj_n_vertices*2] (NULL = all
     * zero).  tex_size: int32[n_textures*2] (width, height).  tex_rgb: the
     * images' 8-bit sRGB RGB texels concatenated, each row-major with its
     * top row first (stb_image order, no flip). */
    const float* obj_texcoords;
    int32_t n_textures;
    const int32_t* tex_size;
    const uint8_t* tex_rgb;
} zgl_scene_desc;

enum { ZGL_SCENE_HOST_ONLY = 1 };

/* Build the scene tables (light power/alias, environment alias tables, Sobol
 * matrices, per-pixel seeds) and, unless flags has ZGL_SCENE_HOST_ONLY, the
 * MTBVH and all device buffers on the current device.  Replaces
 * Scene::createGLContext (src/core/Scene.cpp:133-270). */
zgl_status zgl_scene_create(const zgl_scene_desc* desc, int32_t flags, zgl_scene** out);

/* Copy a named host table into `out` (`bytes` must match exactly):
 *   "light_power" float[nL*3], "light_alias" int32[nL], "light_prob" float[nL],
 *   "env_alias" int32[(W+1)*H], "env_prob" float[(W+1)*H],
 *   "env_texels" float[W*H*3] (after RGB16F rounding), "sobol" uint32[256*32],
 *   "noise" float[filmW*filmH*2], "pixel_seeds" uint32[filmW*filmH*2],
 *   "camera" float[19] (front, right, up, inverse camera matrix column-major,
 *   tan(fov/2)), "scalars" float[4] (lightSum, envSum as used by the shaders,
 *   objPrimCount, nLightTriangles), "info" int64[13] (film width, film
 *   height, vertices, object vertices, triangles, object triangles, light
 *   triangles, materials, environment width, environment height, textures,
 *   texture layer width, texture layer height), the
 *   flattened "vertices" and "normals"
 *   float[nv*3], "indices" uint32[ntri*3], "mat_tex" int32[objPrimCount],
 *   "materials" float[nmat*16], "tex_scale" float[n_textures*2] (image size /
 *   largest image size, Texture.cpp:163-170), "texcoords"
 *   float[object vertices*2], "tex_texels" uint32[textures*layer height*layer
 *   width] (RGB8 in the low three bytes, images in the top-left corner of
 *   their layer) and "srgb_lut" float[256] (the linear value of each 8-bit
 *   sRGB code). */
zgl_status zgl_scene_export(const zgl_scene* scene, const char* table, void* out, size_t bytes);

/* Scene::load (src/core/Scene.cpp:58-127) + createGLContext: read a scene XML
 * file (integrator size, sampler, camera, model instances with transforms,
 * materials or light radiance, environment map) and build the scene.  Models
 * are Wavefront OBJ files (texcoords flipped as aiProcess_FlipUVs does, one
 * material slot per `usemtl` with the .mtl's Kd and map_Kd; an instance's
 * <material> replaces every slot's parameters and keeps the textures), albedo
 * textures are binary/ASCII PPM or uncompressed BMP images (a texture that
 * cannot be read leaves its faces untextured, as Resource::addImage does) and
 * the environment map is a PFM image (the reference uses assimp and
 * stb_image, which this library does not include).  `flags` as for
 * zgl_scene_create.  Malformed files give ZGL_ERR_PARSE. */
zgl_status zgl_scene_load_xml(const char* path, int32_t flags, zgl_scene** out);

zgl_status zgl_scene_destroy(zgl_scene* scene);

/* Alias table of a discrete pdf (Walker/Vose), host only: alias int32[n] and
 * prob float[n].  Same construction as AliasTable::build<int32_t>
 * (src/math/AliasTable.h:12-54), which the light-selection table uses. */
zgl_status zgl_alias_table_build(const float* pdf, size_t n, int32_t* alias, float* prob);

/* ------------------------------------------------------------------------ */
/* Integrators (class Integrator, src/core/Integrator.h:25-52)               */
/* ------------------------------------------------------------------------ */

typedef struct zgl_integrator zgl_integrator;

/* ZGL_INTEGRATOR_PATH: NaivePathIntegrator (path_integ_naive.glsl);
 * ZGL_INTEGRATOR_LIGHT: LightPathIntegrator, the particle tracer
 * (light_path_integ.glsl, LightPath.cpp); ZGL_INTEGRATOR_TRIPLE:
 * TriplePathIntegrator, the MIS-weighted (s=0)+(s=1)+(t=1) integrator
 * (triple_path_pass_{pt,lpt}.glsl, TriplePath.cpp).  The light and triple
 * integrators need at least one light triangle. */
enum { ZGL_INTEGRATOR_PATH = 0, ZGL_INTEGRATOR_LIGHT = 1, ZGL_INTEGRATOR_TRIPLE = 2 };

/* Parameters of PathIntegParam / LightPathIntegParam / TriplePathIntegParam
 * (src/core/Integrator.h:56-143) plus rr_start_depth: Russian roulette runs
 * from this bounce on (1 = every bounce, the reference's behaviour).
 * blocks_per_pass: light paths per pass are blocks_per_pass x 1536 (0 = the
 * reference default, 32 for the light tracer and 64 for the triple
 * integrator); loops_per_pass: light paths per thread of the triple
 * integrator (LPTLoopsPerPass, 1). */
typedef struct zgl_integrator_params {
    int32_t max_depth;                /* 4 */
    int32_t russian_roulette;         /* 0 */
    int32_t rr_start_depth;           /* 1 */
    int32_t sample_light;             /* 1 */
    int32_t light_env_uniform_sample; /* 0 */
    float light_portion;              /* 0.5 */
    int32_t finite_sample;            /* 0 */
    int32_t max_sample;               /* 64 */
    int32_t blocks_per_pass;          /* 0 = kind default */
    int32_t loops_per_pass;           /* 1 */
} zgl_integrator_params;

/* Fill the reference defaults. */
zgl_status zgl_integrator_params_default(zgl_integrator_params* params);

/* Integrator::init (NaivePath.cpp:69-75): allocate the frame (film size of
 * the scene) on the scene's device.  The scene must outlive the integrator. */
zgl_status zgl_integrator_create(zgl_scene* scene, int32_t kind, const zgl_integrator_params* params,
                                 zgl_integrator** out);

/* Integrator::renderOnePass (NaivePath.cpp:77-105): one sample per pixel,
 * accumulated into the frame; asynchronous on `stream`. */
zgl_status zgl_integrator_render_pass(zgl_integrator* integ, void* stream);

/* `passes` consecutive calls of zgl_integrator_render_pass in one go: the
 * frame, sample count and counters end exactly as after those calls.  The
 * path tracer renders all of them in one launch (per-pass radiance in a
 * device scratch buffer of filmW*filmH*3*passes floats kept by the
 * integrator, then added to the frame in pass order), which fills the GPU at
 * small film sizes; the light and triple integrators run one pass at a time.
 * No counterpart in the reference (one dispatch per pass). */
zgl_status zgl_integrator_render_passes(zgl_integrator* integ, int32_t passes, void* stream);

/* Integrator::reset (NaivePath.cpp:107-115): the next pass restarts the
 * progressive sum at sample 0. */
zgl_status zgl_integrator_reset(zgl_integrator* integ);

/* Integrator::getFrame: the frame holds the running SUM of samples, RGBA
 * float[filmW*filmH*4], row y = 0 first (GL convention: bottom row).  `out`
 * may be host or device memory; spp (may be NULL) receives the passes done.
 * Synchronous for host memory. */
zgl_status zgl_integrator_frame(zgl_integrator* integ, float* out, int32_t* spp, void* stream);

/* Integrator::resultScale: 1 / (samples + 1) for the path tracer
 * (Integrator.h:79) and 1 / samplePerPixel for the light and triple
 * integrators (Integrator.h:114, :156), with the reference's bookkeeping of
 * samplePerPixel (LightPath.cpp:113-134, TriplePath.cpp:303-322). */
zgl_status zgl_integrator_result_scale(const zgl_integrator* integ, float* out);

zgl_status zgl_integrator_destroy(zgl_integrator* integ);

/* Checkpoint / resume (no counterpart in the reference, whose
 * Scene::saveToFile is empty, Scene.cpp:129-131).  An integrator's whole
 * progressive state is its running sum plus the counters below; the samplers
 * are counter-based, so an integrator restored from a checkpoint continues
 * exactly like one that never stopped (the path tracer bit for bit).  The
 * sum holds zgl_integrator_state_size floats: the path tracer's RGBA frame
 * (filmW*filmH*4) or the light / triple integrators' RGB film
 * (filmW*filmH*3).  `sum` may be host or device memory; both calls return
 * after the copy.  A checkpoint restores into any integrator of the same
 * kind on a scene with the same film size. */
typedef struct zgl_integrator_state {
    int32_t kind;             /* ZGL_INTEGRATOR_* of the saving integrator */
    int32_t cur_sample;       /* passes rendered since the last reset */
    int32_t free_counter;     /* the rand() seed counter */
    int32_t finished;         /* the finite-sample limit was reached */
    float sample_per_pixel;   /* light / triple bookkeeping of resultScale */
} zgl_integrator_state;
zgl_status zgl_integrator_state_size(const zgl_integrator* integ, size_t* floats);
zgl_status zgl_integrator_save(const zgl_integrator* integ, zgl_integrator_state* state, float* sum,
                               void* stream);
zgl_status zgl_integrator_restore(zgl_integrator* integ, const zgl_integrator_state* state, const float* sum,
                                  void* stream);

/* ------------------------------------------------------------------------ */
/* Batched rendering: many requests in persistent launches                   */
/* ------------------------------------------------------------------------ */

/* One render request: `spp` path-tracer samples per pixel of `scene` (its film
 * size and camera) into `frame`, a DEVICE buffer of filmW*filmH RGBA floats
 * that receives the running sum, exactly what zgl_integrator_frame returns
 * after `spp` passes of a fresh ZGL_INTEGRATOR_PATH integrator with `params`.
 * No counterpart in the reference (its queue experiments
 * pt_global_queue_*.glsl / pt_shared_queue.glsl are the nearest). */
typedef struct zgl_render_request {
    zgl_scene* scene;
    int32_t spp;
    zgl_integrator_params params;
    float* frame;
} zgl_render_request;

/* Schedule of the batched renderer; 0 picks the default (or, after
 * zgl_batch_autotune, the tuned value).  schedule: ZGL_BATCH_FLAT (one grid of
 * 16x8 pixel tiles over every sample of every request, straight-line path
 * code per thread; the default), ZGL_BATCH_PERSISTENT (persistent warps
 * with per-bounce path state and path regeneration) or ZGL_BATCH_QUEUE
 * (persistent blocks of 256 threads whose paths put their closest-hit and
 * shadow rays into dense queues in shared memory, traced by the whole block
 * between shading rounds; the reference's nearest relative is
 * src/shader/pt_shared_queue.glsl).  For the persistent and queue
 * schedules: block_size 64, 128 or 256 threads (256 for the queue);
 * queue_capacity: work items a warp claims per atomic fetch;
 * regen_threshold: idle lanes a warp waits for before refilling them
 * (1-32).  Every schedule renders every sample of a
 * group of up to 64 requests in one launch (chunks of sample indices when the
 * per-sample scratch would exceed scratch_mib), followed by the in-order frame
 * updates; the CUDA graph holds these launches. */
enum { ZGL_BATCH_DEFAULT = 0, ZGL_BATCH_FLAT = 1, ZGL_BATCH_PERSISTENT = 2, ZGL_BATCH_QUEUE = 3 };
typedef struct zgl_batch_config {
    int32_t block_size;
    int32_t queue_capacity;
    int32_t regen_threshold;
    int32_t schedule;
    int32_t scratch_mib;  /* per-sample scratch budget in MiB (0 = 8192); fixed at zgl_batch_create */
} zgl_batch_config;

typedef struct zgl_batch zgl_batch;

zgl_status zgl_batch_config_default(zgl_batch_config* config);

/* Validates the requests and uploads their descriptors.  Scenes and frames
 * are borrowed and must outlive the batch. */
zgl_status zgl_batch_create(const zgl_render_request* requests, int32_t n, const zgl_batch_config* config,
                            zgl_batch** out);

/* Renders every request (all samples) as one CUDA graph, captured on the
 * first call and replayed afterwards; ordered after prior work on `stream`,
 * and later work on `stream` waits for it. */
zgl_status zgl_batch_render(zgl_batch* batch, void* stream);

/* Times the flat schedule and every combination of block size, queue
 * capacity and regeneration threshold of the persistent one on the first
 * samples of the batch, keeps the fastest for later renders and returns it
 * in `chosen` (may be NULL).  Overwrites the frames. */
zgl_status zgl_batch_autotune(zgl_batch* batch, void* stream, zgl_batch_config* chosen);

zgl_status zgl_batch_set_config(zgl_batch* batch, const zgl_batch_config* config);
zgl_status zgl_batch_get_config(const zgl_batch* batch, zgl_batch_config* out);
zgl_status zgl_batch_destroy(zgl_batch* batch);

/* ------------------------------------------------------------------------ */
/* Differentiable path tracing (path replay adjoint)                         */
/* ------------------------------------------------------------------------ */

/* A differentiable renderer over `scene` with the path tracer's `params`
 * (NULL = defaults) and `spp` samples per pixel.  Its image is the mean of
 * the path tracer's first `spp` samples: after zgl_diff_forward it equals
 * zgl_integrator_frame / spp of a fresh ZGL_INTEGRATOR_PATH integrator with
 * the same params after `spp` passes (up to float summation order of the
 * RGB channels).  Parameters, in order: per material baseColor r, g, b,
 * roughness (before the 0.0134..1 remap), metallic, specular (Lambertian
 * materials use only baseColor); then per light instance power r, g, b.
 * zgl_diff_backward returns d(sum(d_image * image)) / d(params) by path
 * replay with detached sampling, pdfs, MIS weights and Russian roulette;
 * visibility changes are not differentiated.  No counterpart in the
 * reference. */
typedef struct zgl_diff zgl_diff;

zgl_status zgl_diff_create(zgl_scene* scene, const zgl_integrator_params* params, int32_t spp, zgl_diff** out);
zgl_status zgl_diff_param_count(const zgl_diff* diff, int32_t* n);
/* Current parameter values into `out` (host, param_count floats). */
zgl_status zgl_diff_get_params(const zgl_diff* diff, float* out);
/* Writes parameters (host or device array) into the scene: its material
 * records and light tables change for every user of the scene.  Waits for
 * all work queued on the device first (it may read the scene or produce
 * `params`). */
zgl_status zgl_diff_set_params(zgl_diff* diff, const float* params);
/* Renders the image: `image` is a DEVICE buffer of filmW*filmH RGB floats.
 * Besides the per-sample radiance, keeps each path's ray-cast results in
 * device memory (hit triangle and distance of its first 9 bounces, one
 * occlusion bit per light sample) when they fit in 4 GiB, so that the next
 * zgl_diff_backward replays the paths without tracing them again. */
zgl_status zgl_diff_forward(zgl_diff* diff, float* image, void* stream);
/* d_image: DEVICE filmW*filmH RGB adjoint of the image; d_params: DEVICE
 * param_count floats, overwritten with the gradient.  Uses the per-sample
 * radiance and the ray casts kept by the last zgl_diff_forward (bounces past
 * the kept ones, or all of them when the casts did not fit or
 * zgl_diff_set_params ran since, are traced again; the gradient is the same
 * either way up to float atomic order). */
zgl_status zgl_diff_backward(zgl_diff* diff, const float* d_image, float* d_params, void* stream);

/* One inverse-rendering step of the image loss
 *   loss = loss_scale * sum over pixels and channels of (image - target)^2
 * (new, no counterpart in the reference): zgl_diff_forward into `image`,
 * the loss and dloss/dimage = 2 loss_scale (image - target) in one
 * elementwise kernel, then zgl_diff_backward of that adjoint, all queued on
 * `stream` with no host synchronisation.  d_params receives the gradient,
 * `loss` one float.  target and image are device float[H*W*3]. */
zgl_status zgl_diff_step_l2(zgl_diff* diff, const float* target, float loss_scale, float* image,
                            float* d_params, float* loss, void* stream);
zgl_status zgl_diff_destroy(zgl_diff* diff);

/* ------------------------------------------------------------------------ */
/* Display                                                                   */
/* ------------------------------------------------------------------------ */

/* The reference's display pass (src/shader/post_proc.glsl, set up in
 * Application.cpp:361-363, 652-660): out = pow(tone(clamp(frame * result_scale,
 * 0, 1e30)), 1/2.2) per channel, alpha 1.  tone_mapper: 0 none, 1 filmic,
 * 2 ACES.  `frame` is a DEVICE RGBA32F film of (width / preview_scale) x
 * (height / preview_scale) texels (preview_scale 1 = full size; the reference's
 * preview frame); `out` a DEVICE RGBA32F image of width x height.  Output
 * pixel (x, y) reads texel (x / s, y / s); a texel past the film reads as 0.
 * Asynchronous on `stream`. */
zgl_status zgl_postprocess(const float* frame, int32_t width, int32_t height, int32_t preview_scale,
                           float result_scale, int32_t tone_mapper, float* out, void* stream);

/* ------------------------------------------------------------------------ */
/* Measurement                                                               */
/* ------------------------------------------------------------------------ */

/* L2 read bandwidth of the current device in GB/s: a `bytes`-sized buffer
 * (a multiple of 16 in [1 MiB, 1 GiB]; keep it below the L2 size) is read
 * `passes` times by all SMs with 16-byte L1-bypassing loads after two
 * untimed passes; CUDA events time the passes on `stream`.  Synchronous.
 * The traversal roofline uses it as the L2 peak.  No counterpart in the
 * reference. */
zgl_status zgl_measure_l2_read(size_t bytes, int32_t passes, double* gbs, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ZGL_H */
