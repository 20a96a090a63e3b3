/*
 * rendu_gb300 -- C-ABI of the GB300 (sm_103a) BVH raycaster and offline path tracer.
 *
 * This is the drop-in boundary for Rendu's offline rendering path. Every entry point
 * replaces one member of the reference's C++ API (cited per function as file:line of
 * kosua20/Rendu) with a batched, device-backed equivalent:
 *
 *   Raycaster  (src/engine/raycaster/Raycaster.hpp:51-97)  ->  rt_*
 *   PathTracer (src/apps/pathtracer/PathTracer.hpp:18-29)   ->  pt_*
 *
 * Conventions
 *  - Plain pointers and sizes only; no C++ or framework types cross this boundary.
 *  - Every call returns an int status (RT_OK == 0). The reference reports errors with
 *    log lines and early returns (PathTracer.cpp:162-168); here they are status codes,
 *    and rt_last_error() gives the message of the calling thread's last failure.
 *  - Host pointers are the default: the library copies inputs in and results out on its
 *    own stream, and the call returns when the results are in host memory. With
 *    RT_FLAG_DEVICE_PTRS the ray/hit/image pointers are CUDA device pointers and the work
 *    is ordered on `stream` (a cudaStream_t passed as void*; NULL is the CUDA default
 *    stream, as everywhere in CUDA); rt_* queries then return without waiting.
 *  - Matrices are 4x4 column-major float[16] (glm layout), NULL meaning identity.
 *  - A context is bound to the CUDA device given at creation. Calls on one context must
 *    not overlap from several host threads, and device-pointer queries on one context
 *    must be ordered on one stream.
 */
#ifndef RENDU_GB300_H
#define RENDU_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define RT_API __attribute__((visibility("default")))
#else
#define RT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------- */
#define RT_OK 0
#define RT_ERR_ARG 1     /* invalid argument (null pointer, bad index, bad size)          */
#define RT_ERR_OOM 2     /* device or host allocation failed                               */
#define RT_ERR_CUDA 3    /* a CUDA runtime call failed                                     */
#define RT_ERR_TIMEOUT 4 /* a bounded device loop gave up (status word set by the kernel) */
#define RT_ERR_STATE 5   /* call out of order (e.g. intersect before update_hierarchy)    */
#define RT_ERR_OVERFLOW 6 /* a device traversal stack or queue exceeded its capacity       */

/* ---- flags -------------------------------------------------------------------------- */
#define RT_FLAG_DEVICE_PTRS 0x1u /* ray/hit/image pointers are device pointers (async)   */

/* Marks a miss in rt_hit.prim. */
#define RT_NO_HIT 0xFFFFFFFFu

/* A ray: origin + [tmin, tmax] distance window + direction (need not be normalised;
 * the library normalises it exactly as Ray::Ray does, Intersection.cpp:3-5). 32 bytes.
 * The window is the (mini, maxi) pair of Raycaster::intersects (Raycaster.hpp:64);
 * the reference defaults are tmin = 1e-4f, tmax = 1e8f. */
typedef struct rt_ray {
    float ox, oy, oz, tmin;
    float dx, dy, dz, tmax;
} rt_ray;

/* A closest-hit record, 16 bytes. Replaces Raycaster::Hit (Raycaster.hpp:16-42):
 *   hit    = (prim != RT_NO_HIT)
 *   dist   = t          (FLT_MAX on a miss, like Hit::Hit())
 *   u, v   = barycentrics, w = 1 - u - v
 *   prim   = global triangle id in addMesh order; rt_prim_info() maps it back to
 *            (meshId, localId) with localId = 3 * triangle index inside the mesh. */
typedef struct rt_hit {
    float t, u, v;
    uint32_t prim;
} rt_hit;

/* Build / memory statistics of a context. */
typedef struct rt_stats {
    uint64_t triangles;
    uint64_t vertices;
    uint64_t meshes;
    uint64_t nodes;       /* inner nodes of the device hierarchy                         */
    uint64_t leaves;
    uint64_t device_bytes; /* bytes held by the hierarchy + triangle arrays              */
    float build_ms;       /* device time of the last rt_update_hierarchy                 */
    float sah_cost;       /* surface-area cost of the hierarchy (traversal quality)      */
} rt_stats;

typedef struct rt_ctx rt_ctx;

/* Create a raycaster on CUDA device `device`. Replaces Raycaster::Raycaster()
 * (Raycaster.hpp:46). */
RT_API int rt_create(rt_ctx **ctx, int device);

/* Release all device and host memory of the context. */
RT_API int rt_destroy(rt_ctx *ctx);

/* Append a triangle mesh, its vertices transformed by `model` (skipped when NULL or the
 * identity, as at Raycaster.cpp:22-26). positions: vertex_count x 3 floats; indices:
 * index_count uint32 (a multiple of 3, each < vertex_count). *mesh_id receives the mesh
 * index (addMesh call order). Replaces Raycaster::addMesh (Raycaster.cpp:14-52). */
RT_API int rt_add_mesh(rt_ctx *ctx, const float *positions, size_t vertex_count, const uint32_t *indices,
                size_t index_count, const float *model, uint32_t *mesh_id);

/* Build the device hierarchy over every mesh added so far. Replaces
 * Raycaster::updateHierarchy (Raycaster.cpp:54-142); the hierarchy differs (a 4-wide GPU
 * hierarchy: a Morton radix tree for one mesh, locally-ordered clustering for several, with
 * surface-area leaf collapsing and 4-wide conversion) but every query answers the same. */
RT_API int rt_update_hierarchy(rt_ctx *ctx);

/* Closest hit for n rays. Replaces Raycaster::intersects(origin, direction, mini, maxi)
 * (Raycaster.cpp:144-185) for a batch. Ties at exactly equal distance go to the smaller
 * prim id (the reference keeps the first found in its own traversal order). With host
 * buffers the call reports device-side failures itself; with RT_FLAG_DEVICE_PTRS it returns
 * before the kernel has run, and rt_get_status reports them (as for rt_intersect_any,
 * rt_visible and rt_count_visits). */
RT_API int rt_intersect(rt_ctx *ctx, const rt_ray *rays, size_t n, rt_hit *hits, void *stream, uint32_t flags);

/* Occlusion for n rays: occluded[i] = 1 if any triangle is hit inside (tmin, tmax).
 * Replaces Raycaster::intersectsAny (Raycaster.cpp:187-224). */
RT_API int rt_intersect_any(rt_ctx *ctx, const rt_ray *rays, size_t n, uint8_t *occluded, void *stream, uint32_t flags);

/* Segment visibility for n point pairs: segs is n x 6 floats {p0.xyz, p1.xyz};
 * visible[i] = 1 when nothing is hit between them. Replaces Raycaster::visible
 * (Raycaster.cpp:226-230): window (1e-4, |p1 - p0|). */
RT_API int rt_visible(rt_ctx *ctx, const float *segs, size_t n, uint8_t *visible, void *stream, uint32_t flags);

/* Largest batch rt_visible_noalloc accepts. */
#define RT_NOALLOC_MAX_SEGMENTS 262144

/* rt_visible for callers that cannot allocate device memory (cudaMalloc forbidden or too
 * slow where they run: fixed-budget frame loops and callbacks, plugin hosts that own every
 * allocation, code that must avoid the implicit synchronisation of cudaMalloc/cudaFree).
 * No counterpart in the reference (its Raycaster::visible is a single CPU query).
 * segs (n x 6 floats) and visible (n bytes) are DEVICE pointers; the work is ordered on
 * `stream` (NULL = CUDA default stream) and the call returns without waiting. The call
 * allocates nothing: its scratch (converted rays, fetch counter) is one static device
 * array of 8 MiB + 256 B that every GPU loading the library holds until exit, so n must not
 * exceed RT_NOALLOC_MAX_SEGMENTS (RT_ERR_ARG otherwise). All calls share that array: calls
 * that overlap on the GPU race and must be serialised by the caller. The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress, once per device); make
 * it before any stream capture. A traversal stack overflow (only possible under
 * rt_set_traversal_stack) is recorded in the context's status word for asynchronous calls:
 * rt_get_status(ctx, stream, ...) reports it as RT_ERR_OVERFLOW. */
RT_API int rt_visible_noalloc(rt_ctx *ctx, const float *segs, size_t n, uint8_t *visible, void *stream);

/* Map a global triangle id to (meshId, localId) as stored in Raycaster::Hit. */
RT_API int rt_prim_info(const rt_ctx *ctx, uint32_t prim, uint32_t *mesh_id, uint32_t *local_id);

/* The Raycaster::Hit fields meshId and localId (Raycaster.hpp:16-30, set at
 * Raycaster.cpp:177-179) for a batch of closest hits from rt_intersect: mesh_ids[i] = the
 * addMesh index of the hit triangle's mesh, local_ids[i] = 3 x its triangle index inside that
 * mesh (the first index of the triangle in the mesh's own index buffer); both RT_NO_HIT on a
 * miss. Either output may be NULL. Host buffers by default; device buffers with
 * RT_FLAG_DEVICE_PTRS (ordered on `stream`, returns without waiting). */
RT_API int rt_hit_info(rt_ctx *ctx, const rt_hit *hits, size_t n, uint32_t *mesh_ids, uint32_t *local_ids,
                       void *stream, uint32_t flags);

/* Failures the device found during asynchronous calls. The reference logs and returns
 * (PathTracer.cpp:162-168); here host-buffer calls return RT_ERR_OVERFLOW / RT_ERR_TIMEOUT
 * themselves, while calls that return without waiting (RT_FLAG_DEVICE_PTRS queries on the
 * caller's stream, rt_visible_noalloc) record them in a status word of the context. This
 * call waits for `stream`, returns RT_ERR_OVERFLOW (a traversal stack overflowed: the
 * affected rays ended early) or RT_ERR_TIMEOUT (a bounded device loop gave up) if any such
 * call since the last rt_get_status failed, else RT_OK, puts the raw bits in *word (may be
 * NULL) and clears them. */
RT_API int rt_get_status(rt_ctx *ctx, void *stream, uint32_t *word);

/* Cap the traversal stack of the queries at `entries` (1..256; 0 = automatic, the exact
 * bound of the current hierarchy, which never overflows). The queries then run the smallest
 * compiled stack (2, 64 or 256 entries) that holds the cap; rays that need more stop early
 * and the call reports RT_ERR_OVERFLOW. A diagnostic: it lets tests and callers exercise the
 * overflow path, which the automatic bound never reaches. */
RT_API int rt_set_traversal_stack(rt_ctx *ctx, uint32_t entries);

/* Statistics of the current hierarchy. */
RT_API int rt_get_stats(const rt_ctx *ctx, rt_stats *out);

/* Count, for each ray, the inner nodes and triangles the device traversal visits
 * (closest-hit mode). node_visits / tri_visits are n uint32 each (host or device per
 * flags). Used to state the algorithmic bytes per ray of the roofline. */
RT_API int rt_count_visits(rt_ctx *ctx, const rt_ray *rays, size_t n, uint32_t *node_visits, uint32_t *tri_visits,
                    void *stream, uint32_t flags);

/* Hierarchy inspection (the geometry of RaycasterVisualisation::getAllLevels,
 * RaycasterVisualisation.cpp:9-33, for this library's own hierarchy): the box of every node
 * in breadth-first order, the root's first. boxes: count x 6 floats {lo.xyz, hi.xyz}; info:
 * count x 2 int32 {depth (root 0), triangles (0 for an inner node, > 0 for a leaf)}. At most
 * `capacity` entries are written; *count receives the total (NULL arrays: count only). */
RT_API int rt_hierarchy_boxes(const rt_ctx *ctx, float *boxes, int32_t *info, size_t capacity, size_t *count);

/* The boxes one ray enters, in visiting order, and its closest hit
 * (RaycasterVisualisation::getRayLevels, RaycasterVisualisation.cpp:35-81): a host walk of
 * the device hierarchy with the device traversal's order and arithmetic; *hit equals what
 * rt_intersect returns for the ray. boxes / info / capacity / count as rt_hierarchy_boxes. */
RT_API int rt_ray_levels(const rt_ctx *ctx, const rt_ray *ray, float *boxes, int32_t *info, size_t capacity,
                         size_t *count, rt_hit *hit);

/* Message of the calling thread's last failed call ("" if none). */
RT_API const char *rt_last_error(void);

/* ======================================================================================
 * Path tracer
 * ====================================================================================== */

/* Material types, numbered as Material::Type (src/engine/scene/Material.hpp:68-80). The
 * path tracer shades Emissive as an emitter and every other type as the Lambert+GGX
 * Regular material (PathTracer.cpp:228-276). */
#define PT_MAT_REGULAR 1
#define PT_MAT_EMISSIVE 8

/* Background modes, numbered as Scene::Background (src/engine/scene/Scene.hpp:70-75). */
#define PT_BG_COLOR 0
#define PT_BG_IMAGE 1
#define PT_BG_SKYBOX 2
#define PT_BG_ATMOSPHERE 3

/* Light types (src/engine/scene/lights/). */
#define PT_LIGHT_POINT 0
#define PT_LIGHT_DIRECTIONAL 1
#define PT_LIGHT_SPOT 2

/* One mesh with the per-vertex attributes the path tracer reads (Mesh.hpp:126-132).
 * normals/tangents/bitangents: vertex_count x 3 floats (required); texcoords:
 * vertex_count x 2 floats or NULL (an object whose mesh has no texcoords does not use
 * them, Object.cpp:4-8). */
typedef struct pt_mesh_desc {
    const float *positions;
    const float *normals;
    const float *tangents;
    const float *bitangents;
    const float *texcoords;
    size_t vertex_count;
    const uint32_t *indices;
    size_t index_count;
} pt_mesh_desc;

/* A material: its type, alpha masking and three textures ids from pt_scene_add_texture:
 * tex[0] albedo+alpha (or emitted colour), tex[1] normal map, tex[2] roughness/metalness/AO
 * (Material.hpp:12-16). */
typedef struct pt_material_desc {
    int32_t type;
    int32_t masked;
    uint32_t tex[3];
} pt_material_desc;

/* An analytic light (PointLight.cpp:68-87, DirectionalLight.cpp:40-44, SpotLight.cpp:52-78).
 * Spot angles are the (inner, outer) half angles in radians. */
typedef struct pt_light_desc {
    int32_t type;
    int32_t cast_shadows;
    float color[3];
    float position[3];
    float direction[3];
    float radius;
    float inner_angle, outer_angle;
} pt_light_desc;

/* A pinhole camera as Camera::pose + projection (Camera.cpp:10-25); the image-plane
 * corner and steps are derived as in Camera::pixelShifts (Camera.cpp:42-49). */
typedef struct pt_camera_desc {
    float eye[3];
    float center[3];
    float up[3];
    float fov;   /* vertical field of view, radians (default 1.3) */
    float ratio; /* width / height */
} pt_camera_desc;

/* Kernel classes of pt_render_stats.kernel_ms. */
#define PT_KERNEL_RAYGEN 0     /* wave set-up and camera rays                              */
#define PT_KERNEL_TRACE 1      /* closest-hit traversal of the path rays                   */
#define PT_KERNEL_SHADE 2      /* hit shading, light sampling, next rays                   */
#define PT_KERNEL_SHADOW 3     /* shadow rays (any hit, or the walk through cut-outs)       */
#define PT_KERNEL_ACCUMULATE 4 /* per-pixel accumulation of the wave's samples             */
#define PT_KERNEL_KINDS 5

/* Per-render counters. rays = primary + bounce + shadow rays cast. */
typedef struct pt_render_stats {
    uint64_t primary_rays;
    uint64_t bounce_rays;
    uint64_t shadow_rays;
    uint64_t paths;
    float device_ms;
    float kernel_ms[PT_KERNEL_KINDS]; /* device time of each kernel class, measured with CUDA
                                         events between the launches when the render ran with
                                         pt_render_options.profile (else 0)                  */
} pt_render_stats;

typedef struct pt_scene pt_scene;

/* Create an empty scene on CUDA device `device`. */
RT_API int pt_scene_create(pt_scene **scene, int device);
RT_API int pt_scene_destroy(pt_scene *scene);

/* Add a float image (width x height x channels, row-major, channels 1..4) used as a
 * texture; sampled with bilinear wrap filtering as Image::rgbal (Image.cpp:86-106). */
RT_API int pt_scene_add_texture(pt_scene *scene, uint32_t width, uint32_t height, uint32_t channels, const float *pixels,
                         uint32_t *tex_id);
RT_API int pt_scene_add_mesh(pt_scene *scene, const pt_mesh_desc *mesh, uint32_t *mesh_id);
RT_API int pt_scene_add_material(pt_scene *scene, const pt_material_desc *mat, uint32_t *material_id);
/* Add an object (Object.hpp:25): mesh + material + model matrix. */
RT_API int pt_scene_add_object(pt_scene *scene, uint32_t mesh_id, uint32_t material_id, const float *model,
                        uint32_t *object_id);
RT_API int pt_scene_add_light(pt_scene *scene, const pt_light_desc *light);
/* COLOR: color[3] used; IMAGE: tex[0]; SKYBOX: tex[0..5] = +x,-x,+y,-y,+z,-z faces
 * (Texture.cpp:141-191); ATMOSPHERE: color[3] = the sun direction (normalised, as Sky does,
 * Sky.cpp:16,35), the sky of MaterialSky::eval (MaterialSky.cpp:6-87) seen by every miss. */
RT_API int pt_scene_set_background(pt_scene *scene, int32_t mode, const float *color, const uint32_t *tex);

/* ATMOSPHERE's scattering table, width x height RGBA floats (x = relative height, y =
 * cosine of the sun's vertical angle). NULL restores the default: the table the reference
 * ships (resources/common/scattering-precomputed.exr), i.e. AtmosphereApp::precomputeTable
 * (AtmosphereApp.cpp:145-188) at 512 x 512 with 256 steps, in half precision, computed on
 * the device at commit. */
RT_API int pt_scene_set_sky_table(pt_scene *scene, const float *rgba, uint32_t width, uint32_t height);

/* Upload the scene and build its raycaster: every object's mesh is added in object order
 * (so meshId == object index) and the hierarchy is built. Replaces
 * PathTracer::PathTracer(scene) (PathTracer.cpp:11-21). */
RT_API int pt_scene_commit(pt_scene *scene);

/* Render `samples` (rounded to a power of two as at PathTracer.cpp:169-173) paths of at
 * most `depth` segments per pixel and ACCUMULATE the normalised result into `image`
 * (width x height x components floats, components >= 3, RGB in the first three), as
 * PathTracer::render(camera, samples, depth, image) does (PathTracer.cpp:159-299):
 * image.rgb = (image.rgb + sum_s min(L_s, 5)) / spp. `seed` selects the random sequence.
 * Host pointer by default; device pointer with RT_FLAG_DEVICE_PTRS (work ordered on
 * `stream`). The call returns when the image is final. */
RT_API int pt_render(pt_scene *scene, const pt_camera_desc *camera, uint32_t samples, uint32_t depth, uint64_t seed,
              float *image, uint32_t width, uint32_t height, uint32_t components, void *stream, uint32_t flags);

/* Estimators of pt_render_ex. */
#define PT_MODE_REFERENCE 0 /* PathTracer::render's estimator, as pt_render                        */
#define PT_MODE_EXTENDED 1  /* + next-event estimation on emissive triangles and on the environment
                               map, each combined with BSDF sampling by multiple importance sampling
                               (power heuristic); no counterpart in the reference                  */

typedef struct pt_render_options {
    int32_t mode;  /* PT_MODE_REFERENCE or PT_MODE_EXTENDED                                      */
    float clamp;   /* per-sample radiance clamp; the reference uses 5 (PathTracer.cpp:288);
                      <= 0 disables it                                                            */
    int32_t accum_fp64; /* accumulate the samples of each pixel in double precision (for
                           high-spp reference images); the image itself stays float       */
    float *aov;    /* optional feature buffer, width x height x 8 floats (host or device like
                      the image): first-hit albedo (rgb), shading normal (xyz), distance,
                      averaged over the pixel's samples, and the standard error of the
                      pixel's mean luminance (Rec. 709 weights, of the clamped samples:
                      sqrt((E[L^2] - E[L]^2) / spp)); overwritten, not accumulated        */
    uint32_t ranks; /* pixel split over cooperating processes (one per GPU): 0 or 1 renders
                       every pixel; otherwise the image's pixels (row-major) form tiles of
                       PT_RANK_TILE_PIXELS and tile k belongs to rank k % ranks. This call
                       renders the tiles of `rank` only, as pt_render would, and sets every
                       component of every other pixel (and its aov entries) to 0, so that
                       the element-wise sum of all ranks' images is the whole render, bit
                       for bit. The reference splits rows over threads instead
                       (System::forParallel, System.hpp:72-104, PathTracer.cpp:186). */
    uint32_t rank;  /* this process's rank, < ranks                                       */
    int32_t profile; /* nonzero: launch every wave's kernels directly instead of the captured
                        CUDA graph, with CUDA events between them, and report the time of
                        each kernel class in pt_render_stats.kernel_ms (slower)            */
} pt_render_options;

/* Pixels per tile of the pt_render_options rank split. */
#define PT_RANK_TILE_PIXELS 4096

/* Environment map for PT_MODE_EXTENDED: an equirectangular float image (texture id from
 * pt_scene_add_texture; u = phi / 2pi with phi = atan2(z, x), v = theta / pi from +y),
 * scaled by `intensity`. It replaces the background for every miss in that mode and is
 * importance-sampled by luminance x sin(theta). No counterpart in the reference, whose
 * backgrounds are COLOR / IMAGE / SKYBOX / ATMOSPHERE (Scene.hpp:70-75). */
RT_API int pt_scene_set_environment(pt_scene *scene, uint32_t tex_id, float intensity);

/* pt_render with options (NULL = the reference estimator, clamp 5). */
RT_API int pt_render_ex(pt_scene *scene, const pt_camera_desc *camera, uint32_t samples, uint32_t depth, uint64_t seed,
                        float *image, uint32_t width, uint32_t height, uint32_t components,
                        const pt_render_options *options, void *stream, uint32_t flags);

/* ---- batched rendering ---------------------------------------------------------------
 * Many renders of different scenes, resolutions, sample counts and depths in one call:
 * their pixels x samples are cut into tiles and packed into shared waves; one CUDA graph
 * launch loops over the waves on the device (a conditional while node whose body is the
 * whole per-wave launch sequence: ray generation, the persistent traversal, shading, shadow
 * rays, accumulation). Each job's image is exactly
 * what pt_render of that job alone gives (same random stream, same summation order). No
 * counterpart in the reference, which renders one image per PathTracer::render call. */
typedef struct pt_batch pt_batch;

typedef struct pt_batch_job {
    pt_scene *scene; /* committed scene                                                */
    pt_camera_desc camera;
    uint32_t samples, depth;
    uint64_t seed;
    float *image; /* width x height x components floats, accumulated into as pt_render  */
    uint32_t width, height, components;
} pt_batch_job;

/* Wave capacity (paths), pixels per tile, most samples of a pixel in one wave. */
typedef struct pt_batch_tuning {
    uint32_t wave_paths, tile_pixels, max_samples;
} pt_batch_tuning;

RT_API int pt_batch_create(pt_batch **batch, int device);
RT_API int pt_batch_destroy(pt_batch *batch);

/* Render all jobs (host images, or device images with RT_FLAG_DEVICE_PTRS on `stream`);
 * returns when every image is final. tuning NULL: the cached autotuned values for this
 * device if any, else defaults. */
RT_API int pt_batch_render(pt_batch *batch, const pt_batch_job *jobs, size_t n, const pt_render_options *options,
                           const pt_batch_tuning *tuning, void *stream, uint32_t flags);

/* Time the batch (images discarded) under candidate tunings, one parameter at a time
 * (samples per wave, wave capacity, tile size, samples per wave again), cache the fastest
 * for this device in `cache_path` (NULL: $RENDU_GB300_TUNING, else
 * ~/.cache/rendu_gb300/batch_tuning.json) and return it in *out. */
RT_API int pt_batch_autotune(pt_batch *batch, const pt_batch_job *jobs, size_t n, const pt_render_options *options,
                             const char *cache_path, pt_batch_tuning *out);

/* Counters of the last pt_batch_render. */
RT_API int pt_batch_get_stats(const pt_batch *batch, pt_render_stats *out);

/* Counters of the last pt_render on this scene. */
RT_API int pt_get_render_stats(const pt_scene *scene, pt_render_stats *out);

/* MaterialGGX::eval (src/apps/pathtracer/MaterialGGX.cpp:94-101) for n cases on device
 * `device`: cases = n x 11 floats {wo.xyz, base.rgb, roughness, metalness, wi.xyz} (local
 * frame, host memory); out = n x 3 floats. */
RT_API int pt_material_eval(const float *cases, size_t n, float *out, int device);

/* MaterialGGX::sampleAndEval (MaterialGGX.cpp:54-92) for n cases on device `device`:
 * cases = n x 8 floats {wo.xyz, base.rgb, roughness, metalness}; uniforms = n x 3 floats,
 * the three numbers the reference draws (lobe choice, then the two lobe coordinates);
 * out = n x 6 floats {weight.rgb, wi.xyz}. */
RT_API int pt_material_sample(const float *cases, const float *uniforms, size_t n, float *out, int device);

/* Write a render to disk as the reference's command-line renderer does after
 * PathTracer::render (main.cpp:106-119): a path ending in ".exr" gets the linear image as
 * half-precision channels (Image::saveAsHDR, Image.cpp:162-290; at least 16 x 16 pixels);
 * any other path a PNG of 8-bit sRGB-approximated values (Image::saveAsLDR, Image.cpp:
 * 126-160: v^(1/2.2), 255 v clamped and truncated; alpha 255), after the tone map
 * 1 - exp(-c) of main.cpp:109-116 when `tonemap` != 0. image: width x height x components
 * floats (host; 3 or 4 components for PNG, 1 to 4 for EXR). */
RT_API int pt_image_save(const float *image, uint32_t width, uint32_t height, uint32_t components, const char *path,
                         int32_t tonemap);

/* Scene textures: the scanline filters of a PNG (sub)image undone on the host, the step of
 * the PNG decoding behind Image::loadLDR (Image.cpp:291-333) that is sequential along each
 * row. filtered: rows x (1 + row_bytes) bytes, a filter type byte (0..4) before each row;
 * pixel_bytes: bytes per complete pixel (1 for bit depths below 8); out: rows x row_bytes.
 * RT_ERR_ARG for a filter type above 4. */
RT_API int pt_png_unfilter(const uint8_t *filtered, uint32_t rows, uint32_t row_bytes, uint32_t pixel_bytes,
                           uint8_t *out);

/* Scene textures: decode a JPEG file held in memory (Image::loadLDR, Image.cpp:291-333, reads
 * .jpg / .jpeg textures through stb_image): sequential or progressive Huffman JPEG with 1 or 3
 * components, as width x height x channels bytes (channels 1..4: grey, grey + alpha, RGB,
 * RGBA with alpha 255). With out == NULL only *width and *height are filled. RT_ERR_ARG for
 * data it does not decode (arithmetic coding, lossless, 12-bit, CMYK) or a small buffer. */
RT_API int pt_jpeg_decode(const uint8_t *data, size_t size, uint32_t channels, uint8_t *out, size_t out_capacity,
                          uint32_t *width, uint32_t *height);

/* AtmosphereApp::precomputeTable on device `device`: res x res RGBA floats into `out` (host),
 * `samples` march steps, rounded to half precision when half_precision != 0. */
RT_API int pt_sky_table(uint32_t res, uint32_t samples, int32_t half_precision, float *out, int device);

/* MaterialSky::eval (MaterialSky.cpp:6-87) for n cases on device `device`: cases = n x 9
 * floats {ray origin.xyz, normalised direction.xyz, normalised sun direction.xyz} (host);
 * out = n x 3 radiance. table = width x height RGBA floats, or NULL for the default table. */
RT_API int pt_sky_eval(const float *table, uint32_t width, uint32_t height, const float *cases, size_t n, float *out,
                       int device);

/* The raycaster built by pt_scene_commit (PathTracer::raycaster(), PathTracer.hpp:29). */
RT_API rt_ctx *pt_scene_raycaster(pt_scene *scene);

/* ==== Learned denoiser (dn_*) ==============================================================
 * No counterpart in the reference (its only image filter is the real-time bilateral blur of
 * src/engine/processing/BilateralBlur.cpp:7-11): a U-Net that maps a few-sample render and
 * its first-hit feature buffers to a converged image, trained here on path-tracer output.
 *
 * Network: 5 levels of two 3x3 convolutions + ReLU with 32, 48, 64, 96, 128 channels, 2x2
 * max pooling down, nearest 2x upsampling + skip concatenation up, a final 3x3 convolution to
 * 16 channels of which the first 3 are a correction of log(1 + radiance). Activations are
 * NHWC BF16, accumulation FP32 (tensor-core implicit GEMMs); master weights FP32.
 * Features: per pixel DN_FEATURES floats {radiance rgb, albedo rgb, normal xyz, distance,
 * standard error of the mean luminance} (pt_render's image + its 8-float feature buffer).
 * Output: max(exp(log(1 + radiance) + correction) - 1, 0), so a zero correction returns the
 * input radiance exactly. Images of any size are padded to multiples of 16 for inference;
 * training crops must be multiples of 16.
 * Parameters (flat FP32): for each layer in dn_layer order, weights [3][3][cin][cout]
 * (tap-major: tap = 3 dy + dx over the 3x3 window, then input, then output channel)
 * followed by bias [cout]. Loss: the relative squared error ((x - t) / (x' + 0.01))^2 of
 * the output x against the target t, averaged over pixels and channels, x' being x held
 * constant (the relative RMSE the output is judged by; unbiased for noisy targets).
 * Optimiser: Adam. */
#define DN_FEATURES 11
typedef struct dn_net dn_net;

typedef struct dn_layer {
    uint32_t cin0;   /* channels of the first input (half resolution when up0)          */
    uint32_t cin1;   /* channels of the concatenated skip input (0: none)                */
    uint32_t cout;
    int32_t up0;     /* 1: first input upsampled 2x (nearest)                            */
    int32_t relu;
    int32_t level;   /* resolution level: width and height divided by 2^level            */
    uint64_t weight_offset; /* into the flat parameter vector                            */
    uint64_t bias_offset;
} dn_layer;

/* Create the network on `device` with He-initialised parameters (seed 0). */
RT_API int dn_create(dn_net **out, int device);
RT_API int dn_destroy(dn_net *net);
/* Re-initialise parameters (He normal, seeded) and reset the optimiser state. */
RT_API int dn_init(dn_net *net, uint64_t seed);
RT_API int dn_layer_count(const dn_net *net, uint32_t *count);
RT_API int dn_layer_info(const dn_net *net, uint32_t layer, dn_layer *out);
RT_API int dn_param_count(const dn_net *net, size_t *count);
/* Host copies of the FP32 parameters / the last computed gradients (count = dn_param_count). */
RT_API int dn_get_params(dn_net *net, float *out, size_t count);
RT_API int dn_set_params(dn_net *net, const float *in, size_t count); /* also resets Adam */
RT_API int dn_get_grads(dn_net *net, float *out, size_t count);
/* The gradient buffer for data-parallel training (each process computes the gradients of its
 * share of a batch with dn_backward, the processes sum them, dn_adam_step applies them):
 * dn_read_grads copies the last gradients to `out`, dn_write_grads replaces them with `in`
 * (count = dn_param_count floats). Device pointers with RT_FLAG_DEVICE_PTRS (ordered on
 * `stream`, asynchronous); host pointers otherwise (blocking). */
RT_API int dn_read_grads(dn_net *net, float *out, size_t count, void *stream, uint32_t flags);
RT_API int dn_write_grads(dn_net *net, const float *in, size_t count, void *stream, uint32_t flags);

/* Denoise `batch` images: features (batch, height, width, DN_FEATURES) -> out (batch,
 * height, width, 3) radiance. Host pointers by default (blocking); device pointers with
 * RT_FLAG_DEVICE_PTRS (ordered on `stream`). */
RT_API int dn_denoise(dn_net *net, const float *features, uint32_t width, uint32_t height, uint32_t batch, float *out,
                      void *stream, uint32_t flags);
/* Loss and parameter gradients for one batch of crops (width, height multiples of 16):
 * target (batch, height, width, 3) converged radiance. *loss (may be NULL: no read-back,
 * no synchronisation for device pointers) receives the loss. */
RT_API int dn_backward(dn_net *net, const float *features, const float *target, uint32_t width, uint32_t height,
                       uint32_t batch, float *loss, void *stream, uint32_t flags);
/* One Adam step (beta 0.9, 0.999, eps 1e-8) with learning rate lr on the last gradients,
 * ordered on `stream` (NULL: on the network's own stream after all work already queued on
 * the device, including the legacy default stream's; the call blocks). */
RT_API int dn_adam_step(dn_net *net, float lr, void *stream);
/* dn_backward + dn_adam_step. */
RT_API int dn_train_step(dn_net *net, const float *features, const float *target, uint32_t width, uint32_t height,
                         uint32_t batch, float lr, float *loss, void *stream, uint32_t flags);

/* One 3x3 convolution layer on device buffers, ordered on `stream` (the network's building
 * block, exported for tests and custom networks). Input: x0 (batch, height >> up0, width >>
 * up0, c0) BF16 NHWC, then x1 (batch, height, width, c1) BF16 (NULL when c1 = 0), channels
 * concatenated; weights BF16 [3][3][c0 + c1][cout]; bias FP32 [cout] or NULL. out (batch,
 * height, width, cout) BF16, or FP32 when out_fp32. c0, c1, cout multiples of 8; pointers
 * 16-byte aligned. */
RT_API int dn_conv3x3(const void *x0, uint32_t c0, int32_t up0, const void *x1, uint32_t c1, uint32_t batch,
                      uint32_t height, uint32_t width, const void *weights, const float *bias, uint32_t cout,
                      int32_t relu, void *out, int32_t out_fp32, void *stream);
/* Gradients of dn_conv3x3 (without bias or ReLU) for the output gradient gy (batch, height,
 * width, cout) BF16: dx (batch, height, width, c0 + c1) FP32 with respect to the
 * concatenated, upsampled input (NULL: skipped) and dw [3][3][c0 + c1][cout] FP32 (NULL:
 * skipped); weights FP32 [3][3][c0 + c1][cout]. Scratch is allocated on `stream`. */
RT_API int dn_conv3x3_backward(const void *x0, uint32_t c0, int32_t up0, const void *x1, uint32_t c1, uint32_t batch,
                               uint32_t height, uint32_t width, const float *weights, uint32_t cout, const void *gy,
                               float *dx, float *dw, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* RENDU_GB300_H */
