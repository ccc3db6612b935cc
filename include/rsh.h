/*
 * rsh.h — C ABI of the GB300 (sm_103a) ray-space-hierarchy (CRSH) secondary-ray pipeline.
 *
 * This is the drop-in boundary for the CUDA-Engine per-frame path of nuno-tiago-reis/ray-tracer.
 * The reference exports plain `extern "C"` wrappers taking raw device pointers
 * (projects/CUDA-Engine/source/RayTracer.cu:2042-3301, redeclared in main.cpp:192-590).
 * Each entry point below names the wrapper (or host routine) it replaces.
 *
 * Conventions (all entry points):
 *  - Plain C types only: raw device pointers, sizes, host structs passed by pointer.
 *  - Every call returns an rsh_status and never exits the process (the reference called
 *    Utility::checkCUDAError -> exit(1), Utility.h:72-81).
 *  - Every call that launches work takes an explicit stream; NULL means the legacy default stream.
 *  - Counts produced on the GPU stay on the GPU (a device `uint32_t*`); the reference instead did a
 *    blocking cudaMemcpy of one count after most stages (RayTracer.cu:2316, 2364, 2649, 2720, 2832).
 *  - The caller owns inputs and outputs; the context owns its scratch buffers, which it allocates
 *    from an HBM budget (RSH_ERR_OOM past the budget).
 *  - One context per host thread; several contexts may share a device.
 */
#ifndef RSH_H
#define RSH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* rsh_stream_t; /* a cudaStream_t */

typedef enum rsh_status {
    RSH_OK = 0,
    RSH_ERR_OOM = 1,       /* allocation failed or HBM budget exceeded */
    RSH_ERR_OVERFLOW = 2,  /* a bounded buffer (candidates, keys) was too small */
    RSH_ERR_TIMEOUT = 3,   /* a bounded device-side wait (decoupled look-back) gave up */
    RSH_ERR_INVALID = 4,   /* bad argument */
    RSH_ERR_CUDA = 5       /* a CUDA runtime call failed; see rsh_last_error_string */
} rsh_status;

/* Key of an empty ray slot (a pixel with no surface, or a back-facing light). Valid keys use at most
 * 31 bits, so they never equal this value. The reference used a separate head flag of 1 for "no ray"
 * (RayTracer.cu:739). */
#define RSH_KEY_NONE 0xFFFFFFFFu
/* Closest-hit record of a ray that hit nothing. */
#define RSH_HIT_NONE 0xFFFFFFFFFFFFFFFFull
/* Shadow flag of an occluded ray (RayTracer.cu:1611 stores UINT_MAX). Unoccluded = 0. */
#define RSH_OCCLUDED 0xFFFFFFFFu

/* A ray: origin (already offset by epsilon along the direction, as the reference does before every
 * test, RayTracer.cu:1607, 1765), the accepted parameter interval (tmin, tmax) and a unit direction.
 * 32 bytes, two 16-byte halves. */
typedef struct rsh_ray {
    float o[3];
    float tmin;
    float d[3];
    float tmax;
} rsh_ray;

/* A ray-space-hierarchy node: a sphere holding every ray origin below it, a cone holding every
 * direction, and `reach`, a bound on how far from the sphere centre any ray below it can travel
 * (infinity for unbounded rays). Replaces the 2 x float4 node of RayTracer.cu:1105-1107. */
typedef struct rsh_node {
    float c[3];
    float radius;
    float axis[3];
    float cos_spread;   /* <= 0 means "wider than a half-space": the cone test always passes */
    float sin_spread;
    float reach;
    uint32_t first;     /* first sorted ray index covered */
    uint32_t count;     /* rays covered (0 = empty node) */
} rsh_node;

/* Object-sphere-hierarchy node as exported for inspection: the reference's
 * {centre, radius, firstTri, lastTri} record (main.cpp:2455-2459) extended with its children. */
typedef struct rsh_object_node {
    float c[3];
    float radius;
    uint32_t first_tri;   /* in cluster order */
    uint32_t tri_count;
    uint32_t first_child; /* index into the next lower level; leaves: 0 */
    uint32_t child_count; /* leaves: 0 */
} rsh_object_node;

/* Hash parameters: key = tag | morton3(origin cell) | morton2(octahedral direction bin).
 * cell[i] = clamp(floor((o[i] - lo[i]) * scale[i]), 0, 2^grid_bits - 1). */
typedef struct rsh_hash_params {
    float lo[3];
    float scale[3];
    uint32_t grid_bits;  /* 1..10 bits per axis */
    uint32_t dir_log2;   /* 2^dir_log2 octahedral bins per axis, 1..6 */
    uint32_t tag_bits;   /* bits reserved above the hash for the light / segment tag */
    uint32_t key_bits;   /* tag_bits + 3*grid_bits + 2*dir_log2, at most 31 */
} rsh_hash_params;

/* Point light (main.cpp:2596-2623: position, colour, diffuse and specular intensity). */
typedef struct rsh_light {
    float position[3];
    float color[3];
    float diffuse_intensity;
    float specular_intensity;
} rsh_light;

/* Pinhole camera as the engine keeps it (Camera.cpp:91-133): eye, direction scaled by the target
 * distance, right scaled by the half width, up scaled by the half height. The primary ray of pixel
 * (x, y) is normalize(direction + right*(x/W - 0.5) + up*(y/H - 0.5)) (RayTracer.cu:666-667). */
typedef struct rsh_camera {
    float eye[3];
    float direction[3];
    float right[3];
    float up[3];
} rsh_camera;

/* Material (main.cpp:2432-2441): diffuse rgb + reflectance in w; specular rgb + shininess in w. */
typedef struct rsh_material {
    float diffuse[4];
    float specular[4];
} rsh_material;

/* Scene description in host memory. Triangle soup: triangle i has vertices positions[3i..3i+2]
 * (float4, w ignored) and vertex normals normals[3i..3i+2]; the engine packs every object into this
 * layout (main.cpp:2398-2427). */
typedef struct rsh_scene_desc {
    const float* positions;      /* float4 x 3 per triangle */
    const float* normals;        /* float4 x 3 per triangle (NULL: flat normals) */
    const uint32_t* material_ids;/* one per triangle (NULL: all 0) */
    const uint32_t* object_ids;  /* one per triangle (NULL: all 0) */
    const rsh_material* materials;
    uint32_t triangle_count;
    uint32_t material_count;
} rsh_scene_desc;

/* Runtime configuration; replaces the compile-time macros of Constants.h:9-29. */
typedef struct rsh_config {
    uint32_t grid_bits;        /* hash origin grid bits per axis (default 4) */
    uint32_t dir_log2;         /* hash direction bins per axis, log2 (default 6) */
    uint32_t packet_size;      /* rays per hierarchy leaf: 8, 16 or 32 (default 8; Constants.h:29) */
    uint32_t cluster_size;     /* most triangles per object-hierarchy leaf: 1..64 (default 6; batched form <= 32) */
    float epsilon;             /* ray offset (default 0.01; RayTracer.cu:34) */
    uint64_t hbm_budget;       /* bytes the context may allocate (0: 90% of free memory) */
    uint64_t candidate_capacity; /* plain-path traversal candidates per pass (0: automatic) */
    uint32_t flags;            /* RSH_FLAG_* */
    float reflect_jitter;      /* 0: mirror reflections; >0: cosine-lobe perturbation weight */
    uint32_t seed;             /* seed of the reflection perturbation */
    uint32_t ray_level;        /* batched form: object-tree level at and below which rays leave their packet
                                  and descend one by one (0: packets down to the clusters; at or above the tree depth:
                                  from the root, no packet phase, no ray hierarchy; default 15) */
    uint32_t plain_ray_level;  /* plain per-frame path: object-tree level at and below which the traversal
                                  emits per-ray candidates (0: packet candidates only; default 4) */
    uint32_t fused_blocks;     /* batched form: CTAs of the persistent traversal launch per SM (0: as many
                                  as fit, the default; fewer share each SM's L1 among fewer rays) */
} rsh_config;

#define RSH_FLAG_STAGE_TIMERS 1u   /* record per-stage CUDA events (TestManager timers) */
#define RSH_FLAG_FUSED 2u          /* rsh_render_frame traces each bounce through the batched form */
/* rsh_render_frame casts 16 shadow rays per light from the reference's soft-shadow grid around the light
 * and shades with its sample weights and log2(1 + 2 s) factor (SOFT_SHADOWS, RayTracer.cu:1550-1603,
 * 1680-1696); shadow slots per pixel = lights x 16. Each sample is traced exactly (the reference tests the
 * samples only against the centre ray's candidate triangles). */
#define RSH_FLAG_SOFT_SHADOWS 8u
/* Batched form: sort the hashed slots directly instead of their runs of equal keys (no compression or
 * decompression), for incoherent batches whose keys hardly repeat; rsh_autotune_scenes tries both. */
#define RSH_FLAG_NO_COMPRESS 16u
/* Batched form: every ray is traced by one lane from its first step to its last. By default, once a warp
 * of the rays-only kernel has no ray left to take and at most 16 of its lanes still trace one, its idle
 * lanes take subtrees (stack entries) of those rays, which shortens launches that would end on a few long
 * rays (scenes with long sight lines); results are the same either way. The default costs the steps about
 * 4% (the kernel runs at its register limit) and changes the node and triangle test counts through the
 * order the hits are met in; with this flag the counts equal a sequential traversal's, ray by ray, and
 * scenes whose launches end evenly run faster. */
#define RSH_FLAG_SEQUENTIAL_RAYS 32u
#define RSH_FLAG_RAH 4u            /* plain path: ray-hierarchy ablation without hashing/sorting: packets
                                      of consecutive trimmed rays (the reference's algorithm 1 "RAH",
                                      main.cpp:1016-1037) */

/* Per-frame statistics (TestManager::dump, TestManager.cpp:229-313, as a struct). */
typedef struct rsh_frame_stats {
    uint64_t primary_rays;
    uint64_t shadow_rays;        /* traced after trimming, all bounces */
    uint64_t reflection_rays;    /* traced after trimming, all bounces */
    uint64_t chunks;             /* compressed runs, all secondary batches */
    uint64_t candidates;         /* (packet, cluster) pairs emitted by traversal */
    uint64_t node_tests;         /* node tests executed (packet-node x sphere; a single ray x node box);
                                    rsh_render_frame: secondary rays only */
    uint64_t tri_tests;          /* ray x triangle tests executed (rsh_render_frame: secondary rays only) */
    float secondary_ms;          /* first secondary raygen .. last secondary intersection */
    float frame_ms;
    float stage_ms[12];          /* see RSH_STAGE_* */
    uint32_t overflow_passes;    /* traversal restarts after a full candidate buffer */
} rsh_frame_stats;

enum {
    RSH_STAGE_PRIMARY = 0, RSH_STAGE_RAYGEN = 1, RSH_STAGE_COMPRESS = 2, RSH_STAGE_SORT = 3,
    RSH_STAGE_DECOMPRESS = 4, RSH_STAGE_BUILD = 5, RSH_STAGE_TRAVERSE = 6, RSH_STAGE_INTERSECT = 7,
    RSH_STAGE_SHADE = 8, RSH_STAGE_COUNT = 9
};

typedef struct rsh_ctx rsh_ctx;
typedef struct rsh_scene rsh_scene;

/* ---------------------------------------------------------------- context, memory, errors */

void rsh_config_default(rsh_config* cfg);
/* Creates a context on the current device. Replaces the global state set up by init()/reshape()
 * (main.cpp:2343-2659, 1371-1520) and MemoryPreparationWrapper (RayTracer.cu:2093-2157). */
rsh_status rsh_create(const rsh_config* cfg, rsh_ctx** out);
rsh_status rsh_destroy(rsh_ctx* ctx);
rsh_status rsh_get_config(const rsh_ctx* ctx, rsh_config* out);
rsh_status rsh_set_config(rsh_ctx* ctx, const rsh_config* cfg);
const char* rsh_last_error_string(void);
/* Device error word (bounded waits that timed out, buffer overflows) raised since the last reset. */
rsh_status rsh_check_device_errors(rsh_ctx* ctx, rsh_stream_t stream);

/* Self-test of the device-side wait limit: runs one sort pass whose first tile never publishes its
 * look-back status, so the second tile's wait can only end by giving up after spin_limit polls
 * (1..4,194,304; a few thousand take a few milliseconds). Returns RSH_ERR_TIMEOUT when the wait gave up
 * and reported it as designed (the context stays usable, the error word is cleared), anything else on a
 * failure of the mechanism. No counterpart in the reference, whose kernels never wait on each other. */
rsh_status rsh_selftest_wait_timeout(rsh_ctx* ctx, uint32_t spin_limit, rsh_stream_t stream);
uint64_t rsh_bytes_allocated(const rsh_ctx* ctx);

/* Small helpers so that callers without a CUDA runtime binding can move data. */
rsh_status rsh_malloc(void** ptr, size_t bytes);
rsh_status rsh_free(void* ptr);
rsh_status rsh_malloc_host(void** ptr, size_t bytes);   /* pinned */
rsh_status rsh_free_host(void* ptr);
rsh_status rsh_memcpy_h2d(void* dst, const void* src, size_t bytes, rsh_stream_t stream);
rsh_status rsh_memcpy_d2h(void* dst, const void* src, size_t bytes, rsh_stream_t stream);
rsh_status rsh_memset(void* dst, int value, size_t bytes, rsh_stream_t stream);
rsh_status rsh_stream_create(rsh_stream_t* out);
rsh_status rsh_stream_destroy(rsh_stream_t s);
rsh_status rsh_stream_synchronize(rsh_stream_t s);
rsh_status rsh_device_synchronize(void);
/* Elapsed milliseconds of `fn`-free timing: events recorded on `stream`. */
rsh_status rsh_event_create(void** ev);
rsh_status rsh_event_destroy(void* ev);
rsh_status rsh_event_record(void* ev, rsh_stream_t stream);
rsh_status rsh_event_elapsed(void* start, void* stop, float* ms);
int rsh_device_count(void);
int rsh_sm_count(void);
/* Free and total memory of the current device (cudaMemGetInfo), e.g. to size an HBM budget. */
rsh_status rsh_device_memory(uint64_t* free_bytes, uint64_t* total_bytes);
/* Number of this library's kernels launched by this process so far (all contexts). */
uint64_t rsh_kernel_launches(void);

/* ---------------------------------------------------------------- scene, lights, camera */

/* Uploads a scene and builds its object-sphere hierarchy on the GPU (synchronous).
 * Replaces the flat-array packing + cudaMalloc/H2D + texture binds of main.cpp:2374-2586 and the
 * per-mesh Miniball spheres of BoundingSphere.cpp:9-63. */
rsh_status rsh_scene_upload(rsh_ctx* ctx, const rsh_scene_desc* desc, rsh_scene** out);

/* A scene read from a Wavefront OBJ file (+ its MTL files), in host memory, ready for rsh_scene_upload:
 * desc's arrays are float4 x 3 per triangle (w = 1 for positions, 0 for normals), one material id and one
 * object id per triangle; material 0 is the reader's default (0.75 grey, shininess 100), the MTL file's
 * materials follow in file order with their Kd, Ks, Ns and reflectance 0.5. */
typedef struct rsh_obj_data {
    rsh_scene_desc desc;
    uint32_t object_count;  /* "o" / "g" groups that hold faces */
    void* owner;            /* internal */
} rsh_obj_data;

/* Reads an OBJ file: v, vn, f (v, v/vt, v//vn, v/vt/vn; 1-based or negative indices; polygons fanned into
 * triangles), o/g, mtllib (relative to the OBJ file), usemtl. Faces without normals get their geometric
 * normal. Replaces OBJ_Reader::loadMesh / loadMaterial (OBJ_Reader.cpp:60-389, 395-470), which read
 * triangles only and stored zero normals where the file had none. Host only; free with rsh_obj_free. */
rsh_status rsh_obj_load(const char* obj_path, rsh_obj_data** out);
void rsh_obj_free(rsh_obj_data* data);
rsh_status rsh_scene_destroy(rsh_ctx* ctx, rsh_scene* scene);
/* Scene bounds (exact min/max over all vertices). */
/* Per-frame object transforms: every vertex of object k (rsh_scene_desc.object_ids; objects = 1 + the
 * largest id) is multiplied by model_matrices[16k..16k+15] and every normal by normal_matrices[16k..]
 * (NULL: the model matrix; normals renormalised), row-major, out[i] = sum_j M[4i + j] v[j] -- UpdateVertex
 * (RayTracer.cu:448-511) as main.cpp:1131-1196 drives it. Transforms apply to the pose uploaded first
 * (the rest pose), not to the previous frame's; the scene bounds and the object-sphere hierarchy are then
 * rebuilt on the GPU (replacing UpdateBoundingSphere, :513-570). */
rsh_status rsh_scene_set_transforms(rsh_ctx* ctx, rsh_scene* scene, const float* model_matrices,
                                    const float* normal_matrices, uint32_t object_count, rsh_stream_t stream);

/* Rebuilds the scene's bounds and object-sphere hierarchy from its current triangles with the context's
 * cluster_size (rsh_scene_upload and rsh_scene_set_transforms call it). Replaces the per-object
 * BoundingSphere::calculateMiniball (BoundingSphere.cpp:9-63) of the engine's init. */
rsh_status rsh_build_object_hierarchy(rsh_ctx* ctx, rsh_scene* scene, rsh_stream_t stream);
rsh_status rsh_scene_bounds(const rsh_scene* scene, float lo[3], float hi[3]);
uint32_t rsh_scene_triangle_count(const rsh_scene* scene);
/* Object hierarchy inspection: level 0 = leaves (triangle clusters). */
uint32_t rsh_scene_levels(const rsh_scene* scene);
uint32_t rsh_scene_level_size(const rsh_scene* scene, uint32_t level);
rsh_status rsh_scene_get_level(const rsh_scene* scene, uint32_t level, rsh_object_node* host_out);
/* Original triangle id of each cluster-order slot (host copy). */
rsh_status rsh_scene_get_order(const rsh_scene* scene, uint32_t* host_out);
/* The scene's single-ray box tree (built with the object hierarchy; the batched form's rays-only traversal
 * descends it): returns its slot count (slot 0 unused) and writes its root's stack entry; copies its slots
 * (2 float4 each: padded box lo + link word, hi + count word) and its triangles (3 float4 each, in the
 * tree's depth-first order, w of the first = original id bits) to host memory when the pointers are not
 * NULL. An 8-wide tree built by PLOC clustering: no counterpart in the reference, whose rays test
 * per-triangle bounding spheres (CreateTriangleBoundingSphere, RayTracer.cu:301-376). */
uint32_t rsh_scene_box_tree(const rsh_scene* scene, uint32_t* root, float* host_boxes, float* host_tris);
/* Device pointers for stage-level calls: cluster-order vertices (3 float4 per triangle, w of the
 * first = original id bits) and the per-level sphere arrays. */
const void* rsh_scene_device_triangles(const rsh_scene* scene);

/* Replaces the light packing + bind*Texture calls (main.cpp:2596-2656). At most 8 lights. */
rsh_status rsh_lights_set(rsh_ctx* ctx, const rsh_light* lights, uint32_t count);
/* Replaces the camera uniforms passed to every wrapper (eye/direction/right/up, Camera.cpp:91-133). */
rsh_status rsh_camera_set(rsh_ctx* ctx, const rsh_camera* camera);
/* Builds the engine camera from eye/target/up and a vertical field of view in degrees, the way
 * Camera::loadView does (Camera.cpp:108-133). */
rsh_status rsh_camera_look_at(const float eye[3], const float target[3], const float up[3],
                              float fov_degrees, uint32_t width, uint32_t height, rsh_camera* out);

/* ---------------------------------------------------------------- the per-frame path */

/* Renders one frame headless: primary rays, then `depth` bounces of shadow + reflection batches, each
 * through hash -> compress -> sort -> decompress -> build -> traverse -> intersect, then shading into
 * `rgba_out` (device, width*height uint32 RGBA8). Replaces display() stages 2-4 (main.cpp:1077-1303)
 * with the GL rasteriser replaced by a primary ray cast. rgba_out may be NULL (no shading). */
rsh_status rsh_render_frame(rsh_ctx* ctx, const rsh_scene* scene, uint32_t width, uint32_t height,
                            uint32_t depth, uint32_t* rgba_out, rsh_stream_t stream);
/* Statistics of the last rsh_render_frame (synchronises the stream it ran on). */
rsh_status rsh_frame_stats_get(rsh_ctx* ctx, rsh_frame_stats* out);
/* The context's test counters, accumulated by every traversal and intersection since the last reset
 * (rsh_render_frame resets them): node tests and ray x triangle tests, the work the reference's
 * TestManager totals count (TestManager.cpp:276-281). Waits for `stream`; reset != 0 then zeroes them. */
rsh_status rsh_test_counters(rsh_ctx* ctx, uint64_t* node_tests, uint64_t* tri_tests, int32_t reset,
                             rsh_stream_t stream);
/* Device buffers of the last frame, for parity checks: per-bounce closest-hit records and shadow
 * flags. Sizes: width*height and width*height*lights. bounce < depth; bounce -1 = primary hits. */
rsh_status rsh_frame_hits(rsh_ctx* ctx, int32_t bounce, uint64_t* host_out);
rsh_status rsh_frame_shadow(rsh_ctx* ctx, int32_t bounce, uint32_t* host_out);
rsh_status rsh_frame_rays(rsh_ctx* ctx, int32_t bounce, int32_t shadow, rsh_ray* host_out);
rsh_status rsh_frame_surface(rsh_ctx* ctx, int32_t bounce, float* host_pos, float* host_nrm);

/* Writes an RGBA8 image (host memory) as PNG (stored deflate blocks). */
rsh_status rsh_write_png(const char* path, const uint32_t* rgba, uint32_t width, uint32_t height);

/* ---------------------------------------------------------------- stage-level entry points */

rsh_status rsh_hash_params_make(const float lo[3], const float hi[3], uint32_t grid_bits,
                                uint32_t dir_log2, uint32_t tag_bits, rsh_hash_params* out);

/* Primary (camera) rays in 8x8 pixel-tile order, tile rows from the image's middle outwards (rows m, m-1,
 * m+1, m-2, ... with m = tile rows / 2; the longest primary rays, usually in the view's centre band, are
 * traced first): ray k belongs to pixel pixel_of_ray[k] (0xFFFFFFFF: padding of a partial tile, no ray).
 * Replaces the GL rasteriser of the G-buffer (FrameBuffer.cpp:55-140). */
rsh_status rsh_raygen_primary(const rsh_camera* cam, uint32_t width, uint32_t height,
                              rsh_ray* rays, uint32_t* pixel_of_ray, rsh_stream_t stream);

/* Shadow rays with their hash keys. Slot of (pixel x, y, light l) = x + W*(l + L*y)
 * (RayTracer.cu:700-702). surface_pos.w != 0 marks a surface; surface_nrm.xyz its normal.
 * Replaces ShadowRayCreationWrapper / CreateShadowRays (RayTracer.cu:2210-2241, 682-740). */
rsh_status rsh_raygen_shadow(const float* surface_pos, const float* surface_nrm, uint32_t width,
                             uint32_t height, const rsh_light* lights_host, uint32_t light_count,
                             float epsilon, const rsh_hash_params* hp, rsh_ray* rays, uint32_t* keys,
                             rsh_stream_t stream);

/* Soft-shadow rays: 16 per (pixel, light) from the 4x4 grid around the light without its centre
 * (RayTracer.cu:1550-1599). Slot of (x, y, light l, sample k) = x + W*((16 l + k) + 16 L y); sample k =
 * i + 4 j sits at light + axis0 (a - 2) / 8 + axis1 (b - 2) / 8 with a = i, b = j skipping 2; the hash tag
 * is 16 l + k, so hp->tag_bits must cover 16 L. Rays exist where the centre ray of rsh_raygen_shadow does. */
rsh_status rsh_raygen_soft_shadow(const float* surface_pos, const float* surface_nrm, uint32_t width,
                                  uint32_t height, const rsh_light* lights_host, uint32_t light_count,
                                  float epsilon, const rsh_hash_params* hp, rsh_ray* rays, uint32_t* keys,
                                  rsh_stream_t stream);

/* Reflection rays from a surface buffer. prev_rays == NULL: the surface is the primary G-buffer and
 * the incident direction is (p - eye); otherwise it is prev_rays[slot].d (the ray that hit it).
 * jitter > 0 perturbs the mirror direction by a cosine lobe (seeded per slot and bounce).
 * Replaces CreateReflectionRays (RayTracer.cu:742-791) and the ray-creation half of
 * ColorAndCreateReflectionRay (RayTracer.cu:1995-2016). */
rsh_status rsh_raygen_reflect(const float* surface_pos, const float* surface_nrm,
                              const rsh_ray* prev_rays, const float eye[3], uint32_t width,
                              uint32_t height, float epsilon, float jitter, uint32_t seed,
                              uint32_t bounce, const rsh_hash_params* hp, rsh_ray* rays,
                              uint32_t* keys, rsh_stream_t stream);

/* Refraction rays from a surface buffer: direction refract(i, n, eta) by GLSL's formula (eta = 1/1.52 in
 * the reference), i = normalize(p - eye) (prev_rays == NULL) or prev_rays[slot].d; no ray where the
 * formula gives total internal reflection. Replaces CreateRefractionRays (RayTracer.cu:793-842), which
 * the reference creates but never casts; the hash is the one of every other ray (the reference's
 * CreateRefractionRayIndex, :200-227, hashes atan2(x, x), a constant). */
rsh_status rsh_raygen_refract(const float* surface_pos, const float* surface_nrm, const rsh_ray* prev_rays,
                              const float eye[3], uint32_t width, uint32_t height, float epsilon, float eta,
                              const rsh_hash_params* hp, rsh_ray* rays, uint32_t* keys, rsh_stream_t stream);

/* Hash of arbitrary rays; rays with tmax <= tmin get RSH_KEY_NONE. tag goes above the hash bits. */
rsh_status rsh_hash(const rsh_ray* rays, uint32_t n, const rsh_hash_params* hp, uint32_t tag,
                    uint32_t* keys, rsh_stream_t stream);

/* Trim + compress (reduce-then-scan over 4096-slot tiles): keeps slots whose key != RSH_KEY_NONE in slot
 * order (trimmed_ids = their slot indices), and cuts the trimmed keys into runs of equal keys.
 * Outputs chunk_keys[c], chunk_bases[c] (trimmed index of the run head; chunk_bases[C] = R) and, if
 * non-NULL, chunk_sizes[c]; counts[0] = R (rays), counts[1] = C (chunks), device memory.
 * Replaces RayTrimmingWrapper + RayCompressionWrapper (RayTracer.cu:2276-2383) and kernels
 * CreateTrimmedRays / CreateChunkFlags / CreateChunkBases / CreateChunkSizes (:844-991). */
rsh_status rsh_compress(rsh_ctx* ctx, const uint32_t* keys, uint32_t n_slots, uint32_t* trimmed_ids,
                        uint32_t* chunk_keys, uint32_t* chunk_bases, uint32_t* chunk_sizes,
                        uint32_t* counts, rsh_stream_t stream);

/* rsh_compress without allocating: same outputs and semantics, no context, no cudaMalloc/cudaFree.
 * For callers that may not allocate device memory themselves or let a library do it: hosts that own and
 * pre-partition all device memory, and loops that allocate once at start-up and must not allocate while
 * they run. No counterpart in the reference. The scratch (per-tile summaries and prefixes) is a static
 * device array of 196,684 bytes that every GPU loading the library keeps until the process exits;
 * n_slots above 16,777,216 is rejected with RSH_ERR_INVALID. The
 * first call on a device looks up the array's device address (call it once before any stream capture);
 * that address is kept for the process, so a cudaDeviceReset of that device invalidates it.
 * All calls share the array: calls that overlap on the GPU race, so serialise them on one stream. */
rsh_status rsh_compress_noalloc(const uint32_t* keys, uint32_t n_slots, uint32_t* trimmed_ids,
                                uint32_t* chunk_keys, uint32_t* chunk_bases, uint32_t* chunk_sizes,
                                uint32_t* counts, rsh_stream_t stream);

/* Stable LSD radix sort (onesweep) of (key, value) pairs by the low key_bits bits of the key.
 * n = *d_count if d_count != NULL (device), else n_max. vals_in == NULL means values 0..n-1.
 * Replaces RaySortingWrapper / cub::DeviceRadixSort::SortPairs (RayTracer.cu:2385-2409). */
rsh_status rsh_sort_pairs(rsh_ctx* ctx, const uint32_t* keys_in, const uint32_t* vals_in,
                          uint32_t* keys_out, uint32_t* vals_out, uint32_t n_max,
                          const uint32_t* d_count, uint32_t key_bits, rsh_stream_t stream);

/* Expands sorted chunks back to rays: sorted_ids[k] = trimmed_ids[chunk_bases[v] + j] for the j-th
 * ray of the chunk at sorted position x (v = sorted_chunk_vals[x]); sorted_keys likewise (nullable).
 * counts = the device counts written by rsh_compress. Replaces RayDecompressionWrapper
 * (RayTracer.cu:2411-2467), CreateSortedRaySkeleton and CreateSortedRays (:993-1059). */
rsh_status rsh_decompress(rsh_ctx* ctx, const uint32_t* sorted_chunk_keys,
                          const uint32_t* sorted_chunk_vals, const uint32_t* chunk_bases,
                          const uint32_t* trimmed_ids, const uint32_t* counts, uint32_t max_rays,
                          uint32_t* sorted_keys, uint32_t* sorted_ids, rsh_stream_t stream);

/* Node capacity of a 3-level hierarchy over up to max_rays rays: level offsets into one node array. */
uint32_t rsh_hierarchy_capacity(uint32_t max_rays, uint32_t packet_size, uint32_t offsets[4]);

/* Builds the ray-space hierarchy: level 0 = packets of packet_size consecutive sorted rays, level 1 =
 * 8 packets, level 2 = 64 packets. sorted_ids == NULL: identity. n = *d_count (device) or max_rays.
 * Replaces HierarchyCreationWrapper (RayTracer.cu:2469-2535), CreateHierarchyLevel0/N (:1061-1150).*/
rsh_status rsh_build_rsh(const rsh_ray* rays, const uint32_t* sorted_ids, uint32_t max_rays,
                         const uint32_t* d_count, uint32_t packet_size, rsh_node* nodes,
                         rsh_stream_t stream);

/* Hierarchy-vs-hierarchy traversal: every (packet, cluster) pair whose packet node passes the
 * sphere/cone test against the cluster and all its ancestors is written to candidates as
 * (uint64)packet << 32 | cluster, in no particular order; *d_cand_count (device) receives the count.
 * Returns RSH_ERR_OVERFLOW if more than capacity pairs exist (the first capacity are kept).
 * Replaces HierarchyTraversalWarmUpWrapper + HierarchyTraversalWrapper (RayTracer.cu:2537-2852). */
rsh_status rsh_traverse(rsh_ctx* ctx, const rsh_scene* scene, const rsh_node* nodes,
                        uint32_t max_rays, const uint32_t* d_count, uint32_t packet_size,
                        uint64_t* candidates, uint64_t capacity, uint64_t* d_cand_count,
                        rsh_stream_t stream);

/* Any-hit (shadow) intersection of the candidates: flags[slot] = RSH_OCCLUDED for every ray with a
 * hit in (tmin, tmax); untouched otherwise (caller zeroes). Replaces ShadowRayIntersectionWrapper /
 * CalculateShadowRayIntersections (RayTracer.cu:2874-2925, 1498-1614). */
rsh_status rsh_intersect_any(const rsh_scene* scene, const rsh_ray* rays, const uint32_t* sorted_ids,
                             uint32_t max_rays, const uint32_t* d_count, uint32_t packet_size,
                             const uint64_t* candidates, const uint64_t* d_cand_count,
                             uint32_t* flags, rsh_stream_t stream);

/* Closest-hit intersection: hits[slot] = min over candidates of (float bits of t) << 32 | original
 * triangle id, by 64-bit atomicMin (caller fills with RSH_HIT_NONE). Replaces
 * ReflectionRayIntersectionWrapper / CalculateReflectionRayIntersections (RayTracer.cu:2977-3031,
 * 1711-1774), whose 32-bit key quantised t to 0.1 (RayTracer.cu:1770). */
rsh_status rsh_intersect_closest(const rsh_scene* scene, const rsh_ray* rays,
                                 const uint32_t* sorted_ids, uint32_t max_rays,
                                 const uint32_t* d_count, uint32_t packet_size,
                                 const uint64_t* candidates, const uint64_t* d_cand_count,
                                 uint64_t* hits, rsh_stream_t stream);

/* Resolves closest hits into a surface buffer (position.w = 1 on a hit, normal.w = material id bits).
 * Replaces the hit-point / barycentric-normal half of ColorReflectionRay (RayTracer.cu:1806-1843). */
rsh_status rsh_resolve_hits(const rsh_scene* scene, const rsh_ray* rays, const uint64_t* hits,
                            const uint32_t* pixel_of_ray, uint32_t n, float* surface_pos,
                            float* surface_nrm, rsh_stream_t stream);

/* Ray-by-ray trace through the whole pipeline (hash .. intersect) of an arbitrary ray set:
 * closest-hit records (any_hit == 0) or shadow flags (any_hit != 0), indexed like `rays`.
 * Rays with tmax <= tmin are skipped. Output buffers are filled by the call. */
rsh_status rsh_trace_rays(rsh_ctx* ctx, const rsh_scene* scene, const rsh_ray* rays, uint32_t n,
                          int any_hit, uint64_t* hits, uint32_t* flags, rsh_stream_t stream);

/* ---------------------------------------------------------------- batched form */

/* One batch segment: n rays (device) against a resident scene. */
typedef struct rsh_batch_segment {
    const rsh_scene* scene;
    const rsh_ray* rays;
    uint32_t n;
    int any_hit;
    uint64_t* hits;     /* closest-hit output (any_hit == 0) */
    uint32_t* flags;    /* shadow output (any_hit != 0) */
} rsh_batch_segment;

/* Traces many ray batches of uneven size over several resident scenes: one hash, one compress, one
 * sort and one decompress over all segments (the segment index is the key's tag), one hierarchy
 * build, then ONE persistent fused traversal + intersection launch. Without host synchronisation,
 * so the whole call can be captured in a CUDA graph (rsh_batch_graph_*). */
rsh_status rsh_batch_trace(rsh_ctx* ctx, const rsh_batch_segment* segments, uint32_t count,
                           rsh_stream_t stream);
/* Captures rsh_batch_trace for a fixed segment list into a CUDA graph; replays with _launch. */
rsh_status rsh_batch_graph_create(rsh_ctx* ctx, const rsh_batch_segment* segments, uint32_t count,
                                  rsh_stream_t stream, void** graph_exec);
rsh_status rsh_batch_graph_launch(void* graph_exec, rsh_stream_t stream);
rsh_status rsh_batch_graph_destroy(void* graph_exec);
/* Statistics of the last rsh_batch_trace (synchronises): reflection_rays = rays traced, chunks, node and
 * triangle tests, and with RSH_FLAG_STAGE_TIMERS stage_ms (RAYGEN = gather + hash, COMPRESS, SORT,
 * DECOMPRESS, BUILD, TRAVERSE = the fused traversal + intersection launch). */
rsh_status rsh_batch_stats_get(rsh_ctx* ctx, rsh_frame_stats* out);

/* Autotuner: times rsh_batch_trace on `segments` for each (grid_bits, dir_log2, packet_size) in the
 * given lists and stores the fastest in the context's configuration (and in *best). */
rsh_status rsh_autotune(rsh_ctx* ctx, const rsh_batch_segment* segments, uint32_t count,
                        const uint32_t* grid_bits, uint32_t n_grid, const uint32_t* dir_log2,
                        uint32_t n_dir, const uint32_t* packet_sizes, uint32_t n_packet,
                        rsh_stream_t stream, rsh_config* best);

/* Per-scene tuning of the batched form (rsh_batch_trace, its graphs and the server): origin-grid bits,
 * direction bins (dir_log2) and the object-tree level at which rays leave their packets (at or above the
 * tree's depth for every segment of a batch: the rays-only kernel, no ray hierarchy built). A field equal
 * to RSH_TUNE_DEFAULT takes the context's value. The plain per-frame path ignores it. No counterpart in
 * the reference (its hash has no parameters, RayTracer.cu:147-198). */
#define RSH_TUNE_DEFAULT 0xFFFFFFFFu
typedef struct rsh_scene_tuning {
    uint32_t grid_bits;   /* 1..10 */
    uint32_t dir_log2;    /* 1..6 */
    uint32_t ray_level;   /* 0..15 */
} rsh_scene_tuning;
rsh_status rsh_scene_set_tuning(rsh_scene* scene, const rsh_scene_tuning* tuning);
rsh_status rsh_scene_get_tuning(const rsh_scene* scene, rsh_scene_tuning* out);

/* Search space of rsh_autotune_scenes. Any list may be empty (that parameter stays as it is). */
typedef struct rsh_tune_space {
    const uint32_t* grid_bits;    uint32_t n_grid;
    const uint32_t* dir_log2;     uint32_t n_dir;
    const uint32_t* ray_levels;   uint32_t n_ray_level;
    const uint32_t* packet_sizes; uint32_t n_packet;
    uint32_t reps;                /* timed repetitions per point after one warm-up (0: 2) */
    const uint32_t* fused_blocks; uint32_t n_fused_blocks;  /* CTAs per SM of the traversal launch */
} rsh_tune_space;
/* Per-scene autotuner: coordinate descent over the space. The packet size (shared by every segment of a
 * batch) is chosen on the whole batch; then, for each distinct scene, grid bits, direction bins and the
 * switch level are chosen on that scene's segments alone, one parameter at a time, and stored in the
 * scene (rsh_scene_set_tuning); then every scene at switch level 15 at once is tried against that (the
 * rays-only kernel, which skips the ray hierarchy, runs only when no segment uses packets below the root);
 * last, the packet size, the traversal launch's CTAs per SM, run compression on or off
 * (RSH_FLAG_NO_COMPRESS) and the shared launch ends on or off (RSH_FLAG_SEQUENTIAL_RAYS) are chosen with
 * the scenes tuned. The search keeps the untuned configuration
 * when its result is not faster on the whole batch. Points whose hash does not fit beside the batch's
 * segment tag in 31 bits are skipped. *best_ms (optional) is the whole batch's time with the final
 * choice, *untuned_ms (optional) its time with the context's configuration and no scene tuning. */
rsh_status rsh_autotune_scenes(rsh_ctx* ctx, const rsh_batch_segment* segments, uint32_t count,
                               const rsh_tune_space* space, rsh_stream_t stream, float* best_ms,
                               float* untuned_ms);

/* Ray-by-ray trace through the fused persistent kernel (one segment); same outputs as
 * rsh_trace_rays. */
rsh_status rsh_trace_rays_fused(rsh_ctx* ctx, const rsh_scene* scene, const rsh_ray* rays,
                                uint32_t n, int any_hit, uint64_t* hits, uint32_t* flags,
                                rsh_stream_t stream);

/* ---------------------------------------------------------------- serving */

typedef struct rsh_server rsh_server;

typedef struct rsh_request {
    uint32_t scene_index;     /* index into the scenes given to rsh_server_create */
    rsh_camera camera;
    uint32_t width, height;
    uint32_t depth;           /* bounces, 1..4 */
    uint32_t light_count;     /* 1..8 */
    rsh_light lights[8];
} rsh_request;

typedef struct rsh_request_result {
    uint64_t id;
    int32_t status;           /* rsh_status */
    double submit_ms, start_ms, finish_ms;   /* server clock */
    uint64_t rays;            /* secondary (shadow + reflection) rays traced, after trimming */
} rsh_request_result;

/* A continuous-batching request loop on its own host thread: requests are admitted while their
 * device memory fits the HBM budget; every step traces the next stage (primary rays, or one bounce) of
 * the oldest in-flight requests, up to a ray budget per step (rsh_server_set_step_rays), in one batched
 * launch; requests leave as they finish and new ones join between steps. A finished request keeps its
 * device memory (its results) until rsh_server_wait collects it. */
rsh_status rsh_server_create(rsh_ctx* ctx, const rsh_scene* const* scenes, uint32_t scene_count,
                             uint64_t hbm_budget, uint32_t max_inflight, rsh_server** out);
rsh_status rsh_server_submit(rsh_server* srv, const rsh_request* req, uint64_t* id_out);
/* Device bytes the server reserves for a request while it is in flight (what admission counts against
 * the HBM budget); host arithmetic only. RSH_ERR_INVALID for a request that rsh_server_submit rejects
 * on its own fields (scene index aside): zero size, depth outside 1..4, lights outside 1..8, or
 * width x height x lights of 2^31 or more. */
rsh_status rsh_server_request_bytes(const rsh_request* req, uint64_t* bytes);
/* Waits up to timeout_ms for request `id`; copies its closest-hit records per bounce
 * (depth x width*height) and shadow flags (depth x width*height*lights) if the pointers are
 * non-NULL. RSH_ERR_TIMEOUT if not finished. */
rsh_status rsh_server_wait(rsh_server* srv, uint64_t id, uint32_t timeout_ms,
                           rsh_request_result* result, uint64_t* hits_host, uint32_t* flags_host);
rsh_status rsh_server_cancel(rsh_server* srv, uint64_t id);
/* Rays one step may generate (a stage of width*height primary rays or width*height*(lights + 1) bounce
 * rays per request; at least one request per step), taken oldest first; 0 (the default) = every
 * in-flight request each step. A budget bounds a step's length when requests are large. */
rsh_status rsh_server_set_step_rays(rsh_server* srv, uint64_t rays);
rsh_status rsh_server_stats(rsh_server* srv, uint64_t* completed, uint64_t* steps,
                            uint64_t* peak_inflight, uint64_t* peak_bytes);
rsh_status rsh_server_destroy(rsh_server* srv);

#ifdef __cplusplus
}
#endif

#endif /* RSH_H */
