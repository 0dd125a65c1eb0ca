/*
 * wf_api.h — C ABI of the GB300 wavefront path tracer (libwfgpu.so).
 *
 * This is the drop-in boundary for the per-bounce loop of the CPU renderer
 * fhidargue/wavefront-renderer.  Every entry point below names the reference
 * interface it replaces (file:line in that project).  The reference has no
 * FFI of its own: its loop is a set of C++ types and member functions
 * (WavefrontRenderer, RayQueue, ShadingQueue, EmbreeAccelerator) compiled into
 * one executable.  The C++17 mirror in `wf/wavefront.hpp` presents those types
 * again on top of this ABI.
 *
 * Conventions
 *  - Every function returns an int status: WF_OK (0) or a negative WF_ERR_*.
 *    No C++ exception crosses the ABI.  wf_last_error() gives the message of
 *    the last failure on a context (the reference reported errors through
 *    exceptions caught in main, src/main.cpp:218-222).
 *  - The library owns device memory behind opaque handles; the caller owns
 *    every host buffer it passes.  Calls on one context are externally
 *    serialised (one host thread per context); each context owns one CUDA
 *    stream.
 *  - Host arrays are plain pointers plus element counts.  Float columns are
 *    IEEE binary32, index columns int32, exactly as the reference's
 *    std::vector<float>/std::vector<int> columns.
 */
#ifndef WF_API_H
#define WF_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WF_API_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define WF_OK 0
#define WF_ERR_INVALID_ARGUMENT (-1) /* null pointer, size out of range      */
#define WF_ERR_CUDA (-2)             /* a CUDA runtime call failed            */
#define WF_ERR_OUT_OF_MEMORY (-3)    /* device allocation or HBM budget       */
#define WF_ERR_STATE (-4)            /* e.g. stage called before scene upload */
#define WF_ERR_DEVICE_CHECK (-5)     /* a kernel's own bounds check tripped   */
#define WF_ERR_NO_DEVICE (-6)        /* no CUDA device visible                */
#define WF_ERR_CAPACITY (-7)         /* queue or static buffer too small      */

/* ---- enums mirroring the reference ------------------------------------- */
/* MaterialType, reference include/shading/Material.h:9-17 (same order). */
enum {
    WF_MATERIAL_DIFFUSE = 0,
    WF_MATERIAL_METAL = 1,
    WF_MATERIAL_EMISSIVE = 2,
    WF_MATERIAL_SPOTLIGHT = 3,
    WF_MATERIAL_GLASS = 4,
    WF_MATERIAL_PLASTIC = 5
};

/* SchedulingPolicy, reference include/scheduling/ShadingQueue.h:18-24. */
enum {
    WF_POLICY_NONE = 0,
    WF_POLICY_MATERIAL_AWARE = 1,
    WF_POLICY_TEXTURE_AWARE = 2,
    WF_POLICY_COST_BENEFIT_AWARE = 3
};

/* Texel formats.  RGB32F is the reference's Texture::pixels (linear float
 * RGB, include/shading/Texture.h:19).  RGBA8_SRGB is an 8-bit source that the
 * reference's Texture::load decodes with srgbToLinear (src/shading/Texture.cpp
 * :20-27,47-53); the device keeps the bytes and decodes through a 256-entry
 * table built on the host with that same formula, so sampled values agree bit
 * for bit with the decoded float texture. */
enum { WF_TEXEL_RGB32F = 0, WF_TEXEL_RGBA8_SRGB = 1 };

/* ---- scene description --------------------------------------------------- */

/* Material, reference include/shading/Material.h:19-41 without the uuid
 * string.  48 bytes, the device layout as well. */
typedef struct wf_material {
    int32_t type;               /* WF_MATERIAL_*                          */
    float albedo[3];            /* Material::albedo                       */
    float roughness;            /* Material::roughness                    */
    float emission;             /* Material::emission (strength)          */
    int32_t texture_id;         /* Material::textureID, -1 = none         */
    float ior;                  /* Material::indexOfRefraction            */
    float spot_outer_deg;       /* Material::spotOuterAngle               */
    float spot_falloff_deg;     /* Material::spotFalloffAngle             */
    int32_t use_spatial_checker;/* Material::useSpatialChecker            */
    float checker_cell_size;    /* Material::spatialCheckerCellSize       */
} wf_material;

/* Texture, reference include/shading/Texture.h:15-55. */
typedef struct wf_texture {
    int32_t width;
    int32_t height;
    int32_t format;   /* WF_TEXEL_*                                        */
    const void* data; /* width*height texels, row-major (y*width + x)      */
} wf_texture;

/* EnvironmentMap, reference include/core/EnvironmentMap.h:7-24: equirect
 * float RGB, nearest texel; width == 0 means "not loaded" and the miss path
 * uses the gradient sky of WavefrontRenderer::getSkyColor (.cpp:879-888). */
typedef struct wf_environment {
    int32_t width;
    int32_t height;
    const float* rgb;        /* width*height*3 floats                     */
    float intensity_scale;   /* EnvironmentMap::intensityScale            */
    float tint[3];           /* EnvironmentMap::tint                      */
} wf_environment;

/* DirectionalLight, reference include/core/Scene.h:57-62. */
typedef struct wf_directional_light {
    float direction[3];
    float color[3];
    float intensity; /* 0 disables directional NEE (WavefrontRenderer.cpp:713) */
} wf_directional_light;

/* Scene, reference include/core/Scene.h:14-46 (SceneGeometry flat arrays)
 * plus materials/textures/lights.  Mesh i owns indices
 * [mesh_index_offsets[i], mesh_index_offsets[i] + mesh_index_counts[i]);
 * its triangles are geomID i, primID 0.. in that order (the reference gives
 * each Mesh its own Embree geometry, src/accelerator/Embree.cpp:77-113). */
typedef struct wf_scene_desc {
    int32_t num_vertices;
    const float* positions_x;      /* SceneGeometry::allPositionsX        */
    const float* positions_y;
    const float* positions_z;
    int32_t num_indices;           /* 3 per triangle                       */
    const int32_t* indices;        /* SceneGeometry::allIndices (global)  */
    int32_t num_meshes;
    const int32_t* mesh_index_offsets; /* SceneGeometry::meshIndexOffsets */
    const int32_t* mesh_index_counts;  /* SceneGeometry::meshIndexCounts  */
    const int32_t* mesh_material_ids;  /* SceneGeometry::meshMaterialIDs  */
    /* Mesh::triangleUVsU/V (include/geometry/Mesh.h:11-12), one value per
     * triangle corner, aligned with indices[].  NULL when no mesh has UVs. */
    const float* corner_u;
    const float* corner_v;
    const uint8_t* mesh_has_uv;    /* per mesh; NULL = none has UVs        */
    int32_t num_materials;
    const wf_material* materials;
    int32_t num_textures;
    const wf_texture* textures;
    wf_environment environment;
    wf_directional_light directional;
} wf_scene_desc;

/* Camera, reference include/core/Camera.h:6-41 (its four public fields). */
typedef struct wf_camera {
    float origin[3];
    float top_left[3];
    float horizontal[3];
    float vertical[3];
} wf_camera;

/* ---- render parameters ---------------------------------------------------- */

/* The public fields of WavefrontRenderer (include/render/WavefrontRenderer.h
 * :19-34) that change the image, plus device-only batching fields. */
typedef struct wf_render_params {
    int32_t width;
    int32_t height;
    int32_t samples_per_pixel;     /* samplesPerPixel                       */
    int32_t max_depth;             /* maxDepth                              */
    int32_t rr_min_depth;          /* rrMinDepth (the reference fixes 3)    */
    int32_t policy;                /* WF_POLICY_*                           */
    int32_t enable_ray_sort;       /* enableRaySort                         */
    int32_t enable_cost_aware_rr;  /* enableCostAwareRR (frozen costs)      */
    float firefly_threshold;       /* fireflyThreshold (10)                 */
    uint32_t seed_lo;              /* counter-based RNG key                 */
    uint32_t seed_hi;
    int32_t first_sample;          /* samples [first, first+spp) are drawn  */
    int32_t spp_per_wave;          /* samples per wavefront; 0 = automatic  */
    /* Environment-map next-event estimation with balance-heuristic MIS.
     * No reference counterpart (the reference only adds throughput * sky on
     * a miss, WavefrontRenderer.cpp:256-265); 0 keeps that estimator, 1 adds
     * an importance-sampled environment shadow ray at Diffuse and Plastic
     * hits and weights the misses after them: same mean, lower variance. */
    int32_t enable_env_nee;
    /* enableAdaptiveSampling / adaptiveSamplingThreshold
     * (WavefrontRenderer.h:31-33, AdaptiveSampler.h:27-105): per-pixel
     * Welford statistics of each sample's luminance, a convergence check
     * after every 16th sample once a pixel has 32 (standard error of the
     * mean < threshold * (mean + 0.01)); converged pixels trace no more
     * paths, the render stops when none is left, and each pixel is divided
     * by its own sample count.  0 = every pixel gets samples_per_pixel. */
    int32_t enable_adaptive_sampling;
    float adaptive_threshold;      /* 0.05 in the reference                 */
    /* Live CostTracker (include/render/CostTracker.h:8-63, fed as in
     * WavefrontRenderer.cpp:612-625, 742-760, 800-844): a quarter of the
     * shaded hits time their scatter (and, when textured, their surface
     * colour lookup) in SM clock cycles; after every bounce each material's
     * and texture's mean enters its EMA (weight 0.05) once per sample of the
     * wave (the reference records once per bounce of a one-sample pass),
     * and relativeCost
     * (1.0 below 50 records) drives cost-aware RR and the material /
     * costBenefit orders of the next bounce, as in the reference.  Takes
     * precedence over rel_cost_*.  Single renders only. */
    int32_t enable_cost_tracking;
    int32_t reserved0;
    /* CostTracker::relativeCost per material / texture, frozen for the
     * render (include/render/CostTracker.h:42-55).  NULL = 1.0 for all. */
    const double* rel_cost_material;
    const double* rel_cost_texture;
    wf_camera camera;
} wf_render_params;

/* Counters of one render, mirroring the stat blocks of renderScene
 * (WavefrontRenderer.cpp:317-389) plus ray counts. */
typedef struct wf_render_stats {
    uint64_t closest_rays;      /* closest-hit rays traced (all bounces)  */
    uint64_t shadow_rays;       /* shadow (any-hit) rays traced           */
    uint64_t shaded_hits;       /* total shaded hits                      */
    uint64_t misses;            /* rays that left the scene               */
    uint64_t sorted_elements;   /* keys sorted (ray sort + shade sort)    */
    double ms_total;            /* device time of the render              */
    double ms_ray_sort;         /* "Total ray sort time (ms)"             */
    double ms_intersect;        /* "Total intersect time (ms)"            */
    double ms_shade;            /* "Total shade time (ms)" incl. shadows  */
    double ms_schedule;         /* ShadingQueue schedule + materialize    */
    int32_t waves;              /* wavefronts launched                    */
    int32_t bounces;            /* bounce iterations over all waves       */
    int64_t kernel_launches;    /* kernels this library launched          */
    int32_t samples_run;        /* samplesActuallyRun (adaptive stop)     */
    int32_t active_pixels;      /* pixels still unconverged at the end    */
} wf_render_stats;

/* ---- library / context ------------------------------------------------------- */

typedef struct wf_ctx wf_ctx;

typedef struct wf_config {
    int32_t device;              /* CUDA ordinal                            */
    int64_t max_paths_per_wave;  /* queue capacity; 0 = automatic           */
} wf_config;

/* Library version (WF_API_VERSION). */
int wf_version(void);

/* Creates a context on a device: stream, events, scratch.  Replaces the
 * construction of WavefrontRenderer (include/render/WavefrontRenderer.h:36-39)
 * and EmbreeAccelerator (src/accelerator/Embree.cpp:9-14). */
int wf_create(const wf_config* config, wf_ctx** out_ctx);
/* Destroys a context.  Its servers and device queues must be destroyed
 * before it (the Python binding's Context.close does so). */
int wf_destroy(wf_ctx* ctx);
/* Message of the last failing call on ctx ("" when none). */
const char* wf_last_error(const wf_ctx* ctx);

/* Camera::Camera(lookFrom, lookAt, up, vfov, w, h), include/core/Camera.h
 * :13-33.  Host arithmetic only (no context needed). */
int wf_camera_make(const float look_from[3], const float look_at[3], const float up[3],
                   float vfov_degrees, int32_t image_width, int32_t image_height,
                   wf_camera* out_camera);

/* Uploads the scene and builds the device BVH (Morton/LBVH).  Replaces
 * Scene::buildAccelerator (src/core/Scene.cpp:79-113) with
 * EmbreeAccelerator::build (src/accelerator/Embree.cpp:66-119).  Bounds and
 * the emissive-mesh list are derived exactly as the reference does. */
int wf_scene_upload(wf_ctx* ctx, const wf_scene_desc* scene);

/* Scene facts after upload: bounds (Scene::computeBounds, Scene.cpp:59-77),
 * total emissive area (Scene::totalEmissiveArea, Scene.cpp:162-190), BVH
 * node count and build time (EmbreeAccelerator::m_buildTimeMs). */
typedef struct wf_scene_info {
    float bounds_min[3];
    float bounds_max[3];
    float total_emissive_area;
    int32_t num_triangles;
    int32_t num_meshes;
    int32_t num_emissive_meshes;
    int32_t bvh_nodes;
    double bvh_build_ms;
    int64_t device_bytes;
    int32_t bvh_builder;   /* wf_tuning::bvh_builder that built the tree  */
    int32_t bvh_depth;     /* interior levels below the root              */
} wf_scene_info;
int wf_scene_get_info(wf_ctx* ctx, wf_scene_info* out_info);

/* Launch tuning of a context (the autotuner's knobs).  trace_variant: 0 = no
 * occupancy hint on the traversal kernels (the closest-hit kernel of a
 * single-job render whose binary tree and triangles exceed L2, and multi-job
 * waves over a dense scene, run as 1), 1 = 9 blocks of 128 threads per SM
 * (56 registers, no spills).
 * persistent_blocks_per_sm: resident blocks launched per
 * SM by the persistent traversal kernels (0 = 16).  graph_mode: whether a
 * wave's bounce chain is captured once as a CUDA graph and replayed. */
typedef struct wf_tuning {
    int32_t trace_variant;
    int32_t persistent_blocks_per_sm;
    int32_t graph_mode;  /* 0 = graphs for batches and the server, 1 = also for
                            single renders, 2 = never (policy != none never);
                            without a graph a batch of one job issues its
                            bounces with device-side counts, as a single
                            render does */
    int32_t bvh_builder; /* scenes uploaded afterwards: 0 = PLOC binary tree
                            (locally-ordered clustering, default; leaves by
                            the surface area heuristic below 4096 triangles,
                            else every subtree of <= 4 triangles), 1 = LBVH
                            binary tree (Karras radix tree), 3 = the PLOC tree
                            collapsed into 4-wide nodes (full-precision boxes,
                            128 bytes each), 4 = the PLOC binary tree with
                            surface-area leaves at any size (2, a compressed
                            8-wide tree, was taken out); a PLOC tree deeper
                            than its traversal stack falls back to LBVH */
    int32_t sort_min_queue; /* sort-or-skip: the ray sort and the shading
                            policies run on a bounce only when its queue holds
                            at least this many entries (0 = always, as the
                            reference does); skipping reorders nothing that
                            changes the image */
    int32_t reserved2;   /* must be 0 */
    int32_t reserved;    /* must be 0 */
    int32_t ray_sort_bits; /* the render loop's ray sort uses the top bits of
                            RayQueue::sortKey's 33 (0 = all 33; fewer bits =
                            fewer 8-bit passes, coarser grouping); the host
                            entry point always sorts by the full key */
} wf_tuning;
int wf_set_tuning(wf_ctx* ctx, const wf_tuning* tuning);
int wf_get_tuning(const wf_ctx* ctx, wf_tuning* out_tuning);

/* Autotuner (no reference counterpart): renders one wave of `params` on the
 * current scene (samples capped at one wave, adaptive sampling and cost
 * tracking off) under every combination of trace_variant {0, 1} (block
 * occupancy), persistent_blocks_per_sm {4, 8, 12, 16, 24} and graph_mode
 * {2, 1}, each once untimed and twice
 * timed on the device; then, when params sort rays or shading, the
 * sort-or-skip threshold sort_min_queue over {0, 2^18, 2^20, 2^22, never}
 * and, with the ray sort on, its key width ray_sort_bits over {24, 16}, with
 * the best launch settings.  Keeps the fastest on the context
 * (bvh_builder is left as it is) and returns it with its time per wave.
 * Images and statistics of the trial renders are discarded. */
int wf_autotune(wf_ctx* ctx, const wf_render_params* params, wf_tuning* out_tuning, double* out_wave_ms);

/* ---- ray batches (host buffers) --------------------------------------------- */

/* Closest hit of n rays, t in [tmin, tmax].  Replaces
 * EmbreeAccelerator::intersect4 / intersect (src/accelerator/Embree.cpp
 * :122-256) and the HitRecord they fill (include/core/HitRecord.h:6-22).
 * Output columns (all length n, any may be NULL): geom_id (-1 on miss),
 * prim_id (HitRecord::triangleIndex), distance, bary_u/bary_v (raw
 * barycentrics), point xyz, normal xyz (face-forwarded), front_face, u/v
 * (Mesh::interpolateUV), material_id, texture_id. */
typedef struct wf_hit_columns {
    int32_t* geom_id;
    int32_t* prim_id;
    float* distance;
    float* bary_u;
    float* bary_v;
    float* point_x;
    float* point_y;
    float* point_z;
    float* normal_x;
    float* normal_y;
    float* normal_z;
    uint8_t* front_face;
    float* u;
    float* v;
    int32_t* material_id;
    int32_t* texture_id;
} wf_hit_columns;
int wf_trace_closest_host(wf_ctx* ctx, int64_t n, const float* origins_x,
                          const float* origins_y, const float* origins_z, const float* dirs_x,
                          const float* dirs_y, const float* dirs_z, float tmin, float tmax,
                          wf_hit_columns* out);

/* Any hit with t in [0.001, max_distance - 0.001].  Replaces
 * EmbreeAccelerator::occluded (src/accelerator/Embree.cpp:258-280).
 * out_occluded[i] = 1 when ray i is blocked. */
int wf_trace_occluded_host(wf_ctx* ctx, int64_t n, const float* origins_x,
                           const float* origins_y, const float* origins_z, const float* dirs_x,
                           const float* dirs_y, const float* dirs_z, const float* max_distance,
                           uint8_t* out_occluded);

/* Camera rays of WavefrontRenderer::generatePrimaryRays (.cpp:401-457) for
 * samples [first_sample, first_sample + nspp) of every pixel, jittered by the
 * counter-based RNG keyed (seed, pixel, sample).  Output order: sample-major,
 * then pixel (y*width + x).  Columns of length width*height*nspp. */
int wf_generate_primary_host(wf_ctx* ctx, const wf_camera* camera, int32_t width,
                             int32_t height, uint32_t seed_lo, uint32_t seed_hi,
                             int32_t first_sample, int32_t nspp, float* origins_x,
                             float* origins_y, float* origins_z, float* dirs_x, float* dirs_y,
                             float* dirs_z, int32_t* pixel_indices, int32_t* sample_indices);

/* RayQueue sort for callers that cannot allocate device memory.  This entry
 * point has no counterpart in the reference.  It computes the same keys and
 * permutation as wf_ray_schedule_host, but the ray columns and the outputs
 * are DEVICE pointers owned by the caller, while bounds_min / bounds_max are
 * HOST arrays of 3 floats read during the call.  It needs no context and calls
 * no cudaMalloc,
 * cudaFree or other allocating routine: its scratch is one file-scope device
 * array sized for WF_STATIC_SCHEDULE_MAX_RAYS rays (~25 MB, held by every GPU
 * that loads the library until the process exits).  Callers it is for: code
 * running under a framework that owns the device heap, loops with a
 * no-allocation rule, code preparing work during stream capture.
 *  - Work is enqueued on `stream` (a cudaStream_t; NULL = the legacy default
 *    stream) of the CURRENT device; the call returns without waiting.
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress); make that first call before any stream capture.
 *  - All calls share the one array, which keeps the last call's contents:
 *    calls whose GPU work overlaps (other streams, other host threads) race.
 *    Serialise them on one stream.
 *  - n > WF_STATIC_SCHEDULE_MAX_RAYS returns WF_ERR_CAPACITY and enqueues
 *    nothing.  out_keys may be NULL.
 *  - A launch error already pending on the calling thread (left by earlier,
 *    unrelated work) is not cleared: the call returns WF_ERR_CUDA and
 *    enqueues nothing.  WF_ERR_CUDA after work was enqueued means one of this
 *    call's own launches failed. */
#define WF_STATIC_SCHEDULE_MAX_RAYS (1 << 20)
int wf_ray_schedule_static(void* stream, int64_t n, const float* origins_x, const float* origins_y,
                           const float* origins_z, const float* dirs_x, const float* dirs_y,
                           const float* dirs_z, const float bounds_min[3], const float bounds_max[3],
                           int32_t* out_sorted_indices, uint64_t* out_keys);

/* ---- scheduling (host buffers) ---------------------------------------------- */

/* RayQueue::sortKey + RayQueue::schedule (include/scheduling/RayQueue.h
 * :135-179): key = octant << 30 | morton3(origin quantised to the scene
 * bounds).  Writes the sort permutation (sortedIndices) and, if not NULL,
 * the keys.  The permutation is that of a stable sort of the keys. */
int wf_ray_schedule_host(wf_ctx* ctx, int64_t n, const float* origins_x,
                         const float* origins_y, const float* origins_z, const float* dirs_x,
                         const float* dirs_y, const float* dirs_z, const float bounds_min[3],
                         const float bounds_max[3], int32_t* out_sorted_indices,
                         uint64_t* out_keys);

/* ShadingQueue::schedule (include/scheduling/ShadingQueue.h:90-141,277-329,
 * 437-550) for one queue.  Inputs are the queue columns the policies read;
 * texture_bytes[t] is Texture::memoryBytes() of texture t.  rel_cost_* are
 * frozen CostTracker::relativeCost values (NULL = no tracker, i.e. 1.0 for
 * materials and 0 texture cost, as the reference does with a null tracker).
 * Writes sortedIndices: the permutation of a stable sort under the policy's
 * comparator. */
int wf_shading_schedule_host(wf_ctx* ctx, int32_t policy, int64_t n,
                             const int32_t* material_ids, const int32_t* texture_ids,
                             const float* throughputs_r, const float* throughputs_g,
                             const float* throughputs_b, const float* hit_points_x,
                             const float* hit_points_y, const float* hit_points_z,
                             int32_t num_materials, const wf_material* materials,
                             int32_t num_textures, const int64_t* texture_bytes,
                             const double* rel_cost_material, const double* rel_cost_texture,
                             int32_t* out_sorted_indices);

/* ---- full render -------------------------------------------------------------- */

/* WavefrontRenderer::renderScene (src/render/WavefrontRenderer.cpp:94-399)
 * with adaptive sampling off: renders samples_per_pixel samples of every
 * pixel and writes the averaged image (accumulator / spp, the reference's
 * writeAveragedImage) to image_rgb (width*height*3 floats, host memory).
 * The scene must have been uploaded.  stats may be NULL. */
int wf_render(wf_ctx* ctx, const wf_render_params* params, float* image_rgb,
              wf_render_stats* stats);

/* Same loop, but leaves the per-pixel sums (not divided by spp) on the
 * device and returns them in accum_rgb (host) — the form used to merge
 * batches of samples. */
int wf_render_accumulate(wf_ctx* ctx, const wf_render_params* params, float* accum_rgb,
                         wf_render_stats* stats);

/* Same loop; the averaged image stays in a context-owned device buffer
 * (no host copy) until wf_image_download.  The form a resident render
 * service uses between progressive frames. */
int wf_render_device(wf_ctx* ctx, const wf_render_params* params, wf_render_stats* stats);
/* Copies the image of the last wf_render_device (width*height*3 floats). */
int wf_image_download(wf_ctx* ctx, float* image_rgb, int64_t num_floats);

/* Page-locked host memory (device addition): images and queue mirrors in it
 * are copied by DMA at full link speed, without staging through the driver's
 * buffers.  wf_host_alloc returns WF_ERR_OUT_OF_MEMORY (or WF_ERR_NO_DEVICE)
 * and leaves *out_ptr NULL on failure; wf_host_free(NULL) is a no-op. */
int wf_host_alloc(size_t bytes, void** out_ptr);
int wf_host_free(void* ptr);

/* Relative costs (CostTracker::relativeCost) of the live trackers after
 * the last render with enable_cost_tracking: num_materials doubles, then
 * num_textures doubles (either pointer may be NULL). */
int wf_cost_tracker_state(wf_ctx* ctx, double* rel_material, int32_t num_materials, double* rel_texture,
                          int32_t num_textures);

/* Replays recorded cost samples through the device CostTracker: for step
 * k = 0..steps-1, every item i with counts[k*items+i] > 0 records the mean
 * sums[k*items+i] / counts[k*items+i] (CostTracker::record), in item order;
 * rel_out (items doubles) receives relativeCost afterwards.  The update
 * kernel is the one the render loop runs after each bounce. */
int wf_cost_tracker_replay(wf_ctx* ctx, int32_t items, int32_t steps, const uint64_t* sums,
                           const uint32_t* counts, double* rel_out);

/* Per-pixel sample counts of the last render (AdaptiveSampler::
 * getSampleCount, AdaptiveSampler.h:85-88): width*height int32 values.  Every
 * pixel holds samples_per_pixel when the render was not adaptive. */
int wf_adaptive_sample_counts(wf_ctx* ctx, int32_t* counts, int64_t num_pixels);

/* The context's CUDA stream (a cudaStream_t), so a caller can record its own
 * events around library calls. */
int wf_get_stream(wf_ctx* ctx, void** out_stream);

/* CUDA-event timer on the context's stream: wf_timer_begin records the start
 * event, wf_timer_end records the stop event, waits for it and returns the
 * elapsed device time in milliseconds. */
int wf_timer_begin(wf_ctx* ctx);
int wf_timer_end(wf_ctx* ctx, double* out_ms);

/* ---- per-bounce stages on device-resident queues ------------------------------
 *
 * The reference's loop body (WavefrontRenderer::renderScene, src/render/
 * WavefrontRenderer.cpp:141-268) as separate calls on queues that live in
 * device memory, so a caller can drive its own loop, stage by stage, with no
 * host copy between stages:
 *
 *   wf_stage_begin(ctx, &params)                 renderScene's setup (:94-140)
 *   for sample: wf_generate_primary(...)         generatePrimaryRays (:401-457)
 *     for depth:
 *       wf_ray_queue_schedule / _materialize     RayQueue::schedule / materialize (:159-168)
 *       wf_intersect(rays, hits, misses)         intersectAll (:459-567)
 *       wf_shading_queue_schedule / _materialize ShadingQueue::schedule / materialize (:183-185)
 *       wf_shade(hits, next, shadows)            shadeAll (:569-877), emission into the sums
 *       wf_trace_occluded(shadows)               shadeAll's occluded() calls (:676, :720)
 *       wf_miss(misses)                          the miss loop (:256-265)
 *       swap rays <-> next                       currentQueue = nextQueue (:267)
 *   wf_stage_image(ctx, image)                   writeAveragedImage (:127-137)
 *
 * Queue sizes live on the device: stages chain on the context's stream
 * without waiting; only the calls marked "waits" synchronise.  Paths draw the
 * same random numbers as in wf_render (streams keyed by pixel, sample, depth),
 * so a loop driven this way renders wf_render's image up to the order of
 * float additions into the pixel sums.  The stages share the context's
 * scratch with the full-render entry points: do not interleave them with
 * wf_render* between wf_stage_begin and wf_stage_image.
 *
 * Device layout differences, stated:
 *  - a wf_shading_queue holds, per hit, the ray's index in the ray queue it
 *    came from plus (leaf triangle, t, barycentrics); the other 20 of the
 *    reference's 24 columns are rebuilt from the scene when read (shading,
 *    scheduling, wf_shading_queue_download).  The ray queue given to
 *    wf_intersect must stay unchanged until the hits are shaded.
 *  - misses go to a wf_ray_queue as copies of the missed rays, as in the
 *    reference; wf_intersect with misses == NULL adds their sky terms at once.
 *  - shadow rays are a queue of their own (origin, direction, max distance,
 *    the unoccluded contribution, pixel): the reference calls occluded()
 *    inline; the contribution is added when the ray is found unoccluded. */

typedef struct wf_ray_queue wf_ray_queue;         /* RayQueue, RayQueue.h:63-245 */
typedef struct wf_shading_queue wf_shading_queue; /* ShadingQueue, ShadingQueue.h:27-551 */
typedef struct wf_shadow_queue wf_shadow_queue;   /* shadow rays of one bounce */

/* Host SoA view of a RayQueue (RayQueue.h:65-90: originsX/Y/Z, dirsX/Y/Z,
 * throughputsR/G/B, pixelIndices, depths, pdfs; sampleIndices is a device
 * addition).  accumLight is always 0 and alive always true in the reference's
 * loop, so neither is stored.  NULL columns are skipped (download) or
 * defaulted (upload: throughput 1, depth 0, pdf -1, sample 0). */
typedef struct wf_ray_columns {
    float* origins_x;
    float* origins_y;
    float* origins_z;
    float* dirs_x;
    float* dirs_y;
    float* dirs_z;
    float* throughputs_r;
    float* throughputs_g;
    float* throughputs_b;
    float* pdfs;
    int32_t* pixel_indices;
    int32_t* depths;
    int32_t* sample_indices;
} wf_ray_columns;

/* Queues of `capacity` entries on the context's device.  A shadow queue
 * needs up to 3 entries per hit (area light, directional light, environment
 * map).  Freed queues must not be in use by queued work. */
int wf_ray_queue_alloc(wf_ctx* ctx, int64_t capacity, wf_ray_queue** out);
int wf_ray_queue_free(wf_ray_queue* q);
int wf_shading_queue_alloc(wf_ctx* ctx, int64_t capacity, wf_shading_queue** out);
int wf_shading_queue_free(wf_shading_queue* q);
int wf_shadow_queue_alloc(wf_ctx* ctx, int64_t capacity, wf_shadow_queue** out);
int wf_shadow_queue_free(wf_shadow_queue* q);

/* Entries in a queue (waits). */
int wf_ray_queue_size(wf_ray_queue* q, int64_t* n);
int wf_shading_queue_size(wf_shading_queue* q, int64_t* n);
int wf_shadow_queue_size(wf_shadow_queue* q, int64_t* n);

/* RayQueue::add / addPrimary for n rays from host columns (replaces the
 * queue's contents); wf_ray_queue_download copies up to `capacity` entries
 * back in queue order and returns the count (waits). */
int wf_ray_queue_upload(wf_ray_queue* q, const wf_ray_columns* host, int64_t n);
int wf_ray_queue_download(wf_ray_queue* q, wf_ray_columns* host, int64_t capacity, int64_t* n);

/* The ShadingQueue's columns in queue order (waits): hit columns as
 * wf_trace_closest_host writes them (HitRecord + geomID) and the ray columns
 * of each hit's ray (origins, dirs, throughputs, pixel, depth, pdf). */
int wf_shading_queue_download(wf_shading_queue* q, wf_hit_columns* hits, wf_ray_columns* rays,
                              int64_t capacity, int64_t* n);

/* The render the stages serve: its parameters (the reference's public
 * WavefrontRenderer fields and the camera; adaptive sampling and live cost
 * tracking are not used here) and zeroed per-pixel sums.  Needs an uploaded
 * scene. */
int wf_stage_begin(wf_ctx* ctx, const wf_render_params* params);

/* generatePrimaryRays for samples [first_sample, first_sample + nspp) of
 * every pixel, pixel-major (a pixel's samples are consecutive), throughput 1,
 * depth 0, pdf -1.  Replaces the queue's contents.  Capacity must hold
 * width * height * nspp rays. */
int wf_generate_primary(wf_ctx* ctx, int32_t first_sample, int32_t nspp, wf_ray_queue* out);

/* RayQueue::schedule (RayQueue.h:165-179): sortedIndices = the stable sort of
 * sortKey (octant << 30 | Morton code of the origin in [bounds_min,
 * bounds_max], host arrays of 3 floats), kept in the queue; if not NULL,
 * sorted_indices_host receives it (waits).  Reads the queue's size (waits).
 * RayQueue::materialize (:182-215) gathers every column by it and resets it
 * to the identity. */
int wf_ray_queue_schedule(wf_ray_queue* q, const float bounds_min[3], const float bounds_max[3],
                          int32_t* sorted_indices_host);
int wf_ray_queue_materialize(wf_ray_queue* q);

/* intersectAll: closest hit of every ray of `rays` (t in [0.001, 1e9]); the
 * hits fill `hits` in ray order, the misses `misses` (or, with misses ==
 * NULL, their sky / environment terms go into the sums at once). */
int wf_intersect(wf_ctx* ctx, wf_ray_queue* rays, wf_shading_queue* hits, wf_ray_queue* misses);

/* ShadingQueue::schedule (ShadingQueue.h:90-141, 277-329, 437-550) under
 * `policy` with frozen CostTracker::relativeCost vectors (NULL = no tracker):
 * sortedIndices kept in the queue, copied to sorted_indices_host if not NULL.
 * Reads the hit count (waits).  ShadingQueue::materialize (:233-275) puts the
 * queue in that order and resets sortedIndices to the identity. */
int wf_shading_queue_schedule(wf_shading_queue* q, int32_t policy, const double* rel_cost_material,
                              const double* rel_cost_texture, int32_t* sorted_indices_host);
int wf_shading_queue_materialize(wf_shading_queue* q);

/* shadeAll for every hit of `hits`: emission with MIS into the sums,
 * area / directional (/ environment) NEE as shadow rays, Material::scatter,
 * Russian roulette, next rays.  Replaces the contents of `next` and
 * `shadows`. */
int wf_shade(wf_ctx* ctx, wf_shading_queue* hits, wf_ray_queue* next, wf_shadow_queue* shadows);

/* The occluded() test of every shadow ray; the contribution of an
 * unoccluded one goes into the sums. */
int wf_trace_occluded(wf_ctx* ctx, wf_shadow_queue* shadows);

/* The miss loop: throughput x getSkyColor (or the environment map) of every
 * ray of `misses` into the sums. */
int wf_miss(wf_ctx* ctx, wf_ray_queue* misses);

/* writeAveragedImage: sums / samples_per_pixel into image_rgb (host,
 * width*height*3 floats); also reports a tripped device check (waits). */
int wf_stage_image(wf_ctx* ctx, float* image_rgb, int64_t num_floats);

/* ---- resident scenes, jobs, batches ------------------------------------------ */

/* More scenes kept resident beside the current one (slot 0, set by
 * wf_scene_upload): BVH, triangles, materials and textures stay on the device
 * so jobs over several scenes can share one wavefront.  No counterpart in the
 * reference (it renders one Scene per process). */
int wf_scene_add(wf_ctx* ctx, const wf_scene_desc* scene, int32_t* out_scene_id);
int wf_scene_remove(wf_ctx* ctx, int32_t scene_id);
int wf_scene_get_info_id(wf_ctx* ctx, int32_t scene_id, wf_scene_info* out_info);

/* One render request: a renderScene call (WavefrontRenderer.cpp:94-399,
 * adaptive sampling off, policy none) on a resident scene. */
typedef struct wf_job {
    int32_t scene_id;
    int32_t width;
    int32_t height;
    int32_t samples_per_pixel;
    int32_t max_depth;
    int32_t rr_min_depth;
    int32_t enable_cost_aware_rr;
    float firefly_threshold;
    uint32_t seed_lo;
    uint32_t seed_hi;
    int32_t first_sample;
    int32_t enable_env_nee;          /* as wf_render_params::enable_env_nee */
    const double* rel_cost_material; /* frozen relativeCost per material or NULL */
    wf_camera camera;
} wf_job;

/* Renders njobs jobs to completion with the rays of all jobs sharing each
 * wave (per-ray job ids); each job's random streams are keyed by its own
 * seed, so its image equals a wf_render of it alone up to the order of float
 * additions.  images[j] (host, width*height*3 floats) receives job j's
 * averaged image; NULL skips it. */
int wf_render_batch(wf_ctx* ctx, const wf_job* jobs, int32_t njobs, float* const* images,
                    wf_render_stats* stats);

/* ---- serving loop ------------------------------------------------------------- */

/* A render service on one context.  Jobs are admitted in arrival order while
 * their pixel sums fit the HBM budget.  The server owns a streaming wave: a
 * ray queue of max_paths_per_wave paths that every step advances by 8 bounce
 * iterations, replacing the paths that ended by camera rays of the next
 * frames (frame_spp samples of every pixel of one job, appended round robin
 * over the running jobs, first frames ahead of the others).  A frame's sums
 * join its job's once every one of its paths has ended (max_depth iterations
 * after its last one started), so a progressive image is always the average
 * of whole frames.  Budget = the queue (276 B per path) + the jobs' sums + a
 * share for frame sums (an eighth of the rest, at least 6 floats per queued
 * path).  The queue keeps paths between steps: the server's buffers are its
 * own, apart from the context's.  A job whose last frame ends in a step has
 * its sums freed at the end of that step and its image copied out while the
 * next step runs; it turns WF_JOB_DONE (and leaves `running`) in that next
 * step, or at once when wf_server_image or wf_server_cancel asks for it.
 * Times are seconds on the server's monotonic clock.  No counterpart in the reference
 * (it renders one image per process; its GUI polls a preview file). */
typedef struct wf_server wf_server;
typedef struct wf_server_config {
    int64_t hbm_budget_bytes;   /* queue + job sums + frame sums            */
    int64_t max_paths_per_wave; /* queue capacity; 0 = 2^24 (or the
                                   context's wave size, if smaller)         */
    int32_t frame_spp;          /* samples per progressive frame (8)        */
    int32_t reserved[7];
} wf_server_config;
enum {
    WF_JOB_QUEUED = 0,
    WF_JOB_RUNNING = 1,
    WF_JOB_DONE = 2,
    WF_JOB_CANCELLED = 3,
    WF_JOB_REJECTED = 4 /* larger than the whole budget */
};
typedef struct wf_job_status {
    int32_t state;
    int32_t samples_done;
    int32_t frames;
    int32_t reserved;
    double t_submit;
    double t_admit;
    double t_first_frame;
    double t_done;
} wf_job_status;
typedef struct wf_server_step_info {
    int32_t queued;
    int32_t running;
    int32_t completed_this_step;
    int32_t jobs_in_wave;       /* jobs with frames still running           */
    int64_t paths_in_wave;      /* paths started in this step               */
    uint64_t rays_traced;       /* closest + shadow rays of this step       */
    double step_ms;             /* device time of the step's iterations     */
    int64_t budget_used_bytes;
} wf_server_step_info;
int wf_server_create(wf_ctx* ctx, const wf_server_config* config, wf_server** out_server);
int wf_server_destroy(wf_server* server);
int wf_server_submit(wf_server* server, const wf_job* job, int64_t* out_job_id);
int wf_server_step(wf_server* server, wf_server_step_info* out_info);
int wf_server_status(wf_server* server, int64_t job_id, wf_job_status* out_status);
/* The job's current averaged image (progressive) or final image. */
int wf_server_image(wf_server* server, int64_t job_id, float* image_rgb, int64_t num_floats);
int wf_server_cancel(wf_server* server, int64_t job_id);
double wf_server_clock(const wf_server* server);

/* ---- procedural scenes (host only) ------------------------------------------- */

/* The synthetic workloads that stand in for the reference's stress scenes:
 *   0  Cornell box, 0.55 m, 36 triangles in 18 meshes (one per quad, as the
 *      reference's CornellBox::addQuad/addRotatedBox build it)
 *   1  config-0 room plus a displaced icosphere (subdivision 8, 1,310,720
 *      triangles) split into Lambert / metal / glass regions
 *   3  a job scene of the batched workload: seeded variant `seed` of config 0
 *      (albedos, metal roughness, light position, camera jitter)
 * 100  config 1 at subdivision 4 (5,132 triangles), for fast tests
 * The scene owns its arrays until wf_host_scene_free. */
typedef struct wf_host_scene wf_host_scene;
int wf_host_scene_generate(int32_t config, uint64_t seed, wf_host_scene** out_scene);
int wf_host_scene_describe(const wf_host_scene* scene, wf_scene_desc* out_desc);
/* The camera the workload is rendered with at the given image size. */
int wf_host_scene_camera(const wf_host_scene* scene, int32_t width, int32_t height,
                         wf_camera* out_camera);
int wf_host_scene_free(wf_host_scene* scene);

/* ---- scene files and images (host only) -------------------------------------- */

/* The reference loads scenes through OpenUSD (src/scene/UsdSceneLoader.cpp)
 * and writes images through OpenImageIO, neither of which this build links.
 * A scene file holds what the render path consumes — the flat
 * Scene/SceneGeometry arrays, materials, textures, environment map,
 * directional light — plus a default camera (look_from, look_at, up, vfov).
 * wf_scene_load returns a wf_host_scene for wf_host_scene_describe /
 * wf_host_scene_camera / wf_host_scene_free.  The layout is documented in
 * wavefront-renderer_gb300/csrc/wf_scene_io.cpp. */
int wf_scene_save(const char* path, const wf_scene_desc* desc, const float look_from[3], const float look_at[3],
                  const float up[3], float vfov);
int wf_scene_load(const char* path, wf_host_scene** out_scene);
/* width*height*3 floats, top row first, as a little-endian PFM. */
int wf_image_write_pfm(const char* path, const float* image_rgb, int32_t width, int32_t height);

#ifdef __cplusplus
}
#endif

#endif /* WF_API_H */
