/*
 * wf_oracle.h — CPU oracle of the wavefront path tracer.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load this library,
 * and only as the checker or as the timed CPU baseline.  The product
 * (libwfgpu.so) never links or calls it.
 *
 * What it is: a plain C++17 restatement of the reference's per-bounce loop
 * (fhidargue/wavefront-renderer, src/render/WavefrontRenderer.cpp:94-889 and
 * the functions it calls), with three deliberate substitutions that the GPU
 * path shares:
 *   1. Randomness: the reference draws from a thread_local std::mt19937
 *      (include/math/Random.h:6-18), so its output depends on thread
 *      scheduling.  The oracle draws from Philox4x32-10 (Salmon et al.,
 *      SC'11) keyed by (seed) with counter (block, purpose|depth, pixel,
 *      sample), exactly as the GPU does.  Same estimator, reproducible
 *      streams: a GPU path and an oracle path see the same random numbers.
 *   2. Intersection: Embree 4 is absent, so closest/any hit use the
 *      reference's own Moller-Trumbore (include/geometry/Triangle.h:6-43)
 *      over a CPU BVH.  The closest hit is the one brute force over all
 *      meshes in order returns (Scene::hit fallback, src/core/Scene.cpp
 *      :120-160): smallest t, and on equal t the later triangle.
 *   3. Threads: pixels are split over std::threads; each pixel's samples are
 *      accumulated in the reference's order (sample, then bounce), so the
 *      float sums are reproducible.
 * Floating point is compiled with -ffp-contract=off so no multiply-add is
 * fused: the arithmetic is the reference's, operation by operation.
 *
 * Parity pins: the known-answer cases of the reference's own tests
 * (tests/scheduling/*, tests/accelerator/EmbreeTest.cpp, tests/geometry/
 * TriangleTest.cpp, ...) and the reference sources compiled unmodified with
 * shims (oracle/_ref, see oracle/Makefile) — tests/ compare this port with
 * both.
 */
#ifndef WF_ORACLE_H
#define WF_ORACLE_H

#include <stdint.h>
#include "../include/wf_api.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene orc_scene;

/* Builds the oracle's scene (flat copy + CPU BVH). */
orc_scene* orc_scene_create(const wf_scene_desc* desc);
void orc_scene_destroy(orc_scene* scene);
void orc_scene_bounds(const orc_scene* scene, float bmin[3], float bmax[3]);
float orc_scene_total_emissive_area(const orc_scene* scene);

/* Philox4x32-10 block: out[4] = philox(ctr[4], key[2]). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Camera::getRay(u, v), include/core/Camera.h:35-40. */
void orc_camera_get_ray(const wf_camera* cam, float u, float v, float origin[3], float dir[3]);

/* generatePrimaryRays with the Philox jitter; layout as
 * wf_generate_primary_host. */
void orc_generate_primary(const wf_camera* cam, int32_t width, int32_t height, uint32_t seed_lo,
                          uint32_t seed_hi, int32_t first_sample, int32_t nspp, float* ox,
                          float* oy, float* oz, float* dx, float* dy, float* dz, int32_t* pixel,
                          int32_t* sample);

/* Closest hit (Embree intersect4 mapping) for n rays; columns as
 * wf_hit_columns. */
void orc_trace_closest(const orc_scene* scene, int64_t n, const float* ox, const float* oy,
                       const float* oz, const float* dx, const float* dy, const float* dz,
                       float tmin, float tmax, wf_hit_columns* out);

/* Brute force over all meshes in order, Scene::hit fallback semantics
 * (Mesh::hit), for cross-checking the BVH. Same columns. */
void orc_trace_closest_brute(const orc_scene* scene, int64_t n, const float* ox, const float* oy,
                             const float* oz, const float* dx, const float* dy, const float* dz,
                             float tmin, float tmax, wf_hit_columns* out);

/* EmbreeAccelerator::occluded. */
void orc_trace_occluded(const orc_scene* scene, int64_t n, const float* ox, const float* oy,
                        const float* oz, const float* dx, const float* dy, const float* dz,
                        const float* max_distance, uint8_t* out_occluded);

/* RayQueue::sortKey for n rays, and the stable-sort permutation. */
void orc_ray_sort_keys(int64_t n, const float* ox, const float* oy, const float* oz,
                       const float* dx, const float* dy, const float* dz, const float bmin[3],
                       const float bmax[3], uint64_t* keys);
void orc_ray_schedule(int64_t n, const float* ox, const float* oy, const float* oz,
                      const float* dx, const float* dy, const float* dz, const float bmin[3],
                      const float bmax[3], int32_t* sorted_indices);

/* ShadingQueue::schedule; arguments as wf_shading_schedule_host. */
void orc_shading_schedule(int32_t policy, int64_t n, const int32_t* material_ids,
                          const int32_t* texture_ids, const float* tr, const float* tg,
                          const float* tb, const float* px, const float* py, const float* pz,
                          int32_t num_materials, const wf_material* materials,
                          int32_t num_textures, const int64_t* texture_bytes,
                          const double* rel_cost_material, const double* rel_cost_texture,
                          int32_t* sorted_indices);

/* The whole loop (renderScene with adaptive sampling off) for the pixel
 * window [x0, x0+w) x [y0, y0+h) of a width x height image.  accum_rgb gets
 * the per-pixel sums (not divided by spp), w*h*3 floats, row-major over the
 * window.  threads <= 0: hardware concurrency.  Counters may be NULL. */
typedef struct orc_counters {
    uint64_t closest_rays;
    uint64_t shadow_rays;
    uint64_t shaded_hits;
    uint64_t misses;
} orc_counters;
void orc_render_window(const orc_scene* scene, const wf_render_params* params, int32_t x0,
                       int32_t y0, int32_t w, int32_t h, int32_t threads, float* accum_rgb,
                       orc_counters* counters);
/* Same with AdaptiveSampler when params->enable_adaptive_sampling: counts
 * (w*h, may be null) receives each pixel's sample count. */
void orc_render_window_counts(const orc_scene* scene, const wf_render_params* params, int32_t x0, int32_t y0,
                              int32_t w, int32_t h, int32_t threads, float* accum, int32_t* counts,
                              orc_counters* counters);

/* CostTracker (include/render/CostTracker.h:8-63): feeds cost samples
 * (id, ns) in order and returns relativeCost for every id. */
void orc_cost_tracker_relative(int32_t item_count, int64_t n_samples, const int32_t* ids,
                               const double* costs_ns, double* out_relative);

#ifdef __cplusplus
}
#endif

#endif /* WF_ORACLE_H */
