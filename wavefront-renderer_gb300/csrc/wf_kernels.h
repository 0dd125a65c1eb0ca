// wf_kernels.h — launchers of the render kernels (wf_render.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "wf_device.cuh"

namespace wf {

using ull = unsigned long long;

// Shading parameters fixed for one render (WavefrontRenderer public fields).
struct ShadeParams {
    uint32_t seed_lo, seed_hi;
    float firefly;
    int32_t rr_min_depth;
    int32_t cost_aware_rr;
    const float* rel_cost_material;  // device, float(relativeCost) per material, or null
};

// Build it as LaunchCfg{grid, block} and assign the other members by name.
// Multi-job waves over a scene whose tree + triangles reach this size run
// the traversal kernels at 9 blocks per SM under variant 0 (wf_render.cu).
constexpr int64_t kDenseSceneBytes = int64_t(16) << 20;

struct LaunchCfg {
    int grid;
    int block;
    int variant = 0;   // kernel variant (traversal occupancy hint / stack placement)
    int64_t l2_bytes = 0;  // the device's L2 size (variant 0 of a larger scene runs at 9 blocks per SM)
    int64_t max_scene_bytes = 0;  // largest resident tree + triangles (variant 0 of multi-job waves)
    int lean_multi = 0;  // no resident scene has an environment map, textures or a directional light
    int ray_order = 0;    // 1 = hit records at their rays' indices, listed by k_compact_hits
    int shade_grid = 0;        // k_shade's grid (one full wave of resident blocks); 0 = grid
    int shade_grid_other = 0;  // the same for its multi-job and cost-timed forms
};

// Resident blocks of 128 threads per SM of k_shade from the occupancy
// calculator: the plain single-job form (plain = true) or the smaller of the
// multi-job and cost-timed forms.
int shade_blocks_per_sm(bool plain);

// Camera rays of n = width*height*nspp paths, sample-major.
void launch_camera(const wf_camera& cam, int width, int height, uint32_t seed_lo, uint32_t seed_hi,
                   int first_sample, int nspp, RayQueueDev rq, cudaStream_t s);

// Closest hit for the host API: per-ray HitRecord columns (device buffers).
struct HitColumnsDev {
    int32_t *geom, *prim;
    float *t, *bu, *bv, *px, *py, *pz, *nx, *ny, *nz;
    uint8_t* front;
    float *u, *v;
    int32_t *mat, *tex;
};
void launch_trace_api(const DeviceScene& S, int64_t n, const float* ox, const float* oy,
                      const float* oz, const float* dx, const float* dy, const float* dz,
                      float tmin, float tmax, HitColumnsDev out, int* err, LaunchCfg cfg,
                      cudaStream_t s);
void launch_occluded_api(const DeviceScene& S, int64_t n, const float* ox, const float* oy,
                         const float* oz, const float* dx, const float* dy, const float* dz,
                         const float* maxd, uint8_t* out, int* err, LaunchCfg cfg, cudaStream_t s);

// Render loop stages over a job table and a scene table (device memory).
// Counts live in device memory; accumulators at accum + job.accum_offset.
// header[0] = paths in the wave, header[1] = chunks (device memory, so a
// captured wave can be replayed for any job mix).
void launch_camera_chunks(const WaveChunk* chunks, const long long* header, const DeviceJob* jobs, RayQueueDev rq,
                          LaunchCfg cfg, cudaStream_t s);
// The job and scene tables of a wave.  multi = false: a single job (job0 on
// scene0, passed by value); true: rays look up their job and scene.
struct WaveTables {
    const DeviceScene* scenes;
    const DeviceJob* jobs;
    DeviceScene scene0;
    DeviceJob job0;
    bool multi;
    int tree;  // tree format of the scenes (TreeFormat)
};
void launch_trace_render(const WaveTables& t, RayQueueDev rq, const ull* d_n, HitQueueDev hq, ull* hq_n,
                         float* accum, ull* work, int* err, LaunchCfg cfg, cudaStream_t s);
void launch_shade(const WaveTables& t, RayQueueDev rq, HitQueueDev hq, const ull* hq_n, ShadowQueueDev sh,
                  ull* sh_n, RayQueueDev next, ull* next_n, float* accum, int* err, LaunchCfg cfg, cudaStream_t s);
// After a ray-order trace: lists the rays that hit in hq.ray, counting them
// into *hq_n (zero before the launch).
void launch_compact_hits(const WaveTables& t, RayQueueDev rq, const ull* d_n, HitQueueDev hq, ull* hq_n,
                         float* accum, LaunchCfg cfg, cudaStream_t s);
void launch_occluded_render(const WaveTables& t, ShadowQueueDev sh, const ull* sh_n, float* accum, ull* work,
                            int* err, LaunchCfg cfg, cudaStream_t s);
// End of a bounce of a device-counted chain: tally[0..3] += rays, hits,
// shadow rays, (rays > 0) of the bounce just run; the next bounce's ray
// count into counters[0]; counters[1..5] zeroed.
void launch_bounce_end(ull* counters, ull* tally, cudaStream_t s);

// Streaming waves: after a bounce's shading, plan the refill (one thread:
// new rays = min(capacity - next rays, paths left), cursor advanced,
// counters[3] raised by them, log[iter] = the cursor after it), then write
// those camera rays into the next queue behind the surviving rays.
void launch_stream_plan(ull* counters, StreamState* st, int64_t capacity, int64_t* log, int iter, cudaStream_t s);
void launch_camera_refill(const WaveChunk* chunks, const StreamState* st, const DeviceJob* jobs, RayQueueDev rq,
                          LaunchCfg cfg, cudaStream_t s);
// dst[i] += src[i] (a finished frame's sums into its job's sums).
void launch_add_floats(float* dst, const float* src, int64_t n, cudaStream_t s);

// RayQueue::sortKey over the queue (each ray's scene bounds), (key, index)
// pairs for the radix sort.
void launch_ray_keys(const DeviceScene* scenes, const DeviceJob* jobs, RayQueueDev rq, const ull* d_n,
                     uint64_t* keys, uint32_t* vals, LaunchCfg cfg, cudaStream_t s);
void launch_ray_keys_raw(int64_t n, const float* ox, const float* oy, const float* oz,
                         const float* dx, const float* dy, const float* dz, const float bmin[3],
                         const float bmax[3], uint64_t* keys, uint32_t* vals, LaunchCfg cfg,
                         cudaStream_t s);
// out[i] = in[perm[i]] for every column (RayQueue::materialize).
void launch_gather_rays(RayQueueDev in, const uint32_t* perm, const ull* d_n, RayQueueDev out,
                        LaunchCfg cfg, cudaStream_t s);

// ShadingQueue scheduling on plain columns.
struct ShadeColumnsDev {
    const int32_t* mat;
    const int32_t* tex;
    const float *tr, *tg, *tb;
    const float *px, *py, *pz;
};
// Per material type: hit count, texture bytes, first queue index.
void launch_type_stats(ShadeColumnsDev c, const ull* d_n, const wf_material* mats, int num_tex,
                       const int64_t* tex_bytes, ull* counts, ull* mem, int* first, LaunchCfg cfg,
                       cudaStream_t s);
// Material / texture policy keys: type_rank[type] << shift | secondary rank.
void launch_policy_keys(ShadeColumnsDev c, const ull* d_n, const wf_material* mats, int policy,
                        const int* type_rank8, const int* cost_rank, const int* tex_rank,
                        int num_tex, int shift, uint64_t* keys, uint32_t* vals, LaunchCfg cfg,
                        cudaStream_t s);
// Cost-benefit: per material luminance sums and hit-point bounds.
void launch_cb_reduce(ShadeColumnsDev c, const ull* d_n, double* benefit, int* present,
                      unsigned* bounds6, int num_materials, LaunchCfg cfg, cudaStream_t s);
void launch_cb_keys(ShadeColumnsDev c, const ull* d_n, const wf_material* mats,
                    const int* prio_rank, int prio_bits, const unsigned* bounds6, uint64_t* keys,
                    uint32_t* vals, LaunchCfg cfg, cudaStream_t s);
// Columns of the render loop's hit queue for the schedulers.
struct ShadeColumnsMut {
    int32_t* mat;
    int32_t* tex;
    float *tr, *tg, *tb, *px, *py, *pz;
};
// full: the throughput and hit point columns too (costBenefit); scene: the
// scene of every hit when the wave has one job (device pointer), else null.
void launch_hit_columns(const DeviceScene* scenes, const DeviceJob* jobs, const DeviceScene* scene, bool full,
                        RayQueueDev rq, HitQueueDev hq, const ull* d_n, ShadeColumnsMut out, LaunchCfg cfg,
                        cudaStream_t s);
void launch_permute_hits(HitQueueDev in, const uint32_t* perm, const ull* d_n, HitQueueDev out,
                         LaunchCfg cfg, cudaStream_t s);

// Per-bounce stages on caller-held queues.  After a trace with ray_order 2
// (records at the rays' indices, misses left alone): the hits listed in
// hq.ray (k_compact_hits) and the misses in miss_list; the counts must be
// zero before the launch.
void launch_split_hits(const WaveTables& t, RayQueueDev rq, const ull* d_n, HitQueueDev hq, ull* hq_n,
                       uint32_t* miss_list, ull* miss_n, LaunchCfg cfg, cudaStream_t s);
// The miss loop over a queue of missed rays (single job t.job0 on t.scene0).
void launch_miss_queue(const WaveTables& t, RayQueueDev misses, const ull* d_n, float* accum, LaunchCfg cfg,
                       cudaStream_t s);
// out[i] = in[perm ? perm[i] : i] in list layout (records at list positions);
// at_ray: in's records sit at their rays' indices.
void launch_materialize_hits(HitQueueDev in, bool at_ray, const uint32_t* perm, const ull* d_n, HitQueueDev out,
                             LaunchCfg cfg, cudaStream_t s);
// The ShadingQueue's columns of every entry (HitRecord + the ray's columns).
void launch_shading_columns(const DeviceScene& S, RayQueueDev rq, HitQueueDev hq, bool at_ray, const ull* d_n,
                            HitColumnsDev out, RayQueueDev rays_out, LaunchCfg cfg, cudaStream_t s);

// image = accum / spp.
void launch_finalize(const float* accum, int64_t nfloats, float spp, float* image, cudaStream_t s);

// Adaptive sampling: fold a wave's per-sample sums into the pixel sums and
// Welford statistics (the wave's samples sit in slots slot0, slot0+1, ...
// modulo wave_spp of the per-sample buffer); mark converged pixels; list the
// active ones in index order; divide by per-pixel sample counts; fill an int
// array (or iota).
void launch_adaptive_fold(float* sample_buf, int64_t np, int nspp, int slot0, int wave_spp, float* accum,
                          float* mean, float* m2, int32_t* count, const int32_t* active, int32_t n_active,
                          cudaStream_t s);
void launch_adaptive_check(const float* mean, const float* m2, const int32_t* count, const int32_t* active,
                           int32_t n_active, float threshold, int32_t* flag, cudaStream_t s);
void launch_compact_active(const int32_t* flag, int64_t np, int32_t* pos, int32_t* block_sums, int32_t* out,
                           int32_t* n_out, cudaStream_t s);
void launch_finalize_counts(const float* accum, const int32_t* count, int64_t np, float* image, cudaStream_t s);
void launch_fill_i32(int32_t* a, int64_t n, int32_t v, bool identity, cudaStream_t s);

// Live CostTracker: fold the last bounce's timings into both trackers
// (`repeat` records of the bounce mean per item).
void launch_cost_update(const CostTrackerDev& mat, const CostTrackerDev& tex, int repeat, cudaStream_t s);

}  // namespace wf
