// wf_loop.cpp — the wavefront render loop behind wf_render*, wf_render_batch
// and the serving loop (reference src/render/WavefrontRenderer.cpp:94-399).
//
// A wave is a set of chunks — (job, range of samples) — whose paths are
// generated together and bounce together: trace, shade, shadow rays, once
// per depth.  Two executors run a wave:
//   host loop  one host round trip per bounce (counts read back); needed for
//              the ShadingQueue policies, whose type order is decided on the
//              host, and for per-stage timings;
//   graph      the whole bounce chain captured once as a CUDA graph (all
//              counts stay on the device; empty bounces cost only launches)
//              and replayed for every wave with the same depth.
// Jobs share waves through the job table: each ray carries its job id, the
// job names its resident scene, RNG seed and accumulator offset.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <vector>

#include "../../include/wf_api.h"
#include "wf_ctx.h"
#include "wf_kernels.h"
#include "wf_sort.h"

using namespace wf;

namespace wf {

int validate_job(wf_ctx* c, const wf_job& j)
{
    if (j.scene_id < 0 || j.scene_id >= (int)c->scenes.size() || !c->scenes[j.scene_id].live)
        return set_err(c, WF_ERR_STATE, "job names a scene that is not resident");
    if (j.width < 2 || j.height < 2)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "width and height must be >= 2 (u = x/(width-1))");
    if ((int64_t)j.width * j.height > (int64_t)1 << 28)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "image larger than 2^28 pixels");
    if (j.samples_per_pixel < 1) return set_err(c, WF_ERR_INVALID_ARGUMENT, "samples_per_pixel < 1");
    if (j.max_depth < 0 || j.max_depth > 0xFFFF) return set_err(c, WF_ERR_INVALID_ARGUMENT, "max_depth out of range");
    return WF_OK;
}

// Device job: cost-aware RR reads float(relativeCost) per material
// (WavefrontRenderer.cpp:781-785) from a table copied here.
int make_device_job(wf_ctx* c, const wf_job& j, int64_t accum_offset, DeviceJob& dj)
{
    std::memset(&dj, 0, sizeof(dj));
    dj.scene = j.scene_id;
    dj.width = j.width;
    dj.height = j.height;
    dj.max_depth = j.max_depth;
    dj.rr_min_depth = j.rr_min_depth;
    dj.cost_aware_rr = j.enable_cost_aware_rr;
    dj.firefly = j.firefly_threshold;
    dj.seed_lo = j.seed_lo;
    dj.seed_hi = j.seed_hi;
    dj.env_nee = j.enable_env_nee ? 1 : 0;
    dj.accum_offset = accum_offset;
    dj.camera = j.camera;
    if (j.enable_cost_aware_rr && j.rel_cost_material) {
        const int nm = c->scenes[j.scene_id].S.num_materials;
        std::vector<float> f(nm);
        for (int m = 0; m < nm; ++m) f[m] = (float)j.rel_cost_material[m];
        float* d = nullptr;
        WF_CK(c, wf_dalloc(c->rel_cost_allocs, &d, nm));
        WF_CK(c, cudaMemcpyAsync(d, f.data(), sizeof(float) * nm, cudaMemcpyHostToDevice, c->stream));
        dj.rel_cost_material = d;
    }
    return WF_OK;
}

int upload_jobs(wf_ctx* c, const std::vector<DeviceJob>& jobs)
{
    int rc = ensure_job_tables(c, (int)jobs.size(), 1);
    if (rc) return rc;
    WF_CK(c, cudaMemcpyAsync(c->d_jobs, jobs.data(), sizeof(DeviceJob) * jobs.size(), cudaMemcpyHostToDevice,
                             c->stream));
    return WF_OK;
}

// Chunks of the next wave and the device header (total paths, chunk count).
int upload_wave(wf_ctx* c, const std::vector<WaveChunk>& chunks, int64_t total)
{
    int rc = ensure_job_tables(c, 1, (int)chunks.size());
    if (rc) return rc;
    WF_CK(c, cudaMemcpyAsync(c->d_chunks, chunks.data(), sizeof(WaveChunk) * chunks.size(), cudaMemcpyHostToDevice,
                             c->stream));
    long long hdr[2] = {(long long)total, (long long)chunks.size()};
    WF_CK(c, cudaMemcpyAsync(c->d_wave_header, hdr, sizeof(hdr), cudaMemcpyHostToDevice, c->stream));
    // a pageable source may be read after the call returns; make it safe
    WF_CK(c, cudaStreamSynchronize(c->stream));
    return WF_OK;
}

}  // namespace wf

namespace {

// The render loop's ray sort orders by the top wf_tuning::ray_sort_bits of
// RayQueue::sortKey's 33 bits (octant, then Morton code of the origin): the
// order only groups rays, so a coarser key sorts in fewer 8-bit passes.  The
// host entry point wf_ray_schedule_host always sorts by the full key.
int ray_key_begin(const wf_ctx* c)
{
    const int bits = c->tuning.ray_sort_bits > 0 ? std::min(33, c->tuning.ray_sort_bits) : 33;
    return 33 - bits;
}

// Whether a bounce shades its hits in ray order: without a shading policy.
// Against shading the compact queue in the traversal's completion order this
// measured +4% (dense mesh), +10% (lattice), +9% (batched jobs): coalesced ray
// reads, and next rays and shadow rays that stay in queue order, so later
// bounces trace coherent runs of rays.
int hits_in_ray_order(int policy) { return policy == WF_POLICY_NONE ? 1 : 0; }

// The tree format of the resident scenes (TreeFormat); a wave's kernels use
// one traversal, so the formats must not be mixed.
int table_tree(wf_ctx* c, int& tree)
{
    int seen = -1;
    for (const auto& r : c->scenes) {
        if (!r.live || r.S.num_tris <= 0) continue;
        const int f = tree_format(r.S);
        if (seen >= 0 && f != seen)
            return set_err(c, WF_ERR_STATE,
                           "resident scenes were built with different BVH formats (wf_tuning::bvh_builder)");
        seen = f;
    }
    tree = seen < 0 ? kTreeBinary : seen;
    return WF_OK;
}

// One wave, one host round trip per bounce.  policy / ray sort as in the
// reference (RayQueue::schedule + ShadingQueue::schedule), materials of
// scene `policy_scene`.
int wave_host(wf_ctx* c, int64_t total, int max_depth, int policy, bool ray_sort, int policy_scene,
              const double* rc_mat, const double* rc_tex, const DeviceJob* single_job, wf_render_stats& stats,
              bool track_costs = false, int cost_records = 1)
{
    std::vector<double> live_mat, live_tex;  // relativeCost of the live trackers, for the policies
    cudaStream_t s = c->stream;
    WaveTables T{c->d_scene_table, c->d_jobs, DeviceScene{}, DeviceJob{}, single_job == nullptr, kTreeBinary};
    if (single_job) {
        T.job0 = *single_job;
        T.scene0 = c->scenes[single_job->scene].S;
        T.tree = tree_format(T.scene0);
    } else {
        int rc = table_tree(c, T.tree);
        if (rc) return rc;
    }
    // Without a shading policy the hits are shaded in ray order (records at
    // their rays' indices): coalesced ray reads, and the next rays and shadow
    // rays keep the queue's order.  A policy sorts the compact hit queue.
    LaunchCfg PC = persist_cfg(c);
    PC.ray_order = hits_in_ray_order(policy);
    const LaunchCfg WC = wide_cfg(c);
    cudaEvent_t* ev = c->ev;
    float ms = 0.0f;
    int cur = 0;
    launch_camera_chunks(c->d_chunks, c->d_wave_header, c->d_jobs, c->rq[cur], WC, s);
    stats.kernel_launches += 1;
    ull hc = (ull)total;
    WF_CK(c, cudaMemcpyAsync(c->counters, &hc, sizeof(ull), cudaMemcpyHostToDevice, s));
    int64_t count = total;
    stats.waves++;
    for (int depth = 0; depth < max_depth && count > 0; ++depth) {
        stats.bounces++;
        stats.closest_rays += (uint64_t)count;
        const bool sort_rays = ray_sort && count >= (int64_t)c->tuning.sort_min_queue;
        if (sort_rays) {  // RayQueue::schedule + materialize (.cpp:159-168)
            WF_CK(c, cudaEventRecord(ev[2], s));
            launch_ray_keys(c->d_scene_table, c->d_jobs, c->rq[cur], c->counters, c->keys, c->vals, WC, s);
            uint64_t* rk;
            uint32_t* rv;
            RadixSortArgs a{c->keys, c->vals,    c->keys_tmp, c->vals_tmp, c->hist, c->counters,
                            c->nb,   ray_key_begin(c), 33,          &rk,         &rv};
            radix_sort_pairs(a, s);
            launch_gather_rays(c->rq[cur], rv, c->counters, c->rq[1 - cur], WC, s);
            stats.kernel_launches += 2 + kSortKernelsPerPass * ((33 - ray_key_begin(c) + 7) / 8);
            cur = 1 - cur;
            WF_CK(c, cudaEventRecord(ev[3], s));
            stats.sorted_elements += (uint64_t)count;
        }
        WF_CK(c, cudaMemsetAsync(c->counters + 1, 0, sizeof(ull) * 5, s));
        WF_CK(c, cudaEventRecord(ev[4], s));
        launch_trace_render(T, c->rq[cur], c->counters, c->hq[0], c->counters + 1, c->arena, c->counters + 4,
                            c->err_flag, PC, s);
        if (PC.ray_order) {
            launch_compact_hits(T, c->rq[cur], c->counters, c->hq[0], c->counters + 1, c->arena, WC, s);
            stats.kernel_launches += 1;
        }
        WF_CK(c, cudaEventRecord(ev[5], s));
        HitQueueDev hq_use = c->hq[0];
        ull hits = 0;
        if (policy != WF_POLICY_NONE) {
            WF_CK(c, cudaMemcpyAsync(&hits, c->counters + 1, sizeof(ull), cudaMemcpyDeviceToHost, s));
            WF_CK(c, cudaStreamSynchronize(s));
        }
        if (policy != WF_POLICY_NONE && hits >= (ull)c->tuning.sort_min_queue) {
            ShadeColumnsMut cm{c->col_mat, c->col_tex, c->col_tr, c->col_tg, c->col_tb, c->col_px, c->col_py, c->col_pz};
            launch_hit_columns(c->d_scene_table, c->d_jobs, single_job ? c->d_scene_table + single_job->scene : nullptr,
                               policy == WF_POLICY_COST_BENEFIT_AWARE, c->rq[cur], c->hq[0], c->counters + 1, cm, WC,
                               s);
            ShadeColumnsDev cd{c->col_mat, c->col_tex, c->col_tr, c->col_tg, c->col_tb, c->col_px, c->col_py, c->col_pz};
            const ResidentScene& R = c->scenes[policy_scene];
            if (track_costs) {  // the trackers' state after the previous bounce
                live_mat.resize((size_t)std::max(c->ct_mat.items, 1));
                live_tex.resize((size_t)std::max(c->ct_tex.items, 1));
                WF_CK(c, cudaMemcpyAsync(live_mat.data(), c->ct_mat.rel, sizeof(double) * live_mat.size(),
                                         cudaMemcpyDeviceToHost, s));
                WF_CK(c, cudaMemcpyAsync(live_tex.data(), c->ct_tex.rel, sizeof(double) * live_tex.size(),
                                         cudaMemcpyDeviceToHost, s));
                WF_CK(c, cudaStreamSynchronize(s));
                rc_mat = live_mat.data();
                rc_tex = live_tex.data();
            }
            uint32_t* perm = nullptr;
            int rc = schedule_columns(c, policy, c->counters + 1, (int64_t)hits, cd, R.S.materials, R.S.num_materials,
                                      R.mats, R.S.num_textures, R.d_tex_bytes, R.tex_bytes, rc_mat, rc_tex, &perm);
            if (rc) return rc;
            // ShadingQueue::materialize's gather.  A material or texture order
            // keeps long runs of the list order (a stable sort by a few type and
            // cost ranks), so k_shade reads the hits through the permutation
            // (C2 material +5.8%, dense mesh material +8.7%); costBenefit's
            // Morton sub-order scatters them, and a separate gather is faster
            // there (shading through it measured 12 ms slower per C2 step).
            if (policy == WF_POLICY_COST_BENEFIT_AWARE) {
                launch_permute_hits(c->hq[0], perm, c->counters + 1, c->hq[1], WC, s);
                stats.kernel_launches += c->last_schedule_launches + 2;
                hq_use = c->hq[1];
            } else {
                stats.kernel_launches += c->last_schedule_launches + 1;
                hq_use.order = perm;
            }
            stats.sorted_elements += hits;
        }
        WF_CK(c, cudaEventRecord(ev[6], s));
        launch_shade(T, c->rq[cur], hq_use, c->counters + 1, c->sh, c->counters + 2, c->rq[1 - cur], c->counters + 3,
                     c->arena, c->err_flag, PC, s);
        if (track_costs) {  // the tracker merge at the end of shadeAll (.cpp:800-844)
            launch_cost_update(c->ct_mat, c->ct_tex, cost_records, s);
            stats.kernel_launches += 1;
        }
        launch_occluded_render(T, c->sh, c->counters + 2, c->arena, c->counters + 5, c->err_flag, PC, s);
        stats.kernel_launches += 3;
        WF_CK(c, cudaEventRecord(ev[7], s));
        ull cnt[4];
        WF_CK(c, cudaMemcpyAsync(cnt, c->counters, sizeof(cnt), cudaMemcpyDeviceToHost, s));
        WF_CK(c, cudaMemcpyAsync(c->counters, c->counters + 3, sizeof(ull), cudaMemcpyDeviceToDevice, s));
        WF_CK(c, cudaStreamSynchronize(s));
        if (sort_rays) {
            WF_CK(c, cudaEventElapsedTime(&ms, ev[2], ev[3]));
            stats.ms_ray_sort += ms;
        }
        WF_CK(c, cudaEventElapsedTime(&ms, ev[4], ev[5]));
        stats.ms_intersect += ms;
        WF_CK(c, cudaEventElapsedTime(&ms, ev[5], ev[6]));
        stats.ms_schedule += ms;
        WF_CK(c, cudaEventElapsedTime(&ms, ev[6], ev[7]));
        stats.ms_shade += ms;
        stats.shaded_hits += cnt[1];
        stats.misses += (uint64_t)count - cnt[1];
        stats.shadow_rays += cnt[2];
        count = (int64_t)cnt[3];
        cur = 1 - cur;
    }
    return WF_OK;
}

// The launches of one wave with every count on the device: what a graph
// captures.  Returns the number of kernels.
int record_chain(wf_ctx* c, int max_depth, bool ray_sort, int tree)
{
    cudaStream_t s = c->stream;
    LaunchCfg PC = persist_cfg(c);
    PC.ray_order = hits_in_ray_order(WF_POLICY_NONE);
    const LaunchCfg WC = wide_cfg(c);
    int kernels = 0;
    int cur = 0;
    const WaveTables T{c->d_scene_table, c->d_jobs, DeviceScene{}, DeviceJob{}, true, tree};
    launch_camera_chunks(c->d_chunks, c->d_wave_header, c->d_jobs, c->rq[cur], WC, s);
    cudaMemcpyAsync(c->counters, c->d_wave_header, sizeof(ull), cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(c->counters + 1, 0, sizeof(ull) * 5, s);  // later bounces: k_bounce_end
    kernels += 1;
    for (int depth = 0; depth < max_depth; ++depth) {
        if (ray_sort) {
            launch_ray_keys(c->d_scene_table, c->d_jobs, c->rq[cur], c->counters, c->keys, c->vals, WC, s);
            uint64_t* rk;
            uint32_t* rv;
            RadixSortArgs a{c->keys, c->vals,    c->keys_tmp, c->vals_tmp, c->hist, c->counters,
                            c->nb,   ray_key_begin(c), 33,          &rk,         &rv};
            radix_sort_pairs(a, s);
            launch_gather_rays(c->rq[cur], rv, c->counters, c->rq[1 - cur], WC, s);
            kernels += 2 + kSortKernelsPerPass * ((33 - ray_key_begin(c) + 7) / 8);
            cur = 1 - cur;
        }
        launch_trace_render(T, c->rq[cur], c->counters, c->hq[0], c->counters + 1, c->arena, c->counters + 4,
                            c->err_flag, PC, s);
        if (PC.ray_order) {
            launch_compact_hits(T, c->rq[cur], c->counters, c->hq[0], c->counters + 1, c->arena, WC, s);
            kernels += 1;
        }
        launch_shade(T, c->rq[cur], c->hq[0], c->counters + 1, c->sh, c->counters + 2, c->rq[1 - cur], c->counters + 3,
                     c->arena, c->err_flag, PC, s);
        launch_occluded_render(T, c->sh, c->counters + 2, c->arena, c->counters + 5, c->err_flag, PC, s);
        launch_bounce_end(c->counters, c->tally, s);
        kernels += 4;
        cur = 1 - cur;
    }
    return kernels;
}

int wave_graph(wf_ctx* c, int max_depth, bool ray_sort, wf_render_stats& stats)
{
    cudaStream_t s = c->stream;
    int tree = kTreeBinary;
    int rc = table_tree(c, tree);
    if (rc) return rc;
    const LaunchCfg pc = persist_cfg(c);
    const bool dense = pc.max_scene_bytes >= kDenseSceneBytes;
    CapturedWave* g = nullptr;
    for (auto& x : c->graphs)
        if (x.max_depth == max_depth && x.ray_sort == ray_sort && x.variant == c->tuning.trace_variant &&
            x.key_ptr == c->arena && x.key_cap == c->cap && x.tree == tree && x.lean == pc.lean_multi &&
            x.dense == dense)
            g = &x;
    if (!g) {
        cudaGraph_t graph = nullptr;
        WF_CK(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int k = record_chain(c, max_depth, ray_sort, tree);
        cudaError_t e = cudaStreamEndCapture(s, &graph);
        if (e != cudaSuccess) return set_err(c, WF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        CapturedWave w;
        e = cudaGraphInstantiate(&w.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return set_err(c, WF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        w.max_depth = max_depth;
        w.ray_sort = ray_sort;
        w.variant = c->tuning.trace_variant;
        w.key_ptr = c->arena;
        w.key_cap = c->cap;
        w.tree = tree;
        w.kernels = k;
        w.lean = pc.lean_multi;
        w.dense = dense;
        c->graphs.push_back(w);
        g = &c->graphs.back();
    }
    WF_CK(c, cudaGraphLaunch(g->exec, s));
    stats.waves++;
    stats.kernel_launches += g->kernels;
    return WF_OK;
}

int zero_tally(wf_ctx* c) { WF_CK(c, cudaMemsetAsync(c->tally, 0, sizeof(ull) * 8, c->stream)); return WF_OK; }

int read_tally(wf_ctx* c, wf_render_stats& stats);

// One wave of a single job without a shading policy, every count on the
// device and the bounces issued back to back: no host round trip between
// bounces (wave_host waits for each bounce's counts), with the single-job
// kernels (wave_graph captures the multi-job ones).  All max_depth bounces
// are issued; a bounce whose queue is empty costs only its empty launches.
// Stage times come from per-bounce events read once the wave is done.
int wave_chain(wf_ctx* c, int max_depth, bool ray_sort, const DeviceJob& job, wf_render_stats& stats,
               bool track_costs, int cost_records)
{
    cudaStream_t s = c->stream;
    WaveTables T{c->d_scene_table, c->d_jobs, c->scenes[job.scene].S, job, false, kTreeBinary};
    T.tree = tree_format(T.scene0);
    LaunchCfg PC = persist_cfg(c);
    PC.ray_order = hits_in_ray_order(WF_POLICY_NONE);
    const LaunchCfg WC = wide_cfg(c);
    const size_t nev = (size_t)5 * (size_t)max_depth;
    while (c->stage_ev.size() < nev) {
        cudaEvent_t e = nullptr;
        WF_CK(c, cudaEventCreate(&e));
        c->stage_ev.push_back(e);
    }
    int rc = zero_tally(c);
    if (rc) return rc;
    int cur = 0;
    int64_t kernels = 0;
    launch_camera_chunks(c->d_chunks, c->d_wave_header, c->d_jobs, c->rq[cur], WC, s);
    WF_CK(c, cudaMemcpyAsync(c->counters, c->d_wave_header, sizeof(ull), cudaMemcpyDeviceToDevice, s));
    WF_CK(c, cudaMemsetAsync(c->counters + 1, 0, sizeof(ull) * 5, s));  // later bounces: k_bounce_end
    kernels += 1;
    for (int depth = 0; depth < max_depth; ++depth) {
        cudaEvent_t* E = c->stage_ev.data() + 5 * depth;
        if (ray_sort) {
            WF_CK(c, cudaEventRecord(E[0], s));
            launch_ray_keys(c->d_scene_table, c->d_jobs, c->rq[cur], c->counters, c->keys, c->vals, WC, s);
            uint64_t* rk;
            uint32_t* rv;
            RadixSortArgs a{c->keys, c->vals,    c->keys_tmp, c->vals_tmp, c->hist, c->counters,
                            c->nb,   ray_key_begin(c), 33,          &rk,         &rv};
            radix_sort_pairs(a, s);
            launch_gather_rays(c->rq[cur], rv, c->counters, c->rq[1 - cur], WC, s);
            kernels += 2 + kSortKernelsPerPass * ((33 - ray_key_begin(c) + 7) / 8);
            cur = 1 - cur;
            WF_CK(c, cudaEventRecord(E[1], s));
        }
        WF_CK(c, cudaEventRecord(E[2], s));
        launch_trace_render(T, c->rq[cur], c->counters, c->hq[0], c->counters + 1, c->arena, c->counters + 4,
                            c->err_flag, PC, s);
        launch_compact_hits(T, c->rq[cur], c->counters, c->hq[0], c->counters + 1, c->arena, WC, s);
        WF_CK(c, cudaEventRecord(E[3], s));
        launch_shade(T, c->rq[cur], c->hq[0], c->counters + 1, c->sh, c->counters + 2, c->rq[1 - cur],
                     c->counters + 3, c->arena, c->err_flag, PC, s);
        if (track_costs) {  // the tracker merge at the end of shadeAll (.cpp:800-844)
            launch_cost_update(c->ct_mat, c->ct_tex, cost_records, s);
            kernels += 1;
        }
        launch_occluded_render(T, c->sh, c->counters + 2, c->arena, c->counters + 5, c->err_flag, PC, s);
        WF_CK(c, cudaEventRecord(E[4], s));
        launch_bounce_end(c->counters, c->tally, s);
        kernels += 5;
        cur = 1 - cur;
    }
    const uint64_t rays_before = stats.closest_rays;
    rc = read_tally(c, stats);  // waits for the wave
    if (rc) return rc;
    float ms = 0.0f;
    for (int depth = 0; depth < max_depth; ++depth) {
        cudaEvent_t* E = c->stage_ev.data() + 5 * depth;
        if (ray_sort) {
            WF_CK(c, cudaEventElapsedTime(&ms, E[0], E[1]));
            stats.ms_ray_sort += ms;
        }
        WF_CK(c, cudaEventElapsedTime(&ms, E[2], E[3]));
        stats.ms_intersect += ms;
        WF_CK(c, cudaEventElapsedTime(&ms, E[3], E[4]));
        stats.ms_shade += ms;
    }
    if (ray_sort) stats.sorted_elements += stats.closest_rays - rays_before;  // every bounce sorts its queue
    stats.waves++;
    stats.kernel_launches += kernels;
    return WF_OK;
}

// Scene traits (wave_scene_traits) of the jobs of the multi-job waves about
// to be launched, for the launch configuration while the scope lasts.
struct WaveSceneScope {
    wf_ctx* c;
    WaveSceneScope(wf_ctx* ctx, const std::vector<int32_t>& scene_ids) : c(ctx)
    {
        wave_scene_traits(c, scene_ids.data(), (int)scene_ids.size(), c->wave_scene_bytes, c->wave_lean);
    }
    ~WaveSceneScope()
    {
        c->wave_scene_bytes = -1;
        c->wave_lean = -1;
    }
};

int read_tally(wf_ctx* c, wf_render_stats& stats)
{
    ull t[4];
    WF_CK(c, cudaMemcpyAsync(t, c->tally, sizeof(t), cudaMemcpyDeviceToHost, c->stream));
    WF_CK(c, cudaStreamSynchronize(c->stream));
    stats.closest_rays += t[0];
    stats.shaded_hits += t[1];
    stats.misses += t[0] - t[1];
    stats.shadow_rays += t[2];
    stats.bounces += (int32_t)t[3];
    return WF_OK;
}

bool use_graph(const wf_ctx* c, bool batch, int policy)
{
    if (policy != WF_POLICY_NONE || c->tuning.graph_mode == 2) return false;
    return batch || c->tuning.graph_mode == 1;
}

int validate_params(wf_ctx* c, const wf_render_params* P)
{
    if (!P) return set_err(c, WF_ERR_INVALID_ARGUMENT, "params is null");
    if (P->policy < 0 || P->policy > 3) return set_err(c, WF_ERR_INVALID_ARGUMENT, "unknown policy");
    if (c->scenes.empty() || !c->scenes[0].live) return set_err(c, WF_ERR_STATE, "no scene uploaded");
    wf_job j{};
    j.scene_id = 0;
    j.width = P->width;
    j.height = P->height;
    j.samples_per_pixel = P->samples_per_pixel;
    j.max_depth = P->max_depth;
    if (P->enable_adaptive_sampling) {
        if (!(P->adaptive_threshold > 0.0f))
            return set_err(c, WF_ERR_INVALID_ARGUMENT, "adaptive_threshold must be > 0");
        if ((int64_t)P->width * P->height * 16 > INT32_MAX)
            return set_err(c, WF_ERR_INVALID_ARGUMENT, "adaptive sampling needs width*height*16 < 2^31");
    }
    return validate_job(c, j);
}

// renderScene for the current scene: leaves the per-pixel sums in the arena
// at offset 0 (W*H*3 floats).
int render_single(wf_ctx* c, const wf_render_params* P, wf_render_stats* st)
{
    cudaStream_t s = c->stream;
    const int W = P->width, H = P->height;
    const int64_t np = (int64_t)W * H;
    int spw = P->spp_per_wave > 0 ? P->spp_per_wave : (int)std::max<int64_t>(1, c->paths_per_wave / np);
    spw = std::max(1, std::min(spw, P->samples_per_pixel));
    const bool adaptive = P->enable_adaptive_sampling != 0;
    if (adaptive) {  // waves end on the convergence checks: sample 32, then every 16th
        int p2 = 1;
        while (p2 * 2 <= std::min(spw, 32) && np * (p2 * 2) <= (int64_t)INT32_MAX) p2 *= 2;
        spw = p2;
    }
    int rc = ensure_render_buffers(c, np * spw);
    if (rc) return rc;
    rc = ensure_arena(c, 3 * np);
    if (rc) return rc;
    rc = sync_scene_table(c);
    if (rc) return rc;
    free_all(c->rel_cost_allocs);
    wf_job j{};
    j.scene_id = 0;
    j.width = W;
    j.height = H;
    j.samples_per_pixel = P->samples_per_pixel;
    j.max_depth = P->max_depth;
    j.rr_min_depth = P->rr_min_depth;
    j.enable_cost_aware_rr = P->enable_cost_aware_rr;
    j.firefly_threshold = P->firefly_threshold;
    j.seed_lo = P->seed_lo;
    j.seed_hi = P->seed_hi;
    j.first_sample = P->first_sample;
    j.enable_env_nee = P->enable_env_nee;
    j.rel_cost_material = P->rel_cost_material;
    j.camera = P->camera;
    std::vector<DeviceJob> table(1);
    rc = make_device_job(c, j, 0, table[0]);
    if (rc) return rc;
    int64_t kernels_setup = 0;
    if (adaptive) {
        rc = ensure_adaptive(c, np, 3 * np * spw);
        if (rc) return rc;
        table[0].sample_buf = c->ad_buf;
        table[0].active = c->ad_active;
        table[0].sample0 = P->first_sample;
        table[0].wave_spp = spw;
        WF_CK(c, cudaMemsetAsync(c->ad_buf, 0, sizeof(float) * 3 * (size_t)(np * spw), s));
        WF_CK(c, cudaMemsetAsync(c->ad_mean, 0, sizeof(float) * (size_t)np, s));
        WF_CK(c, cudaMemsetAsync(c->ad_m2, 0, sizeof(float) * (size_t)np, s));
        WF_CK(c, cudaMemsetAsync(c->ad_count, 0, sizeof(int32_t) * (size_t)np, s));
        launch_fill_i32(c->ad_flag, np, 1, false, s);
        launch_fill_i32(c->ad_active, np, 0, true, s);
        kernels_setup = 2;
    }
    const bool tracking = P->enable_cost_tracking != 0;
    if (tracking) {
        const DeviceScene& S0 = c->scenes[0].S;
        rc = reset_cost_trackers(c, S0.num_materials, S0.num_textures);
        if (rc) return rc;
        kernels_setup += 1;
        table[0].cost_sum_mat = c->ct_mat.sum;
        table[0].cost_cnt_mat = c->ct_mat.cnt;
        table[0].cost_sum_tex = c->ct_tex.sum;
        table[0].cost_cnt_tex = c->ct_tex.cnt;
        table[0].rel_cost_material = c->ct_mat.rel_f;
    }
    rc = upload_jobs(c, table);
    if (rc) return rc;
    WF_CK(c, cudaMemsetAsync(c->arena, 0, sizeof(float) * 3 * (size_t)np, s));
    const bool graph = !tracking && use_graph(c, false, P->policy);
    // without a policy (and without a sort-or-skip threshold, a host decision)
    // the bounces need no host round trip
    const bool chain = !graph && P->policy == WF_POLICY_NONE &&
                       !(P->enable_ray_sort && c->tuning.sort_min_queue > 0);
    wf_render_stats stats{};
    stats.kernel_launches = kernels_setup;
    if (graph) {
        rc = zero_tally(c);
        if (rc) return rc;
    }
    float ms = 0.0f;
    int32_t n_active = (int32_t)np;
    int samples_run = P->samples_per_pixel;
    WF_CK(c, cudaEventRecord(c->ev[0], s));
    for (int s0 = 0, nspp = 0; s0 < P->samples_per_pixel; s0 += nspp) {
        nspp = std::min(spw, P->samples_per_pixel - s0);
        if (adaptive) {  // no wave crosses a check (AdaptiveSampler: from 32 samples, every 16)
            const int next_check = s0 < 32 ? 32 : (s0 / 16 + 1) * 16;
            nspp = std::min(nspp, next_check - s0);
        }
        const int64_t pix = adaptive ? (int64_t)n_active : np;
        std::vector<WaveChunk> ch(1);
        ch[0] = WaveChunk{0, P->first_sample + s0, nspp, adaptive ? n_active : 0, 0};
        rc = upload_wave(c, ch, pix * nspp);
        if (rc) return rc;
        if (graph)
            rc = wave_graph(c, P->max_depth, P->enable_ray_sort != 0, stats);
        else if (chain)
            rc = wave_chain(c, P->max_depth, P->enable_ray_sort != 0, table[0], stats, tracking, nspp);
        else
            rc = wave_host(c, pix * nspp, P->max_depth, P->policy, P->enable_ray_sort != 0, 0, P->rel_cost_material,
                           P->rel_cost_texture, &table[0], stats, tracking, nspp);
        if (rc) return rc;
        if (adaptive) {  // renderScene's per-sample adaptive block (.cpp:270-294)
            launch_adaptive_fold(c->ad_buf, np, nspp, s0 % spw, spw, c->arena, c->ad_mean, c->ad_m2, c->ad_count,
                                 c->ad_active, n_active, s);
            stats.kernel_launches += 1;
            if ((s0 + nspp) % 16 == 0) {
                launch_adaptive_check(c->ad_mean, c->ad_m2, c->ad_count, c->ad_active, n_active,
                                      P->adaptive_threshold, c->ad_flag, s);
                launch_compact_active(c->ad_flag, np, c->ad_pos, c->ad_bsums, c->ad_active, c->ad_nactive, s);
                stats.kernel_launches += 5;
                WF_CK(c, cudaMemcpyAsync(&n_active, c->ad_nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
                WF_CK(c, cudaStreamSynchronize(s));
                if (n_active == 0) {
                    samples_run = s0 + nspp;
                    break;
                }
            }
        }
    }
    stats.samples_run = samples_run;
    stats.active_pixels = adaptive ? n_active : (int32_t)np;
    c->last_adaptive = adaptive;
    c->last_np = np;
    c->last_spp = samples_run;
    WF_CK(c, cudaEventRecord(c->ev[1], s));
    WF_CK(c, cudaEventSynchronize(c->ev[1]));
    WF_CK(c, cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
    stats.ms_total = ms;
    if (graph) {
        rc = read_tally(c, stats);
        if (rc) return rc;
    }
    rc = check_device_flag(c);
    if (rc) return rc;
    if (st) *st = stats;
    return WF_OK;
}

// --------------------------------------------------------------------------
// Serving loop
// --------------------------------------------------------------------------

// First-fit allocator of accumulator ranges (floats) inside an arena.
struct RangeAllocator {
    std::map<int64_t, int64_t> free;  // offset -> length
    int64_t base = 0;                 // first float of the range in the arena
    int64_t total = 0;
    int64_t used = 0;
    void reset(int64_t first, int64_t n)
    {
        free.clear();
        base = first;
        if (n > 0) free[first] = n;
        total = n;
        used = 0;
    }
    int64_t alloc(int64_t n)
    {
        for (auto it = free.begin(); it != free.end(); ++it) {
            if (it->second < n) continue;
            const int64_t off = it->first, len = it->second;
            free.erase(it);
            if (len > n) free[off + n] = len - n;
            used += n;
            return off;
        }
        return -1;
    }
    void release(int64_t off, int64_t n)
    {
        used -= n;
        auto it = free.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free.erase(nx);
        }
        if (it != free.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free.erase(it);
            }
        }
    }
};

struct ServedJob {
    wf_job spec{};
    int state = WF_JOB_QUEUED;
    int samples_done = 0;   // samples of finished frames (in the job's sums)
    int scheduled = 0;      // samples handed to frames so far
    int frames = 0;
    int chunks_out = 0;     // frames appended and not yet finished
    int64_t accum_off = -1;
    int64_t accum_floats = 0;
    bool flushing = false;  // image copy in flight (its sums released), done at the next flush_complete
    double t_submit = 0, t_admit = -1, t_first = -1, t_done = -1;
    std::vector<float> final_image;
};

// One frame of a served job in the streaming wave: frame_spp samples of every
// pixel (fewer for the last), accumulated into sums of its own that are added
// to the job's sums once every one of its paths has finished, so the job's
// sums only ever hold whole frames.
struct ServerChunk {
    int64_t job = 0;          // served job id
    int slot = 0;             // device job table entry (the frame's sums)
    int first_sample = 0;
    int nspp = 0;
    int depth = 0;            // the job's max_depth
    bool first = false;       // the job's first frame (laid out ahead of the others)
    int64_t frame_off = 0;    // frame sums (floats into the arena)
    int64_t floats = 0;       // 3 * width * height
    int64_t path_offset = 0;  // absolute path index of its first path
    int64_t len = 0;          // width * height * nspp
    int64_t done_iter = -1;   // iterations after which all its paths have finished
};

// Served jobs by id: ids are 1, 2, 3, ... in submission order, so the table
// is a deque (stable references as it grows, constant-time lookup).
struct JobTable {
    std::deque<ServedJob> v;
    ServedJob& operator[](int64_t id) { return v[(size_t)(id - 1)]; }
    ServedJob* find(int64_t id) { return id >= 1 && id <= (int64_t)v.size() ? &v[(size_t)(id - 1)] : nullptr; }
    int64_t add(ServedJob&& j)
    {
        v.push_back(std::move(j));
        return (int64_t)v.size();
    }
};

double seconds_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Iterations (bounce + refill) per server step; even, so every step starts on
// the same queue of the ping-pong pair.
constexpr int kGroupIters = 8;

// What a step reads back: the tally, the next iteration's ray count, the
// stream state and the cursor after each iteration.
struct StepReadback {
    ull tally[4];
    ull live;
    StreamState st;
    int64_t log[kGroupIters];
};

}  // namespace

struct wf_server {
    wf_ctx* c = nullptr;
    wf_server_config cfg{};
    JobTable jobs;
    std::deque<int64_t> queue;       // submitted, not admitted yet
    std::deque<int64_t> fresh;       // admitted, no frame appended yet
    std::deque<int64_t> to_schedule; // admitted, frames left to append (admission order)
    int64_t running = 0;             // admitted jobs not finished or cancelled
    std::chrono::steady_clock::time_point t0;
    RangeAllocator alloc;    // job sums
    RangeAllocator frames;   // frame sums
    int64_t wave_paths = 0;  // streaming queue capacity
    int64_t wave_bytes = 0;
    float* tmp = nullptr;  // averaged image staging (device)
    int64_t tmp_floats = 0;
    float* host_stage = nullptr;  // finished images (page-locked)
    int64_t host_stage_floats = 0;
    std::vector<int64_t> finishing;  // jobs whose last frame finished this step
    std::vector<int64_t> flushing;   // jobs whose averaged images are being copied into host_stage
    // page-locked sources of the step's uploads (read by the device after the
    // call returns; rewritten only after the step's final wait)
    DeviceJob* job_stage = nullptr;    // one per table entry
    WaveChunk* chunk_stage = nullptr;  // the chunk list
    int64_t* state_stage = nullptr;    // [0] total, [1] nchunks
    // Streaming wave, owned by the server (its queues hold paths between steps)
    std::vector<void*> allocs;
    RayQueueDev rq[2]{};
    HitQueueDev hq{};
    ShadowQueueDev sh{};
    ull* counters = nullptr;  // as the context's: [0] rays [1] hits [2] shadows [3] next [4] [5] work
    ull* tally = nullptr;
    int* err = nullptr;
    float* arena = nullptr;
    DeviceJob* d_jobs = nullptr;
    std::vector<int> free_slots;
    WaveChunk* d_chunks = nullptr;
    int chunks_cap = 0;
    StreamState* d_state = nullptr;
    int64_t* d_log = nullptr;
    StepReadback* rb = nullptr;  // page-locked
    cudaEvent_t ev[3]{};  // [0], [1] around the step's graph, [2] after the finished images' copy
    cudaGraphExec_t exec = nullptr;
    const void* exec_table = nullptr;  // scene table, variant and tree the capture used
    int exec_variant = -1, exec_tree = -1, exec_lean = -1;
    bool exec_dense = false;
    int64_t cursor = 0;       // paths generated (device cursor after the last step)
    int64_t appended = 0;     // paths appended (the list's end)
    int64_t live = 0;         // rays queued for the next iteration
    int64_t iters = 0;        // iterations run
    ull tally_prev[4] = {};
    std::deque<ServerChunk> pending;   // not every path generated yet, in list order
    std::vector<ServerChunk> inflight; // generated, not yet finished
};

namespace {

// Device bytes per path of the streaming wave: two RayQueues (14 columns),
// one hit queue (5) and the shadow queue (3 x 12).
constexpr int64_t kServerPathsPerWave = int64_t(1) << 24;
constexpr int64_t kBytesPerPath = 2 * 14 * 4 + 5 * 4 + 3 * 12 * 4;
constexpr int kServerSlots = 1 << 14;  // frames appended or in flight at once

void server_free(wf_server* sv)
{
    if (sv->exec) cudaGraphExecDestroy(sv->exec);
    sv->exec = nullptr;
    for (auto& e : sv->ev)
        if (e) cudaEventDestroy(e);
    if (sv->rb) cudaFreeHost(sv->rb);
    sv->rb = nullptr;
    for (void* p : {(void*)sv->host_stage, (void*)sv->job_stage, (void*)sv->chunk_stage, (void*)sv->state_stage})
        if (p) cudaFreeHost(p);
    sv->host_stage = nullptr;
    sv->job_stage = nullptr;
    sv->chunk_stage = nullptr;
    sv->state_stage = nullptr;
    free_all(sv->allocs);
    cudaFree(sv->tmp);
    sv->tmp = nullptr;
}

int server_alloc(wf_server* sv, int64_t arena_floats)
{
    wf_ctx* c = sv->c;
    auto& A = sv->allocs;
    const size_t n = (size_t)sv->wave_paths;
    for (int q = 0; q < 2; ++q) {
        RayQueueDev& r = sv->rq[q];
        WF_CK(c, wf_dalloc(A, &r.ox, n)); WF_CK(c, wf_dalloc(A, &r.oy, n)); WF_CK(c, wf_dalloc(A, &r.oz, n));
        WF_CK(c, wf_dalloc(A, &r.dx, n)); WF_CK(c, wf_dalloc(A, &r.dy, n)); WF_CK(c, wf_dalloc(A, &r.dz, n));
        WF_CK(c, wf_dalloc(A, &r.tr, n)); WF_CK(c, wf_dalloc(A, &r.tg, n)); WF_CK(c, wf_dalloc(A, &r.tb, n));
        WF_CK(c, wf_dalloc(A, &r.pdf, n));
        WF_CK(c, wf_dalloc(A, &r.pixel, n)); WF_CK(c, wf_dalloc(A, &r.depth, n)); WF_CK(c, wf_dalloc(A, &r.sample, n));
        WF_CK(c, wf_dalloc(A, &r.job, n));
        r.capacity = sv->wave_paths;
    }
    HitQueueDev& h = sv->hq;
    WF_CK(c, wf_dalloc(A, &h.ray, n)); WF_CK(c, wf_dalloc(A, &h.tri, n)); WF_CK(c, wf_dalloc(A, &h.t, n));
    WF_CK(c, wf_dalloc(A, &h.bu, n)); WF_CK(c, wf_dalloc(A, &h.bv, n));
    h.capacity = sv->wave_paths;
    const size_t ns = 3 * n;
    ShadowQueueDev& q = sv->sh;
    WF_CK(c, wf_dalloc(A, &q.ox, ns)); WF_CK(c, wf_dalloc(A, &q.oy, ns)); WF_CK(c, wf_dalloc(A, &q.oz, ns));
    WF_CK(c, wf_dalloc(A, &q.dx, ns)); WF_CK(c, wf_dalloc(A, &q.dy, ns)); WF_CK(c, wf_dalloc(A, &q.dz, ns));
    WF_CK(c, wf_dalloc(A, &q.dist, ns));
    WF_CK(c, wf_dalloc(A, &q.cr, ns)); WF_CK(c, wf_dalloc(A, &q.cg, ns)); WF_CK(c, wf_dalloc(A, &q.cb, ns));
    WF_CK(c, wf_dalloc(A, &q.pixel, ns)); WF_CK(c, wf_dalloc(A, &q.job, ns));
    q.capacity = (int64_t)ns;
    WF_CK(c, wf_dalloc(A, &sv->counters, 8));
    WF_CK(c, wf_dalloc(A, &sv->tally, 8));
    WF_CK(c, wf_dalloc(A, &sv->err, 1));
    WF_CK(c, wf_dalloc(A, &sv->arena, (size_t)arena_floats));
    WF_CK(c, wf_dalloc(A, &sv->d_jobs, (size_t)kServerSlots));
    sv->chunks_cap = kServerSlots;
    WF_CK(c, wf_dalloc(A, &sv->d_chunks, (size_t)sv->chunks_cap));
    WF_CK(c, wf_dalloc(A, &sv->d_state, 1));
    WF_CK(c, wf_dalloc(A, &sv->d_log, (size_t)kGroupIters));
    WF_CK(c, cudaMallocHost(&sv->rb, sizeof(StepReadback)));
    WF_CK(c, cudaMallocHost(&sv->job_stage, sizeof(DeviceJob) * (size_t)kServerSlots));
    WF_CK(c, cudaMallocHost(&sv->chunk_stage, sizeof(WaveChunk) * (size_t)sv->chunks_cap));
    WF_CK(c, cudaMallocHost(&sv->state_stage, sizeof(int64_t) * 2));
    for (auto& e : sv->ev) WF_CK(c, cudaEventCreate(&e));
    cudaStream_t s = c->stream;
    WF_CK(c, cudaMemsetAsync(sv->counters, 0, sizeof(ull) * 8, s));
    WF_CK(c, cudaMemsetAsync(sv->tally, 0, sizeof(ull) * 8, s));
    WF_CK(c, cudaMemsetAsync(sv->err, 0, sizeof(int), s));
    WF_CK(c, cudaMemsetAsync(sv->d_state, 0, sizeof(StreamState), s));
    WF_CK(c, cudaStreamSynchronize(s));
    sv->free_slots.clear();
    for (int k = kServerSlots - 1; k >= 0; --k) sv->free_slots.push_back(k);
    return WF_OK;
}

// The iterations of one server step, captured once: every live path does one
// bounce (closest hit, shading, shadow rays) and the paths that ended are
// replaced by camera rays of the next chunks.  Returns the kernel count.
int record_stream_group(wf_server* sv, int tree)
{
    wf_ctx* c = sv->c;
    cudaStream_t s = c->stream;
    LaunchCfg PC = persist_cfg(c);
    PC.ray_order = hits_in_ray_order(WF_POLICY_NONE);
    const LaunchCfg WC = wide_cfg(c);
    const WaveTables T{c->d_scene_table, sv->d_jobs, DeviceScene{}, DeviceJob{}, true, tree};
    ull* n = sv->counters;
    int kernels = 0;
    for (int it = 0; it < kGroupIters; ++it) {
        const int cur = it & 1;
        launch_trace_render(T, sv->rq[cur], n, sv->hq, n + 1, sv->arena, n + 4, sv->err, PC, s);
        launch_compact_hits(T, sv->rq[cur], n, sv->hq, n + 1, sv->arena, WC, s);
        launch_shade(T, sv->rq[cur], sv->hq, n + 1, sv->sh, n + 2, sv->rq[1 - cur], n + 3, sv->arena, sv->err, PC, s);
        launch_occluded_render(T, sv->sh, n + 2, sv->arena, n + 5, sv->err, PC, s);
        launch_stream_plan(n, sv->d_state, sv->wave_paths, sv->d_log, it, s);
        launch_camera_refill(sv->d_chunks, sv->d_state, sv->d_jobs, sv->rq[1 - cur], WC, s);
        launch_bounce_end(n, sv->tally, s);
        kernels += 7;
    }
    return kernels;
}

int ensure_stream_graph(wf_server* sv)
{
    wf_ctx* c = sv->c;
    int tree = kTreeBinary;
    int rc = table_tree(c, tree);
    if (rc) return rc;
    const LaunchCfg pc = persist_cfg(c);
    const bool dense = pc.max_scene_bytes >= kDenseSceneBytes;
    if (sv->exec && sv->exec_table == c->d_scene_table && sv->exec_variant == c->tuning.trace_variant &&
        sv->exec_tree == tree && sv->exec_lean == pc.lean_multi && sv->exec_dense == dense)
        return WF_OK;
    if (sv->exec) cudaGraphExecDestroy(sv->exec);
    sv->exec = nullptr;
    cudaStream_t s = c->stream;
    cudaGraph_t graph = nullptr;
    WF_CK(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    record_stream_group(sv, tree);
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (e != cudaSuccess) return set_err(c, WF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&sv->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return set_err(c, WF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    sv->exec_table = c->d_scene_table;
    sv->exec_variant = c->tuning.trace_variant;
    sv->exec_tree = tree;
    sv->exec_lean = pc.lean_multi;
    sv->exec_dense = dense;
    return WF_OK;
}

// Jobs whose last frame finished this step: their averaged images are made
// together at the end of the step and copied into page-locked memory with no
// wait (their sums are released at once: later work on the stream runs after
// the copy).  flush_complete hands the images over while the next step's
// iterations run, so the host copies overlap the device.
int flush_begin(wf_server* sv)
{
    if (sv->finishing.empty()) return WF_OK;
    wf_ctx* c = sv->c;
    int64_t total = 0;
    for (int64_t id : sv->finishing) total += sv->jobs[id].accum_floats;
    if (total > sv->tmp_floats) {
        cudaFree(sv->tmp);
        sv->tmp = nullptr;
        sv->tmp_floats = 0;
        WF_CK(c, cudaMalloc(&sv->tmp, sizeof(float) * total));
        sv->tmp_floats = total;
    }
    if (total > sv->host_stage_floats) {  // no copy into it is in flight (flush_complete ran first)
        cudaFreeHost(sv->host_stage);
        sv->host_stage = nullptr;
        sv->host_stage_floats = 0;
        WF_CK(c, cudaMallocHost(&sv->host_stage, sizeof(float) * total));
        sv->host_stage_floats = total;
    }
    int64_t o = 0;
    for (int64_t id : sv->finishing) {
        ServedJob& j = sv->jobs[id];
        launch_finalize(sv->arena + j.accum_off, j.accum_floats, (float)j.samples_done, sv->tmp + o, c->stream);
        o += j.accum_floats;
        sv->alloc.release(j.accum_off, j.accum_floats);
        j.accum_off = -1;
        j.flushing = true;
    }
    WF_CK(c, cudaMemcpyAsync(sv->host_stage, sv->tmp, sizeof(float) * total, cudaMemcpyDeviceToHost, c->stream));
    WF_CK(c, cudaEventRecord(sv->ev[2], c->stream));
    sv->flushing.swap(sv->finishing);
    sv->finishing.clear();
    return WF_OK;
}

int flush_complete(wf_server* sv, wf_server_step_info& si)
{
    if (sv->flushing.empty()) return WF_OK;
    wf_ctx* c = sv->c;
    WF_CK(c, cudaEventSynchronize(sv->ev[2]));
    const double now = seconds_since(sv->t0);
    int64_t o = 0;
    for (int64_t id : sv->flushing) {
        ServedJob& j = sv->jobs[id];
        j.final_image.assign(sv->host_stage + o, sv->host_stage + o + j.accum_floats);
        o += j.accum_floats;
        j.flushing = false;
        j.state = WF_JOB_DONE;
        j.t_done = now;
        si.completed_this_step++;
        sv->running--;
    }
    sv->flushing.clear();
    return WF_OK;
}

// Appends the next frame of running job `id` to the streaming wave's chunk
// list: frame sums and a job-table entry (a DeviceJob whose sums are the
// frame's).  room = false when no frame sums or table entry are free.
int append_frame(wf_server* sv, int64_t id, ServedJob& j, bool& room)
{
    wf_ctx* c = sv->c;
    room = false;
    const int left = j.spec.samples_per_pixel - j.scheduled;
    if (j.state != WF_JOB_RUNNING || left <= 0) {
        room = true;
        return WF_OK;
    }
    if (sv->free_slots.empty() || (int)sv->pending.size() >= sv->chunks_cap) return WF_OK;
    const int64_t foff = sv->frames.alloc(j.accum_floats);
    if (foff < 0) return WF_OK;
    ServerChunk k;
    k.job = id;
    k.slot = sv->free_slots.back();
    sv->free_slots.pop_back();
    k.first_sample = j.spec.first_sample + j.scheduled;
    k.nspp = std::min(left, sv->cfg.frame_spp);
    k.depth = j.spec.max_depth;
    k.first = j.scheduled == 0;
    k.frame_off = foff;
    k.floats = j.accum_floats;
    k.len = (int64_t)j.spec.width * j.spec.height * k.nspp;
    k.path_offset = sv->appended;
    DeviceJob& dj = sv->job_stage[k.slot];
    int rc = make_device_job(c, j.spec, foff, dj);
    if (rc) return rc;
    WF_CK(c, cudaMemcpyAsync(sv->d_jobs + k.slot, &dj, sizeof(dj), cudaMemcpyHostToDevice, c->stream));
    WF_CK(c, cudaMemsetAsync(sv->arena + foff, 0, sizeof(float) * (size_t)k.floats, c->stream));
    sv->appended += k.len;
    j.scheduled += k.nspp;
    j.chunks_out++;
    sv->pending.push_back(k);
    room = true;
    return WF_OK;
}

// A frame whose paths have all finished: its sums join the job's (or are
// dropped for a cancelled job); its sums and table entry are freed.
int retire_chunk(wf_server* sv, const ServerChunk& k, double now, wf_server_step_info& si)
{
    wf_ctx* c = sv->c;
    ServedJob& j = sv->jobs[k.job];
    if (j.state == WF_JOB_RUNNING) launch_add_floats(sv->arena + j.accum_off, sv->arena + k.frame_off, k.floats, c->stream);
    sv->frames.release(k.frame_off, k.floats);
    sv->free_slots.push_back(k.slot);
    j.chunks_out--;
    if (j.state == WF_JOB_RUNNING) {
        j.samples_done += k.nspp;
        j.frames++;
        if (j.t_first < 0) j.t_first = now;
        if (j.samples_done >= j.spec.samples_per_pixel) sv->finishing.push_back(k.job);
    } else if (j.chunks_out == 0 && j.accum_off >= 0) {  // cancelled: its sums go once no frame runs
        sv->alloc.release(j.accum_off, j.accum_floats);
        j.accum_off = -1;
    }
    return WF_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

namespace {

// writeAveragedImage (.cpp:127-137) into the context's image buffer.
int finalize_image(wf_ctx* c, const wf_render_params* P, wf_render_stats* st)
{
    const int64_t np = (int64_t)P->width * P->height, nf = 3 * np;
    if (nf > c->image_floats) {
        cudaFree(c->image);
        c->image = nullptr;
        c->image_floats = 0;
        WF_CK(c, cudaMalloc(&c->image, sizeof(float) * nf));
        c->image_floats = nf;
    }
    if (c->last_adaptive)
        launch_finalize_counts(c->arena, c->ad_count, np, c->image, c->stream);
    else
        launch_finalize(c->arena, nf, (float)P->samples_per_pixel, c->image, c->stream);
    if (st) st->kernel_launches += 1;
    return WF_OK;
}

}  // namespace

int wf_render(wf_ctx* c, const wf_render_params* P, float* image, wf_render_stats* st)
{
    if (!c || !image) return set_err(c, WF_ERR_INVALID_ARGUMENT, "null argument");
    int rc = validate_params(c, P);
    if (rc) return rc;
    cudaSetDevice(c->device);
    rc = render_single(c, P, st);
    if (rc) return rc;
    const int64_t nf = 3 * (int64_t)P->width * P->height;
    rc = finalize_image(c, P, st);
    if (rc) return rc;
    WF_CK(c, cudaMemcpyAsync(image, c->image, sizeof(float) * nf, cudaMemcpyDeviceToHost, c->stream));
    WF_CK(c, cudaStreamSynchronize(c->stream));
    return WF_OK;
}

int wf_autotune(wf_ctx* c, const wf_render_params* P, wf_tuning* out, double* out_ms)
{
    if (!c || !P) return set_err(c, WF_ERR_INVALID_ARGUMENT, "null argument");
    int rc = validate_params(c, P);
    if (rc) return rc;
    cudaSetDevice(c->device);
    wf_render_params trial = *P;
    const int64_t np = (int64_t)P->width * P->height;
    int spw = P->spp_per_wave > 0 ? P->spp_per_wave : (int)std::max<int64_t>(1, c->paths_per_wave / np);
    trial.samples_per_pixel = std::max(1, std::min(spw, P->samples_per_pixel));
    trial.spp_per_wave = trial.samples_per_pixel;
    trial.enable_adaptive_sampling = 0;
    trial.enable_cost_tracking = 0;
    const wf_tuning base = c->tuning;
    wf_tuning best = base;
    double best_ms = -1.0;
    const int variants[2] = {0, 1};
    const int blocks[5] = {4, 8, 12, 16, 24};
    const int graphs[2] = {2, 1};
    for (int v : variants)
        for (int b : blocks)
            for (int g : graphs) {
                wf_tuning t = base;
                t.trace_variant = v;
                t.persistent_blocks_per_sm = b;
                t.graph_mode = g;
                c->tuning = t;
                double ms = 0.0;
                for (int rep = 0; rep < 3; ++rep) {
                    wf_render_stats st{};
                    rc = render_single(c, &trial, &st);
                    if (rc) {
                        c->tuning = base;
                        return rc;
                    }
                    if (rep > 0) ms += st.ms_total;
                }
                ms *= 0.5;
                if (best_ms < 0.0 || ms < best_ms) {
                    best_ms = ms;
                    best = t;
                }
            }
    if (P->policy != WF_POLICY_NONE || P->enable_ray_sort) {  // sort-or-skip threshold, ray key width
        const int thresholds[5] = {0, 1 << 18, 1 << 20, 1 << 22, INT32_MAX};
        const int widths[3] = {33, 24, 16};
        const wf_tuning launch = best;
        for (int trial_no = 0; trial_no < 5 + (P->enable_ray_sort ? 2 : 0); ++trial_no) {
            wf_tuning t = launch;
            const int th = trial_no < 5 ? thresholds[trial_no] : 0;
            t.sort_min_queue = th;
            t.ray_sort_bits = trial_no < 5 ? 33 : widths[trial_no - 4];
            c->tuning = t;
            double ms = 0.0;
            for (int rep = 0; rep < 3; ++rep) {
                wf_render_stats st{};
                rc = render_single(c, &trial, &st);
                if (rc) {
                    c->tuning = base;
                    return rc;
                }
                if (rep > 0) ms += st.ms_total;
            }
            ms *= 0.5;
            if (trial_no == 0 || ms < best_ms) {  // the launch winner re-timed at 0 sets the bar
                best_ms = ms;
                best = t;
            }
        }
    }
    c->tuning = best;
    if (out) *out = best;
    if (out_ms) *out_ms = best_ms;
    return WF_OK;
}

int wf_render_device(wf_ctx* c, const wf_render_params* P, wf_render_stats* st)
{
    if (!c) return WF_ERR_INVALID_ARGUMENT;
    int rc = validate_params(c, P);
    if (rc) return rc;
    cudaSetDevice(c->device);
    rc = render_single(c, P, st);
    if (rc) return rc;
    rc = finalize_image(c, P, st);
    if (rc) return rc;
    WF_CK(c, cudaStreamSynchronize(c->stream));
    return WF_OK;
}

int wf_cost_tracker_state(wf_ctx* c, double* rel_mat, int32_t nmat, double* rel_tex, int32_t ntex)
{
    if (!c) return WF_ERR_INVALID_ARGUMENT;
    if ((rel_mat && nmat != c->ct_mat.items) || (rel_tex && ntex != c->ct_tex.items) || !c->ct_mat.rel)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "no tracker of that size (render with enable_cost_tracking)");
    if (rel_mat && nmat > 0)
        WF_CK(c, cudaMemcpyAsync(rel_mat, c->ct_mat.rel, sizeof(double) * nmat, cudaMemcpyDeviceToHost, c->stream));
    if (rel_tex && ntex > 0)
        WF_CK(c, cudaMemcpyAsync(rel_tex, c->ct_tex.rel, sizeof(double) * ntex, cudaMemcpyDeviceToHost, c->stream));
    WF_CK(c, cudaStreamSynchronize(c->stream));
    return WF_OK;
}

int wf_cost_tracker_replay(wf_ctx* c, int32_t items, int32_t steps, const uint64_t* sums, const uint32_t* counts,
                           double* rel_out)
{
    if (!c || items <= 0 || steps < 0 || (steps > 0 && (!sums || !counts)) || !rel_out)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "bad replay arguments");
    cudaSetDevice(c->device);
    int rc = reset_cost_trackers(c, items, 0);
    if (rc) return rc;
    for (int k = 0; k < steps; ++k) {
        WF_CK(c, cudaMemcpyAsync(c->ct_mat.sum, sums + (size_t)k * items, sizeof(uint64_t) * items,
                                 cudaMemcpyHostToDevice, c->stream));
        WF_CK(c, cudaMemcpyAsync(c->ct_mat.cnt, counts + (size_t)k * items, sizeof(uint32_t) * items,
                                 cudaMemcpyHostToDevice, c->stream));
        launch_cost_update(c->ct_mat, c->ct_tex, 1, c->stream);
        WF_CK(c, cudaStreamSynchronize(c->stream));  // the host rows are read before the next step
    }
    WF_CK(c, cudaMemcpyAsync(rel_out, c->ct_mat.rel, sizeof(double) * items, cudaMemcpyDeviceToHost, c->stream));
    WF_CK(c, cudaStreamSynchronize(c->stream));
    return WF_OK;
}

int wf_adaptive_sample_counts(wf_ctx* c, int32_t* counts, int64_t n)
{
    if (!c || !counts) return set_err(c, WF_ERR_INVALID_ARGUMENT, "null argument");
    if (n != c->last_np || n <= 0) return set_err(c, WF_ERR_INVALID_ARGUMENT, "pixel count differs from the last render");
    if (!c->last_adaptive) {
        std::fill(counts, counts + n, c->last_spp);
        return WF_OK;
    }
    WF_CK(c, cudaMemcpyAsync(counts, c->ad_count, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    WF_CK(c, cudaStreamSynchronize(c->stream));
    return WF_OK;
}

int wf_image_download(wf_ctx* c, float* image, int64_t nf)
{
    if (!c || !image || nf < 0) return set_err(c, WF_ERR_INVALID_ARGUMENT, "null argument");
    if (nf > c->image_floats) return set_err(c, WF_ERR_CAPACITY, "no image of that size");
    WF_CK(c, cudaMemcpyAsync(image, c->image, sizeof(float) * (size_t)nf, cudaMemcpyDeviceToHost, c->stream));
    WF_CK(c, cudaStreamSynchronize(c->stream));
    return WF_OK;
}

int wf_render_accumulate(wf_ctx* c, const wf_render_params* P, float* accum_rgb, wf_render_stats* st)
{
    if (!c || !accum_rgb) return set_err(c, WF_ERR_INVALID_ARGUMENT, "null argument");
    int rc = validate_params(c, P);
    if (rc) return rc;
    cudaSetDevice(c->device);
    rc = render_single(c, P, st);
    if (rc) return rc;
    const int64_t nf = 3 * (int64_t)P->width * P->height;
    WF_CK(c, cudaMemcpyAsync(accum_rgb, c->arena, sizeof(float) * nf, cudaMemcpyDeviceToHost, c->stream));
    WF_CK(c, cudaStreamSynchronize(c->stream));
    return WF_OK;
}

int wf_render_batch(wf_ctx* c, const wf_job* jobs, int32_t njobs, float* const* images, wf_render_stats* st)
{
    if (!c || (njobs > 0 && !jobs) || njobs < 0) return set_err(c, WF_ERR_INVALID_ARGUMENT, "null argument");
    if (njobs == 0) return WF_OK;
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    int rc;
    int64_t floats = 0, max_np = 0;
    int max_depth = 0;
    std::vector<int64_t> offs(njobs);
    for (int j = 0; j < njobs; ++j) {
        if ((rc = validate_job(c, jobs[j]))) return rc;
        const int64_t np = (int64_t)jobs[j].width * jobs[j].height;
        offs[j] = floats;
        floats += 3 * np;
        max_np = std::max(max_np, np);
        max_depth = std::max(max_depth, jobs[j].max_depth);
    }
    const int64_t cap = std::max(c->paths_per_wave, max_np);
    if ((rc = ensure_render_buffers(c, cap))) return rc;
    if ((rc = ensure_arena(c, floats))) return rc;
    if ((rc = sync_scene_table(c))) return rc;
    free_all(c->rel_cost_allocs);
    std::vector<DeviceJob> table(njobs);
    for (int j = 0; j < njobs; ++j)
        if ((rc = make_device_job(c, jobs[j], offs[j], table[j]))) return rc;
    if ((rc = upload_jobs(c, table))) return rc;
    WF_CK(c, cudaMemsetAsync(c->arena, 0, sizeof(float) * (size_t)floats, s));
    std::vector<int32_t> scene_ids(njobs);
    for (int j = 0; j < njobs; ++j) scene_ids[j] = jobs[j].scene_id;
    const WaveSceneScope scene_scope(c, scene_ids);
    const bool graph = use_graph(c, true, WF_POLICY_NONE);
    wf_render_stats stats{};
    if (graph && (rc = zero_tally(c))) return rc;
    std::vector<int> done(njobs, 0);
    float ms = 0.0f;
    WF_CK(c, cudaEventRecord(c->ev[0], s));
    int next = 0;  // first job with samples left
    while (next < njobs) {
        std::vector<WaveChunk> chunks;
        int64_t total = 0;
        int wave_depth = 0;
        for (int j = next; j < njobs; ++j) {
            const int64_t np = (int64_t)jobs[j].width * jobs[j].height;
            const int left = jobs[j].samples_per_pixel - done[j];
            if (left <= 0) continue;
            const int64_t room = cap - total;
            if (np > room) break;
            const int nspp = (int)std::min<int64_t>(left, room / np);
            chunks.push_back(WaveChunk{j, jobs[j].first_sample + done[j], nspp, 0, total});
            total += np * nspp;
            done[j] += nspp;
            wave_depth = std::max(wave_depth, jobs[j].max_depth);
        }
        if (chunks.empty()) return set_err(c, WF_ERR_CAPACITY, "no job fits a wave");
        if ((rc = upload_wave(c, chunks, total))) return rc;
        // without graph replay a lone job issues its bounces back to back with
        // device-side counts (the single-job render's chain); several jobs in
        // one wave take the host loop
        if (graph)
            rc = wave_graph(c, max_depth, false, stats);
        else if (njobs == 1)
            rc = wave_chain(c, wave_depth, false, table[0], stats, false, 0);
        else
            rc = wave_host(c, total, wave_depth, WF_POLICY_NONE, false, 0, nullptr, nullptr, nullptr, stats);
        if (rc) return rc;
        while (next < njobs && done[next] >= jobs[next].samples_per_pixel) ++next;
    }
    WF_CK(c, cudaEventRecord(c->ev[1], s));
    WF_CK(c, cudaEventSynchronize(c->ev[1]));
    WF_CK(c, cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
    stats.ms_total = ms;
    if (graph && (rc = read_tally(c, stats))) return rc;
    if ((rc = check_device_flag(c))) return rc;
    if (images) {
        float* tmp = nullptr;
        WF_CK(c, cudaMalloc(&tmp, sizeof(float) * 3 * (size_t)max_np));
        for (int j = 0; j < njobs; ++j) {
            if (!images[j]) continue;
            const int64_t nf = 3 * (int64_t)jobs[j].width * jobs[j].height;
            launch_finalize(c->arena + offs[j], nf, (float)jobs[j].samples_per_pixel, tmp, s);
            cudaMemcpyAsync(images[j], tmp, sizeof(float) * nf, cudaMemcpyDeviceToHost, s);
            stats.kernel_launches += 1;
        }
        cudaError_t e = cudaStreamSynchronize(s);
        cudaFree(tmp);
        if (e != cudaSuccess) return set_err(c, WF_ERR_CUDA, cudaGetErrorString(e));
    }
    if (st) *st = stats;
    return WF_OK;
}

// ---- serving loop ---------------------------------------------------------

int wf_server_create(wf_ctx* c, const wf_server_config* cfg, wf_server** out)
{
    if (!c || !cfg || !out) return WF_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    cudaSetDevice(c->device);
    wf_server* sv = new wf_server();
    sv->c = c;
    sv->cfg = *cfg;
    if (sv->cfg.frame_spp <= 0) sv->cfg.frame_spp = 8;
    // The queue capacity of the streaming wave: every step runs kGroupIters
    // bounces of up to this many paths, so it sets the latency of a step and
    // the time a frame takes to finish (max_depth iterations).  On the served
    // mix 2^24 paths against 2^23: +9% throughput, first frames p99 0.13 s
    // instead of 0.09 s.
    sv->wave_paths = cfg->max_paths_per_wave > 0 ? cfg->max_paths_per_wave
                                                 : std::min<int64_t>(c->paths_per_wave, kServerPathsPerWave);
    sv->wave_bytes = sv->wave_paths * kBytesPerPath;
    const int64_t accum_floats = (cfg->hbm_budget_bytes - sv->wave_bytes) / 4;
    // Frame sums get a share of their own, at least two frames of the largest
    // image a job may have (width*height <= the queue capacity): while no
    // frame is out the whole share is free, so a frame always fits.
    const int64_t frame_floats = std::max<int64_t>(accum_floats / 8, 2 * 3 * sv->wave_paths);
    if (accum_floats - frame_floats <= 0) {
        delete sv;
        return set_err(c, WF_ERR_OUT_OF_MEMORY, "HBM budget smaller than the wave buffers and frame sums");
    }
    int rc = sync_scene_table(c);
    if (!rc) rc = server_alloc(sv, accum_floats);
    if (rc) {
        server_free(sv);
        delete sv;
        return rc;
    }
    sv->alloc.reset(0, accum_floats - frame_floats);
    sv->frames.reset(accum_floats - frame_floats, frame_floats);
    sv->t0 = std::chrono::steady_clock::now();
    *out = sv;
    return WF_OK;
}

int wf_server_destroy(wf_server* sv)
{
    if (!sv) return WF_OK;
    cudaSetDevice(sv->c->device);
    cudaStreamSynchronize(sv->c->stream);
    server_free(sv);
    delete sv;
    return WF_OK;
}

double wf_server_clock(const wf_server* sv) { return sv ? seconds_since(sv->t0) : 0.0; }

int wf_server_submit(wf_server* sv, const wf_job* job, int64_t* out_id)
{
    if (!sv || !job || !out_id) return WF_ERR_INVALID_ARGUMENT;
    int rc = validate_job(sv->c, *job);
    if (rc) return rc;
    ServedJob j;
    j.spec = *job;
    j.spec.rel_cost_material = nullptr;  // a request carries no cost table across calls
    j.spec.enable_cost_aware_rr = 0;
    j.t_submit = seconds_since(sv->t0);
    j.accum_floats = 3 * (int64_t)job->width * job->height;
    const bool reject = j.accum_floats > sv->alloc.total || (int64_t)job->width * job->height > sv->wave_paths;
    if (reject) j.state = WF_JOB_REJECTED;
    const int64_t id = sv->jobs.add(std::move(j));
    if (!reject) sv->queue.push_back(id);
    *out_id = id;
    return WF_OK;
}

// One step of the service: admit jobs, append frames of the running jobs to
// the streaming wave's chunk list, run kGroupIters bounce iterations (a
// captured graph), then retire the frames whose paths have all finished.
int wf_server_step(wf_server* sv, wf_server_step_info* info)
{
    if (!sv) return WF_ERR_INVALID_ARGUMENT;
    wf_ctx* c = sv->c;
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    int rc = sync_scene_table(c);
    if (rc) return rc;
    wf_server_step_info si{};
    // 1. admit in arrival order while the job's sums fit the budget
    while (!sv->queue.empty()) {
        ServedJob& j = sv->jobs[sv->queue.front()];
        if (j.state != WF_JOB_QUEUED) {
            sv->queue.pop_front();
            continue;
        }
        const int64_t off = sv->alloc.alloc(j.accum_floats);
        if (off < 0) break;
        j.accum_off = off;
        j.state = WF_JOB_RUNNING;
        j.t_admit = seconds_since(sv->t0);
        WF_CK(c, cudaMemsetAsync(sv->arena + off, 0, sizeof(float) * (size_t)j.accum_floats, s));
        const int64_t id = sv->queue.front();
        sv->queue.pop_front();
        sv->running++;
        if (j.spec.max_depth == 0) {  // renderScene traces depths 0 .. maxDepth-1: nothing
            j.samples_done = j.scheduled = j.spec.samples_per_pixel;
            j.frames = 1;
            j.t_first = seconds_since(sv->t0);
            sv->finishing.push_back(id);
            continue;
        }
        sv->fresh.push_back(id);
        sv->to_schedule.push_back(id);
    }
    // 2. append frames until the list holds what one step can generate at most
    // (kGroupIters full queues): first the first frame of every job that has
    // none (laid out ahead of the rest, below), then the further frames of
    // the running jobs in admission order, so jobs finish in the order they
    // came while a new one shows a frame a few bounces after it starts.
    const int64_t target = (int64_t)kGroupIters * sv->wave_paths;
    bool room = true;
    while (room && !sv->fresh.empty() && sv->appended - sv->cursor < 2 * target) {
        ServedJob& j = sv->jobs[sv->fresh.front()];
        if (j.state == WF_JOB_RUNNING && j.scheduled == 0) {
            if ((rc = append_frame(sv, sv->fresh.front(), j, room))) return rc;
            if (!room) break;
        }
        sv->fresh.pop_front();
    }
    while (room && !sv->to_schedule.empty() && sv->appended - sv->cursor < target) {
        const int64_t id = sv->to_schedule.front();
        ServedJob& j = sv->jobs[id];
        while (room && j.state == WF_JOB_RUNNING && j.scheduled < j.spec.samples_per_pixel &&
               sv->appended - sv->cursor < target)
            if ((rc = append_frame(sv, id, j, room))) return rc;
        if (j.state != WF_JOB_RUNNING || j.scheduled >= j.spec.samples_per_pixel) sv->to_schedule.pop_front();
        else break;
    }
    // 3. lay the unstarted frames out again, first frames of jobs ahead (the
    // front frame may be partly generated and keeps its place)
    {
        auto first_unstarted = sv->pending.begin();
        if (first_unstarted != sv->pending.end() && first_unstarted->path_offset < sv->cursor) ++first_unstarted;
        std::stable_partition(first_unstarted, sv->pending.end(), [](const ServerChunk& k) { return k.first; });
        int64_t off = first_unstarted == sv->pending.begin() ? sv->cursor
                                                             : sv->pending.front().path_offset + sv->pending.front().len;
        for (auto it = first_unstarted; it != sv->pending.end(); ++it) {
            it->path_offset = off;
            off += it->len;
        }
        sv->appended = sv->pending.empty() ? sv->cursor : off;
        int nchunks = 0;
        for (const auto& k : sv->pending)
            sv->chunk_stage[nchunks++] = WaveChunk{k.slot, k.first_sample, k.nspp, 0, k.path_offset};
        if (nchunks > 0)
            WF_CK(c, cudaMemcpyAsync(sv->d_chunks, sv->chunk_stage, sizeof(WaveChunk) * nchunks, cudaMemcpyHostToDevice, s));
        sv->state_stage[0] = sv->appended;
        sv->state_stage[1] = nchunks;
        WF_CK(c, cudaMemcpyAsync(reinterpret_cast<char*>(sv->d_state) + offsetof(StreamState, total), sv->state_stage,
                                 sizeof(int64_t), cudaMemcpyHostToDevice, s));
        int32_t* nc32 = reinterpret_cast<int32_t*>(sv->state_stage + 1);
        *nc32 = nchunks;
        WF_CK(c, cudaMemcpyAsync(reinterpret_cast<char*>(sv->d_state) + offsetof(StreamState, nchunks), nc32,
                                 sizeof(int32_t), cudaMemcpyHostToDevice, s));
    }
    // 4. run the step's iterations, unless nothing is queued or left to generate
    if (sv->live > 0 || sv->appended > sv->cursor) {
        // the scenes whose rays the queue can hold during the step
        std::vector<int32_t> scene_ids;
        for (const auto& k : sv->inflight) scene_ids.push_back(sv->jobs[k.job].spec.scene_id);
        for (const auto& k : sv->pending) scene_ids.push_back(sv->jobs[k.job].spec.scene_id);
        {
            const WaveSceneScope scene_scope(c, scene_ids);
            if ((rc = ensure_stream_graph(sv))) return rc;
        }
        WF_CK(c, cudaEventRecord(sv->ev[0], s));
        WF_CK(c, cudaGraphLaunch(sv->exec, s));
        WF_CK(c, cudaEventRecord(sv->ev[1], s));
        StepReadback* rb = sv->rb;
        WF_CK(c, cudaMemcpyAsync(rb->tally, sv->tally, sizeof(rb->tally), cudaMemcpyDeviceToHost, s));
        WF_CK(c, cudaMemcpyAsync(&rb->live, sv->counters, sizeof(ull), cudaMemcpyDeviceToHost, s));
        WF_CK(c, cudaMemcpyAsync(&rb->st, sv->d_state, sizeof(StreamState), cudaMemcpyDeviceToHost, s));
        WF_CK(c, cudaMemcpyAsync(rb->log, sv->d_log, sizeof(rb->log), cudaMemcpyDeviceToHost, s));
        if ((rc = flush_complete(sv, si))) return rc;  // the last step's finished jobs, while this one runs
        WF_CK(c, cudaStreamSynchronize(s));
        int flag = 0;
        WF_CK(c, cudaMemcpy(&flag, sv->err, sizeof(int), cudaMemcpyDeviceToHost));
        if (flag) return set_err(c, WF_ERR_DEVICE_CHECK, "device check failed in the streaming wave (flags " +
                                                             std::to_string(flag) + ")");
        float ms = 0.0f;
        WF_CK(c, cudaEventElapsedTime(&ms, sv->ev[0], sv->ev[1]));
        si.step_ms = ms;
        si.rays_traced = (rb->tally[0] - sv->tally_prev[0]) + (rb->tally[2] - sv->tally_prev[2]);
        si.paths_in_wave = rb->st.cursor - sv->cursor;
        std::memcpy(sv->tally_prev, rb->tally, sizeof(sv->tally_prev));
        // frames whose last path was generated in this step: finished
        // max_depth iterations after that one
        const int64_t base_iter = sv->iters;
        sv->iters += kGroupIters;
        while (!sv->pending.empty()) {
            ServerChunk& k = sv->pending.front();
            const int64_t end = k.path_offset + k.len;
            int m = 0;
            while (m < kGroupIters && rb->log[m] < end) ++m;
            if (m == kGroupIters) break;
            k.done_iter = base_iter + m + k.depth + 1;
            sv->inflight.push_back(k);
            sv->pending.pop_front();
        }
        sv->cursor = rb->st.cursor;
        sv->live = (int64_t)rb->live;
    }
    if ((rc = flush_complete(sv, si))) return rc;  // no iterations this step
    // 5. retire finished frames, in the order they were generated
    if (sv->live == 0 && sv->pending.empty())  // every generated path has ended
        for (auto& k : sv->inflight) k.done_iter = std::min<int64_t>(k.done_iter, sv->iters);
    {
        std::vector<int64_t> jobs_seen;
        for (const auto& k : sv->inflight) jobs_seen.push_back(k.job);
        std::sort(jobs_seen.begin(), jobs_seen.end());
        si.jobs_in_wave = (int32_t)(std::unique(jobs_seen.begin(), jobs_seen.end()) - jobs_seen.begin());
    }
    const double now = seconds_since(sv->t0);
    std::vector<ServerChunk> keep;
    keep.reserve(sv->inflight.size());
    for (const auto& k : sv->inflight) {
        if (k.done_iter <= sv->iters) {
            if ((rc = retire_chunk(sv, k, now, si))) return rc;
        } else {
            keep.push_back(k);
        }
    }
    sv->inflight.swap(keep);
    if ((rc = flush_begin(sv))) return rc;
    si.queued = (int32_t)sv->queue.size();
    si.running = (int32_t)sv->running;
    si.budget_used_bytes = sv->wave_bytes + 4 * (sv->alloc.used + sv->frames.used);
    if (info) *info = si;
    return WF_OK;
}

int wf_server_status(wf_server* sv, int64_t id, wf_job_status* out)
{
    if (!sv || !out) return WF_ERR_INVALID_ARGUMENT;
    const ServedJob* jp = sv->jobs.find(id);
    if (!jp) return set_err(sv->c, WF_ERR_INVALID_ARGUMENT, "no such job");
    const ServedJob& j = *jp;
    out->state = j.state;
    out->samples_done = j.samples_done;
    out->frames = j.frames;
    out->reserved = 0;
    out->t_submit = j.t_submit;
    out->t_admit = j.t_admit;
    out->t_first_frame = j.t_first;
    out->t_done = j.t_done;
    return WF_OK;
}

int wf_server_image(wf_server* sv, int64_t id, float* image, int64_t nf)
{
    if (!sv || !image) return WF_ERR_INVALID_ARGUMENT;
    ServedJob* jp = sv->jobs.find(id);
    if (!jp) return set_err(sv->c, WF_ERR_INVALID_ARGUMENT, "no such job");
    ServedJob& j = *jp;
    if (nf < j.accum_floats) return set_err(sv->c, WF_ERR_CAPACITY, "image buffer too small");
    if (!sv->flushing.empty()) {  // this job's image, or a copy out of tmp that must end before tmp is reused
        wf_server_step_info si{};
        const int rc = flush_complete(sv, si);
        if (rc) return rc;
    }
    if (j.state == WF_JOB_DONE) {
        std::memcpy(image, j.final_image.data(), sizeof(float) * j.accum_floats);
        return WF_OK;
    }
    if (j.state != WF_JOB_RUNNING || j.samples_done == 0) return set_err(sv->c, WF_ERR_STATE, "no frame yet");
    wf_ctx* c = sv->c;
    if (j.accum_floats > sv->tmp_floats) {
        cudaFree(sv->tmp);
        sv->tmp = nullptr;
        sv->tmp_floats = 0;
        WF_CK(c, cudaMalloc(&sv->tmp, sizeof(float) * j.accum_floats));
        sv->tmp_floats = j.accum_floats;
    }
    launch_finalize(sv->arena + j.accum_off, j.accum_floats, (float)j.samples_done, sv->tmp, c->stream);
    WF_CK(c, cudaMemcpyAsync(image, sv->tmp, sizeof(float) * j.accum_floats, cudaMemcpyDeviceToHost, c->stream));
    WF_CK(c, cudaStreamSynchronize(c->stream));
    return WF_OK;
}

int wf_server_cancel(wf_server* sv, int64_t id)
{
    if (!sv) return WF_ERR_INVALID_ARGUMENT;
    ServedJob* jp = sv->jobs.find(id);
    if (!jp) return set_err(sv->c, WF_ERR_INVALID_ARGUMENT, "no such job");
    ServedJob& j = *jp;
    if (j.flushing) {  // every frame has finished: the job completes
        wf_server_step_info si{};
        return flush_complete(sv, si);
    }
    if (j.state == WF_JOB_RUNNING) {
        // frames not started yet are dropped; frames already generating run
        // to their end and are discarded (their paths are in the queue)
        const int64_t cursor = sv->cursor;
        std::deque<ServerChunk> keep;
        for (auto& k : sv->pending) {
            if (k.job == id && k.path_offset >= cursor) {
                sv->frames.release(k.frame_off, k.floats);
                sv->free_slots.push_back(k.slot);
                j.chunks_out--;
            } else {
                keep.push_back(k);
            }
        }
        sv->pending.swap(keep);
        // the list's end moves back; the next step lays the frames out again
        int64_t end = cursor;
        for (const auto& k : sv->pending) end = std::max(end, k.path_offset + k.len);
        sv->appended = end;
        sv->running--;
        if (j.chunks_out == 0) {
            sv->alloc.release(j.accum_off, j.accum_floats);
            j.accum_off = -1;
        }
    }
    if (j.state == WF_JOB_RUNNING || j.state == WF_JOB_QUEUED) {
        j.state = WF_JOB_CANCELLED;
        j.t_done = seconds_since(sv->t0);
    }
    return WF_OK;
}

}  // extern "C"
