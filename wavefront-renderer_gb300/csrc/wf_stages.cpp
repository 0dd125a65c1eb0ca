// wf_stages.cpp — the per-bounce stages of the reference's loop as separate
// entry points on device-resident queues (reference src/render/
// WavefrontRenderer.cpp:141-268; include/scheduling/RayQueue.h:165-215,
// ShadingQueue.h:90-141, 233-275).
//
// The stages launch the render loop's own kernels (camera, traversal, hit
// compaction, policy sort, shading, shadow rays) on queues the caller holds,
// so a caller's loop renders what wf_render renders.  Each queue keeps its
// entry count in device memory; a stage reads its input counts there and
// writes its outputs' counts there, so consecutive stages need no host round
// trip.  The calls that return a count or a permutation to the host wait.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/wf_api.h"
#include "wf_ctx.h"
#include "wf_kernels.h"
#include "wf_sort.h"

using namespace wf;

// A RayQueue: the 14 device columns twice (materialize gathers into the
// other copy), the permutation of the last schedule, and counters: [0] the
// entry count, [1] the traversal kernels' ray fetch counter.
struct wf_ray_queue {
    wf_ctx* ctx = nullptr;
    RayQueueDev q[2]{};
    int cur = 0;
    ull* counts = nullptr;
    uint32_t* perm = nullptr;
    bool has_perm = false;
    int64_t capacity = 0;
    std::vector<void*> allocs;
};

// A ShadingQueue: per hit the ray's index in `rays` and (leaf triangle, t,
// barycentrics).  After wf_intersect the records sit at the rays' indices
// (at_ray); after materialize at the list positions.
struct wf_shading_queue {
    wf_ctx* ctx = nullptr;
    HitQueueDev h[2]{};
    int cur = 0;
    bool at_ray = false;
    RayQueueDev rays{};            // the ray columns the entries index
    const wf_ray_queue* source = nullptr;
    ull* counts = nullptr;         // [0] hits, [1] scratch
    uint32_t* perm = nullptr;
    bool has_perm = false;
    int64_t capacity = 0;
    std::vector<void*> allocs;
};

// Shadow rays: [0] count, [1] the any-hit kernel's fetch counter.
struct wf_shadow_queue {
    wf_ctx* ctx = nullptr;
    ShadowQueueDev sh{};
    ull* counts = nullptr;
    int64_t capacity = 0;
    std::vector<void*> allocs;
};

namespace {

int alloc_rays(wf_ctx* c, std::vector<void*>& A, RayQueueDev& r, int64_t cap)
{
    const size_t n = (size_t)cap;
    WF_CK(c, wf_dalloc(A, &r.ox, n)); WF_CK(c, wf_dalloc(A, &r.oy, n)); WF_CK(c, wf_dalloc(A, &r.oz, n));
    WF_CK(c, wf_dalloc(A, &r.dx, n)); WF_CK(c, wf_dalloc(A, &r.dy, n)); WF_CK(c, wf_dalloc(A, &r.dz, n));
    WF_CK(c, wf_dalloc(A, &r.tr, n)); WF_CK(c, wf_dalloc(A, &r.tg, n)); WF_CK(c, wf_dalloc(A, &r.tb, n));
    WF_CK(c, wf_dalloc(A, &r.pdf, n));
    WF_CK(c, wf_dalloc(A, &r.pixel, n)); WF_CK(c, wf_dalloc(A, &r.depth, n)); WF_CK(c, wf_dalloc(A, &r.sample, n));
    WF_CK(c, wf_dalloc(A, &r.job, n));
    r.capacity = cap;
    return WF_OK;
}

int alloc_hits(wf_ctx* c, std::vector<void*>& A, HitQueueDev& h, int64_t cap)
{
    const size_t n = (size_t)cap;
    WF_CK(c, wf_dalloc(A, &h.ray, n)); WF_CK(c, wf_dalloc(A, &h.tri, n)); WF_CK(c, wf_dalloc(A, &h.t, n));
    WF_CK(c, wf_dalloc(A, &h.bu, n)); WF_CK(c, wf_dalloc(A, &h.bv, n));
    h.capacity = cap;
    return WF_OK;
}

// The stage render's tables: a single job on scene 0.
int stage_tables(wf_ctx* c, WaveTables& T)
{
    if (!c->stage_live) return set_err(c, WF_ERR_STATE, "wf_stage_begin has not been called");
    if (c->scenes.empty() || !c->scenes[0].live) return set_err(c, WF_ERR_STATE, "no scene uploaded");
    if (c->arena_floats < 3 * c->stage_pixels)
        return set_err(c, WF_ERR_STATE, "the stage render's pixel sums were released by another render");
    T = WaveTables{c->d_scene_table, c->d_jobs, c->scenes[0].S, c->stage_job, false, kTreeBinary};
    T.tree = tree_format(T.scene0);
    return WF_OK;
}

int read_count(wf_ctx* c, const ull* d, int64_t* n)
{
    ull v = 0;
    WF_CK(c, cudaMemcpyAsync(&v, d, sizeof(ull), cudaMemcpyDeviceToHost, c->stream));
    WF_CK(c, cudaStreamSynchronize(c->stream));
    *n = (int64_t)v;
    return WF_OK;
}

// Scratch of the policy and ray sorts (keys, values, digit counts and the
// scheduling columns) for n entries: the context's render buffers.
int ensure_sort_scratch(wf_ctx* c, int64_t n) { return ensure_render_buffers(c, std::max<int64_t>(n, 1)); }

template <class Q>
int free_queue(Q* q)
{
    if (!q) return WF_OK;
    if (q->ctx) {
        cudaSetDevice(q->ctx->device);
        cudaStreamSynchronize(q->ctx->stream);
    }
    free_all(q->allocs);
    delete q;
    return WF_OK;
}

}  // namespace

extern "C" {

int wf_ray_queue_alloc(wf_ctx* c, int64_t capacity, wf_ray_queue** out)
{
    if (!c || !out || capacity < 1 || capacity > ((int64_t)1 << 31) - 1)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "ray queue capacity must be in [1, 2^31)");
    cudaSetDevice(c->device);
    *out = nullptr;
    auto* q = new wf_ray_queue();
    q->ctx = c;
    q->capacity = capacity;
    int rc = alloc_rays(c, q->allocs, q->q[0], capacity);
    if (!rc) rc = alloc_rays(c, q->allocs, q->q[1], capacity);
    if (!rc && wf_dalloc(q->allocs, &q->counts, 4) != cudaSuccess) rc = set_err(c, WF_ERR_OUT_OF_MEMORY, "counts");
    if (!rc && wf_dalloc(q->allocs, &q->perm, (size_t)capacity) != cudaSuccess)
        rc = set_err(c, WF_ERR_OUT_OF_MEMORY, "permutation");
    if (!rc && cudaMemsetAsync(q->counts, 0, sizeof(ull) * 4, c->stream) != cudaSuccess)
        rc = set_err(c, WF_ERR_CUDA, "memset");
    if (rc) {
        free_all(q->allocs);
        delete q;
        return rc == WF_ERR_CUDA ? WF_ERR_OUT_OF_MEMORY : rc;
    }
    *out = q;
    return WF_OK;
}

int wf_ray_queue_free(wf_ray_queue* q) { return free_queue(q); }

int wf_shading_queue_alloc(wf_ctx* c, int64_t capacity, wf_shading_queue** out)
{
    if (!c || !out || capacity < 1 || capacity > ((int64_t)1 << 31) - 1)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "shading queue capacity must be in [1, 2^31)");
    cudaSetDevice(c->device);
    *out = nullptr;
    auto* q = new wf_shading_queue();
    q->ctx = c;
    q->capacity = capacity;
    int rc = alloc_hits(c, q->allocs, q->h[0], capacity);
    if (!rc) rc = alloc_hits(c, q->allocs, q->h[1], capacity);
    if (!rc && wf_dalloc(q->allocs, &q->counts, 4) != cudaSuccess) rc = set_err(c, WF_ERR_OUT_OF_MEMORY, "counts");
    if (!rc && wf_dalloc(q->allocs, &q->perm, (size_t)capacity) != cudaSuccess)
        rc = set_err(c, WF_ERR_OUT_OF_MEMORY, "permutation");
    if (!rc && cudaMemsetAsync(q->counts, 0, sizeof(ull) * 4, c->stream) != cudaSuccess)
        rc = set_err(c, WF_ERR_CUDA, "memset");
    if (rc) {
        free_all(q->allocs);
        delete q;
        return rc == WF_ERR_CUDA ? WF_ERR_OUT_OF_MEMORY : rc;
    }
    *out = q;
    return WF_OK;
}

int wf_shading_queue_free(wf_shading_queue* q) { return free_queue(q); }

int wf_shadow_queue_alloc(wf_ctx* c, int64_t capacity, wf_shadow_queue** out)
{
    if (!c || !out || capacity < 1 || capacity > ((int64_t)1 << 31) - 1)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "shadow queue capacity must be in [1, 2^31)");
    cudaSetDevice(c->device);
    *out = nullptr;
    auto* q = new wf_shadow_queue();
    q->ctx = c;
    q->capacity = capacity;
    auto& A = q->allocs;
    ShadowQueueDev& s = q->sh;
    const size_t n = (size_t)capacity;
    bool ok = wf_dalloc(A, &s.ox, n) == cudaSuccess && wf_dalloc(A, &s.oy, n) == cudaSuccess &&
              wf_dalloc(A, &s.oz, n) == cudaSuccess && wf_dalloc(A, &s.dx, n) == cudaSuccess &&
              wf_dalloc(A, &s.dy, n) == cudaSuccess && wf_dalloc(A, &s.dz, n) == cudaSuccess &&
              wf_dalloc(A, &s.dist, n) == cudaSuccess && wf_dalloc(A, &s.cr, n) == cudaSuccess &&
              wf_dalloc(A, &s.cg, n) == cudaSuccess && wf_dalloc(A, &s.cb, n) == cudaSuccess &&
              wf_dalloc(A, &s.pixel, n) == cudaSuccess && wf_dalloc(A, &s.job, n) == cudaSuccess &&
              wf_dalloc(A, &q->counts, 4) == cudaSuccess &&
              cudaMemsetAsync(q->counts, 0, sizeof(ull) * 4, c->stream) == cudaSuccess;
    if (!ok) {
        free_all(A);
        delete q;
        return set_err(c, WF_ERR_OUT_OF_MEMORY, "shadow queue");
    }
    s.capacity = capacity;
    *out = q;
    return WF_OK;
}

int wf_shadow_queue_free(wf_shadow_queue* q) { return free_queue(q); }

int wf_ray_queue_size(wf_ray_queue* q, int64_t* n)
{
    if (!q || !n) return WF_ERR_INVALID_ARGUMENT;
    return read_count(q->ctx, q->counts, n);
}

int wf_shading_queue_size(wf_shading_queue* q, int64_t* n)
{
    if (!q || !n) return WF_ERR_INVALID_ARGUMENT;
    return read_count(q->ctx, q->counts, n);
}

int wf_shadow_queue_size(wf_shadow_queue* q, int64_t* n)
{
    if (!q || !n) return WF_ERR_INVALID_ARGUMENT;
    return read_count(q->ctx, q->counts, n);
}

int wf_ray_queue_upload(wf_ray_queue* q, const wf_ray_columns* h, int64_t n)
{
    if (!q || !h || n < 0) return WF_ERR_INVALID_ARGUMENT;
    wf_ctx* c = q->ctx;
    if (n > q->capacity) return set_err(c, WF_ERR_CAPACITY, "more rays than the queue holds");
    if (n > 0 && (!h->origins_x || !h->origins_y || !h->origins_z || !h->dirs_x || !h->dirs_y || !h->dirs_z ||
                  !h->pixel_indices))
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "origins, directions and pixel indices are required");
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    RayQueueDev& r = q->q[q->cur];
    const size_t fb = sizeof(float) * (size_t)n, ib = sizeof(int32_t) * (size_t)n;
    // RayQueue::addPrimary's defaults for the columns not given (RayQueue.h:113-116)
    std::vector<float> one(n > 0 && (!h->throughputs_r || !h->throughputs_g || !h->throughputs_b) ? n : 0, 1.0f);
    std::vector<float> minus_one(n > 0 && !h->pdfs ? n : 0, -1.0f);
    const float* cols_f[10] = {h->origins_x, h->origins_y, h->origins_z, h->dirs_x, h->dirs_y, h->dirs_z,
                               h->throughputs_r ? h->throughputs_r : one.data(),
                               h->throughputs_g ? h->throughputs_g : one.data(),
                               h->throughputs_b ? h->throughputs_b : one.data(),
                               h->pdfs ? h->pdfs : minus_one.data()};
    float* dst_f[10] = {r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, r.tr, r.tg, r.tb, r.pdf};
    if (n > 0) {
        for (int k = 0; k < 10; ++k) WF_CK(c, cudaMemcpyAsync(dst_f[k], cols_f[k], fb, cudaMemcpyHostToDevice, s));
        WF_CK(c, cudaMemcpyAsync(r.pixel, h->pixel_indices, ib, cudaMemcpyHostToDevice, s));
        if (h->depths)
            WF_CK(c, cudaMemcpyAsync(r.depth, h->depths, ib, cudaMemcpyHostToDevice, s));
        else
            WF_CK(c, cudaMemsetAsync(r.depth, 0, ib, s));
        if (h->sample_indices)
            WF_CK(c, cudaMemcpyAsync(r.sample, h->sample_indices, ib, cudaMemcpyHostToDevice, s));
        else
            WF_CK(c, cudaMemsetAsync(r.sample, 0, ib, s));
        WF_CK(c, cudaMemsetAsync(r.job, 0, ib, s));
    }
    const ull cnt = (ull)n;
    WF_CK(c, cudaMemcpyAsync(q->counts, &cnt, sizeof(ull), cudaMemcpyHostToDevice, s));
    WF_CK(c, cudaStreamSynchronize(s));  // the host columns may be freed on return
    q->has_perm = false;
    return WF_OK;
}

int wf_ray_queue_download(wf_ray_queue* q, wf_ray_columns* h, int64_t capacity, int64_t* n)
{
    if (!q || !h || !n) return WF_ERR_INVALID_ARGUMENT;
    wf_ctx* c = q->ctx;
    cudaSetDevice(c->device);
    int64_t cnt = 0;
    int rc = read_count(c, q->counts, &cnt);
    if (rc) return rc;
    *n = cnt;
    if (cnt > capacity) return set_err(c, WF_ERR_CAPACITY, "host columns smaller than the queue");
    const RayQueueDev& r = q->q[q->cur];
    const size_t fb = sizeof(float) * (size_t)cnt, ib = sizeof(int32_t) * (size_t)cnt;
    float* dst_f[10] = {h->origins_x, h->origins_y, h->origins_z, h->dirs_x, h->dirs_y, h->dirs_z,
                        h->throughputs_r, h->throughputs_g, h->throughputs_b, h->pdfs};
    const float* src_f[10] = {r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, r.tr, r.tg, r.tb, r.pdf};
    int32_t* dst_i[3] = {h->pixel_indices, h->depths, h->sample_indices};
    const int32_t* src_i[3] = {r.pixel, r.depth, r.sample};
    if (cnt > 0) {
        for (int k = 0; k < 10; ++k)
            if (dst_f[k]) WF_CK(c, cudaMemcpyAsync(dst_f[k], src_f[k], fb, cudaMemcpyDeviceToHost, c->stream));
        for (int k = 0; k < 3; ++k)
            if (dst_i[k]) WF_CK(c, cudaMemcpyAsync(dst_i[k], src_i[k], ib, cudaMemcpyDeviceToHost, c->stream));
    }
    WF_CK(c, cudaStreamSynchronize(c->stream));
    return check_device_flag(c);
}

int wf_shading_queue_download(wf_shading_queue* q, wf_hit_columns* hits, wf_ray_columns* rays, int64_t capacity,
                              int64_t* n)
{
    if (!q || !n) return WF_ERR_INVALID_ARGUMENT;
    wf_ctx* c = q->ctx;
    cudaSetDevice(c->device);
    int64_t cnt = 0;
    int rc = read_count(c, q->counts, &cnt);
    if (rc) return rc;
    *n = cnt;
    if (cnt > capacity) return set_err(c, WF_ERR_CAPACITY, "host columns smaller than the queue");
    if (cnt == 0) return WF_OK;
    if (c->scenes.empty() || !c->scenes[0].live) return set_err(c, WF_ERR_STATE, "no scene uploaded");
    // rebuild the 24 columns into temporary device columns, then copy
    std::vector<void*> tmp;
    const size_t m = (size_t)cnt;
    HitColumnsDev hd{};
    RayQueueDev rd{};
    bool ok = wf_dalloc(tmp, &hd.geom, m) == cudaSuccess && wf_dalloc(tmp, &hd.prim, m) == cudaSuccess &&
              wf_dalloc(tmp, &hd.t, m) == cudaSuccess && wf_dalloc(tmp, &hd.bu, m) == cudaSuccess &&
              wf_dalloc(tmp, &hd.bv, m) == cudaSuccess && wf_dalloc(tmp, &hd.px, m) == cudaSuccess &&
              wf_dalloc(tmp, &hd.py, m) == cudaSuccess && wf_dalloc(tmp, &hd.pz, m) == cudaSuccess &&
              wf_dalloc(tmp, &hd.nx, m) == cudaSuccess && wf_dalloc(tmp, &hd.ny, m) == cudaSuccess &&
              wf_dalloc(tmp, &hd.nz, m) == cudaSuccess && wf_dalloc(tmp, &hd.front, m) == cudaSuccess &&
              wf_dalloc(tmp, &hd.u, m) == cudaSuccess && wf_dalloc(tmp, &hd.v, m) == cudaSuccess &&
              wf_dalloc(tmp, &hd.mat, m) == cudaSuccess && wf_dalloc(tmp, &hd.tex, m) == cudaSuccess;
    if (ok) ok = alloc_rays(c, tmp, rd, cnt) == WF_OK;
    if (!ok) {
        free_all(tmp);
        return set_err(c, WF_ERR_OUT_OF_MEMORY, "download scratch");
    }
    launch_shading_columns(c->scenes[0].S, q->rays, q->h[q->cur], q->at_ray, q->counts, hd, rd, wide_cfg(c),
                           c->stream);
    auto cp = [&](void* dst, const void* src, size_t bytes) {
        return dst ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream) : cudaSuccess;
    };
    const size_t fb = sizeof(float) * m, ib = sizeof(int32_t) * m;
    cudaError_t e = cudaSuccess;
    if (hits) {
        const void* src[16] = {hd.geom, hd.prim, hd.t, hd.bu, hd.bv, hd.px, hd.py, hd.pz,
                               hd.nx,   hd.ny,   hd.nz, hd.front, hd.u, hd.v, hd.mat, hd.tex};
        void* dst[16] = {hits->geom_id, hits->prim_id, hits->distance, hits->bary_u, hits->bary_v, hits->point_x,
                         hits->point_y, hits->point_z, hits->normal_x, hits->normal_y, hits->normal_z,
                         hits->front_face, hits->u, hits->v, hits->material_id, hits->texture_id};
        for (int k = 0; k < 16 && e == cudaSuccess; ++k) e = cp(dst[k], src[k], k == 11 ? m : (k < 2 || k > 13 ? ib : fb));
    }
    if (rays && e == cudaSuccess) {
        const void* src[13] = {rd.ox, rd.oy, rd.oz, rd.dx, rd.dy, rd.dz, rd.tr, rd.tg, rd.tb, rd.pdf,
                               rd.pixel, rd.depth, rd.sample};
        void* dst[13] = {rays->origins_x, rays->origins_y, rays->origins_z, rays->dirs_x, rays->dirs_y, rays->dirs_z,
                         rays->throughputs_r, rays->throughputs_g, rays->throughputs_b, rays->pdfs,
                         rays->pixel_indices, rays->depths, rays->sample_indices};
        for (int k = 0; k < 13 && e == cudaSuccess; ++k) e = cp(dst[k], src[k], k < 10 ? fb : ib);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    free_all(tmp);
    if (e != cudaSuccess) return set_err(c, WF_ERR_CUDA, cudaGetErrorString(e));
    return check_device_flag(c);
}

int wf_stage_begin(wf_ctx* c, const wf_render_params* P)
{
    if (!c || !P) return set_err(c, WF_ERR_INVALID_ARGUMENT, "null argument");
    if (P->policy < 0 || P->policy > 3) return set_err(c, WF_ERR_INVALID_ARGUMENT, "unknown policy");
    cudaSetDevice(c->device);
    c->stage_live = false;
    if (c->scenes.empty() || !c->scenes[0].live) return set_err(c, WF_ERR_STATE, "no scene uploaded");
    wf_job j{};
    j.scene_id = 0;
    j.width = P->width;
    j.height = P->height;
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
    int rc = validate_job(c, j);
    if (rc) return rc;
    const int64_t np = (int64_t)P->width * P->height;
    if ((rc = ensure_arena(c, 3 * np))) return rc;
    if ((rc = sync_scene_table(c))) return rc;
    free_all(c->rel_cost_allocs);
    if ((rc = make_device_job(c, j, 0, c->stage_job))) return rc;
    if ((rc = upload_jobs(c, {c->stage_job}))) return rc;
    WF_CK(c, cudaMemsetAsync(c->arena, 0, sizeof(float) * 3 * (size_t)np, c->stream));
    WF_CK(c, cudaMemsetAsync(c->err_flag, 0, sizeof(int), c->stream));
    c->stage_params = *P;
    c->stage_pixels = np;
    c->stage_live = true;
    return WF_OK;
}

int wf_generate_primary(wf_ctx* c, int32_t first_sample, int32_t nspp, wf_ray_queue* out)
{
    if (!c || !out || out->ctx != c || nspp < 1 || first_sample < 0)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "bad argument");
    cudaSetDevice(c->device);
    WaveTables T;
    int rc = stage_tables(c, T);
    if (rc) return rc;
    const int64_t total = c->stage_pixels * nspp;
    if (total > out->capacity) return set_err(c, WF_ERR_CAPACITY, "queue smaller than width * height * nspp");
    if ((rc = upload_jobs(c, {c->stage_job}))) return rc;  // the camera kernel reads the job table
    std::vector<WaveChunk> ch(1);
    ch[0] = WaveChunk{0, c->stage_params.first_sample + first_sample, nspp, 0, 0};
    if ((rc = upload_wave(c, ch, total))) return rc;
    launch_camera_chunks(c->d_chunks, c->d_wave_header, c->d_jobs, out->q[out->cur], wide_cfg(c), c->stream);
    WF_CK(c, cudaMemcpyAsync(out->counts, c->d_wave_header, sizeof(ull), cudaMemcpyDeviceToDevice, c->stream));
    out->has_perm = false;
    return WF_OK;
}

int wf_ray_queue_schedule(wf_ray_queue* q, const float bounds_min[3], const float bounds_max[3],
                          int32_t* sorted_indices_host)
{
    if (!q || !bounds_min || !bounds_max) return WF_ERR_INVALID_ARGUMENT;
    wf_ctx* c = q->ctx;
    cudaSetDevice(c->device);
    int64_t n = 0;
    int rc = read_count(c, q->counts, &n);
    if (rc) return rc;
    q->has_perm = true;
    if (n == 0) return WF_OK;
    if ((rc = ensure_sort_scratch(c, n))) return rc;
    cudaStream_t s = c->stream;
    const RayQueueDev& r = q->q[q->cur];
    const LaunchCfg WC = wide_cfg(c);
    // RayQueue::sortKey (RayQueue.h:135-162) with the given bounds, then the
    // stable radix sort of (key, index) over all 33 key bits
    launch_ray_keys_raw(n, r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, bounds_min, bounds_max, c->keys, c->vals, WC, s);
    uint64_t* rk = nullptr;
    uint32_t* rv = nullptr;
    RadixSortArgs a{c->keys, c->vals, c->keys_tmp, c->vals_tmp, c->hist, q->counts, c->nb, 0, 33, &rk, &rv};
    radix_sort_pairs(a, s);
    WF_CK(c, cudaMemcpyAsync(q->perm, rv, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    if (sorted_indices_host) {
        WF_CK(c, cudaMemcpyAsync(sorted_indices_host, q->perm, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, s));
        WF_CK(c, cudaStreamSynchronize(s));
    }
    return WF_OK;
}

int wf_ray_queue_materialize(wf_ray_queue* q)
{
    if (!q) return WF_ERR_INVALID_ARGUMENT;
    wf_ctx* c = q->ctx;
    if (!q->has_perm) return WF_OK;  // no schedule since the last fill: the identity
    cudaSetDevice(c->device);
    launch_gather_rays(q->q[q->cur], q->perm, q->counts, q->q[1 - q->cur], wide_cfg(c), c->stream);
    q->cur = 1 - q->cur;
    q->has_perm = false;
    return WF_OK;
}

int wf_intersect(wf_ctx* c, wf_ray_queue* rays, wf_shading_queue* hits, wf_ray_queue* misses)
{
    if (!c || !rays || !hits || rays->ctx != c || hits->ctx != c || (misses && (misses->ctx != c || misses == rays)))
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "bad argument");
    // records sit at the rays' indices: the hit queue spans the ray queue
    if (hits->capacity < rays->capacity) return set_err(c, WF_ERR_CAPACITY, "hit queue smaller than the ray queue");
    if (misses && misses->capacity < rays->capacity)
        return set_err(c, WF_ERR_CAPACITY, "miss queue smaller than the ray queue");
    cudaSetDevice(c->device);
    WaveTables T;
    int rc = stage_tables(c, T);
    if (rc) return rc;
    cudaStream_t s = c->stream;
    LaunchCfg PC = persist_cfg(c);
    const LaunchCfg WC = wide_cfg(c);
    const RayQueueDev& r = rays->q[rays->cur];
    HitQueueDev& h = hits->h[hits->cur];
    WF_CK(c, cudaMemsetAsync(hits->counts, 0, sizeof(ull), s));
    WF_CK(c, cudaMemsetAsync(rays->counts + 1, 0, sizeof(ull), s));
    float* accum = c->arena;
    if (misses) {
        // records at the rays' indices, misses left alone (ray order 2); then
        // the hit list and the miss list, the missed rays copied out
        PC.ray_order = 2;
        WF_CK(c, cudaMemsetAsync(misses->counts, 0, sizeof(ull), s));
        launch_trace_render(T, r, rays->counts, h, hits->counts, accum, rays->counts + 1, c->err_flag, PC, s);
        launch_split_hits(T, r, rays->counts, h, hits->counts, misses->perm, misses->counts, WC, s);
        launch_gather_rays(r, misses->perm, misses->counts, misses->q[misses->cur], WC, s);
        misses->has_perm = false;
    } else {
        // the render loop's own ray-order bounce: misses shaded on the way
        PC.ray_order = 1;
        launch_trace_render(T, r, rays->counts, h, hits->counts, accum, rays->counts + 1, c->err_flag, PC, s);
        launch_compact_hits(T, r, rays->counts, h, hits->counts, accum, WC, s);
    }
    hits->at_ray = true;
    hits->rays = r;
    hits->source = rays;
    hits->has_perm = false;
    return WF_OK;
}

int wf_shading_queue_schedule(wf_shading_queue* q, int32_t policy, const double* rel_cost_material,
                              const double* rel_cost_texture, int32_t* sorted_indices_host)
{
    if (!q || policy < 0 || policy > 3) return WF_ERR_INVALID_ARGUMENT;
    wf_ctx* c = q->ctx;
    cudaSetDevice(c->device);
    WaveTables T;
    int rc = stage_tables(c, T);
    if (rc) return rc;
    int64_t n = 0;
    if ((rc = read_count(c, q->counts, &n))) return rc;
    q->has_perm = true;
    if (n == 0) return WF_OK;
    if ((rc = ensure_sort_scratch(c, n))) return rc;
    cudaStream_t s = c->stream;
    const LaunchCfg WC = wide_cfg(c);
    if (q->at_ray) {  // the policy keys read the compact list layout
        launch_materialize_hits(q->h[q->cur], true, nullptr, q->counts, q->h[1 - q->cur], WC, s);
        q->cur = 1 - q->cur;
        q->at_ray = false;
    }
    ShadeColumnsMut cm{c->col_mat, c->col_tex, c->col_tr, c->col_tg, c->col_tb, c->col_px, c->col_py, c->col_pz};
    launch_hit_columns(c->d_scene_table, c->d_jobs, nullptr, policy == WF_POLICY_COST_BENEFIT_AWARE, q->rays,
                       q->h[q->cur], q->counts, cm, WC, s);
    ShadeColumnsDev cd{c->col_mat, c->col_tex, c->col_tr, c->col_tg, c->col_tb, c->col_px, c->col_py, c->col_pz};
    const ResidentScene& R = c->scenes[0];
    uint32_t* perm = nullptr;
    if ((rc = schedule_columns(c, policy, q->counts, n, cd, R.S.materials, R.S.num_materials, R.mats,
                               R.S.num_textures, R.d_tex_bytes, R.tex_bytes, rel_cost_material, rel_cost_texture,
                               &perm)))
        return rc;
    WF_CK(c, cudaMemcpyAsync(q->perm, perm, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    if (sorted_indices_host) {
        WF_CK(c, cudaMemcpyAsync(sorted_indices_host, q->perm, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, s));
        WF_CK(c, cudaStreamSynchronize(s));
    }
    return WF_OK;
}

int wf_shading_queue_materialize(wf_shading_queue* q)
{
    if (!q) return WF_ERR_INVALID_ARGUMENT;
    wf_ctx* c = q->ctx;
    if (!q->has_perm) return WF_OK;
    cudaSetDevice(c->device);
    launch_materialize_hits(q->h[q->cur], q->at_ray, q->perm, q->counts, q->h[1 - q->cur], wide_cfg(c), c->stream);
    q->cur = 1 - q->cur;
    q->at_ray = false;
    q->has_perm = false;
    return WF_OK;
}

int wf_shade(wf_ctx* c, wf_shading_queue* hits, wf_ray_queue* next, wf_shadow_queue* shadows)
{
    if (!c || !hits || !next || !shadows || hits->ctx != c || next->ctx != c || shadows->ctx != c)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "bad argument");
    if (!hits->source) return set_err(c, WF_ERR_STATE, "the shading queue holds no hits (wf_intersect)");
    if (next == hits->source) return set_err(c, WF_ERR_INVALID_ARGUMENT, "next must not be the hits' ray queue");
    // a hit emits at most one next ray and three shadow rays
    if (next->capacity < std::min(hits->capacity, hits->source->capacity) ||
        shadows->capacity < 3 * std::min(hits->capacity, hits->source->capacity))
        return set_err(c, WF_ERR_CAPACITY, "next queue below the hits, or shadow queue below 3 x the hits");
    cudaSetDevice(c->device);
    WaveTables T;
    int rc = stage_tables(c, T);
    if (rc) return rc;
    cudaStream_t s = c->stream;
    LaunchCfg PC = persist_cfg(c);
    PC.ray_order = hits->at_ray ? 1 : 0;
    WF_CK(c, cudaMemsetAsync(next->counts, 0, sizeof(ull), s));
    WF_CK(c, cudaMemsetAsync(shadows->counts, 0, sizeof(ull), s));
    launch_shade(T, hits->rays, hits->h[hits->cur], hits->counts, shadows->sh, shadows->counts,
                 next->q[next->cur], next->counts, c->arena, c->err_flag, PC, s);
    next->has_perm = false;
    return WF_OK;
}

int wf_trace_occluded(wf_ctx* c, wf_shadow_queue* shadows)
{
    if (!c || !shadows || shadows->ctx != c) return set_err(c, WF_ERR_INVALID_ARGUMENT, "bad argument");
    cudaSetDevice(c->device);
    WaveTables T;
    int rc = stage_tables(c, T);
    if (rc) return rc;
    WF_CK(c, cudaMemsetAsync(shadows->counts + 1, 0, sizeof(ull), c->stream));
    launch_occluded_render(T, shadows->sh, shadows->counts, c->arena, shadows->counts + 1, c->err_flag,
                           persist_cfg(c), c->stream);
    return WF_OK;
}

int wf_miss(wf_ctx* c, wf_ray_queue* misses)
{
    if (!c || !misses || misses->ctx != c) return set_err(c, WF_ERR_INVALID_ARGUMENT, "bad argument");
    cudaSetDevice(c->device);
    WaveTables T;
    int rc = stage_tables(c, T);
    if (rc) return rc;
    launch_miss_queue(T, misses->q[misses->cur], misses->counts, c->arena, wide_cfg(c), c->stream);
    return WF_OK;
}

int wf_stage_image(wf_ctx* c, float* image, int64_t nf)
{
    if (!c || !image) return set_err(c, WF_ERR_INVALID_ARGUMENT, "null argument");
    cudaSetDevice(c->device);
    WaveTables T;
    int rc = stage_tables(c, T);
    if (rc) return rc;
    const int64_t need = 3 * c->stage_pixels;
    if (nf < need) return set_err(c, WF_ERR_CAPACITY, "image buffer smaller than width * height * 3");
    float* d = nullptr;
    WF_CK(c, cudaMalloc(&d, sizeof(float) * (size_t)need));
    launch_finalize(c->arena, need, (float)c->stage_params.samples_per_pixel, d, c->stream);
    cudaError_t e = cudaMemcpyAsync(image, d, sizeof(float) * (size_t)need, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (e != cudaSuccess) return set_err(c, WF_ERR_CUDA, cudaGetErrorString(e));
    return check_device_flag(c);
}

}  // extern "C"
