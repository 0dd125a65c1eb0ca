// wf_api.cpp — the C ABI (include/wf_api.h): context, resident scenes, the
// stage entry points on host buffers, tuning and timers.  The render loop
// itself (single renders, batches of jobs, the serving loop) is in
// wf_loop.cpp.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "../../include/wf_api.h"
#include "wf_bvh.h"
#include "wf_ctx.h"
#include "wf_device.cuh"
#include "wf_kernels.h"
#include "wf_sort.h"

using namespace wf;

namespace wf {

int set_err(wf_ctx* c, int code, const std::string& msg)
{
    if (c) c->last_error = msg;
    return code;
}

void free_all(std::vector<void*>& v)
{
    for (void* p : v) cudaFree(p);
    v.clear();
}

// The largest tree + triangles among the scenes `ids` (all resident scenes
// when ids is null) and whether none of them has an environment map,
// textures or a directional light (the lean shading instance).
void wave_scene_traits(const wf_ctx* c, const int32_t* ids, int n, int64_t& max_bytes, int& lean)
{
    max_bytes = 0;
    lean = 1;
    const int count = ids ? n : (int)c->scenes.size();
    for (int k = 0; k < count; ++k) {
        const int i = ids ? ids[k] : k;
        if (i < 0 || i >= (int)c->scenes.size() || !c->scenes[i].live) continue;
        const ResidentScene& r = c->scenes[i];
        max_bytes = std::max<int64_t>(max_bytes, (int64_t)r.tree_bytes);
        if (r.S.env_alias_prob || r.S.num_textures > 0 || r.S.directional.intensity > 0.0f) lean = 0;
    }
}

LaunchCfg persist_cfg(const wf_ctx* c)
{
    int per_sm = c->tuning.persistent_blocks_per_sm > 0 ? c->tuning.persistent_blocks_per_sm : 16;
    LaunchCfg cfg{c->num_sms * per_sm, 128};
    cfg.variant = c->tuning.trace_variant;
    cfg.l2_bytes = c->l2_bytes;
    if (c->wave_scene_bytes >= 0 && c->wave_lean >= 0) {
        cfg.max_scene_bytes = c->wave_scene_bytes;
        cfg.lean_multi = c->wave_lean;
    } else {
        wave_scene_traits(c, nullptr, 0, cfg.max_scene_bytes, cfg.lean_multi);
    }
    cfg.shade_grid = c->num_sms * c->shade_per_sm;
    cfg.shade_grid_other = c->num_sms * c->shade_per_sm_other;
    return cfg;
}

LaunchCfg wide_cfg(const wf_ctx* c) { return LaunchCfg{c->num_sms * 8, 256}; }

void drop_graphs(wf_ctx* c)
{
    for (auto& g : c->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
}

int ensure_render_buffers(wf_ctx* c, int64_t paths)
{
    if (paths <= c->cap) return WF_OK;
    free_all(c->render_allocs);
    drop_graphs(c);
    c->cap = 0;
    auto& A = c->render_allocs;
    const size_t n = (size_t)paths;
    for (int q = 0; q < 2; ++q) {
        RayQueueDev& r = c->rq[q];
        WF_CK(c, wf_dalloc(A, &r.ox, n)); WF_CK(c, wf_dalloc(A, &r.oy, n)); WF_CK(c, wf_dalloc(A, &r.oz, n));
        WF_CK(c, wf_dalloc(A, &r.dx, n)); WF_CK(c, wf_dalloc(A, &r.dy, n)); WF_CK(c, wf_dalloc(A, &r.dz, n));
        WF_CK(c, wf_dalloc(A, &r.tr, n)); WF_CK(c, wf_dalloc(A, &r.tg, n)); WF_CK(c, wf_dalloc(A, &r.tb, n));
        WF_CK(c, wf_dalloc(A, &r.pdf, n));
        WF_CK(c, wf_dalloc(A, &r.pixel, n)); WF_CK(c, wf_dalloc(A, &r.depth, n)); WF_CK(c, wf_dalloc(A, &r.sample, n));
        WF_CK(c, wf_dalloc(A, &r.job, n));
        r.capacity = paths;
        HitQueueDev& h = c->hq[q];
        WF_CK(c, wf_dalloc(A, &h.ray, n)); WF_CK(c, wf_dalloc(A, &h.tri, n)); WF_CK(c, wf_dalloc(A, &h.t, n));
        WF_CK(c, wf_dalloc(A, &h.bu, n)); WF_CK(c, wf_dalloc(A, &h.bv, n));
        h.capacity = paths;
    }
    const size_t ns = 3 * n;  // area, directional and environment NEE per hit
    ShadowQueueDev& s = c->sh;
    WF_CK(c, wf_dalloc(A, &s.ox, ns)); WF_CK(c, wf_dalloc(A, &s.oy, ns)); WF_CK(c, wf_dalloc(A, &s.oz, ns));
    WF_CK(c, wf_dalloc(A, &s.dx, ns)); WF_CK(c, wf_dalloc(A, &s.dy, ns)); WF_CK(c, wf_dalloc(A, &s.dz, ns));
    WF_CK(c, wf_dalloc(A, &s.dist, ns));
    WF_CK(c, wf_dalloc(A, &s.cr, ns)); WF_CK(c, wf_dalloc(A, &s.cg, ns)); WF_CK(c, wf_dalloc(A, &s.cb, ns));
    WF_CK(c, wf_dalloc(A, &s.pixel, ns));
    WF_CK(c, wf_dalloc(A, &s.job, ns));
    s.capacity = (int64_t)ns;
    WF_CK(c, wf_dalloc(A, &c->keys, n)); WF_CK(c, wf_dalloc(A, &c->keys_tmp, n));
    WF_CK(c, wf_dalloc(A, &c->vals, n)); WF_CK(c, wf_dalloc(A, &c->vals_tmp, n));
    c->nb = radix_blocks_for(paths, c->num_sms);
    WF_CK(c, wf_dalloc(A, &c->hist, radix_hist_words(c->nb)));
    WF_CK(c, wf_dalloc(A, &c->col_mat, n)); WF_CK(c, wf_dalloc(A, &c->col_tex, n));
    WF_CK(c, wf_dalloc(A, &c->col_tr, n)); WF_CK(c, wf_dalloc(A, &c->col_tg, n)); WF_CK(c, wf_dalloc(A, &c->col_tb, n));
    WF_CK(c, wf_dalloc(A, &c->col_px, n)); WF_CK(c, wf_dalloc(A, &c->col_py, n)); WF_CK(c, wf_dalloc(A, &c->col_pz, n));
    c->cap = paths;
    return WF_OK;
}

int ensure_arena(wf_ctx* c, int64_t floats)
{
    if (floats <= c->arena_floats) return WF_OK;
    drop_graphs(c);
    cudaFree(c->arena);
    c->arena = nullptr;
    c->arena_floats = 0;
    WF_CK(c, cudaMalloc(&c->arena, sizeof(float) * (size_t)floats));
    c->arena_floats = floats;
    return WF_OK;
}

int ensure_adaptive(wf_ctx* c, int64_t np, int64_t buf_floats)
{
    if (np <= c->ad_np_cap && buf_floats <= c->ad_buf_cap) return WF_OK;
    drop_graphs(c);
    free_all(c->adaptive_allocs);
    c->ad_np_cap = c->ad_buf_cap = 0;
    auto& A = c->adaptive_allocs;
    const size_t n = (size_t)np;
    WF_CK(c, wf_dalloc(A, &c->ad_mean, n));
    WF_CK(c, wf_dalloc(A, &c->ad_m2, n));
    WF_CK(c, wf_dalloc(A, &c->ad_count, n));
    WF_CK(c, wf_dalloc(A, &c->ad_active, n));
    WF_CK(c, wf_dalloc(A, &c->ad_flag, n));
    WF_CK(c, wf_dalloc(A, &c->ad_pos, n));
    WF_CK(c, wf_dalloc(A, &c->ad_bsums, (size_t)scan_block_words(np)));
    WF_CK(c, wf_dalloc(A, &c->ad_nactive, 1));
    WF_CK(c, wf_dalloc(A, &c->ad_buf, (size_t)buf_floats));
    c->ad_np_cap = np;
    c->ad_buf_cap = buf_floats;
    return WF_OK;
}

namespace {
int alloc_tracker(wf_ctx* c, CostTrackerDev& T, int cap)
{
    auto& A = c->cost_allocs;
    const size_t n = (size_t)std::max(cap, 1);
    WF_CK(c, wf_dalloc(A, &T.sum, n));
    WF_CK(c, wf_dalloc(A, &T.cnt, n));
    WF_CK(c, wf_dalloc(A, &T.avg, n));
    WF_CK(c, wf_dalloc(A, &T.samples, n));
    WF_CK(c, wf_dalloc(A, &T.init, n));
    WF_CK(c, wf_dalloc(A, &T.total, 1));
    WF_CK(c, wf_dalloc(A, &T.tracked, 1));
    WF_CK(c, wf_dalloc(A, &T.rel, n));
    WF_CK(c, wf_dalloc(A, &T.rel_f, n));
    return WF_OK;
}

int zero_tracker(wf_ctx* c, CostTrackerDev& T, int items)
{
    cudaStream_t s = c->stream;
    const size_t n = (size_t)std::max(items, 1);
    T.items = items;
    WF_CK(c, cudaMemsetAsync(T.sum, 0, sizeof(*T.sum) * n, s));
    WF_CK(c, cudaMemsetAsync(T.cnt, 0, sizeof(*T.cnt) * n, s));
    WF_CK(c, cudaMemsetAsync(T.avg, 0, sizeof(*T.avg) * n, s));
    WF_CK(c, cudaMemsetAsync(T.samples, 0, sizeof(*T.samples) * n, s));
    WF_CK(c, cudaMemsetAsync(T.init, 0, sizeof(*T.init) * n, s));
    WF_CK(c, cudaMemsetAsync(T.total, 0, sizeof(*T.total), s));
    WF_CK(c, cudaMemsetAsync(T.tracked, 0, sizeof(*T.tracked), s));
    return WF_OK;
}
}  // namespace

int reset_cost_trackers(wf_ctx* c, int nmat, int ntex)
{
    if (nmat > c->ct_mat_cap || ntex > c->ct_tex_cap) {
        free_all(c->cost_allocs);
        c->ct_mat = CostTrackerDev{};
        c->ct_tex = CostTrackerDev{};
        c->ct_mat_cap = c->ct_tex_cap = 0;
        int rc = alloc_tracker(c, c->ct_mat, nmat);
        if (rc) return rc;
        rc = alloc_tracker(c, c->ct_tex, ntex);
        if (rc) return rc;
        c->ct_mat_cap = nmat;
        c->ct_tex_cap = ntex;
    }
    int rc = zero_tracker(c, c->ct_mat, nmat);
    if (rc) return rc;
    rc = zero_tracker(c, c->ct_tex, ntex);
    if (rc) return rc;
    launch_cost_update(c->ct_mat, c->ct_tex, 1, c->stream);  // no records yet: relativeCost 1.0
    return WF_OK;
}

int ensure_job_tables(wf_ctx* c, int jobs, int chunks)
{
    if (jobs > c->jobs_cap) {
        drop_graphs(c);
        cudaFree(c->d_jobs);
        c->d_jobs = nullptr;
        c->jobs_cap = 0;
        int cap = std::max(jobs, 64);
        WF_CK(c, cudaMalloc(&c->d_jobs, sizeof(DeviceJob) * (size_t)cap));
        c->jobs_cap = cap;
    }
    if (chunks > c->chunks_cap) {
        drop_graphs(c);
        cudaFree(c->d_chunks);
        c->d_chunks = nullptr;
        c->chunks_cap = 0;
        int cap = std::max(chunks, 64);
        WF_CK(c, cudaMalloc(&c->d_chunks, sizeof(WaveChunk) * (size_t)cap));
        c->chunks_cap = cap;
    }
    return WF_OK;
}

// The device copy of every resident scene's descriptor, indexed by scene id.
int sync_scene_table(wf_ctx* c)
{
    if (!c->scene_table_dirty) return WF_OK;
    const int n = std::max<int>(1, (int)c->scenes.size());
    if (n > c->scene_table_cap) {
        drop_graphs(c);
        cudaFree(c->d_scene_table);
        c->d_scene_table = nullptr;
        c->scene_table_cap = 0;
        int cap = std::max(n, 16);
        WF_CK(c, cudaMalloc(&c->d_scene_table, sizeof(DeviceScene) * (size_t)cap));
        c->scene_table_cap = cap;
    }
    std::vector<DeviceScene> host(n);
    for (int i = 0; i < (int)c->scenes.size(); ++i) host[i] = c->scenes[i].S;
    WF_CK(c, cudaMemcpyAsync(c->d_scene_table, host.data(), sizeof(DeviceScene) * n, cudaMemcpyHostToDevice,
                             c->stream));
    WF_CK(c, cudaStreamSynchronize(c->stream));
    c->scene_table_dirty = false;
    return WF_OK;
}

namespace {
int ensure_rank_buffers(wf_ctx* c, int count)
{
    if (count <= c->rank_cap) return WF_OK;
    if (c->rank_buf) cudaFree(c->rank_buf);
    if (c->benefit) cudaFree(c->benefit);
    if (c->present) cudaFree(c->present);
    c->rank_buf = nullptr;
    c->benefit = nullptr;
    c->present = nullptr;
    WF_CK(c, cudaMalloc(&c->rank_buf, sizeof(int) * (size_t)count));
    WF_CK(c, cudaMalloc(&c->benefit, sizeof(double) * (size_t)count));
    WF_CK(c, cudaMalloc(&c->present, sizeof(int) * (size_t)count));
    c->rank_cap = count;
    return WF_OK;
}

// Dense ranks of values in descending order (equal values share a rank).
std::vector<int> dense_rank_desc(const std::vector<double>& v, int& bits)
{
    std::vector<double> u(v);
    std::sort(u.begin(), u.end(), [](double a, double b) { return a > b; });
    u.erase(std::unique(u.begin(), u.end()), u.end());
    std::vector<int> r(v.size());
    for (size_t i = 0; i < v.size(); ++i)
        r[i] = (int)(std::lower_bound(u.begin(), u.end(), v[i], [](double a, double b) { return a > b; }) - u.begin());
    bits = 1;
    while ((size_t(1) << bits) < u.size() + 1) ++bits;
    return r;
}

// The type order of computeTypeOrder (ShadingQueue.h:277-329): candidate list
// in reverse order of first appearance (the iteration order of the
// reference's unordered_map for these keys), insertion-sorted (stable) by
// count desc with ties on the larger type (material) or by texture bytes desc
// (texture).
void type_ranks(int policy, const ull cnt[8], const ull mem[8], const int first[8], int rank[8])
{
    std::vector<int> types;
    for (int t = 0; t < 8; ++t)
        if (cnt[t]) types.push_back(t);
    std::sort(types.begin(), types.end(), [&](int a, int b) { return first[a] > first[b]; });
    if (policy == WF_POLICY_MATERIAL_AWARE)
        std::stable_sort(types.begin(), types.end(), [&](int a, int b) {
            if (cnt[a] != cnt[b]) return cnt[a] > cnt[b];
            return a > b;
        });
    else
        std::stable_sort(types.begin(), types.end(), [&](int a, int b) { return mem[a] > mem[b]; });
    for (int t = 0; t < 8; ++t) rank[t] = 0;
    for (int r = 0; r < (int)types.size(); ++r) rank[types[r]] = r;
}

}  // namespace

// Sorts the n scheduling columns under the policy; perm (device) receives the
// permutation.  Requires c->keys etc. with capacity >= n and d_n on device.
int schedule_columns(wf_ctx* c, int policy, const ull* d_n, int64_t n, ShadeColumnsDev cols,
                     const wf_material* d_mats, int num_materials, const std::vector<wf_material>& hmats,
                     int num_tex, const int64_t* d_tex_bytes, const std::vector<int64_t>& htex_bytes,
                     const double* rc_mat, const double* rc_tex, uint32_t** perm_out)
{
    cudaStream_t s = c->stream;
    LaunchCfg W = wide_cfg(c);
    uint64_t* rk = nullptr;
    uint32_t* rv = nullptr;
    c->last_schedule_launches = 1;
    if (policy == WF_POLICY_NONE || n == 0) {
        launch_iota(c->vals, d_n, W.grid, s);
        *perm_out = c->vals;
        return WF_OK;
    }
    int rc = ensure_rank_buffers(c, std::max(num_materials, num_tex + 1) + 1);
    if (rc) return rc;
    if (policy == WF_POLICY_COST_BENEFIT_AWARE) {
        WF_CK(c, cudaMemsetAsync(c->benefit, 0, sizeof(double) * num_materials, s));
        WF_CK(c, cudaMemsetAsync(c->present, 0, sizeof(int) * num_materials, s));
        unsigned init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
        WF_CK(c, cudaMemcpyAsync(c->bounds6, init, sizeof(init), cudaMemcpyHostToDevice, s));
        launch_cb_reduce(cols, d_n, c->benefit, c->present, c->bounds6, num_materials, W, s);
        std::vector<double> ben(num_materials);
        std::vector<int> pres(num_materials);
        WF_CK(c, cudaMemcpyAsync(ben.data(), c->benefit, sizeof(double) * num_materials, cudaMemcpyDeviceToHost, s));
        WF_CK(c, cudaMemcpyAsync(pres.data(), c->present, sizeof(int) * num_materials, cudaMemcpyDeviceToHost, s));
        WF_CK(c, cudaStreamSynchronize(s));
        // priority = benefit / max(cost, 1e-6) (ShadingQueue.h:458-471)
        std::vector<double> prio(num_materials, -1.0);
        std::vector<double> present_prio;
        for (int m = 0; m < num_materials; ++m) {
            if (!pres[m]) continue;
            double cost = rc_mat ? rc_mat[m] : 1.0;
            int tid = hmats[m].texture_id;
            double tcost = (rc_tex && tid >= 0) ? rc_tex[tid] : 0.0;
            prio[m] = ben[m] / std::max(cost + tcost, 1e-6);
            present_prio.push_back(prio[m]);
        }
        int bits = 1;
        std::vector<int> pr_present = dense_rank_desc(present_prio, bits);
        std::vector<int> pr(num_materials, 0);
        for (int m = 0, k = 0; m < num_materials; ++m)
            if (pres[m]) pr[m] = pr_present[k++];
        WF_CK(c, cudaMemcpyAsync(c->rank_buf, pr.data(), sizeof(int) * num_materials, cudaMemcpyHostToDevice, s));
        launch_cb_keys(cols, d_n, d_mats, c->rank_buf, bits, c->bounds6, c->keys, c->vals, W, s);
        RadixSortArgs a{c->keys, c->vals, c->keys_tmp, c->vals_tmp, c->hist, d_n, c->nb, 0, 33 + bits,
                        &rk, &rv};
        radix_sort_pairs(a, s);
        c->last_schedule_launches = 2 + kSortKernelsPerPass * ((33 + bits + 7) / 8);
        *perm_out = rv;
        return WF_OK;
    }
    // Material / texture aware
    WF_CK(c, cudaMemsetAsync(c->stats8, 0, sizeof(ull) * 16, s));
    {
        int init[8];
        for (int k = 0; k < 8; ++k) init[k] = 0x7FFFFFFF;
        WF_CK(c, cudaMemcpyAsync(c->first8, init, sizeof(init), cudaMemcpyHostToDevice, s));
    }
    launch_type_stats(cols, d_n, d_mats, num_tex, d_tex_bytes, c->stats8, c->stats8 + 8, c->first8, W, s);
    ull st[16];
    int first[8];
    WF_CK(c, cudaMemcpyAsync(st, c->stats8, sizeof(st), cudaMemcpyDeviceToHost, s));
    WF_CK(c, cudaMemcpyAsync(first, c->first8, sizeof(first), cudaMemcpyDeviceToHost, s));
    WF_CK(c, cudaStreamSynchronize(s));
    int trank[8];
    type_ranks(policy, st, st + 8, first, trank);
    int bits = 1;
    std::vector<int> sec;
    if (policy == WF_POLICY_TEXTURE_AWARE) {
        std::vector<double> sizes(num_tex + 1, 0.0);
        for (int t = 0; t < num_tex; ++t) sizes[t] = (double)htex_bytes[t];
        sizes[num_tex] = 0.0;
        sec = dense_rank_desc(sizes, bits);
    } else {
        std::vector<double> costs(num_materials, 1.0);
        if (rc_mat)
            for (int m = 0; m < num_materials; ++m) costs[m] = rc_mat[m];
        sec = dense_rank_desc(costs, bits);
    }
    WF_CK(c, cudaMemcpyAsync(c->rank_buf, sec.data(), sizeof(int) * sec.size(), cudaMemcpyHostToDevice, s));
    launch_policy_keys(cols, d_n, d_mats, policy, trank, c->rank_buf, c->rank_buf, num_tex, bits,
                       c->keys, c->vals, W, s);
    RadixSortArgs a{c->keys, c->vals, c->keys_tmp, c->vals_tmp, c->hist, d_n, c->nb, 0, bits + 3,
                    &rk, &rv};
    radix_sort_pairs(a, s);
    c->last_schedule_launches = 2 + kSortKernelsPerPass * ((bits + 3 + 7) / 8);
    *perm_out = rv;
    return WF_OK;
}

int check_device_flag(wf_ctx* c)
{
    int flag = 0;
    WF_CK(c, cudaMemcpyAsync(&flag, c->err_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    WF_CK(c, cudaStreamSynchronize(c->stream));
    if (flag) {
        cudaMemsetAsync(c->err_flag, 0, sizeof(int), c->stream);
        return set_err(c, WF_ERR_DEVICE_CHECK,
                       "device check tripped (flag " + std::to_string(flag) +
                           "): 1 traversal stack, 2 hit queue, 4 shadow queue, 8 ray queue");
    }
    return WF_OK;
}

}  // namespace wf

namespace {

// Default builder: scenes below this many triangles get surface-area leaves.
constexpr int kSahLeafTriangles = 4096;

// Bytes per node of a built tree's format.
size_t tree_node_bytes(const BvhBuildOutput& b)
{
    return b.nodes4 ? sizeof(Bvh4Node) : sizeof(BvhNode);
}

// srgbToLinear, reference src/shading/Texture.cpp:20-27.
float srgb_to_linear(float s)
{
    if (s <= 0.04045f) return s / 12.92f;
    return std::pow((s + 0.055f) / 1.055f, 2.4f);
}

struct HostV3 {
    float x, y, z;
};
inline HostV3 hsub(HostV3 a, HostV3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline HostV3 hcross(HostV3 a, HostV3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float hlen(HostV3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

void free_scene_res(ResidentScene& R)
{
    free_all(R.allocs);
    R = ResidentScene{};
}

bool has_scene(const wf_ctx* c) { return !c->scenes.empty() && c->scenes[0].live; }

// Uploads one scene and builds its BVH: Scene::buildAccelerator
// (src/core/Scene.cpp:79-113) + EmbreeAccelerator::build (Embree.cpp:66-119).
// Environment importance sampler (no reference counterpart): texel weights
// luminance(rgb * scale * tint) x cos(elevation of the texel's centre row),
// normalised to p_i = N f_i / sum f (N texels, stored as texel_pdf), and
// Walker's alias table built by Vose's method: texels with p < 1 and p >= 1
// on two stacks in index order; repeatedly pop one of each, give the small
// one (prob = p_s, alias = the large one) and move the large one's excess
// p_l + p_s - 1 back onto the stack it now belongs to; leftovers get
// prob 1.  Returns false when the map carries no energy.
bool build_env_sampler(const wf_environment& e, std::vector<float>& prob, std::vector<int32_t>& alias,
                       std::vector<float>& texel_pdf)
{
    const int64_t W = e.width, H = e.height, N = W * H;
    std::vector<double> p((size_t)N);
    double sum = 0.0;
    const double pi = 3.14159265358979323846;
    for (int64_t y = 0; y < H; ++y) {
        const double ce = std::cos((0.5 - (y + 0.5) / (double)H) * pi);
        for (int64_t x = 0; x < W; ++x) {
            const float* t = e.rgb + 3 * (y * W + x);
            const double r = (double)t[0] * e.intensity_scale * e.tint[0];
            const double g = (double)t[1] * e.intensity_scale * e.tint[1];
            const double b = (double)t[2] * e.intensity_scale * e.tint[2];
            const double f = std::max(0.0, 0.2126 * r + 0.7152 * g + 0.0722 * b) * ce;
            p[(size_t)(y * W + x)] = f;
            sum += f;
        }
    }
    if (!(sum > 0.0) || !std::isfinite(sum)) return false;
    prob.assign((size_t)N, 1.0f);
    alias.resize((size_t)N);
    texel_pdf.resize((size_t)N);
    std::vector<int64_t> small, large;
    for (int64_t i = 0; i < N; ++i) {
        p[(size_t)i] = p[(size_t)i] * (double)N / sum;
        texel_pdf[(size_t)i] = (float)p[(size_t)i];
        alias[(size_t)i] = (int32_t)i;
        (p[(size_t)i] < 1.0 ? small : large).push_back(i);
    }
    while (!small.empty() && !large.empty()) {
        const int64_t sm = small.back(), lg = large.back();
        small.pop_back();
        large.pop_back();
        prob[(size_t)sm] = (float)p[(size_t)sm];
        alias[(size_t)sm] = (int32_t)lg;
        p[(size_t)lg] = (p[(size_t)lg] + p[(size_t)sm]) - 1.0;
        (p[(size_t)lg] < 1.0 ? small : large).push_back(lg);
    }
    return true;
}

int build_scene(wf_ctx* c, const wf_scene_desc* D, ResidentScene& R)
{
    if (!c || !D) return WF_ERR_INVALID_ARGUMENT;
    if (D->num_indices % 3 != 0 || D->num_indices < 0 || D->num_vertices < 0 || D->num_meshes < 0)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "index count must be a multiple of 3");
    if (D->num_materials <= 0 || !D->materials)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "scene needs at least one material");
    const int ntri = D->num_indices / 3;
    if (ntri >= (1 << 28)) return set_err(c, WF_ERR_INVALID_ARGUMENT, "more than 2^28 triangles");
    // Validate meshes: contiguous, in index order, material ids in range.
    int expect = 0;
    for (int m = 0; m < D->num_meshes; ++m) {
        if (D->mesh_index_offsets[m] != expect || D->mesh_index_counts[m] % 3 != 0)
            return set_err(c, WF_ERR_INVALID_ARGUMENT, "meshes must be contiguous in index order");
        if (D->mesh_material_ids[m] < 0 || D->mesh_material_ids[m] >= D->num_materials)
            return set_err(c, WF_ERR_INVALID_ARGUMENT, "mesh material id out of range");
        expect += D->mesh_index_counts[m];
    }
    if (expect != D->num_indices) return set_err(c, WF_ERR_INVALID_ARGUMENT, "meshes do not cover the indices");
    for (int i = 0; i < D->num_indices; ++i)
        if (D->indices[i] < 0 || D->indices[i] >= D->num_vertices)
            return set_err(c, WF_ERR_INVALID_ARGUMENT, "vertex index out of range");
    for (int m = 0; m < D->num_materials; ++m) {
        int t = D->materials[m].type;
        if (t < 0 || t > 5) return set_err(c, WF_ERR_INVALID_ARGUMENT, "unknown material type");
    }
    cudaStream_t s = c->stream;
    auto& A = R.allocs;
    DeviceScene S{};

    // Per-triangle ids, emissive meshes, area, bounds — host, as the reference.
    std::vector<int32_t> tri_geom(ntri), tri_prim(ntri);
    for (int m = 0; m < D->num_meshes; ++m) {
        int first = D->mesh_index_offsets[m] / 3, cnt = D->mesh_index_counts[m] / 3;
        for (int t = 0; t < cnt; ++t) {
            tri_geom[first + t] = m;
            tri_prim[first + t] = t;
        }
    }
    auto vert = [&](int gi) { return HostV3{D->positions_x[gi], D->positions_y[gi], D->positions_z[gi]}; };
    std::vector<EmissiveMesh> em;
    std::vector<float4> etris;
    float total_area = 0.0f;
    for (int m = 0; m < D->num_meshes; ++m) {
        int ty = D->materials[D->mesh_material_ids[m]].type;
        if (ty != WF_MATERIAL_EMISSIVE && ty != WF_MATERIAL_SPOTLIGHT) continue;
        EmissiveMesh e{(int32_t)(etris.size() / 3), D->mesh_index_counts[m] / 3, D->mesh_material_ids[m], 0};
        for (int t = 0; t < e.count; ++t) {
            int base = D->mesh_index_offsets[m] + 3 * t;
            HostV3 a = vert(D->indices[base]), b = vert(D->indices[base + 1]), cc = vert(D->indices[base + 2]);
            etris.push_back(make_float4(a.x, a.y, a.z, 0.0f));
            etris.push_back(make_float4(b.x, b.y, b.z, 0.0f));
            etris.push_back(make_float4(cc.x, cc.y, cc.z, 0.0f));
            total_area += hlen(hcross(hsub(b, a), hsub(cc, a))) * 0.5f;  // Scene.cpp:173-186
        }
        em.push_back(e);
    }
    float bmin[3], bmax[3];
    for (int k = 0; k < 3; ++k) {
        bmin[k] = std::numeric_limits<float>::max();
        bmax[k] = std::numeric_limits<float>::lowest();
    }
    for (int i = 0; i < D->num_vertices; ++i) {
        float p[3] = {D->positions_x[i], D->positions_y[i], D->positions_z[i]};
        for (int k = 0; k < 3; ++k) {
            bmin[k] = std::min(bmin[k], p[k]);
            bmax[k] = std::max(bmax[k], p[k]);
        }
    }

    // Geometry upload + BVH build.
    float *dpx = nullptr, *dpy = nullptr, *dpz = nullptr;
    int32_t *didx = nullptr, *dgeom = nullptr, *dprim = nullptr;
    std::vector<void*> tmp;
    auto cleanup_tmp = [&]() { free_all(tmp); };
    BvhBuildOutput bo{};
    std::string err;
    if (ntri > 0) {
        if (wf_dalloc(tmp, &dpx, D->num_vertices) || wf_dalloc(tmp, &dpy, D->num_vertices) ||
            wf_dalloc(tmp, &dpz, D->num_vertices) || wf_dalloc(tmp, &didx, D->num_indices) ||
            wf_dalloc(tmp, &dgeom, ntri) || wf_dalloc(tmp, &dprim, ntri)) {
            cleanup_tmp();
            return set_err(c, WF_ERR_OUT_OF_MEMORY, "geometry upload allocation failed");
        }
        cudaMemcpyAsync(dpx, D->positions_x, sizeof(float) * D->num_vertices, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dpy, D->positions_y, sizeof(float) * D->num_vertices, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dpz, D->positions_z, sizeof(float) * D->num_vertices, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(didx, D->indices, sizeof(int32_t) * D->num_indices, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dgeom, tri_geom.data(), sizeof(int32_t) * ntri, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dprim, tri_prim.data(), sizeof(int32_t) * ntri, cudaMemcpyHostToDevice, s);
        BvhBuildInput bi{dpx, dpy, dpz, didx, dgeom, dprim, ntri, {bmin[0], bmin[1], bmin[2]}, {bmax[0], bmax[1], bmax[2]}};
        auto b0 = std::chrono::steady_clock::now();
        int brc = -1;
        if (c->tuning.bvh_builder == 0) {
            // Scenes of few triangles (the Cornell-box workloads, whose wall
            // triangles dwarf the rest) get leaves by the surface area
            // heuristic (Cornell box +4.6%); dense scenes keep leaves of up to
            // four triangles (dense mesh with SAH leaves: -1.4%).
            brc = build_ploc(bi, bo, c->num_sms, s, err, ntri < kSahLeafTriangles);
            R.info.bvh_builder = 0;
        } else if (c->tuning.bvh_builder == 3) {
            brc = build_ploc4(bi, bo, c->num_sms, s, err);
            R.info.bvh_builder = 3;
        } else if (c->tuning.bvh_builder == 4) {
            brc = build_ploc(bi, bo, c->num_sms, s, err, true);
            R.info.bvh_builder = 4;
        }
        if (brc) {  // LBVH on request, or when a PLOC tree is too deep for its stack
            brc = build_lbvh(bi, bo, c->num_sms, s, err);
            R.info.bvh_builder = 1;
        }
        auto b1 = std::chrono::steady_clock::now();
        cleanup_tmp();
        if (brc) return set_err(c, WF_ERR_CUDA, "BVH build failed: " + err);
        // Tree nodes and triangles in one allocation, nodes first: one
        // address range the traversal reads.
        {
            const size_t node_bytes = (size_t)bo.num_nodes * tree_node_bytes(bo);
            const size_t tri_bytes = 3 * sizeof(float4) * (size_t)ntri;
            unsigned char* pool = nullptr;
            if (cudaMalloc(&pool, node_bytes + tri_bytes) != cudaSuccess) {
                cudaFree(bo.tris);
                cudaFree(bo.nodes);
                cudaFree(bo.nodes4);
                free_scene_res(R);
                return set_err(c, WF_ERR_OUT_OF_MEMORY, "BVH pool allocation failed");
            }
            const void* src_nodes = bo.nodes4 ? (const void*)bo.nodes4 : (const void*)bo.nodes;
            cudaMemcpyAsync(pool, src_nodes, node_bytes, cudaMemcpyDeviceToDevice, s);
            cudaMemcpyAsync(pool + node_bytes, bo.tris, tri_bytes, cudaMemcpyDeviceToDevice, s);
            cudaStreamSynchronize(s);
            cudaFree(bo.tris);
            cudaFree(bo.nodes);
            cudaFree(bo.nodes4);
            bo.tris = reinterpret_cast<float4*>(pool + node_bytes);
            if (bo.nodes4)
                bo.nodes4 = reinterpret_cast<Bvh4Node*>(pool);
            else
                bo.nodes = reinterpret_cast<BvhNode*>(pool);
            A.push_back(pool);
            R.tree_base = pool;
            R.tree_bytes = node_bytes + tri_bytes;
        }
        R.info.bvh_build_ms = std::chrono::duration<double, std::milli>(b1 - b0).count();
        R.info.bvh_depth = bo.max_depth;
    }
    S.tris = bo.tris;
    S.nodes = bo.nodes;
    S.nodes4 = bo.nodes4;
    S.num_tris = ntri;
    S.num_nodes = bo.num_nodes;
    S.root_is_empty = ntri == 0 ? 1 : 0;
    S.num_meshes = D->num_meshes;

    std::vector<float> env_prob, env_pdf;
    std::vector<int32_t> env_alias;
#define UP(dst, src, count)                                                                     \
    do {                                                                                        \
        if (wf_dalloc(A, &dst, (count)) != cudaSuccess) {                                          \
            free_scene_res(R);                                                                      \
            return set_err(c, WF_ERR_OUT_OF_MEMORY, "scene allocation failed");                 \
        }                                                                                       \
        if ((count) > 0)                                                                        \
            cudaMemcpyAsync((void*)dst, (src), sizeof(*dst) * (size_t)(count), cudaMemcpyHostToDevice, s); \
    } while (0)

    int32_t* d_mesh_mat = nullptr;
    UP(d_mesh_mat, D->mesh_material_ids, D->num_meshes);
    S.mesh_material = d_mesh_mat;
    std::vector<uint8_t> has_uv(std::max(1, D->num_meshes), 0);
    bool any_uv = false;
    if (D->mesh_has_uv && D->corner_u && D->corner_v)
        for (int m = 0; m < D->num_meshes; ++m) {
            has_uv[m] = D->mesh_has_uv[m] ? 1 : 0;
            any_uv = any_uv || has_uv[m];
        }
    uint8_t* d_has_uv = nullptr;
    UP(d_has_uv, has_uv.data(), (int64_t)has_uv.size());
    S.mesh_has_uv = d_has_uv;
    S.has_any_uv = any_uv ? 1 : 0;
    if (any_uv) {
        std::vector<float2> cuv((size_t)D->num_indices);
        for (int i = 0; i < D->num_indices; ++i) cuv[i] = make_float2(D->corner_u[i], D->corner_v[i]);
        float2* d_cuv = nullptr;
        UP(d_cuv, cuv.data(), (int64_t)cuv.size());
        S.corner_uv = d_cuv;
    }
    wf_material* d_mats = nullptr;
    UP(d_mats, D->materials, D->num_materials);
    S.materials = d_mats;
    S.num_materials = D->num_materials;
    R.mats.assign(D->materials, D->materials + D->num_materials);
    // Textures
    std::vector<TexDesc> td(std::max(1, D->num_textures));
    std::vector<float> pool_f;
    std::vector<uint32_t> pool_b;
    R.tex_bytes.assign(D->num_textures, 0);
    for (int t = 0; t < D->num_textures; ++t) {
        const wf_texture& x = D->textures[t];
        if (x.width <= 0 || x.height <= 0 || !x.data) {
            free_scene_res(R);
            return set_err(c, WF_ERR_INVALID_ARGUMENT, "texture without texels");
        }
        size_t n = (size_t)x.width * x.height;
        td[t].width = x.width;
        td[t].height = x.height;
        td[t].format = x.format;
        // Texture::memoryBytes = pixels.size() * sizeof(Color) (Texture.h:51-54)
        R.tex_bytes[t] = (int64_t)(n * 12);
        if (x.format == WF_TEXEL_RGB32F) {
            td[t].offset = (int64_t)pool_f.size();
            const float* f = (const float*)x.data;
            pool_f.insert(pool_f.end(), f, f + 3 * n);
        } else {
            td[t].offset = (int64_t)pool_b.size();
            const uint32_t* b = (const uint32_t*)x.data;
            pool_b.insert(pool_b.end(), b, b + n);
        }
    }
    TexDesc* d_td = nullptr;
    UP(d_td, td.data(), (int64_t)td.size());
    S.textures = d_td;
    S.num_textures = D->num_textures;
    float* d_pf = nullptr;
    UP(d_pf, pool_f.data(), (int64_t)pool_f.size());
    S.tex_f32 = d_pf;
    uint32_t* d_pb = nullptr;
    UP(d_pb, pool_b.data(), (int64_t)pool_b.size());
    S.tex_rgba8 = d_pb;
    float lut[256];
    for (int i = 0; i < 256; ++i) lut[i] = srgb_to_linear((float)i / 255.0f);
    float* d_lut = nullptr;
    UP(d_lut, lut, 256);
    S.srgb_lut = d_lut;
    int64_t* d_tb = nullptr;
    UP(d_tb, R.tex_bytes.data(), (int64_t)R.tex_bytes.size());
    R.d_tex_bytes = d_tb;
    // Lights
    EmissiveMesh* d_em = nullptr;
    UP(d_em, em.data(), (int64_t)em.size());
    S.emissive_meshes = d_em;
    S.num_emissive_meshes = (int32_t)em.size();
    float4* d_et = nullptr;
    UP(d_et, etris.data(), (int64_t)etris.size());
    S.emissive_tris = d_et;
    S.total_emissive_area = total_area;
    S.light_area_pdf = total_area <= 0.0f ? 0.0f : 1.0f / total_area;  // MIS.h:24-31
    S.directional = D->directional;
    // Environment
    if (D->environment.width > 0 && D->environment.rgb) {
        float* d_env = nullptr;
        UP(d_env, D->environment.rgb, 3 * (int64_t)D->environment.width * D->environment.height);
        S.env_rgb = d_env;
        S.env_w = D->environment.width;
        S.env_h = D->environment.height;
        S.env_scale = D->environment.intensity_scale;
        for (int k = 0; k < 3; ++k) S.env_tint[k] = D->environment.tint[k];
        if (build_env_sampler(D->environment, env_prob, env_alias, env_pdf)) {
            float *d_prob = nullptr, *d_pdf = nullptr;
            int32_t* d_alias = nullptr;
            UP(d_prob, env_prob.data(), (int64_t)env_prob.size());
            UP(d_alias, env_alias.data(), (int64_t)env_alias.size());
            UP(d_pdf, env_pdf.data(), (int64_t)env_pdf.size());
            S.env_alias_prob = d_prob;
            S.env_alias = d_alias;
            S.env_texel_pdf = d_pdf;
        }
    }
    for (int k = 0; k < 3; ++k) {
        S.bmin[k] = bmin[k];
        S.bmax[k] = bmax[k];
    }
#undef UP
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        free_scene_res(R);
        return set_err(c, WF_ERR_CUDA, "scene upload failed");
    }
    R.S = S;
    R.live = true;
    wf_scene_info& I = R.info;
    for (int k = 0; k < 3; ++k) {
        I.bounds_min[k] = bmin[k];
        I.bounds_max[k] = bmax[k];
    }
    I.total_emissive_area = total_area;
    I.num_triangles = ntri;
    I.num_meshes = D->num_meshes;
    I.num_emissive_meshes = (int32_t)em.size();
    I.bvh_nodes = bo.num_nodes;
    int64_t bytes = (int64_t)ntri * 48 +
                    (int64_t)bo.num_nodes * (int64_t)tree_node_bytes(bo) +
                    (int64_t)pool_f.size() * 4 + (int64_t)pool_b.size() * 4;
    I.device_bytes = bytes;
    return WF_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int wf_version(void) { return WF_API_VERSION; }

int wf_create(const wf_config* cfg, wf_ctx** out)
{
    if (!out) return WF_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return WF_ERR_NO_DEVICE;
    wf_ctx* c = new wf_ctx();
    c->device = cfg ? cfg->device : 0;
    if (c->device < 0 || c->device >= ndev) {
        delete c;
        return WF_ERR_INVALID_ARGUMENT;
    }
    if (cfg && cfg->max_paths_per_wave > 0) c->paths_per_wave = cfg->max_paths_per_wave;
    if (cudaSetDevice(c->device) != cudaSuccess) {
        delete c;
        return WF_ERR_CUDA;
    }
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, c->device);
    c->num_sms = prop.multiProcessorCount;
    c->l2_bytes = prop.l2CacheSize;
    c->shade_per_sm = shade_blocks_per_sm(true);
    c->shade_per_sm_other = shade_blocks_per_sm(false);
    bool ok = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) == cudaSuccess;
    for (auto& e : c->ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    for (auto& e : c->timer) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    ok = ok && cudaMalloc(&c->counters, sizeof(ull) * 8) == cudaSuccess;
    ok = ok && cudaMalloc(&c->tally, sizeof(ull) * 8) == cudaSuccess;
    ok = ok && cudaMalloc(&c->d_wave_header, sizeof(long long) * 2) == cudaSuccess;
    ok = ok && cudaMalloc(&c->err_flag, sizeof(int)) == cudaSuccess;
    ok = ok && cudaMalloc(&c->stats8, sizeof(ull) * 16) == cudaSuccess;
    ok = ok && cudaMalloc(&c->first8, sizeof(int) * 8) == cudaSuccess;
    ok = ok && cudaMalloc(&c->bounds6, sizeof(unsigned) * 6) == cudaSuccess;
    ok = ok && cudaMemset(c->err_flag, 0, sizeof(int)) == cudaSuccess;
    ok = ok && cudaMemset(c->counters, 0, sizeof(ull) * 8) == cudaSuccess;
    if (!ok) {
        wf_destroy(c);
        return WF_ERR_CUDA;
    }
    *out = c;
    return WF_OK;
}

int wf_destroy(wf_ctx* c)
{
    if (!c) return WF_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    drop_graphs(c);
    for (auto& r : c->scenes) free_scene_res(r);
    free_all(c->render_allocs);
    free_all(c->rel_cost_allocs);
    free_all(c->adaptive_allocs);
    free_all(c->cost_allocs);
    cudaFree(c->d_scene_table);
    cudaFree(c->d_jobs);
    cudaFree(c->d_chunks);
    cudaFree(c->d_wave_header);
    cudaFree(c->arena);
    cudaFree(c->tally);
    cudaFree(c->counters);
    cudaFree(c->err_flag);
    cudaFree(c->stats8);
    cudaFree(c->first8);
    cudaFree(c->bounds6);
    cudaFree(c->rank_buf);
    cudaFree(c->benefit);
    cudaFree(c->present);
    cudaFree(c->image);
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->timer)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->stage_ev)
        if (e) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return WF_OK;
}

const char* wf_last_error(const wf_ctx* c) { return c ? c->last_error.c_str() : ""; }

int wf_host_alloc(size_t bytes, void** out)
{
    if (!out) return WF_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return WF_ERR_NO_DEVICE;
    }
    if (cudaMallocHost(out, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return WF_ERR_OUT_OF_MEMORY;
    }
    return WF_OK;
}

int wf_host_free(void* p)
{
    if (!p) return WF_OK;
    return cudaFreeHost(p) == cudaSuccess ? WF_OK : WF_ERR_INVALID_ARGUMENT;
}

int wf_camera_make(const float look_from[3], const float look_at[3], const float up[3],
                   float vfov, int32_t w, int32_t h, wf_camera* out)
{
    if (!look_from || !look_at || !up || !out || w <= 0 || h <= 0) return WF_ERR_INVALID_ARGUMENT;
    // Camera::Camera, include/core/Camera.h:13-33 (float arithmetic as written).
    float aspect = (float)w / h;
    float theta = vfov * 3.14159265f / 180.0f;
    float vh = 2.0f * std::tan(theta / 2.0f);
    float vw = aspect * vh;
    HostV3 from = {look_from[0], look_from[1], look_from[2]};
    HostV3 at = {look_at[0], look_at[1], look_at[2]};
    HostV3 u = {up[0], up[1], up[2]};
    HostV3 fw = hsub(from, at);
    float lf = hlen(fw);
    fw = {fw.x / lf, fw.y / lf, fw.z / lf};
    HostV3 right = hcross(u, fw);
    float lr = hlen(right);
    right = {right.x / lr, right.y / lr, right.z / lr};
    HostV3 upv = hcross(fw, right);
    HostV3 hz = {right.x * vw, right.y * vw, right.z * vw};
    HostV3 vt = {upv.x * vh, upv.y * vh, upv.z * vh};
    HostV3 tl = {from.x - hz.x / 2.0f, from.y - hz.y / 2.0f, from.z - hz.z / 2.0f};
    tl = {tl.x - vt.x / 2.0f, tl.y - vt.y / 2.0f, tl.z - vt.z / 2.0f};
    tl = hsub(tl, fw);
    float* dsts[4] = {out->origin, out->top_left, out->horizontal, out->vertical};
    HostV3 srcs[4] = {from, tl, hz, vt};
    for (int k = 0; k < 4; ++k) {
        dsts[k][0] = srcs[k].x;
        dsts[k][1] = srcs[k].y;
        dsts[k][2] = srcs[k].z;
    }
    return WF_OK;
}

int wf_scene_upload(wf_ctx* c, const wf_scene_desc* D)
{
    if (!c || !D) return WF_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (c->scenes.empty()) c->scenes.resize(1);
    drop_graphs(c);
    free_scene_res(c->scenes[0]);
    c->scene_table_dirty = true;
    int rc = build_scene(c, D, c->scenes[0]);
    if (rc) return rc;
    return sync_scene_table(c);
}

int wf_scene_add(wf_ctx* c, const wf_scene_desc* D, int32_t* out_id)
{
    if (!c || !D || !out_id) return WF_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (c->scenes.empty()) c->scenes.resize(1);  // slot 0 stays the current scene
    int slot = -1;
    for (int i = 1; i < (int)c->scenes.size(); ++i)
        if (!c->scenes[i].live) {
            slot = i;
            break;
        }
    if (slot < 0) {
        c->scenes.emplace_back();
        slot = (int)c->scenes.size() - 1;
    }
    int rc = build_scene(c, D, c->scenes[slot]);
    if (rc) return rc;
    c->scene_table_dirty = true;
    rc = sync_scene_table(c);
    if (rc) return rc;
    *out_id = slot;
    return WF_OK;
}

int wf_scene_remove(wf_ctx* c, int32_t id)
{
    if (!c || id < 0 || id >= (int)c->scenes.size() || !c->scenes[id].live)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "no such scene");
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    free_scene_res(c->scenes[id]);
    c->scene_table_dirty = true;
    return sync_scene_table(c);
}

int wf_scene_get_info(wf_ctx* c, wf_scene_info* out)
{
    if (!c || !out) return WF_ERR_INVALID_ARGUMENT;
    if (!has_scene(c)) return set_err(c, WF_ERR_STATE, "no scene uploaded");
    *out = c->scenes[0].info;
    return WF_OK;
}

int wf_scene_get_info_id(wf_ctx* c, int32_t id, wf_scene_info* out)
{
    if (!c || !out) return WF_ERR_INVALID_ARGUMENT;
    if (id < 0 || id >= (int)c->scenes.size() || !c->scenes[id].live)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "no such scene");
    *out = c->scenes[id].info;
    return WF_OK;
}

int wf_trace_closest_host(wf_ctx* c, int64_t n, const float* ox, const float* oy, const float* oz,
                          const float* dx, const float* dy, const float* dz, float tmin, float tmax,
                          wf_hit_columns* out)
{
    if (!c || !out || n < 0 || (n > 0 && (!ox || !oy || !oz || !dx || !dy || !dz)))
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "null argument");
    if (!has_scene(c)) return set_err(c, WF_ERR_STATE, "no scene uploaded");
    if (n == 0) return WF_OK;
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    std::vector<void*> tmp;
    float* in[6];
    const float* src[6] = {ox, oy, oz, dx, dy, dz};
    for (int k = 0; k < 6; ++k) {
        WF_CK(c, wf_dalloc(tmp, &in[k], n));
        WF_CK(c, cudaMemcpyAsync(in[k], src[k], sizeof(float) * n, cudaMemcpyHostToDevice, s));
    }
    HitColumnsDev d{};
    WF_CK(c, wf_dalloc(tmp, &d.geom, n)); WF_CK(c, wf_dalloc(tmp, &d.prim, n));
    WF_CK(c, wf_dalloc(tmp, &d.t, n)); WF_CK(c, wf_dalloc(tmp, &d.bu, n)); WF_CK(c, wf_dalloc(tmp, &d.bv, n));
    WF_CK(c, wf_dalloc(tmp, &d.px, n)); WF_CK(c, wf_dalloc(tmp, &d.py, n)); WF_CK(c, wf_dalloc(tmp, &d.pz, n));
    WF_CK(c, wf_dalloc(tmp, &d.nx, n)); WF_CK(c, wf_dalloc(tmp, &d.ny, n)); WF_CK(c, wf_dalloc(tmp, &d.nz, n));
    WF_CK(c, wf_dalloc(tmp, &d.front, n)); WF_CK(c, wf_dalloc(tmp, &d.u, n)); WF_CK(c, wf_dalloc(tmp, &d.v, n));
    WF_CK(c, wf_dalloc(tmp, &d.mat, n)); WF_CK(c, wf_dalloc(tmp, &d.tex, n));
    launch_trace_api(c->scenes[0].S, n, in[0], in[1], in[2], in[3], in[4], in[5], tmin, tmax, d, c->err_flag,
                     persist_cfg(c), s);
    WF_CK(c, cudaGetLastError());
    struct Pair {
        void* host;
        void* dev;
        size_t elem;
    } pairs[] = {{out->geom_id, d.geom, 4}, {out->prim_id, d.prim, 4}, {out->distance, d.t, 4},
                 {out->bary_u, d.bu, 4},   {out->bary_v, d.bv, 4},   {out->point_x, d.px, 4},
                 {out->point_y, d.py, 4},  {out->point_z, d.pz, 4},  {out->normal_x, d.nx, 4},
                 {out->normal_y, d.ny, 4}, {out->normal_z, d.nz, 4}, {out->front_face, d.front, 1},
                 {out->u, d.u, 4},         {out->v, d.v, 4},         {out->material_id, d.mat, 4},
                 {out->texture_id, d.tex, 4}};
    for (auto& p : pairs)
        if (p.host) WF_CK(c, cudaMemcpyAsync(p.host, p.dev, p.elem * (size_t)n, cudaMemcpyDeviceToHost, s));
    WF_CK(c, cudaStreamSynchronize(s));
    free_all(tmp);
    return check_device_flag(c);
}

int wf_trace_occluded_host(wf_ctx* c, int64_t n, const float* ox, const float* oy, const float* oz,
                           const float* dx, const float* dy, const float* dz, const float* maxd,
                           uint8_t* out)
{
    if (!c || n < 0 || (n > 0 && (!ox || !oy || !oz || !dx || !dy || !dz || !maxd || !out)))
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "null argument");
    if (!has_scene(c)) return set_err(c, WF_ERR_STATE, "no scene uploaded");
    if (n == 0) return WF_OK;
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    std::vector<void*> tmp;
    float* in[7];
    const float* src[7] = {ox, oy, oz, dx, dy, dz, maxd};
    for (int k = 0; k < 7; ++k) {
        WF_CK(c, wf_dalloc(tmp, &in[k], n));
        WF_CK(c, cudaMemcpyAsync(in[k], src[k], sizeof(float) * n, cudaMemcpyHostToDevice, s));
    }
    uint8_t* d_out = nullptr;
    WF_CK(c, wf_dalloc(tmp, &d_out, n));
    launch_occluded_api(c->scenes[0].S, n, in[0], in[1], in[2], in[3], in[4], in[5], in[6], d_out, c->err_flag,
                        persist_cfg(c), s);
    WF_CK(c, cudaGetLastError());
    WF_CK(c, cudaMemcpyAsync(out, d_out, (size_t)n, cudaMemcpyDeviceToHost, s));
    WF_CK(c, cudaStreamSynchronize(s));
    free_all(tmp);
    return check_device_flag(c);
}

int wf_generate_primary_host(wf_ctx* c, const wf_camera* cam, int32_t W, int32_t H, uint32_t s0,
                             uint32_t s1, int32_t first_sample, int32_t nspp, float* ox, float* oy,
                             float* oz, float* dx, float* dy, float* dz, int32_t* pixel,
                             int32_t* sample)
{
    if (!c || !cam || W < 2 || H < 2 || nspp < 1) return set_err(c, WF_ERR_INVALID_ARGUMENT, "bad arguments");
    cudaSetDevice(c->device);
    const int64_t n = (int64_t)W * H * nspp;
    cudaStream_t s = c->stream;
    std::vector<void*> tmp;
    RayQueueDev rq{};
    WF_CK(c, wf_dalloc(tmp, &rq.ox, n)); WF_CK(c, wf_dalloc(tmp, &rq.oy, n)); WF_CK(c, wf_dalloc(tmp, &rq.oz, n));
    WF_CK(c, wf_dalloc(tmp, &rq.dx, n)); WF_CK(c, wf_dalloc(tmp, &rq.dy, n)); WF_CK(c, wf_dalloc(tmp, &rq.dz, n));
    WF_CK(c, wf_dalloc(tmp, &rq.tr, n)); WF_CK(c, wf_dalloc(tmp, &rq.tg, n)); WF_CK(c, wf_dalloc(tmp, &rq.tb, n));
    WF_CK(c, wf_dalloc(tmp, &rq.pdf, n)); WF_CK(c, wf_dalloc(tmp, &rq.pixel, n));
    WF_CK(c, wf_dalloc(tmp, &rq.depth, n)); WF_CK(c, wf_dalloc(tmp, &rq.sample, n));
    rq.job = nullptr;
    rq.capacity = n;
    launch_camera(*cam, W, H, s0, s1, first_sample, nspp, rq, s);
    WF_CK(c, cudaGetLastError());
    void* hs[8] = {ox, oy, oz, dx, dy, dz, pixel, sample};
    void* ds[8] = {rq.ox, rq.oy, rq.oz, rq.dx, rq.dy, rq.dz, rq.pixel, rq.sample};
    for (int k = 0; k < 8; ++k)
        if (hs[k]) WF_CK(c, cudaMemcpyAsync(hs[k], ds[k], 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    WF_CK(c, cudaStreamSynchronize(s));
    free_all(tmp);
    return WF_OK;
}

int wf_ray_schedule_host(wf_ctx* c, int64_t n, const float* ox, const float* oy, const float* oz,
                         const float* dx, const float* dy, const float* dz, const float bmin[3],
                         const float bmax[3], int32_t* out_sorted, uint64_t* out_keys)
{
    if (!c || n < 0 || !bmin || !bmax || (n > 0 && (!ox || !oy || !oz || !dx || !dy || !dz || !out_sorted)))
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "null argument");
    if (n == 0) return WF_OK;
    if (n > 0x7FFFFFFF) return set_err(c, WF_ERR_INVALID_ARGUMENT, "too many rays");
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    std::vector<void*> tmp;
    float* in[6];
    const float* src[6] = {ox, oy, oz, dx, dy, dz};
    for (int k = 0; k < 6; ++k) {
        WF_CK(c, wf_dalloc(tmp, &in[k], n));
        WF_CK(c, cudaMemcpyAsync(in[k], src[k], sizeof(float) * n, cudaMemcpyHostToDevice, s));
    }
    uint64_t *k0, *k1;
    uint32_t *v0, *v1, *hist;
    ull* d_n;
    int nb = radix_blocks_for(n, c->num_sms);
    WF_CK(c, wf_dalloc(tmp, &k0, n)); WF_CK(c, wf_dalloc(tmp, &k1, n));
    WF_CK(c, wf_dalloc(tmp, &v0, n)); WF_CK(c, wf_dalloc(tmp, &v1, n));
    WF_CK(c, wf_dalloc(tmp, &hist, radix_hist_words(nb)));
    WF_CK(c, wf_dalloc(tmp, &d_n, 1));
    ull hn = (ull)n;
    WF_CK(c, cudaMemcpyAsync(d_n, &hn, sizeof(hn), cudaMemcpyHostToDevice, s));
    launch_ray_keys_raw(n, in[0], in[1], in[2], in[3], in[4], in[5], bmin, bmax, k0, v0, wide_cfg(c), s);
    if (out_keys) WF_CK(c, cudaMemcpyAsync(out_keys, k0, 8 * (size_t)n, cudaMemcpyDeviceToHost, s));
    uint64_t* rk;
    uint32_t* rv;
    RadixSortArgs a{k0, v0, k1, v1, hist, d_n, nb, 0, 33, &rk, &rv};
    radix_sort_pairs(a, s);
    WF_CK(c, cudaGetLastError());
    WF_CK(c, cudaMemcpyAsync(out_sorted, rv, 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    WF_CK(c, cudaStreamSynchronize(s));
    free_all(tmp);
    return WF_OK;
}

int wf_shading_schedule_host(wf_ctx* c, int32_t policy, int64_t n, const int32_t* mat_ids,
                             const int32_t* tex_ids, const float* tr, const float* tg, const float* tb,
                             const float* px, const float* py, const float* pz, int32_t num_materials,
                             const wf_material* materials, int32_t num_textures,
                             const int64_t* texture_bytes, const double* rc_mat, const double* rc_tex,
                             int32_t* out_sorted)
{
    if (!c || n < 0 || policy < 0 || policy > 3 || num_materials <= 0 || !materials || num_textures < 0 ||
        (num_textures > 0 && !texture_bytes))
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "bad arguments");
    if (n == 0) return WF_OK;
    if (!mat_ids || !tex_ids || !tr || !tg || !tb || !px || !py || !pz || !out_sorted)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "null column");
    for (int64_t i = 0; i < n; ++i)
        if (mat_ids[i] < 0 || mat_ids[i] >= num_materials)
            return set_err(c, WF_ERR_INVALID_ARGUMENT, "material id out of range");
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    int rc = ensure_render_buffers(c, n);
    if (rc) return rc;
    std::vector<void*> tmp;
    WF_CK(c, cudaMemcpyAsync(c->col_mat, mat_ids, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
    WF_CK(c, cudaMemcpyAsync(c->col_tex, tex_ids, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
    WF_CK(c, cudaMemcpyAsync(c->col_tr, tr, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
    WF_CK(c, cudaMemcpyAsync(c->col_tg, tg, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
    WF_CK(c, cudaMemcpyAsync(c->col_tb, tb, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
    WF_CK(c, cudaMemcpyAsync(c->col_px, px, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
    WF_CK(c, cudaMemcpyAsync(c->col_py, py, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
    WF_CK(c, cudaMemcpyAsync(c->col_pz, pz, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
    wf_material* d_mats;
    int64_t* d_tb;
    ull* d_n;
    WF_CK(c, wf_dalloc(tmp, &d_mats, num_materials));
    WF_CK(c, wf_dalloc(tmp, &d_tb, std::max(1, num_textures)));
    WF_CK(c, wf_dalloc(tmp, &d_n, 1));
    WF_CK(c, cudaMemcpyAsync(d_mats, materials, sizeof(wf_material) * num_materials, cudaMemcpyHostToDevice, s));
    if (num_textures > 0)
        WF_CK(c, cudaMemcpyAsync(d_tb, texture_bytes, 8 * (size_t)num_textures, cudaMemcpyHostToDevice, s));
    ull hn = (ull)n;
    WF_CK(c, cudaMemcpyAsync(d_n, &hn, sizeof(hn), cudaMemcpyHostToDevice, s));
    std::vector<wf_material> hm(materials, materials + num_materials);
    std::vector<int64_t> htb(texture_bytes, texture_bytes + num_textures);
    ShadeColumnsDev cd{c->col_mat, c->col_tex, c->col_tr, c->col_tg, c->col_tb, c->col_px, c->col_py, c->col_pz};
    uint32_t* perm = nullptr;
    rc = schedule_columns(c, policy, d_n, n, cd, d_mats, num_materials, hm, num_textures, d_tb, htb, rc_mat,
                          rc_tex, &perm);
    if (rc) {
        free_all(tmp);
        return rc;
    }
    WF_CK(c, cudaGetLastError());
    WF_CK(c, cudaMemcpyAsync(out_sorted, perm, 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    WF_CK(c, cudaStreamSynchronize(s));
    free_all(tmp);
    return WF_OK;
}

int wf_get_stream(wf_ctx* c, void** out)
{
    if (!c || !out) return WF_ERR_INVALID_ARGUMENT;
    *out = (void*)c->stream;
    return WF_OK;
}

int wf_set_tuning(wf_ctx* c, const wf_tuning* t)
{
    if (!c || !t) return WF_ERR_INVALID_ARGUMENT;
    if (t->trace_variant < 0 || t->trace_variant > 1 || t->persistent_blocks_per_sm < 0 ||
        t->persistent_blocks_per_sm > 32 || t->bvh_builder < 0 || t->bvh_builder > 4 || t->bvh_builder == 2 ||
        t->reserved2 != 0 || t->reserved != 0)
        return set_err(c, WF_ERR_INVALID_ARGUMENT, "tuning out of range");
    c->tuning = *t;
    return WF_OK;
}

int wf_get_tuning(const wf_ctx* c, wf_tuning* out)
{
    if (!c || !out) return WF_ERR_INVALID_ARGUMENT;
    *out = c->tuning;
    return WF_OK;
}

int wf_timer_begin(wf_ctx* c)
{
    if (!c) return WF_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    WF_CK(c, cudaEventRecord(c->timer[0], c->stream));
    return WF_OK;
}

int wf_timer_end(wf_ctx* c, double* out_ms)
{
    if (!c || !out_ms) return WF_ERR_INVALID_ARGUMENT;
    WF_CK(c, cudaEventRecord(c->timer[1], c->stream));
    WF_CK(c, cudaEventSynchronize(c->timer[1]));
    float ms = 0.0f;
    WF_CK(c, cudaEventElapsedTime(&ms, c->timer[0], c->timer[1]));
    *out_ms = ms;
    return WF_OK;
}

}  // extern "C"
