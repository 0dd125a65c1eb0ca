// wf_ctx.h — the context behind the C ABI (internal to libwfgpu.so).
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/wf_api.h"
#include "wf_device.cuh"
#include "wf_kernels.h"

namespace wf {

// Paths in flight per wave: 2^27 (134 M paths, ~57 GB of queues at 424 B per
// path) holds all 64 samples of a 1024^2 render, or all 32 of a 2048^2
// render, in one wave, so the bounce tails stay wide and a warp traces the
// samples of one pixel (2^23 measured 30% slower on the dense-mesh workload;
// 2^27 against 2^26 on the 2048^2 lattice: +1.1%).
constexpr int64_t kDefaultPathsPerWave = int64_t(1) << 27;

// A scene kept on the device: BVH, triangles, materials, textures, lights.
struct ResidentScene {
    bool live = false;
    DeviceScene S{};
    std::vector<void*> allocs;
    wf_scene_info info{};
    std::vector<wf_material> mats;
    std::vector<int64_t> tex_bytes;
    int64_t* d_tex_bytes = nullptr;
    const void* tree_base = nullptr;  // tree nodes followed by triangles
    size_t tree_bytes = 0;
};

// A captured bounce chain (one wave, fixed depth), replayed for every wave.
struct CapturedWave {
    cudaGraphExec_t exec = nullptr;
    int max_depth = 0;
    bool ray_sort = false;
    int variant = 0;
    const void* key_ptr = nullptr;  // buffers the capture baked in
    int64_t key_cap = 0;
    int tree = kTreeBinary;         // tree format (TreeFormat) of the traversal
    int kernels = 0;                // kernels per replay
    int lean = 0;                   // LaunchCfg::lean_multi of the capture
    bool dense = false;             // LaunchCfg::max_scene_bytes >= kDenseSceneBytes at the capture
};

}  // namespace wf

struct wf_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 1;
    int64_t l2_bytes = 0;  // L2 cache size of the device
    int shade_per_sm = 0;        // k_shade's resident blocks per SM (0 = unknown: use the persistent grid)
    int shade_per_sm_other = 0;  // the same for its multi-job and cost-timed forms
    std::string last_error;
    int64_t paths_per_wave = wf::kDefaultPathsPerWave;
    // The scenes of the multi-job wave about to be launched (render_batch and
    // the server set them from their jobs; -1 = every resident scene): the
    // largest tree + triangles and whether all fit the lean shading instance.
    int64_t wave_scene_bytes = -1;
    int wave_lean = -1;

    // Resident scenes; slot 0 is the scene of wf_scene_upload (the "current"
    // scene of the single-scene entry points).
    std::vector<wf::ResidentScene> scenes;
    wf::DeviceScene* d_scene_table = nullptr;
    int scene_table_cap = 0;
    bool scene_table_dirty = true;

    // Job table and wave chunks (device), grown on demand
    wf::DeviceJob* d_jobs = nullptr;
    int jobs_cap = 0;
    wf::WaveChunk* d_chunks = nullptr;
    int chunks_cap = 0;
    long long* d_wave_header = nullptr;  // [0] total paths, [1] chunk count

    // Render buffers (grown on demand)
    int64_t cap = 0;
    wf::RayQueueDev rq[2]{};
    wf::HitQueueDev hq[2]{};
    wf::ShadowQueueDev sh{};
    uint64_t *keys = nullptr, *keys_tmp = nullptr;
    uint32_t *vals = nullptr, *vals_tmp = nullptr, *hist = nullptr;
    int nb = 1;
    int32_t *col_mat = nullptr, *col_tex = nullptr;
    float *col_tr = nullptr, *col_tg = nullptr, *col_tb = nullptr, *col_px = nullptr, *col_py = nullptr,
          *col_pz = nullptr;
    std::vector<void*> render_allocs;

    // Accumulator arena (per-job pixel sums live at offsets inside it)
    float* arena = nullptr;
    int64_t arena_floats = 0;

    // Small device state
    wf::ull* counters = nullptr;  // [0] rays [1] hits [2] shadows [3] next [4] work [5] work2
    wf::ull* tally = nullptr;     // [0] rays [1] hits [2] shadows [3] bounces (graph mode)
    int* err_flag = nullptr;
    wf::ull* stats8 = nullptr;    // type counts [8], mem [8]
    int* first8 = nullptr;        // first index per type
    int* rank_buf = nullptr;      // cost / texture / priority ranks
    int rank_cap = 0;
    double* benefit = nullptr;    // per material
    int* present = nullptr;       // per material
    unsigned* bounds6 = nullptr;
    std::vector<void*> rel_cost_allocs;  // float(relativeCost) tables of jobs
    int last_schedule_launches = 0;
    // Image of the last wf_render_device
    float* image = nullptr;
    int64_t image_floats = 0;

    // Adaptive sampling state (AdaptiveSampler) of the last single render:
    // per-pixel Welford mean / M2 / count, active flags and list, and the
    // per-sample sums of one wave.
    std::vector<void*> adaptive_allocs;
    int64_t ad_np_cap = 0, ad_buf_cap = 0;
    float *ad_mean = nullptr, *ad_m2 = nullptr, *ad_buf = nullptr;
    int32_t *ad_count = nullptr, *ad_active = nullptr, *ad_nactive = nullptr;
    int32_t *ad_flag = nullptr, *ad_pos = nullptr, *ad_bsums = nullptr;
    bool last_adaptive = false;
    int64_t last_np = 0;
    int32_t last_spp = 0;

    // Live CostTrackers (materials, textures) of the last single render
    std::vector<void*> cost_allocs;
    wf::CostTrackerDev ct_mat{}, ct_tex{};
    int ct_mat_cap = 0, ct_tex_cap = 0;

    std::vector<wf::CapturedWave> graphs;

    cudaEvent_t ev[8]{};
    cudaEvent_t timer[2]{};
    std::vector<cudaEvent_t> stage_ev;  // per-bounce stage events of the device-counted chain
    wf_tuning tuning{};


    // The render served by the per-bounce stage entry points (wf_stage_begin):
    // its parameters, its device job (slot 0 of the job table, scene 0) and
    // its pixel sums at offset 0 of the arena.
    bool stage_live = false;
    wf_render_params stage_params{};
    wf::DeviceJob stage_job{};
    int64_t stage_pixels = 0;
};

namespace wf {

int set_err(wf_ctx* c, int code, const std::string& msg);
void free_all(std::vector<void*>& v);
void wave_scene_traits(const wf_ctx* c, const int32_t* ids, int n, int64_t& max_bytes, int& lean);
LaunchCfg persist_cfg(const wf_ctx* c);
LaunchCfg wide_cfg(const wf_ctx* c);
int ensure_render_buffers(wf_ctx* c, int64_t paths);
int ensure_arena(wf_ctx* c, int64_t floats);
int ensure_adaptive(wf_ctx* c, int64_t np, int64_t buf_floats);
// Cost trackers for nmat materials and ntex textures, reset to their initial
// state (relativeCost 1.0) on the context's stream.
int reset_cost_trackers(wf_ctx* c, int nmat, int ntex);
int ensure_job_tables(wf_ctx* c, int jobs, int chunks);
int sync_scene_table(wf_ctx* c);
int check_device_flag(wf_ctx* c);
// Job setup shared by the render loop and the per-bounce stage entry points
// (wf_loop.cpp): a job's limits; its device form (accumulator at
// accum_offset floats); the job table; a wave's chunks and header.
int validate_job(wf_ctx* c, const wf_job& j);
int make_device_job(wf_ctx* c, const wf_job& j, int64_t accum_offset, DeviceJob& dj);
int upload_jobs(wf_ctx* c, const std::vector<DeviceJob>& jobs);
int upload_wave(wf_ctx* c, const std::vector<WaveChunk>& chunks, int64_t total);
void drop_graphs(wf_ctx* c);
// Sorts n scheduling columns under a ShadingQueue policy; *perm_out gets the
// permutation (device).  Materials and texture sizes of one scene.
int schedule_columns(wf_ctx* c, int policy, const ull* d_n, int64_t n, ShadeColumnsDev cols,
                     const wf_material* d_mats, int num_materials, const std::vector<wf_material>& hmats,
                     int num_tex, const int64_t* d_tex_bytes, const std::vector<int64_t>& htex_bytes,
                     const double* rc_mat, const double* rc_tex, uint32_t** perm_out);

}  // namespace wf

#define WF_CK(ctx, x)                                                                            \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess)                                                                   \
            return ::wf::set_err(ctx, WF_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
cudaError_t wf_dalloc(std::vector<void*>& owner, T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
    if (e == cudaSuccess) owner.push_back((void*)*p);
    return e;
}
