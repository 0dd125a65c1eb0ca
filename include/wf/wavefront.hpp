// wavefront.hpp — C++17 mirror of the reference's per-bounce-loop API over the
// C ABI of libwfgpu.so (include/wf_api.h).  Header-only.
//
// Same type and member names as fhidargue/wavefront-renderer, so code written
// against the reference's loop ports by changing includes and passing a
// wf::Context (the GPU and its resident scene):
//   RayQueue          include/scheduling/RayQueue.h:63-245
//   ShadingQueue      include/scheduling/ShadingQueue.h:27-551
//   SchedulingPolicy  include/scheduling/ShadingQueue.h:18-24
//   HitRecord         include/core/HitRecord.h:6-22 (plus geomID)
//   WavefrontRenderer include/render/WavefrontRenderer.h:16-56
// Errors: the reference throws from deep inside and catches in main
// (src/main.cpp:218-222); here every failing ABI call throws wf::Error with
// the library's message.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../wf_api.h"

namespace wf {

enum class SchedulingPolicy {
    None = WF_POLICY_NONE,
    MaterialAware = WF_POLICY_MATERIAL_AWARE,
    TextureAware = WF_POLICY_TEXTURE_AWARE,
    CostBenefitAware = WF_POLICY_COST_BENEFIT_AWARE,
};

class Error : public std::runtime_error {
  public:
    Error(int code, const std::string& msg) : std::runtime_error(msg), code(code) {}
    int code;
};

inline void check(int rc, const wf_ctx* ctx, const char* what)
{
    if (rc != WF_OK)
        throw Error(rc, std::string(what) + " failed (" + std::to_string(rc) + "): " + (ctx ? wf_last_error(ctx) : ""));
}

// One GPU, one stream, one resident scene.
class Context {
  public:
    explicit Context(int device = 0, int64_t maxPathsPerWave = 0)
    {
        wf_config cfg{device, maxPathsPerWave};
        check(wf_create(&cfg, &h_), nullptr, "wf_create");
    }
    ~Context() { wf_destroy(h_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    Context(Context&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
    Context& operator=(Context&& o) noexcept
    {
        if (this != &o) {
            wf_destroy(h_);
            h_ = std::exchange(o.h_, nullptr);
        }
        return *this;
    }
    // Scene::buildAccelerator + EmbreeAccelerator::build
    wf_scene_info upload(const wf_scene_desc& desc)
    {
        check(wf_scene_upload(h_, &desc), h_, "wf_scene_upload");
        wf_scene_info info{};
        check(wf_scene_get_info(h_, &info), h_, "wf_scene_get_info");
        return info;
    }
    wf_ctx* handle() const { return h_; }

  private:
    wf_ctx* h_ = nullptr;
};

struct HitRecord {
    float point[3] = {0, 0, 0};
    float normal[3] = {0, 0, 0};
    float distance = 0.0f;
    int materialID = -1;
    int textureID = -1;
    int triangleIndex = -1;
    float u = 0.0f, v = 0.0f;
    bool frontFace = false;
    int geomID = -1;  // device addition: the mesh index (Embree geomID)
};

namespace detail {
template <class V>
void permute(V& a, const std::vector<int>& idx)
{
    V out(idx.size());
    for (size_t i = 0; i < idx.size(); ++i) out[i] = a[idx[i]];
    a = std::move(out);
}
}  // namespace detail

// include/scheduling/RayQueue.h:63-245
struct RayQueue {
    std::vector<float> originsX, originsY, originsZ;
    std::vector<float> dirsX, dirsY, dirsZ;
    std::vector<float> throughputsR, throughputsG, throughputsB;
    std::vector<float> accumLightR, accumLightG, accumLightB;
    std::vector<int> pixelIndices;
    std::vector<int> depths;
    std::vector<bool> alive;
    std::vector<float> pdfs;
    std::vector<int> sortedIndices;

    void add(const float o[3], const float d[3], const float t[3], const float a[3], int pixel, int depth,
             bool isAlive, float pdf)
    {
        originsX.push_back(o[0]); originsY.push_back(o[1]); originsZ.push_back(o[2]);
        dirsX.push_back(d[0]); dirsY.push_back(d[1]); dirsZ.push_back(d[2]);
        throughputsR.push_back(t[0]); throughputsG.push_back(t[1]); throughputsB.push_back(t[2]);
        accumLightR.push_back(a[0]); accumLightG.push_back(a[1]); accumLightB.push_back(a[2]);
        pixelIndices.push_back(pixel);
        depths.push_back(depth);
        alive.push_back(isAlive);
        pdfs.push_back(pdf);
    }
    void addPrimary(const float o[3], const float d[3], int pixel)
    {
        const float one[3] = {1, 1, 1}, zero[3] = {0, 0, 0};
        add(o, d, one, zero, pixel, 0, true, -1.0f);
    }
    int size() const { return (int)originsX.size(); }
    bool empty() const { return originsX.empty(); }
    void clear() { *this = RayQueue{}; }

    // RayQueue::schedule on the GPU: sortedIndices = stable sort of sortKey.
    void schedule(Context& ctx, const float sceneMin[3], const float sceneMax[3])
    {
        sortedIndices.assign(size(), 0);
        if (empty()) return;
        check(wf_ray_schedule_host(ctx.handle(), size(), originsX.data(), originsY.data(), originsZ.data(),
                                   dirsX.data(), dirsY.data(), dirsZ.data(), sceneMin, sceneMax,
                                   sortedIndices.data(), nullptr),
              ctx.handle(), "wf_ray_schedule_host");
    }
    // RayQueue::materialize: gather every column, reset the identity.
    void materialize()
    {
        if ((int)sortedIndices.size() != size()) return;
        for (auto* c : {&originsX, &originsY, &originsZ, &dirsX, &dirsY, &dirsZ, &throughputsR, &throughputsG,
                        &throughputsB, &accumLightR, &accumLightG, &accumLightB, &pdfs})
            detail::permute(*c, sortedIndices);
        detail::permute(pixelIndices, sortedIndices);
        detail::permute(depths, sortedIndices);
        detail::permute(alive, sortedIndices);
        for (int i = 0; i < size(); ++i) sortedIndices[i] = i;
    }
};

// include/scheduling/ShadingQueue.h:27-551
struct ShadingQueue {
    std::vector<float> hitPointsX, hitPointsY, hitPointsZ;
    std::vector<float> hitNormalsX, hitNormalsY, hitNormalsZ;
    std::vector<float> hitDistances, hitU, hitV;
    std::vector<int> hitTriangleIndex;
    std::vector<int> materialIDs, textureIDs;
    std::vector<float> originsX, originsY, originsZ;
    std::vector<float> dirsX, dirsY, dirsZ;
    std::vector<float> throughputsR, throughputsG, throughputsB;
    std::vector<int> pixelIndices, depths;
    std::vector<float> pdfs;
    std::vector<int> sortedIndices;
    std::vector<int> geomIDs;       // device addition
    std::vector<uint8_t> frontFaces; // carried (the reference's getHitRecord drops it)
    SchedulingPolicy policy;

    explicit ShadingQueue(SchedulingPolicy p = SchedulingPolicy::None) : policy(p) {}

    void add(const RayQueue& r, int i, const HitRecord& h)
    {
        hitPointsX.push_back(h.point[0]); hitPointsY.push_back(h.point[1]); hitPointsZ.push_back(h.point[2]);
        hitNormalsX.push_back(h.normal[0]); hitNormalsY.push_back(h.normal[1]); hitNormalsZ.push_back(h.normal[2]);
        hitDistances.push_back(h.distance); hitU.push_back(h.u); hitV.push_back(h.v);
        hitTriangleIndex.push_back(h.triangleIndex);
        materialIDs.push_back(h.materialID); textureIDs.push_back(h.textureID);
        originsX.push_back(r.originsX[i]); originsY.push_back(r.originsY[i]); originsZ.push_back(r.originsZ[i]);
        dirsX.push_back(r.dirsX[i]); dirsY.push_back(r.dirsY[i]); dirsZ.push_back(r.dirsZ[i]);
        throughputsR.push_back(r.throughputsR[i]); throughputsG.push_back(r.throughputsG[i]);
        throughputsB.push_back(r.throughputsB[i]);
        pixelIndices.push_back(r.pixelIndices[i]); depths.push_back(r.depths[i]); pdfs.push_back(r.pdfs[i]);
        geomIDs.push_back(h.geomID);
        frontFaces.push_back(h.frontFace ? 1 : 0);
    }
    int size() const { return (int)materialIDs.size(); }
    bool empty() const { return materialIDs.empty(); }

    // ShadingQueue::schedule on the GPU.  textureBytes[t] = Texture::memoryBytes();
    // relative costs are frozen CostTracker::relativeCost values (null = 1.0).
    void schedule(Context& ctx, const std::vector<wf_material>& materials, const std::vector<int64_t>& textureBytes,
                  const std::vector<double>* relCostMaterial = nullptr,
                  const std::vector<double>* relCostTexture = nullptr)
    {
        sortedIndices.assign(size(), 0);
        if (empty()) return;
        check(wf_shading_schedule_host(ctx.handle(), (int32_t)policy, size(), materialIDs.data(), textureIDs.data(),
                                       throughputsR.data(), throughputsG.data(), throughputsB.data(),
                                       hitPointsX.data(), hitPointsY.data(), hitPointsZ.data(),
                                       (int32_t)materials.size(), materials.data(), (int32_t)textureBytes.size(),
                                       textureBytes.data(), relCostMaterial ? relCostMaterial->data() : nullptr,
                                       relCostTexture ? relCostTexture->data() : nullptr, sortedIndices.data()),
              ctx.handle(), "wf_shading_schedule_host");
    }
    HitRecord getHitRecord(int pos) const
    {
        int i = sortedIndices.empty() ? pos : sortedIndices[pos];
        HitRecord h;
        h.point[0] = hitPointsX[i]; h.point[1] = hitPointsY[i]; h.point[2] = hitPointsZ[i];
        h.normal[0] = hitNormalsX[i]; h.normal[1] = hitNormalsY[i]; h.normal[2] = hitNormalsZ[i];
        h.distance = hitDistances[i]; h.u = hitU[i]; h.v = hitV[i];
        h.triangleIndex = hitTriangleIndex[i]; h.materialID = materialIDs[i]; h.textureID = textureIDs[i];
        h.geomID = geomIDs[i]; h.frontFace = frontFaces[i] != 0;
        return h;
    }
    int getPixelIndex(int pos) const { return pixelIndices[sortedIndices.empty() ? pos : sortedIndices[pos]]; }
    void materialize()
    {
        if ((int)sortedIndices.size() != size()) return;
        for (auto* c : {&hitPointsX, &hitPointsY, &hitPointsZ, &hitNormalsX, &hitNormalsY, &hitNormalsZ,
                        &hitDistances, &hitU, &hitV, &originsX, &originsY, &originsZ, &dirsX, &dirsY, &dirsZ,
                        &throughputsR, &throughputsG, &throughputsB, &pdfs})
            detail::permute(*c, sortedIndices);
        for (auto* c : {&hitTriangleIndex, &materialIDs, &textureIDs, &pixelIndices, &depths, &geomIDs})
            detail::permute(*c, sortedIndices);
        detail::permute(frontFaces, sortedIndices);
        for (int i = 0; i < size(); ++i) sortedIndices[i] = i;
    }
};

// WavefrontRenderer::intersectAll (.cpp:459-567): closest hits of a queue on
// the GPU, split into a ShadingQueue of hits and a RayQueue of misses.
inline void intersectAll(Context& ctx, const RayQueue& in, ShadingQueue& hits, RayQueue& misses)
{
    const int n = in.size();
    if (n == 0) return;
    std::vector<int32_t> geom(n), prim(n), mat(n), tex(n);
    std::vector<float> t(n), px(n), py(n), pz(n), nx(n), ny(n), nz(n), u(n), v(n);
    std::vector<uint8_t> front(n);
    wf_hit_columns cols{geom.data(), prim.data(), t.data(), nullptr, nullptr, px.data(), py.data(), pz.data(),
                        nx.data(), ny.data(), nz.data(), front.data(), u.data(), v.data(), mat.data(), tex.data()};
    check(wf_trace_closest_host(ctx.handle(), n, in.originsX.data(), in.originsY.data(), in.originsZ.data(),
                                in.dirsX.data(), in.dirsY.data(), in.dirsZ.data(), 0.001f, 1e9f, &cols),
          ctx.handle(), "wf_trace_closest_host");
    for (int i = 0; i < n; ++i) {
        if (geom[i] < 0) {
            const float o[3] = {in.originsX[i], in.originsY[i], in.originsZ[i]};
            const float d[3] = {in.dirsX[i], in.dirsY[i], in.dirsZ[i]};
            const float T[3] = {in.throughputsR[i], in.throughputsG[i], in.throughputsB[i]};
            const float A[3] = {in.accumLightR[i], in.accumLightG[i], in.accumLightB[i]};
            misses.add(o, d, T, A, in.pixelIndices[i], in.depths[i], true, in.pdfs[i]);
            continue;
        }
        HitRecord h;
        h.point[0] = px[i]; h.point[1] = py[i]; h.point[2] = pz[i];
        h.normal[0] = nx[i]; h.normal[1] = ny[i]; h.normal[2] = nz[i];
        h.distance = t[i]; h.u = u[i]; h.v = v[i];
        h.materialID = mat[i]; h.textureID = tex[i]; h.triangleIndex = prim[i]; h.geomID = geom[i];
        h.frontFace = front[i] != 0;
        hits.add(in, i, h);
    }
}

// ---- queues in device memory (the stage-level entry points) ---------------

namespace detail {
template <class H, int (*Free)(H*)>
class DeviceHandle {
  public:
    DeviceHandle() = default;
    DeviceHandle(const DeviceHandle&) = delete;
    DeviceHandle& operator=(const DeviceHandle&) = delete;
    DeviceHandle(DeviceHandle&& o) noexcept : h_(std::exchange(o.h_, nullptr)), ctx_(o.ctx_) {}
    DeviceHandle& operator=(DeviceHandle&& o) noexcept
    {
        if (this != &o) {
            if (h_) Free(h_);
            h_ = std::exchange(o.h_, nullptr);
            ctx_ = o.ctx_;
        }
        return *this;
    }
    ~DeviceHandle()
    {
        if (h_) Free(h_);
    }
    H* handle() const { return h_; }

  protected:
    H* h_ = nullptr;
    wf_ctx* ctx_ = nullptr;
};
}  // namespace detail

// RayQueue kept on the GPU: schedule / materialize run there; upload and
// download move it to and from the host mirror above.
class DeviceRayQueue : public detail::DeviceHandle<wf_ray_queue, wf_ray_queue_free> {
  public:
    DeviceRayQueue(Context& ctx, int64_t capacity)
    {
        ctx_ = ctx.handle();
        check(wf_ray_queue_alloc(ctx_, capacity, &h_), ctx_, "wf_ray_queue_alloc");
    }
    int64_t size() const
    {
        int64_t n = 0;
        check(wf_ray_queue_size(h_, &n), ctx_, "wf_ray_queue_size");
        return n;
    }
    // RayQueue::schedule (sortedIndices stay on the device; `sorted` gets a copy if given)
    void schedule(const float sceneMin[3], const float sceneMax[3], std::vector<int>* sorted = nullptr)
    {
        if (sorted) sorted->assign((size_t)size(), 0);
        check(wf_ray_queue_schedule(h_, sceneMin, sceneMax, sorted ? sorted->data() : nullptr), ctx_,
              "wf_ray_queue_schedule");
    }
    void materialize() { check(wf_ray_queue_materialize(h_), ctx_, "wf_ray_queue_materialize"); }
    void upload(const RayQueue& q)
    {
        wf_ray_columns c{const_cast<float*>(q.originsX.data()), const_cast<float*>(q.originsY.data()),
                         const_cast<float*>(q.originsZ.data()), const_cast<float*>(q.dirsX.data()),
                         const_cast<float*>(q.dirsY.data()), const_cast<float*>(q.dirsZ.data()),
                         const_cast<float*>(q.throughputsR.data()), const_cast<float*>(q.throughputsG.data()),
                         const_cast<float*>(q.throughputsB.data()), const_cast<float*>(q.pdfs.data()),
                         const_cast<int*>(q.pixelIndices.data()), const_cast<int*>(q.depths.data()), nullptr};
        check(wf_ray_queue_upload(h_, &c, q.size()), ctx_, "wf_ray_queue_upload");
    }
    RayQueue download() const
    {
        const int64_t n = size();
        RayQueue q;
        for (auto* v : {&q.originsX, &q.originsY, &q.originsZ, &q.dirsX, &q.dirsY, &q.dirsZ, &q.throughputsR,
                        &q.throughputsG, &q.throughputsB, &q.pdfs, &q.accumLightR, &q.accumLightG, &q.accumLightB})
            v->assign((size_t)n, 0.0f);
        q.pixelIndices.assign((size_t)n, 0);
        q.depths.assign((size_t)n, 0);
        q.alive.assign((size_t)n, true);
        wf_ray_columns c{q.originsX.data(), q.originsY.data(), q.originsZ.data(), q.dirsX.data(), q.dirsY.data(),
                         q.dirsZ.data(), q.throughputsR.data(), q.throughputsG.data(), q.throughputsB.data(),
                         q.pdfs.data(), q.pixelIndices.data(), q.depths.data(), nullptr};
        int64_t got = 0;
        check(wf_ray_queue_download(h_, &c, n, &got), ctx_, "wf_ray_queue_download");
        return q;
    }
};

// ShadingQueue kept on the GPU (its entries index the ray queue they were
// intersected from, which must stay unchanged until they are shaded).
class DeviceShadingQueue : public detail::DeviceHandle<wf_shading_queue, wf_shading_queue_free> {
  public:
    DeviceShadingQueue(Context& ctx, int64_t capacity, SchedulingPolicy p = SchedulingPolicy::None) : policy(p)
    {
        ctx_ = ctx.handle();
        check(wf_shading_queue_alloc(ctx_, capacity, &h_), ctx_, "wf_shading_queue_alloc");
    }
    int64_t size() const
    {
        int64_t n = 0;
        check(wf_shading_queue_size(h_, &n), ctx_, "wf_shading_queue_size");
        return n;
    }
    // ShadingQueue::schedule with frozen relative costs (null = no tracker)
    void schedule(const std::vector<double>* relCostMaterial = nullptr,
                  const std::vector<double>* relCostTexture = nullptr, std::vector<int>* sorted = nullptr)
    {
        if (sorted) sorted->assign((size_t)size(), 0);
        check(wf_shading_queue_schedule(h_, (int32_t)policy, relCostMaterial ? relCostMaterial->data() : nullptr,
                                        relCostTexture ? relCostTexture->data() : nullptr,
                                        sorted ? sorted->data() : nullptr),
              ctx_, "wf_shading_queue_schedule");
    }
    void materialize() { check(wf_shading_queue_materialize(h_), ctx_, "wf_shading_queue_materialize"); }
    SchedulingPolicy policy;
};

class DeviceShadowQueue : public detail::DeviceHandle<wf_shadow_queue, wf_shadow_queue_free> {
  public:
    DeviceShadowQueue(Context& ctx, int64_t capacity)
    {
        ctx_ = ctx.handle();
        check(wf_shadow_queue_alloc(ctx_, capacity, &h_), ctx_, "wf_shadow_queue_alloc");
    }
};

// include/render/WavefrontRenderer.h:16-56, with the reference's defaults:
// adaptive sampling on (threshold 0.05), cost-aware RR on with costs from the
// live device CostTracker, ray sort on.  Frozen relative costs (for
// reproducible runs) replace the live tracker when given.  envNEE is a
// device addition (environment next-event estimation, same mean).
class WavefrontRenderer {
  public:
    int samplesPerPixel;
    int maxDepth;
    int rrMinDepth = 3;
    SchedulingPolicy policy;
    bool enableCostAwareRR = true;
    bool enableRaySort = true;
    bool enableAdaptiveSampling = true;
    float adaptiveSamplingThreshold = 0.05f;
    float fireflyThreshold = 10.0f;
    bool envNEE = false;
    uint64_t seed = 1;
    std::vector<double> relativeCostMaterial;  // frozen CostTracker::relativeCost; empty = live tracker
    std::vector<double> relativeCostTexture;
    wf_render_stats lastStats{};

    WavefrontRenderer(int samples, int maxDepth, SchedulingPolicy policy, int rrMinDepth_ = 3)
        : samplesPerPixel(samples), maxDepth(maxDepth), rrMinDepth(rrMinDepth_), policy(policy)
    {
    }

    // renderScene: writes the averaged image (width*height*3 floats; with
    // adaptive sampling each pixel over its own sample count) and returns
    // the total shade milliseconds, as the reference does.
    double renderScene(Context& ctx, const wf_camera& camera, int width, int height, std::vector<float>& pixels)
    {
        wf_render_params p{};
        p.width = width;
        p.height = height;
        p.samples_per_pixel = samplesPerPixel;
        p.max_depth = maxDepth;
        p.rr_min_depth = rrMinDepth;
        p.policy = (int32_t)policy;
        p.enable_ray_sort = enableRaySort ? 1 : 0;
        p.enable_cost_aware_rr = enableCostAwareRR ? 1 : 0;
        p.firefly_threshold = fireflyThreshold;
        p.seed_lo = (uint32_t)seed;
        p.seed_hi = (uint32_t)(seed >> 32);
        p.enable_env_nee = envNEE ? 1 : 0;
        p.enable_adaptive_sampling = enableAdaptiveSampling ? 1 : 0;
        p.adaptive_threshold = adaptiveSamplingThreshold;
        const bool frozen = !relativeCostMaterial.empty() || !relativeCostTexture.empty();
        p.enable_cost_tracking = frozen ? 0 : 1;
        p.rel_cost_material = relativeCostMaterial.empty() ? nullptr : relativeCostMaterial.data();
        p.rel_cost_texture = relativeCostTexture.empty() ? nullptr : relativeCostTexture.data();
        p.camera = camera;
        pixels.assign((size_t)width * height * 3, 0.0f);
        check(wf_render(ctx.handle(), &p, pixels.data(), &lastStats), ctx.handle(), "wf_render");
        return lastStats.ms_shade;
    }

    // renderScene's loop (WavefrontRenderer.cpp:141-268) written out stage by
    // stage over queues that stay on the GPU, in the reference's order: one
    // sample of every pixel per pass; per bounce the optional ray sort,
    // intersectAll, the ShadingQueue's schedule + materialize, shadeAll with
    // its occluded() calls, the miss loop, currentQueue = nextQueue.  With
    // the same parameters it renders renderScene's image (adaptive sampling
    // and the live cost tracker are renderScene's; here frozen relative costs
    // or none).  sceneMin / sceneMax: the scene bounds the ray sort uses.
    double renderSceneStaged(Context& ctx, const wf_camera& camera, int width, int height, std::vector<float>& pixels,
                             const float sceneMin[3], const float sceneMax[3])
    {
        wf_render_params p{};
        p.width = width;
        p.height = height;
        p.samples_per_pixel = samplesPerPixel;
        p.max_depth = maxDepth;
        p.rr_min_depth = rrMinDepth;
        p.policy = (int32_t)policy;
        p.enable_cost_aware_rr = enableCostAwareRR && !relativeCostMaterial.empty() ? 1 : 0;
        p.firefly_threshold = fireflyThreshold;
        p.seed_lo = (uint32_t)seed;
        p.seed_hi = (uint32_t)(seed >> 32);
        p.enable_env_nee = envNEE ? 1 : 0;
        p.rel_cost_material = relativeCostMaterial.empty() ? nullptr : relativeCostMaterial.data();
        p.rel_cost_texture = relativeCostTexture.empty() ? nullptr : relativeCostTexture.data();
        p.camera = camera;
        wf_ctx* h = ctx.handle();
        check(wf_stage_begin(h, &p), h, "wf_stage_begin");
        const int64_t n = (int64_t)width * height;
        DeviceRayQueue current(ctx, n), next(ctx, n), misses(ctx, n);
        DeviceShadingQueue hits(ctx, n, policy);
        DeviceShadowQueue shadows(ctx, 3 * n);
        const std::vector<double>* rcm = relativeCostMaterial.empty() ? nullptr : &relativeCostMaterial;
        const std::vector<double>* rct = relativeCostTexture.empty() ? nullptr : &relativeCostTexture;
        for (int sample = 0; sample < samplesPerPixel; ++sample) {
            check(wf_generate_primary(h, sample, 1, current.handle()), h, "wf_generate_primary");
            for (int depth = 0; depth < maxDepth && current.size() > 0; ++depth) {
                if (enableRaySort) {
                    current.schedule(sceneMin, sceneMax);
                    current.materialize();
                }
                check(wf_intersect(h, current.handle(), hits.handle(), misses.handle()), h, "wf_intersect");
                hits.schedule(rcm, rct);
                hits.materialize();
                check(wf_shade(h, hits.handle(), next.handle(), shadows.handle()), h, "wf_shade");
                check(wf_trace_occluded(h, shadows.handle()), h, "wf_trace_occluded");
                check(wf_miss(h, misses.handle()), h, "wf_miss");
                std::swap(current, next);
            }
        }
        pixels.assign((size_t)n * 3, 0.0f);
        check(wf_stage_image(h, pixels.data(), (int64_t)pixels.size()), h, "wf_stage_image");
        return 0.0;
    }

    // AdaptiveSampler::getSampleCount of every pixel of the last render.
    std::vector<int32_t> sampleCounts(Context& ctx, int width, int height) const
    {
        std::vector<int32_t> n((size_t)width * height);
        check(wf_adaptive_sample_counts(ctx.handle(), n.data(), (int64_t)n.size()), ctx.handle(),
              "wf_adaptive_sample_counts");
        return n;
    }
};

}  // namespace wf
