// C++ tests of the C++17 mirror (include/wf/wavefront.hpp) on the GPU, in the
// shape of the reference's GoogleTest cases (tests/scheduling/RayQueueTest.cpp,
// ShadingQueueTest.cpp, tests/render/WavefrontRendererTest.cpp).  Exit status
// 0 = all passed.  Built and run by tests/test_cpp_mirror.py.
#include <wf/wavefront.hpp>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

static int failures = 0;
#define EXPECT(c)                                                         \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);    \
            ++failures;                                                   \
        }                                                                 \
    } while (0)

static wf_material material(int type)
{
    wf_material m{};
    m.type = type;
    m.albedo[0] = m.albedo[1] = m.albedo[2] = 1.0f;
    m.roughness = 0.5f;
    m.emission = 1.0f;
    m.texture_id = -1;
    m.ior = 1.5f;
    m.spot_outer_deg = 45.0f;
    m.spot_falloff_deg = 30.0f;
    m.checker_cell_size = 1.0f;
    return m;
}

int main()
{
    wf::Context ctx(0);
    const float smin[3] = {-10, -10, -10}, smax[3] = {10, 10, 10};
    {  // RayQueueTest ScheduleOrdersRaysBySpatialProximityWithinSameOctant
        wf::RayQueue q;
        const float d[3] = {0, 0, 1};
        const float a[3] = {5, 0, 0}, b[3] = {-5, 0, 0}, c[3] = {0, 0, 0};
        q.addPrimary(a, d, 100);
        q.addPrimary(b, d, 200);
        q.addPrimary(c, d, 300);
        q.schedule(ctx, smin, smax);
        q.materialize();
        EXPECT(q.pixelIndices[0] == 200 && q.pixelIndices[1] == 300 && q.pixelIndices[2] == 100);
        EXPECT(q.sortedIndices[0] == 0 && q.sortedIndices[2] == 2);
    }
    {  // RayQueueTest ScheduleOnEmptyQueueDoesNotCrash
        wf::RayQueue q;
        q.schedule(ctx, smin, smax);
        EXPECT(q.size() == 0 && q.sortedIndices.empty());
    }
    std::vector<wf_material> mats;
    for (int t = 0; t < 6; ++t) mats.push_back(material(t));
    std::vector<int64_t> texBytes = {12, 48, 192};
    auto queueWith = [&](wf::SchedulingPolicy p, std::vector<int> mids, std::vector<int> tids = {}) {
        wf::RayQueue r;
        const float o[3] = {0, 0, 0}, d[3] = {0, 0, -1};
        for (size_t i = 0; i < mids.size(); ++i) r.addPrimary(o, d, (int)i);
        wf::ShadingQueue q(p);
        for (size_t i = 0; i < mids.size(); ++i) {
            wf::HitRecord h;
            h.materialID = mids[i];
            h.textureID = tids.empty() ? 0 : tids[i];
            h.distance = 1.0f;
            q.add(r, (int)i, h);
        }
        q.schedule(ctx, mats, texBytes);
        return q;
    };
    {  // ShadingQueueTest MaterialAwareSortsByMaterialIDAscending / GroupsSameMaterialTogether
        auto q = queueWith(wf::SchedulingPolicy::MaterialAware, {2, 0, 1});
        EXPECT(q.getHitRecord(0).materialID == 2 && q.getHitRecord(1).materialID == 1 && q.getHitRecord(2).materialID == 0);
        auto g = queueWith(wf::SchedulingPolicy::MaterialAware, {1, 0, 1, 0, 1});
        g.materialize();
        EXPECT(g.materialIDs == std::vector<int>({1, 1, 1, 0, 0}));
        auto n = queueWith(wf::SchedulingPolicy::None, {2, 0, 1});
        EXPECT(n.getHitRecord(0).materialID == 2 && n.getHitRecord(2).materialID == 1);
        auto t = queueWith(wf::SchedulingPolicy::TextureAware, {0, 1, 0}, {0, 2, 1});
        EXPECT(t.getHitRecord(0).textureID == 2 && t.getHitRecord(1).textureID == 1 && t.getHitRecord(2).textureID == 0);
    }
    {  // intersectAll + WavefrontRendererTest-style render of the Cornell box
        wf_host_scene* hs = nullptr;
        wf::check(wf_host_scene_generate(0, 1, &hs), nullptr, "generate");
        wf_scene_desc desc;
        wf_host_scene_describe(hs, &desc);
        ctx.upload(desc);
        wf_camera cam;
        wf_host_scene_camera(hs, 16, 16, &cam);
        wf::RayQueue prim;
        for (int y = 0; y < 16; ++y)
            for (int x = 0; x < 16; ++x) {
                float u = x / 15.0f, v = 1.0f - y / 15.0f, d[3];
                for (int k = 0; k < 3; ++k) d[k] = cam.top_left[k] + cam.horizontal[k] * u + cam.vertical[k] * v - cam.origin[k];
                float l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                for (float& c : d) c /= l;
                prim.addPrimary(cam.origin, d, y * 16 + x);
            }
        wf::ShadingQueue hits(wf::SchedulingPolicy::MaterialAware);
        wf::RayQueue misses;
        wf::intersectAll(ctx, prim, hits, misses);
        EXPECT(hits.size() + misses.size() == 256);
        EXPECT(hits.size() > 160);  // 195 of the 16x16 grid hit; the border looks past the room
        wf::WavefrontRenderer r(8, 8, wf::SchedulingPolicy::MaterialAware);
        std::vector<float> px;
        r.renderScene(ctx, cam, 16, 16, px);
        int black = 0;
        double mean = 0.0;
        bool finite = true;
        for (size_t i = 0; i < px.size(); i += 3) {
            if (px[i] == 0 && px[i + 1] == 0 && px[i + 2] == 0) ++black;
            mean += px[i];
            finite = finite && std::isfinite(px[i]) && px[i] >= 0;
        }
        EXPECT(black < 128);  // "fewer than half the pixels are black"
        EXPECT(finite);
        EXPECT(mean > 0);
        EXPECT(r.lastStats.closest_rays > 0);
        // the reference's defaults: adaptive sampling (no pixel stops before
        // 32 samples) and cost-aware RR fed by the live tracker
        const std::vector<int32_t> counts = r.sampleCounts(ctx, 16, 16);
        EXPECT(counts.size() == 256 && counts[0] == 8 && counts[255] == 8);
        // the same loop stage by stage on device-resident queues: renderScene's
        // image up to the order of float additions (1e-4 relative on 99% of
        // pixels), policy and ray sort included
        wf::WavefrontRenderer a(4, 8, wf::SchedulingPolicy::MaterialAware);
        a.enableAdaptiveSampling = false;
        a.enableCostAwareRR = false;
        a.relativeCostMaterial.assign((size_t)desc.num_materials, 1.0);
        a.relativeCostTexture.assign(1, 1.0);
        std::vector<float> whole, staged;
        a.renderScene(ctx, cam, 16, 16, whole);
        wf_scene_info info{};
        wf_scene_get_info(ctx.handle(), &info);
        a.renderSceneStaged(ctx, cam, 16, 16, staged, info.bounds_min, info.bounds_max);
        int close = 0;
        for (size_t i = 0; i < whole.size(); i += 3) {
            bool ok = true;
            for (int k = 0; k < 3; ++k)
                ok = ok && std::fabs(whole[i + k] - staged[i + k]) <= 1e-6f + 1e-4f * std::fabs(whole[i + k]);
            close += ok ? 1 : 0;
        }
        EXPECT(close >= 253);  // 99% of 256 pixels
        // RayQueue round trip through the device queue, schedule on the device
        wf::DeviceRayQueue dq(ctx, 256);
        dq.upload(prim);
        std::vector<int> sorted;
        dq.schedule(info.bounds_min, info.bounds_max, &sorted);
        wf::RayQueue hostSorted = prim;
        hostSorted.schedule(ctx, info.bounds_min, info.bounds_max);
        EXPECT(sorted == hostSorted.sortedIndices);
        dq.materialize();
        wf::RayQueue back = dq.download();
        hostSorted.materialize();
        EXPECT(back.pixelIndices == hostSorted.pixelIndices && back.dirsX == hostSorted.dirsX);
        wf_host_scene_free(hs);
    }
    std::printf("%s (%d failures)\n", failures ? "FAIL" : "OK", failures);
    return failures ? 1 : 0;
}
