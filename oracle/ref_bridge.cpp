// ref_bridge.cpp — C entry points over the reference's own C++ sources
// (compiled in place with the shims of oracle/shims), used by tests/ in the
// development container to pin the oracle port and to make golden fixtures.
// TEST INFRASTRUCTURE ONLY; built into oracle/_ref/libwfref.so by
// oracle/Makefile, never shipped or called by the product.
#include <core/Camera.h>
#include <core/Image.h>
#include <core/Scene.h>
#include <geometry/Mesh.h>
#include <geometry/Triangle.h>
#include <math/Random.h>
#include <render/CostTracker.h>
#include <render/WavefrontRenderer.h>
#include <scheduling/RayQueue.h>
#include <scheduling/ShadingQueue.h>

#include <csignal>
#include <iostream>
#include <sstream>

#include "../include/wf_api.h"

namespace {

Material to_material(const wf_material& m)
{
    Material r;
    r.type = (MaterialType)m.type;
    r.albedo = Color(m.albedo[0], m.albedo[1], m.albedo[2]);
    r.roughness = m.roughness;
    r.emission = m.emission;
    r.textureID = m.texture_id;
    r.spotOuterAngle = m.spot_outer_deg;
    r.spotFalloffAngle = m.spot_falloff_deg;
    r.indexOfRefraction = m.ior;
    r.useSpatialChecker = m.use_spatial_checker != 0;
    r.spatialCheckerCellSize = m.checker_cell_size;
    return r;
}

float srgb_to_linear(float s)
{
    if (s <= 0.04045f) return s / 12.92f;
    return std::pow((s + 0.055f) / 1.055f, 2.4f);
}

struct Silence {
    std::stringstream sink;
    std::streambuf* old;
    Silence() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~Silence() { std::cout.rdbuf(old); }
};

}  // namespace

extern "C" {

void ref_set_seed(unsigned long long seed) { wfshim::set_seed(seed); }
void ref_set_threads(int n) { wfshim::set_num_workers(n); }

// Scene from the flat description: one reference Mesh per mesh, vertices
// copied from the global arrays (Scene::addMesh rebuilds the flat arrays).
void* ref_scene_create(const wf_scene_desc* d, int build_accelerator)
{
    Scene* s = new Scene();
    for (int m = 0; m < d->num_materials; ++m) s->addMaterial(to_material(d->materials[m]));
    for (int t = 0; t < d->num_textures; ++t) {
        const wf_texture& x = d->textures[t];
        Texture tex(x.width, x.height);
        for (int i = 0; i < x.width * x.height; ++i) {
            if (x.format == WF_TEXEL_RGB32F) {
                const float* f = (const float*)x.data;
                tex.pixels[i] = Color(f[3 * i], f[3 * i + 1], f[3 * i + 2]);
            } else {
                const uint8_t* b = (const uint8_t*)x.data;
                tex.pixels[i] = Color(srgb_to_linear(b[4 * i] / 255.0f), srgb_to_linear(b[4 * i + 1] / 255.0f),
                                      srgb_to_linear(b[4 * i + 2] / 255.0f));
            }
        }
        s->addTexture(tex);
    }
    for (int m = 0; m < d->num_meshes; ++m) {
        Mesh mesh;
        mesh.materialID = d->mesh_material_ids[m];
        std::vector<int> local(d->num_vertices, -1);
        const int off = d->mesh_index_offsets[m], cnt = d->mesh_index_counts[m];
        for (int i = off; i < off + cnt; ++i) {
            int g = d->indices[i];
            if (local[g] < 0) {
                local[g] = (int)mesh.vertexPositions.size();
                mesh.vertexPositions.push_back(Point3(d->positions_x[g], d->positions_y[g], d->positions_z[g]));
            }
            mesh.triangleIndices.push_back(local[g]);
            if (d->mesh_has_uv && d->mesh_has_uv[m] && d->corner_u) {
                mesh.triangleUVsU.push_back(d->corner_u[i]);
                mesh.triangleUVsV.push_back(d->corner_v[i]);
            }
        }
        s->addMesh(mesh);
    }
    s->directionalLight.direction = Vec3(d->directional.direction[0], d->directional.direction[1], d->directional.direction[2]);
    s->directionalLight.color = Color(d->directional.color[0], d->directional.color[1], d->directional.color[2]);
    s->directionalLight.intensity = d->directional.intensity;
    Silence q;
    if (build_accelerator) {
        s->buildAccelerator();
    } else {
        // the parts of buildAccelerator that do not touch the accelerator
        for (int i = 0; i < (int)s->meshes.size(); ++i) {
            MaterialType t = s->materials[s->meshes[i].materialID].type;
            if (t == MaterialType::Emissive || t == MaterialType::SpotLight) s->emissiveMeshIndices.push_back(i);
        }
        s->totalEmissiveArea();
        s->computeBounds();
    }
    return s;
}

void ref_scene_destroy(void* s) { delete (Scene*)s; }

void ref_scene_bounds(void* sp, float bmin[3], float bmax[3])
{
    Scene* s = (Scene*)sp;
    bmin[0] = s->boundsMin.x; bmin[1] = s->boundsMin.y; bmin[2] = s->boundsMin.z;
    bmax[0] = s->boundsMax.x; bmax[1] = s->boundsMax.y; bmax[2] = s->boundsMax.z;
}

float ref_scene_total_emissive_area(void* s) { return ((Scene*)s)->totalEmissiveArea(); }

// Camera::Camera -> its four public fields (12 floats).
void ref_camera(const float f[3], const float a[3], const float u[3], float vfov, int w, int h, float out[12])
{
    Camera c(Point3(f[0], f[1], f[2]), Point3(a[0], a[1], a[2]), Vec3(u[0], u[1], u[2]), vfov, w, h);
    const Vec3* v[4] = {&c.origin, &c.topLeftCorner, &c.horizontal, &c.vertical};
    for (int k = 0; k < 4; ++k) {
        out[3 * k] = v[k]->x;
        out[3 * k + 1] = v[k]->y;
        out[3 * k + 2] = v[k]->z;
    }
}

static Camera camera_from12(const float c12[12])
{
    Camera c(Point3(0, 0, 1), Point3(0, 0, 0), Vec3(0, 1, 0), 40.0f, 2, 2);
    c.origin = Point3(c12[0], c12[1], c12[2]);
    c.topLeftCorner = Point3(c12[3], c12[4], c12[5]);
    c.horizontal = Vec3(c12[6], c12[7], c12[8]);
    c.vertical = Vec3(c12[9], c12[10], c12[11]);
    return c;
}

void ref_camera_get_ray(const float c12[12], float u, float v, float o[3], float d[3])
{
    Ray r = camera_from12(c12).getRay(u, v);
    o[0] = r.origin.x; o[1] = r.origin.y; o[2] = r.origin.z;
    d[0] = r.direction.x; d[1] = r.direction.y; d[2] = r.direction.z;
}

// HitRecord columns; mode 0 = Scene::hit (brute force when the accelerator
// is not built, else EmbreeAccelerator::intersect), mode 1 =
// EmbreeAccelerator::intersect4 over a RayQueue in packets of four.
void ref_trace(void* sp, int mode, long long n, const float* ox, const float* oy, const float* oz,
               const float* dx, const float* dy, const float* dz, float tmin, float tmax, wf_hit_columns* out)
{
    Scene* s = (Scene*)sp;
    auto put = [&](long long i, const HitRecord* r) {
        if (out->geom_id) out->geom_id[i] = r ? 0 : -1;  // the reference HitRecord has no geomID
        if (out->prim_id) out->prim_id[i] = r ? r->triangleIndex : -1;
        if (out->distance) out->distance[i] = r ? r->distance : 0.0f;
        if (out->point_x) out->point_x[i] = r ? r->point.x : 0.0f;
        if (out->point_y) out->point_y[i] = r ? r->point.y : 0.0f;
        if (out->point_z) out->point_z[i] = r ? r->point.z : 0.0f;
        if (out->normal_x) out->normal_x[i] = r ? r->normal.x : 0.0f;
        if (out->normal_y) out->normal_y[i] = r ? r->normal.y : 0.0f;
        if (out->normal_z) out->normal_z[i] = r ? r->normal.z : 0.0f;
        if (out->front_face) out->front_face[i] = r ? (uint8_t)r->frontFace : 0;
        if (out->u) out->u[i] = r ? r->u : 0.0f;
        if (out->v) out->v[i] = r ? r->v : 0.0f;
        if (out->material_id) out->material_id[i] = r ? r->materialID : -1;
        if (out->texture_id) out->texture_id[i] = r ? r->textureID : -1;
    };
    if (mode == 0) {
        for (long long i = 0; i < n; ++i) {
            HitRecord r;
            Ray ray(Point3(ox[i], oy[i], oz[i]), Vec3(dx[i], dy[i], dz[i]));
            put(i, s->hit(ray, tmin, tmax, r) ? &r : nullptr);
        }
        return;
    }
    RayQueue q;
    for (long long i = 0; i < n; ++i) q.addPrimary(Ray(Point3(ox[i], oy[i], oz[i]), Vec3(dx[i], dy[i], dz[i])), (int)i);
    for (long long i = 0; i < n; i += 4) {
        int cnt = (int)std::min<long long>(4, n - i);
        HitRecord rec[4];
        int mask = s->accelerator.intersect4(q, (int)i, cnt, rec);
        for (int j = 0; j < cnt; ++j) put(i + j, (mask & (1 << j)) ? &rec[j] : nullptr);
    }
}

void ref_occluded(void* sp, long long n, const float* ox, const float* oy, const float* oz, const float* dx,
                  const float* dy, const float* dz, const float* maxd, uint8_t* out)
{
    Scene* s = (Scene*)sp;
    for (long long i = 0; i < n; ++i)
        out[i] = s->accelerator.occluded(Point3(ox[i], oy[i], oz[i]), Vec3(dx[i], dy[i], dz[i]), maxd[i]) ? 1 : 0;
}

// intersectTriangle (include/geometry/Triangle.h) for one ray/triangle.
int ref_intersect_triangle(const float o[3], const float d[3], const float v0[3], const float v1[3],
                           const float v2[3], float tmin, float tmax, float out[3])
{
    Ray r(Point3(o[0], o[1], o[2]), Vec3(d[0], d[1], d[2]));
    float t = 0, u = 0, v = 0;
    bool hit = intersectTriangle(r, Point3(v0[0], v0[1], v0[2]), Point3(v1[0], v1[1], v1[2]),
                                 Point3(v2[0], v2[1], v2[2]), tmin, tmax, t, u, v);
    out[0] = t;
    out[1] = u;
    out[2] = v;
    return hit ? 1 : 0;
}

// RayQueue::schedule -> sortedIndices (and sortKey per ray).
void ref_ray_schedule(long long n, const float* ox, const float* oy, const float* oz, const float* dx,
                      const float* dy, const float* dz, const float bmin[3], const float bmax[3], int* sorted,
                      unsigned long long* keys)
{
    RayQueue q;
    for (long long i = 0; i < n; ++i) q.addPrimary(Ray(Point3(ox[i], oy[i], oz[i]), Vec3(dx[i], dy[i], dz[i])), (int)i);
    Point3 mn(bmin[0], bmin[1], bmin[2]), mx(bmax[0], bmax[1], bmax[2]);
    q.schedule(mn, mx);
    for (long long i = 0; i < n; ++i) {
        sorted[i] = q.sortedIndices[i];
        if (keys) keys[i] = q.sortKey((int)i, mn, mx);
    }
}

// CostTracker fed with (id, ns) samples in order.
static void feed(CostTracker& t, long long n, const int* ids, const double* ns)
{
    for (long long i = 0; i < n; ++i) t.record(ids[i], ns[i]);
}

void ref_cost_tracker_relative(int items, long long n, const int* ids, const double* ns, double* out)
{
    CostTracker t(items);
    feed(t, n, ids, ns);
    for (int i = 0; i < items; ++i) out[i] = t.relativeCost(i);
}

// ShadingQueue::schedule with trackers built from cost samples (a tracker
// with no samples is neutral, relativeCost 1).  textures: (width, height)
// pairs; only memoryBytes matters to the policies.
void ref_shading_schedule(int policy, long long n, const int* mat_ids, const int* tex_ids, const float* tr,
                          const float* tg, const float* tb, const float* px, const float* py, const float* pz,
                          int num_materials, const wf_material* mats, int num_textures, const int* tex_wh,
                          long long n_mat_samples, const int* mat_sample_ids, const double* mat_sample_ns,
                          long long n_tex_samples, const int* tex_sample_ids, const double* tex_sample_ns,
                          int use_trackers, int* sorted)
{
    std::vector<Material> materials;
    for (int m = 0; m < num_materials; ++m) materials.push_back(to_material(mats[m]));
    std::vector<Texture> textures;
    for (int t = 0; t < num_textures; ++t) textures.emplace_back(tex_wh[2 * t], tex_wh[2 * t + 1]);
    CostTracker mt(num_materials), tt(num_textures);
    feed(mt, n_mat_samples, mat_sample_ids, mat_sample_ns);
    feed(tt, n_tex_samples, tex_sample_ids, tex_sample_ns);
    ShadingQueue q((SchedulingPolicy)policy);
    RayQueue rays;
    for (long long i = 0; i < n; ++i)
        rays.add(Ray(Point3(0, 0, 0), Vec3(0, 0, -1)), Color(tr[i], tg[i], tb[i]), Color(0, 0, 0), (int)i, 0, true, -1.0f);
    for (long long i = 0; i < n; ++i) {
        HitRecord h;
        h.point = Point3(px[i], py[i], pz[i]);
        h.normal = Vec3(0, 1, 0);
        h.distance = 1.0f;
        h.materialID = mat_ids[i];
        h.textureID = tex_ids[i];
        h.triangleIndex = (int)i;
        h.u = 0;
        h.v = 0;
        h.frontFace = true;
        q.add(rays, (int)i, h);
    }
    if (use_trackers)
        q.schedule(materials, textures, &mt, &tt);
    else
        q.schedule(materials, textures);
    for (long long i = 0; i < n; ++i) sorted[i] = q.sortedIndices[i];
}

// WavefrontRenderer::renderScene with adaptive sampling and cost-aware RR
// off; writes the averaged image (width*height*3).  env_path (may be null)
// names a PFM the renderer loads as its environment map.
void ref_render(void* sp, const float c12[12], int w, int h, int spp, int max_depth, int policy, int ray_sort,
                float firefly, const char* env_path, float* image_out)
{
    Scene* s = (Scene*)sp;
    Camera cam = camera_from12(c12);
    Image img(w, h);
    WavefrontRenderer r(spp, max_depth, (SchedulingPolicy)policy);
    r.enableAdaptiveSampling = false;
    r.enableCostAwareRR = false;
    r.enableRaySort = ray_sort != 0;
    r.enableSampleLogging = true;
    r.fireflyThreshold = firefly;
    if (env_path) r.environmentMapPath = env_path;
    void (*old_term)(int) = std::signal(SIGTERM, SIG_DFL);
    void (*old_int)(int) = std::signal(SIGINT, SIG_DFL);
    wfshim::set_render_scene(s);
    {
        Silence q;
        r.renderScene(*s, cam, img);
    }
    std::signal(SIGTERM, old_term);
    std::signal(SIGINT, old_int);
    for (int i = 0; i < w * h; ++i) {
        image_out[3 * i] = img.pixels[i].x;
        image_out[3 * i + 1] = img.pixels[i].y;
        image_out[3 * i + 2] = img.pixels[i].z;
    }
}

// renderScene in the reference's default sampling mode: adaptive sampling
// on (threshold as given), cost-aware RR off, no ray sort.
void ref_render_adaptive(void* sp, const float c12[12], int w, int h, int spp, int max_depth, float threshold,
                         float* image_out)
{
    Scene* s = (Scene*)sp;
    Camera cam = camera_from12(c12);
    Image img(w, h);
    WavefrontRenderer r(spp, max_depth, SchedulingPolicy::None);
    r.enableAdaptiveSampling = true;
    r.adaptiveSamplingThreshold = threshold;
    r.enableCostAwareRR = false;
    r.enableRaySort = false;
    r.enableSampleLogging = true;
    void (*old_term)(int) = std::signal(SIGTERM, SIG_DFL);
    void (*old_int)(int) = std::signal(SIGINT, SIG_DFL);
    wfshim::set_render_scene(s);
    {
        Silence q;
        r.renderScene(*s, cam, img);
    }
    std::signal(SIGTERM, old_term);
    std::signal(SIGINT, old_int);
    for (int i = 0; i < w * h; ++i) {
        image_out[3 * i] = img.pixels[i].x;
        image_out[3 * i + 1] = img.pixels[i].y;
        image_out[3 * i + 2] = img.pixels[i].z;
    }
}

// Rebuilt hit records whose frontFace the shim could not resolve, and those
// settled by the hit point (shims/core/HitRecord.h), over the last render.
void ref_front_face_stats(long long* unresolved, long long* ambiguous)
{
    *unresolved = wfshim::front_face_unresolved();
    *ambiguous = wfshim::front_face_ambiguous();
}

}  // extern "C"
