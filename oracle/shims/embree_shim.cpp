// CPU stand-in for EmbreeAccelerator (see shims/accelerator/Embree.h).
#include <accelerator/Embree.h>
#include <core/Scene.h>
#include <geometry/Mesh.h>
#include <geometry/Triangle.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <numeric>

EmbreeAccelerator::EmbreeAccelerator() = default;
EmbreeAccelerator::~EmbreeAccelerator() = default;
EmbreeAccelerator::EmbreeAccelerator(EmbreeAccelerator&& o) noexcept { *this = std::move(o); }
EmbreeAccelerator& EmbreeAccelerator::operator=(EmbreeAccelerator&& o) noexcept
{
    if (this != &o) {
        m_sourceScene = o.m_sourceScene;
        m_built = o.m_built;
        m_meshCount = o.m_meshCount;
        m_totalTriangles = o.m_totalTriangles;
        m_totalVertices = o.m_totalVertices;
        m_buildTimeMs = o.m_buildTimeMs;
        m_nodes = std::move(o.m_nodes);
        m_tris = std::move(o.m_tris);
        o.m_sourceScene = nullptr;
        o.m_built = false;
    }
    return *this;
}

namespace {
struct Box
{
    float lo[3], hi[3];
};
}  // namespace

void EmbreeAccelerator::build(const Scene& scene)
{
    auto t0 = std::chrono::high_resolution_clock::now();
    m_sourceScene = &scene;
    m_tris.clear();
    m_nodes.clear();
    m_meshCount = 0;
    m_totalTriangles = 0;
    m_totalVertices = 0;
    int global = 0;
    for (int m = 0; m < (int)scene.meshes.size(); ++m) {
        const Mesh& mesh = scene.meshes[m];
        for (int t = 0; t < mesh.triangleCount(); ++t) m_tris.push_back({m, t, global++});
        m_meshCount++;
        m_totalTriangles += mesh.triangleCount();
        m_totalVertices += (int)mesh.vertexPositions.size();
    }
    const int n = (int)m_tris.size();
    std::vector<Box> boxes(n);
    std::vector<float> cen(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        const Mesh& mesh = scene.meshes[m_tris[i].mesh];
        const Point3* v[3];
        for (int k = 0; k < 3; ++k) v[k] = &mesh.vertexPositions[mesh.triangleIndices[3 * m_tris[i].prim + k]];
        for (int a = 0; a < 3; ++a) {
            float c0 = a == 0 ? v[0]->x : a == 1 ? v[0]->y : v[0]->z;
            float c1 = a == 0 ? v[1]->x : a == 1 ? v[1]->y : v[1]->z;
            float c2 = a == 0 ? v[2]->x : a == 1 ? v[2]->y : v[2]->z;
            boxes[i].lo[a] = std::min({c0, c1, c2});
            boxes[i].hi[a] = std::max({c0, c1, c2});
            cen[3 * (size_t)i + a] = 0.5f * (boxes[i].lo[a] + boxes[i].hi[a]);
        }
    }
    if (n > 0) {
        std::vector<int> order(n);
        std::iota(order.begin(), order.end(), 0);
        struct Job
        {
            int node, first, count;
        };
        std::vector<Job> stack{{0, 0, n}};
        m_nodes.push_back(Node{});
        while (!stack.empty()) {
            Job j = stack.back();
            stack.pop_back();
            Box b{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
            float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int i = j.first; i < j.first + j.count; ++i)
                for (int a = 0; a < 3; ++a) {
                    b.lo[a] = std::min(b.lo[a], boxes[order[i]].lo[a]);
                    b.hi[a] = std::max(b.hi[a], boxes[order[i]].hi[a]);
                    clo[a] = std::min(clo[a], cen[3 * (size_t)order[i] + a]);
                    chi[a] = std::max(chi[a], cen[3 * (size_t)order[i] + a]);
                }
            Node& nd = m_nodes[j.node];
            for (int a = 0; a < 3; ++a) {
                float pad = std::max(std::fabs(b.lo[a]), std::fabs(b.hi[a])) * 1e-5f + 1e-6f;
                nd.lo[a] = b.lo[a] - pad;
                nd.hi[a] = b.hi[a] + pad;
            }
            if (j.count <= 4) {
                nd.first = j.first;
                nd.count = j.count;
                continue;
            }
            int axis = 0;
            for (int a = 1; a < 3; ++a)
                if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
            int mid = j.first + j.count / 2;
            std::nth_element(order.begin() + j.first, order.begin() + mid, order.begin() + j.first + j.count,
                             [&](int x, int y) {
                                 float cx = cen[3 * (size_t)x + axis], cy = cen[3 * (size_t)y + axis];
                                 return cx < cy || (cx == cy && x < y);
                             });
            int left = (int)m_nodes.size();
            m_nodes.push_back(Node{});
            m_nodes.push_back(Node{});
            m_nodes[j.node].left = left;
            m_nodes[j.node].right = left + 1;
            stack.push_back({left, j.first, mid - j.first});
            stack.push_back({left + 1, mid, j.first + j.count - mid});
        }
        std::vector<Tri> reordered(n);
        for (int i = 0; i < n; ++i) reordered[i] = m_tris[order[i]];
        m_tris.swap(reordered);
    }
    m_built = true;
    auto t1 = std::chrono::high_resolution_clock::now();
    m_buildTimeMs = std::chrono::duration<double, std::milli>(t1 - t0).count();
}

namespace {
inline bool slab(const EmbreeAccelerator::Node& nd, const Ray& r, const float inv[3], float tmin, float tmax)
{
    const float o[3] = {r.origin.x, r.origin.y, r.origin.z};
    float a = tmin, b = tmax;
    for (int k = 0; k < 3; ++k) {
        float t0 = (nd.lo[k] - o[k]) * inv[k], t1 = (nd.hi[k] - o[k]) * inv[k];
        a = std::max(a, std::min(t0, t1));
        b = std::min(b, std::max(t0, t1));
    }
    return a <= b;
}
inline float inv_of(float d)
{
    if (std::fabs(d) < 1e-20f) d = std::copysign(1e-20f, d);
    return 1.0f / d;
}
}  // namespace

EmbreeAccelerator::Closest EmbreeAccelerator::closest(const Ray& ray, float tmin, float tmax) const
{
    Closest best;
    if (m_nodes.empty()) return best;
    float inv[3] = {inv_of(ray.direction.x), inv_of(ray.direction.y), inv_of(ray.direction.z)};
    float best_t = tmax;
    int best_global = -1;
    std::vector<int> stack{0};
    while (!stack.empty()) {
        const Node& nd = m_nodes[stack.back()];
        stack.pop_back();
        if (!slab(nd, ray, inv, tmin, best_t)) continue;
        if (nd.count == 0) {
            stack.push_back(nd.left);
            stack.push_back(nd.right);
            continue;
        }
        for (int i = nd.first; i < nd.first + nd.count; ++i) {
            const Tri& tr = m_tris[i];
            const Mesh& mesh = m_sourceScene->meshes[tr.mesh];
            const Point3& v0 = mesh.vertexPositions[mesh.triangleIndices[3 * tr.prim + 0]];
            const Point3& v1 = mesh.vertexPositions[mesh.triangleIndices[3 * tr.prim + 1]];
            const Point3& v2 = mesh.vertexPositions[mesh.triangleIndices[3 * tr.prim + 2]];
            float t, u, v;
            if (intersectTriangle(ray, v0, v1, v2, tmin, best_t, t, u, v)) {
                if (t < best_t || best.tri < 0 || tr.global > best_global) {
                    best.tri = i;
                    best.t = t;
                    best.u = u;
                    best.v = v;
                    best_t = t;
                    best_global = tr.global;
                }
            }
        }
    }
    return best;
}

// HitRecord mapping of EmbreeAccelerator::intersect (reference Embree.cpp:153-176).
void EmbreeAccelerator::fill(const Ray& ray, const Closest& c, HitRecord& record) const
{
    const Tri& tr = m_tris[c.tri];
    const Mesh& mesh = m_sourceScene->meshes[tr.mesh];
    const Point3& v0 = mesh.vertexPositions[mesh.triangleIndices[3 * tr.prim + 0]];
    const Point3& v1 = mesh.vertexPositions[mesh.triangleIndices[3 * tr.prim + 1]];
    const Point3& v2 = mesh.vertexPositions[mesh.triangleIndices[3 * tr.prim + 2]];
    record.distance = c.t;
    record.point = ray.at(c.t);
    record.materialID = mesh.materialID;
    record.triangleIndex = tr.prim;
    mesh.interpolateUV(tr.prim, c.u, c.v, record.u, record.v);
    Vec3 edge1 = v1 - v0;
    Vec3 edge2 = v2 - v0;
    record.setFaceNormal(ray, edge1.cross(edge2).normalized());
}

bool EmbreeAccelerator::intersect(const Ray& ray, float minDistance, float maxDistance, HitRecord& record) const
{
    Closest c = closest(ray, minDistance, maxDistance);
    if (c.tri < 0) return false;
    fill(ray, c, record);
    return true;
}

// intersect4 (reference Embree.cpp:180-256): tnear 0.001, tfar 1e9, and the
// material's textureID on every hit.
int EmbreeAccelerator::intersect4(const RayQueue& queue, int startIndex, int count, HitRecord* hitRecords) const
{
    int mask = 0;
    for (int i = 0; i < count; ++i) {
        Ray ray = queue.getRay(startIndex + i);
        Closest c = closest(ray, 0.001f, 1e9f);
        if (c.tri < 0) continue;
        mask |= 1 << i;
        fill(ray, c, hitRecords[i]);
        hitRecords[i].textureID = m_sourceScene->materials[hitRecords[i].materialID].textureID;
    }
    return mask;
}

bool EmbreeAccelerator::occluded(const Point3& origin, const Vec3& direction, float maxDistance) const
{
    if (m_nodes.empty()) return false;
    Ray ray(origin, direction);
    const float tmin = 0.001f, tmax = maxDistance - 0.001f;
    float inv[3] = {inv_of(direction.x), inv_of(direction.y), inv_of(direction.z)};
    std::vector<int> stack{0};
    while (!stack.empty()) {
        const Node& nd = m_nodes[stack.back()];
        stack.pop_back();
        if (!slab(nd, ray, inv, tmin, tmax)) continue;
        if (nd.count == 0) {
            stack.push_back(nd.left);
            stack.push_back(nd.right);
            continue;
        }
        for (int i = nd.first; i < nd.first + nd.count; ++i) {
            const Tri& tr = m_tris[i];
            const Mesh& mesh = m_sourceScene->meshes[tr.mesh];
            float t, u, v;
            if (intersectTriangle(ray, mesh.vertexPositions[mesh.triangleIndices[3 * tr.prim + 0]],
                                  mesh.vertexPositions[mesh.triangleIndices[3 * tr.prim + 1]],
                                  mesh.vertexPositions[mesh.triangleIndices[3 * tr.prim + 2]], tmin, tmax, t, u, v))
                return true;
        }
    }
    return false;
}

// frontFace of a HitRecord rebuilt by ShadingQueue::getHitRecord (see
// shims/core/HitRecord.h).  The record keeps its material, its triangle index
// within the mesh and the face-forwarded geometric normal that fill()
// computed; the meshes with that material that own such a triangle are the
// candidates, and the one whose outward normal equals the record's normal
// (frontFace true) or its negation (false) answers.  Candidates that agree
// need no further test; if they disagree, the triangle whose plane holds the
// hit point decides.
namespace wfshim {
namespace {
std::atomic<const Scene*> g_render_scene{nullptr};
std::vector<std::vector<int>> g_meshes_of_material;
std::atomic<long long> g_unresolved{0}, g_ambiguous{0};

inline bool same(const Vec3& a, const Vec3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
}  // namespace

void set_render_scene(const Scene* scene)
{
    g_meshes_of_material.clear();
    if (scene) {
        g_meshes_of_material.resize(scene->materials.size());
        for (int m = 0; m < (int)scene->meshes.size(); ++m) {
            int mat = scene->meshes[m].materialID;
            if (mat >= 0 && mat < (int)g_meshes_of_material.size()) g_meshes_of_material[mat].push_back(m);
        }
    }
    g_unresolved = 0;
    g_ambiguous = 0;
    g_render_scene = scene;
}

long long front_face_unresolved() { return g_unresolved.load(); }
long long front_face_ambiguous() { return g_ambiguous.load(); }

bool rebuilt_front_face(const HitRecord& r)
{
    const Scene* s = g_render_scene.load();
    if (!s || r.materialID < 0 || r.materialID >= (int)g_meshes_of_material.size()) {
        ++g_unresolved;
        return true;
    }
    int yes = 0, no = 0;
    bool best_answer = true;
    float best_dist = INFINITY;
    for (int m : g_meshes_of_material[r.materialID]) {
        const Mesh& mesh = s->meshes[m];
        if (r.triangleIndex < 0 || r.triangleIndex >= mesh.triangleCount()) continue;
        const Point3& v0 = mesh.vertexPositions[mesh.triangleIndices[3 * r.triangleIndex + 0]];
        const Point3& v1 = mesh.vertexPositions[mesh.triangleIndices[3 * r.triangleIndex + 1]];
        const Point3& v2 = mesh.vertexPositions[mesh.triangleIndices[3 * r.triangleIndex + 2]];
        Vec3 edge1 = v1 - v0;
        Vec3 edge2 = v2 - v0;
        Vec3 outward = edge1.cross(edge2).normalized();
        bool answer;
        if (same(r.normal, outward))
            answer = true;
        else if (same(r.normal, outward * -1.0f))
            answer = false;
        else
            continue;
        (answer ? yes : no)++;
        float dist = std::fabs((r.point - v0).dot(outward));
        if (dist < best_dist) {
            best_dist = dist;
            best_answer = answer;
        }
    }
    if (yes + no == 0) {
        ++g_unresolved;
        return true;
    }
    if (yes && no) ++g_ambiguous;
    return yes && !no ? true : (no && !yes ? false : best_answer);
}
}  // namespace wfshim
