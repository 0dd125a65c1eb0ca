// Shim for the reference's include/accelerator/Embree.h: Embree 4 is not
// available, so EmbreeAccelerator keeps its public interface (Embree.h:10-41)
// but traces with a CPU BVH whose leaves call the reference's own
// intersectTriangle (include/geometry/Triangle.h).  Closest hits follow the
// brute-force order of Scene::hit (smallest t; on equal t the later mesh /
// triangle), and the HitRecord mapping is that of src/accelerator/Embree.cpp
// (intersect without textureID, intersect4 with it).
#pragma once

#include <vector>
#include <core/HitRecord.h>
#include <scheduling/RayQueue.h>

struct Scene;

namespace wfshim {
// The scene whose rebuilt hit records resolve frontFace (core/HitRecord.h shim);
// set by the bridge before WavefrontRenderer::renderScene.
void set_render_scene(const Scene* scene);
// Rebuilt records whose triangle could not be found (0 in a correct run), and
// those whose candidate triangles disagreed and were settled by the hit point.
long long front_face_unresolved();
long long front_face_ambiguous();
}  // namespace wfshim

class EmbreeAccelerator
{
  public:
    EmbreeAccelerator();
    ~EmbreeAccelerator();
    EmbreeAccelerator(const EmbreeAccelerator&) = delete;
    EmbreeAccelerator& operator=(const EmbreeAccelerator&) = delete;
    EmbreeAccelerator(EmbreeAccelerator&& other) noexcept;
    EmbreeAccelerator& operator=(EmbreeAccelerator&& other) noexcept;

    void build(const Scene& scene);
    int intersect4(const RayQueue& queue, int startIndex, int count, HitRecord* hitRecords) const;
    bool intersect(const Ray& ray, float minDistance, float maxDistance, HitRecord& record) const;
    bool occluded(const Point3& origin, const Vec3& direction, float maxDistance) const;

    const Scene* m_sourceScene = nullptr;
    bool m_built = false;
    int m_meshCount = 0;
    int m_totalTriangles = 0;
    int m_totalVertices = 0;
    double m_buildTimeMs = 0.0;

    struct Node
    {
        float lo[3], hi[3];
        int left = -1, right = -1, first = 0, count = 0;
    };
    struct Tri
    {
        int mesh, prim, global;
    };

  private:
    struct Closest
    {
        int tri = -1;
        float t = 0.0f, u = 0.0f, v = 0.0f;
    };
    Closest closest(const Ray& ray, float tmin, float tmax) const;
    void fill(const Ray& ray, const Closest& c, HitRecord& record) const;
    std::vector<Node> m_nodes;
    std::vector<Tri> m_tris;
};
