// Shim for the reference's include/core/HitRecord.h (HitRecord.h:6-22): same
// members, names and setFaceNormal; only the type of `frontFace` differs.
//
// Why: ShadingQueue::getHitRecord (include/scheduling/ShadingQueue.h:144-158)
// rebuilds a HitRecord without assigning frontFace, which HitRecord.h:15
// leaves uninitialised, and Material::scatter's Glass branch
// (src/shading/Material.cpp:214-215) reads it.  The reference's glass
// therefore reads an indeterminate bool: its image moves with the worker
// count and the compiler.  Here frontFace is a flag that remembers whether it
// was assigned; a record rebuilt without it answers with the value
// setFaceNormal computed when the ray hit that triangle (the hit-time
// definition of src/accelerator/Embree.cpp:252), found from the record's
// material, triangle index, face-forwarded normal and point
// (wfshim::rebuilt_front_face, oracle/shims/embree_shim.cpp).  Every other
// member and every other material behaves exactly as in the reference.
#pragma once

#include <cstddef>

#include <core/Ray.h>
#include <math/Vec3.h>

struct HitRecord;

namespace wfshim {
bool rebuilt_front_face(const HitRecord& record);
}  // namespace wfshim

struct FrontFaceFlag
{
    signed char state = -1;  // -1: never assigned; else 0 / 1
    FrontFaceFlag& operator=(bool b)
    {
        state = b ? 1 : 0;
        return *this;
    }
    inline operator bool() const;
};

struct HitRecord
{
    Point3 point;
    Vec3 normal;
    float distance;
    int materialID = -1;
    int textureID = -1;
    int triangleIndex = -1;
    float u, v;
    FrontFaceFlag frontFace;

    void setFaceNormal(const Ray& ray, const Vec3& outwardNormal)
    {
        frontFace = ray.direction.dot(outwardNormal) < 0.0f;
        normal = frontFace ? outwardNormal : outwardNormal * -1.0f;
    }
};

inline FrontFaceFlag::operator bool() const
{
    if (state >= 0) return state != 0;
    const HitRecord* r =
        reinterpret_cast<const HitRecord*>(reinterpret_cast<const char*>(this) - offsetof(HitRecord, frontFace));
    return wfshim::rebuilt_front_face(*r);
}
