// wf_traverse.cuh — BVH2 traversal (closest hit and any hit).
//
// Closest hit follows the brute-force semantics of the reference's
// Scene::hit / Mesh::hit (src/core/Scene.cpp:120-160, src/geometry/Mesh.cpp
// :9-44): among triangles accepted by Moller-Trumbore in [tmin, tmax] the
// smallest t wins, and on equal t the later triangle (larger global index,
// i.e. later mesh, then later primitive).  Because node boxes are padded and
// a node is entered when its entry distance is <= the current best t, the
// result does not depend on traversal order: the GPU and the CPU oracle
// return the same triangle and the same t bit for bit.
//
// Any hit (EmbreeAccelerator::occluded, src/accelerator/Embree.cpp:258-280)
// stops at the first accepted triangle.
#pragma once

#include "wf_device.cuh"

namespace wf {

struct TraceResult {
    int leafpos;  // -1 = miss
    float t, bu, bv;
};

// Slab test of both children of a node; FMA form t = lo*inv - o*inv (the
// padded boxes absorb the rounding difference).
__device__ __forceinline__ void slab2(const BvhNode& nd, V3 inv, V3 oi, float tmin, float tmax,
                                      float& tn0, float& tn1, bool& h0, bool& h1)
{
    float lx0 = __fmaf_rn(nd.c0xy.x, inv.x, -oi.x), hx0 = __fmaf_rn(nd.c0xy.y, inv.x, -oi.x);
    float ly0 = __fmaf_rn(nd.c0xy.z, inv.y, -oi.y), hy0 = __fmaf_rn(nd.c0xy.w, inv.y, -oi.y);
    float lz0 = __fmaf_rn(nd.cz.x, inv.z, -oi.z), hz0 = __fmaf_rn(nd.cz.y, inv.z, -oi.z);
    float lx1 = __fmaf_rn(nd.c1xy.x, inv.x, -oi.x), hx1 = __fmaf_rn(nd.c1xy.y, inv.x, -oi.x);
    float ly1 = __fmaf_rn(nd.c1xy.z, inv.y, -oi.y), hy1 = __fmaf_rn(nd.c1xy.w, inv.y, -oi.y);
    float lz1 = __fmaf_rn(nd.cz.z, inv.z, -oi.z), hz1 = __fmaf_rn(nd.cz.w, inv.z, -oi.z);
    tn0 = fmaxf(fmaxf(fminf(lx0, hx0), fminf(ly0, hy0)), fmaxf(fminf(lz0, hz0), tmin));
    float tf0 = fminf(fminf(fmaxf(lx0, hx0), fmaxf(ly0, hy0)), fminf(fmaxf(lz0, hz0), tmax));
    tn1 = fmaxf(fmaxf(fminf(lx1, hx1), fminf(ly1, hy1)), fmaxf(fminf(lz1, hz1), tmin));
    float tf1 = fminf(fminf(fmaxf(lx1, hx1), fmaxf(ly1, hy1)), fminf(fmaxf(lz1, hz1), tmax));
    h0 = tn0 <= tf0;
    h1 = tn1 <= tf1;
}

__device__ __forceinline__ BvhNode load_node(const BvhNode* nodes, uint32_t i)
{
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    BvhNode nd;
    nd.c0xy = __ldg(p + 0);
    nd.c1xy = __ldg(p + 1);
    nd.cz = __ldg(p + 2);
    float4 k = __ldg(p + 3);
    nd.kids = make_int4(__float_as_int(k.x), __float_as_int(k.y), 0, 0);
    return nd;
}

// Returns false (and sets *err_flag) only if the stack would overflow, which
// the build rules out by checking the tree depth.
template <bool kAnyHit>
__device__ __forceinline__ bool traverse(const DeviceScene& S, V3 o, V3 d, float tmin, float tmax,
                                         TraceResult& res, int* err_flag)
{
    res.leafpos = -1;
    if (S.root_is_empty) return true;
    V3 inv = {safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
    V3 oi = {o.x * inv.x, o.y * inv.y, o.z * inv.z};
    uint32_t stack[kStackSize];
    int sp = 0;
    uint32_t cur = 0;
    float best_t = tmax;
    int best_g = -1;
    for (;;) {
        if (!(cur & kLeafFlag)) {
            BvhNode nd = load_node(S.nodes, cur);
            float tn0, tn1;
            bool h0, h1;
            slab2(nd, inv, oi, tmin, best_t, tn0, tn1, h0, h1);
            uint32_t c0 = (uint32_t)nd.kids.x, c1 = (uint32_t)nd.kids.y;
            if (h0 && h1) {
                uint32_t nearc = c0, farc = c1;
                if (tn1 < tn0) {
                    nearc = c1;
                    farc = c0;
                }
                if (sp >= kStackSize) {
                    atomicOr(err_flag, 1);
                    return false;
                }
                stack[sp++] = farc;
                cur = nearc;
                continue;
            } else if (h0) {
                cur = c0;
                continue;
            } else if (h1) {
                cur = c1;
                continue;
            }
        } else {
            int first = (int)((cur & ~kLeafFlag) >> 3);
            int cnt = (int)(cur & 7u) + 1;
            for (int k = 0; k < cnt; ++k) {
                int lp = first + k;
                float4 a = __ldg(S.tris + 3 * lp + 0);
                float4 b = __ldg(S.tris + 3 * lp + 1);
                float4 c = __ldg(S.tris + 3 * lp + 2);
                float th, uh, vh;
                if (intersect_triangle(o, d, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z),
                                       tmin, best_t, th, uh, vh)) {
                    if (kAnyHit) {
                        res.leafpos = lp;
                        res.t = th;
                        res.bu = uh;
                        res.bv = vh;
                        return true;
                    }
                    int g = __float_as_int(a.w);
                    if (th < best_t || res.leafpos < 0 || g > best_g) {
                        res.leafpos = lp;
                        res.t = th;
                        res.bu = uh;
                        res.bv = vh;
                        best_t = th;
                        best_g = g;
                    }
                }
            }
        }
        if (sp == 0) break;
        cur = stack[--sp];
    }
    return true;
}

}  // namespace wf
