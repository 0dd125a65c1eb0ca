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

constexpr uint32_t kSentinel = 0xFFFFFFFFu;

// Resumable while-while traversal (Aila & Laine, "Understanding the
// efficiency of ray traversal on GPUs", HPG 2009).  One call of round() walks
// interior nodes down to a leaf, then leaves until it pops an interior node or
// the stack's sentinel, so the lanes of a warp reconverge after every round
// and a persistent kernel can hand a finished lane a new ray between rounds.
template <bool kAnyHit>
struct Traversal {
    V3 o, d, inv, oi;
    float tmin, best_t;
    int best_g;
    uint32_t cur;
    int sp;
    bool overflow;
    TraceResult res;

    // The stack lives outside the struct (a dynamically indexed array would
    // pull the whole struct into local memory); stack[0] holds the sentinel.
    __device__ __forceinline__ void init(const DeviceScene& S, uint32_t* stack, V3 o_, V3 d_, float tmin_,
                                         float tmax_)
    {
        o = o_;
        d = d_;
        inv = v3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
        oi = v3(o.x * inv.x, o.y * inv.y, o.z * inv.z);
        tmin = tmin_;
        best_t = tmax_;
        best_g = -1;
        res.leafpos = -1;
        sp = 0;
        stack[sp++] = kSentinel;
        cur = S.root_is_empty ? kSentinel : 0u;
        overflow = false;
    }
    __device__ __forceinline__ bool done() const { return cur == kSentinel; }

    // nodes / tris of the ray's scene: from the kernel's parameter bank when
    // every ray shares one scene, else from the scene table.
    __device__ __forceinline__ void round(const BvhNode* __restrict__ nodes, const float4* __restrict__ tris,
                                          uint32_t* stack)
    {
        while (!(cur & kLeafFlag)) {
            const BvhNode nd = load_node(nodes, cur);
            float tn0, tn1;
            bool h0, h1;
            slab2(nd, inv, oi, tmin, best_t, tn0, tn1, h0, h1);
            const uint32_t c0 = (uint32_t)nd.kids.x, c1 = (uint32_t)nd.kids.y;
            if (h0 && h1) {
                const bool swap = tn1 < tn0;
                const uint32_t farc = swap ? c0 : c1;
                cur = swap ? c1 : c0;
                if (sp < kStackSize)
                    stack[sp++] = farc;
                else
                    overflow = true;
            } else if (h0 || h1) {
                cur = h0 ? c0 : c1;
            } else {
                cur = stack[--sp];
            }
        }
        while (cur != kSentinel) {
            if (!(cur & kLeafFlag)) break;
            const int first = (int)((cur & ~kLeafFlag) >> 3);
            const int cnt = (int)(cur & 7u) + 1;
            bool stop = false;
            for (int k = 0; k < cnt; ++k) {
                const int lp = first + k;
                const float4 a = __ldg(tris + 3 * lp + 0);
                const float4 b = __ldg(tris + 3 * lp + 1);
                const float4 c = __ldg(tris + 3 * lp + 2);
                float th, uh, vh;
                if (intersect_triangle(o, d, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z), tmin,
                                       best_t, th, uh, vh)) {
                    const int g = __float_as_int(a.w);
                    if (kAnyHit || th < best_t || res.leafpos < 0 || g > best_g) {
                        res.leafpos = lp;
                        res.t = th;
                        res.bu = uh;
                        res.bv = vh;
                        best_t = th;
                        best_g = g;
                        if (kAnyHit) stop = true;
                    }
                }
            }
            cur = stop ? kSentinel : stack[--sp];
        }
    }
};

// Whole traversal of one ray (host-API kernels).  Returns false (and sets
// *err_flag) only if the stack would overflow, which the build rules out by
// checking the tree depth.
template <bool kAnyHit>
__device__ __forceinline__ bool traverse(const DeviceScene& S, V3 o, V3 d, float tmin, float tmax,
                                         TraceResult& res, int* err_flag)
{
    Traversal<kAnyHit> tr;
    uint32_t stack[kStackSize];
    tr.init(S, stack, o, d, tmin, tmax);
    while (!tr.done()) tr.round(S.nodes, S.tris, stack);
    res = tr.res;
    if (tr.overflow) atomicOr(err_flag, 1);
    return !tr.overflow;
}

}  // namespace wf
