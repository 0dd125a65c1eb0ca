// wf_traverse.cuh — BVH traversal (closest hit and any hit) over the binary
// and 4-wide trees.
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

// Entry / exit distance of a slab test over three axes (an explicit
// three-operand PTX min / max measured no faster than the nested pair).
__device__ __forceinline__ float fmax3(float a, float b, float c) { return fmaxf(fmaxf(a, b), c); }
__device__ __forceinline__ float fmin3(float a, float b, float c) { return fminf(fminf(a, b), c); }

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
    tn0 = fmax3(fminf(lx0, hx0), fminf(ly0, hy0), fmaxf(fminf(lz0, hz0), tmin));
    float tf0 = fmin3(fmaxf(lx0, hx0), fmaxf(ly0, hy0), fminf(fmaxf(lz0, hz0), tmax));
    tn1 = fmax3(fminf(lx1, hx1), fminf(ly1, hy1), fmaxf(fminf(lz1, hz1), tmin));
    float tf1 = fmin3(fmaxf(lx1, hx1), fmaxf(ly1, hy1), fminf(fmaxf(lz1, hz1), tmax));
    h0 = tn0 <= tf0;
    h1 = tn1 <= tf1;
}

// Two float4 in one 32-byte read-only load (sm_100 and later); p must be
// 32-byte aligned.
__device__ __forceinline__ void ldg_v8(const float4* p, float4& a, float4& b)
{
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

// A node in two 32-byte loads: the tree starts its allocation (aligned to 256
// bytes) and nodes are 64 bytes.
__device__ __forceinline__ BvhNode load_node(const BvhNode* nodes, uint32_t i)
{
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    BvhNode nd;
    float4 k;
    ldg_v8(p, nd.c0xy, nd.c1xy);
    ldg_v8(p + 2, nd.cz, k);
    nd.kids = make_int4(__float_as_int(k.x), __float_as_int(k.y), 0, 0);
    return nd;
}

constexpr uint32_t kSentinel = 0xFFFFFFFFu;

// Resumable while-while traversal (Aila & Laine, "Understanding the
// efficiency of ray traversal on GPUs", HPG 2009).  One call of round() walks
// interior nodes down to a leaf, then leaves until it pops an interior node or
// the stack's sentinel, so the lanes of a warp reconverge after every round
// and a persistent kernel can hand a finished lane a new ray between rounds.
template <bool kAnyHit, bool kFarFirst = false>
struct Traversal {
    using Entry = uint32_t;
    static constexpr int kStack = kStackSize;
    V3 o, d, inv, oi;
    float tmin, best_t;
    int best_g;
    uint32_t cur;
    uint32_t top;  // the entry the next pop returns (binary traversal)
    int sp;
    bool overflow;
    TraceResult res;

    // The stack lives outside the struct (a dynamically indexed array would
    // pull the whole struct into local memory); stack[0] holds the sentinel.
    template <class Stk>
    __device__ __forceinline__ void init(const DeviceScene& S, Stk stack, V3 o_, V3 d_, float tmin_, float tmax_)
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
        top = kSentinel;
        cur = S.root_is_empty ? kSentinel : 0u;
        overflow = false;
    }
    __device__ __forceinline__ bool done() const { return cur == kSentinel; }
    __device__ __forceinline__ void idle() { cur = kSentinel; }

    // Binary-traversal stack with its top entry in a register: entries
    // 0 .. sp-2 are in memory, entry sp-1 is `top`.  A pop returns the
    // register at once and reloads `top` for the pop after it, so the next
    // node fetch never waits on a local-memory load.
    template <class Stk>
    __device__ __forceinline__ void push(Stk stack, uint32_t e)
    {
        if (sp < kStackSize) {
            stack[sp - 1] = top;
            top = e;
            ++sp;
        } else {
            overflow = true;
        }
    }
    template <class Stk>
    __device__ __forceinline__ uint32_t pop(Stk stack)
    {
        const uint32_t r = top;
        --sp;
        top = sp > 0 ? stack[sp - 1] : kSentinel;
        return r;
    }
    template <class Stk>
    __device__ __forceinline__ void round(const DeviceScene& S, Stk stack)
    {
        round(S.nodes, S.tris, stack);
    }

    // nodes / tris of the ray's scene: from the kernel's parameter bank when
    // every ray shares one scene, else from the scene table.
    template <class Stk>
    __device__ __forceinline__ void round(const BvhNode* __restrict__ nodes, const float4* __restrict__ tris,
                                          Stk stack)
    {
        // While-while: walk interior nodes down to a leaf, then test leaves
        // until an interior node or the sentinel comes off the stack.
        while (!(cur & kLeafFlag)) {
            const BvhNode nd = load_node(nodes, cur);
            float tn0, tn1;
            bool h0, h1;
            slab2(nd, inv, oi, tmin, best_t, tn0, tn1, h0, h1);
            const uint32_t c0 = (uint32_t)nd.kids.x, c1 = (uint32_t)nd.kids.y;
            if (h0 && h1) {
                const bool swap = child_order_swap(tn0, tn1);
                const uint32_t farc = swap ? c0 : c1;
                cur = swap ? c1 : c0;
                push(stack, farc);
            } else if (h0 || h1) {
                cur = h0 ? c0 : c1;
            } else {
                cur = pop(stack);
            }
        }
        while (cur != kSentinel && (cur & kLeafFlag)) {
            const uint32_t leaf = cur;
            cur = pop(stack);
            if (test_leaf(tris, leaf)) {
                cur = kSentinel;
                return;
            }
        }
    }

    // Which hit child to visit first: the nearer one for closest hit; for
    // any hit (shadow rays) the nearer one, or with kFarFirst the farther
    // one, which reaches the occluders between the surface and the light
    // before the geometry around the ray's own origin, where a shadow ray
    // leaving its surface finds nothing.  (Visiting the first child or the
    // larger box first measured 0.5-3% slower on the dense mesh.)
    __device__ __forceinline__ static bool child_order_swap(float tn0, float tn1)
    {
        if (kAnyHit && kFarFirst) return !(tn1 < tn0);
        return tn1 < tn0;
    }

    // The triangles of one leaf; true when an any-hit query may stop.
    __device__ __forceinline__ bool test_leaf(const float4* __restrict__ tris, uint32_t leaf)
    {
        const int first = (int)((leaf & ~kLeafFlag) >> 3);
        const int cnt = (int)(leaf & 7u) + 1;
        for (int k = 0; k < cnt; ++k) {
            const int lp = first + k;
            const float4 a = __ldg(tris + 3 * lp + 0);
            const float4 b = __ldg(tris + 3 * lp + 1);
            const float4 c = __ldg(tris + 3 * lp + 2);
            float th, uh, vh;
            if (intersect_triangle(o, d, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z), tmin, best_t, th,
                                   uh, vh)) {
                const int g = __float_as_int(a.w);
                if (kAnyHit || th < best_t || res.leafpos < 0 || g > best_g) {
                    res.leafpos = lp;
                    res.t = th;
                    res.bu = uh;
                    res.bv = vh;
                    best_t = th;
                    best_g = g;
                    if (kAnyHit) return true;
                }
            }
        }
        return false;
    }
};

// While-while traversal of the 4-wide tree (Bvh4Node): the four child boxes
// of a node are slab-tested together; the hit children are ordered by entry
// distance with a sorting network over keys (distance bits with the slot in
// the low two bits, misses all ones), the nearest is visited next and the
// others are pushed farthest first.  Same state, leaf test and acceptance
// rule as the binary traversal, so the result does not depend on the tree.
template <bool kAnyHit, bool kFarFirst = false>
struct Traversal4 : Traversal<kAnyHit> {
    static constexpr int kStack = kStack4;

    template <class Stk>
    __device__ __forceinline__ void round(const DeviceScene& S, Stk stack)
    {
        round4(S.nodes4, S.tris, stack);
    }

    __device__ __forceinline__ uint32_t slab_key(float lx, float hx, float ly, float hy, float lz, float hz,
                                                 int kid, uint32_t slot) const
    {
        const float tlx = __fmaf_rn(lx, this->inv.x, -this->oi.x), thx = __fmaf_rn(hx, this->inv.x, -this->oi.x);
        const float tly = __fmaf_rn(ly, this->inv.y, -this->oi.y), thy = __fmaf_rn(hy, this->inv.y, -this->oi.y);
        const float tlz = __fmaf_rn(lz, this->inv.z, -this->oi.z), thz = __fmaf_rn(hz, this->inv.z, -this->oi.z);
        const float tn = fmax3(fminf(tlx, thx), fminf(tly, thy), fmaxf(fminf(tlz, thz), this->tmin));
        const float tf = fmin3(fmaxf(tlx, thx), fmaxf(tly, thy), fminf(fmaxf(tlz, thz), this->best_t));
        // tn >= tmin: for tmin >= 0 the bits order like the distances (the
        // order only steers the walk, never the result); kFarFirst (shadow
        // rays of dense scenes) inverts them, so the farthest hit child
        // comes first (its keys keep the top bit, a miss stays all ones)
        const uint32_t bits = kAnyHit && kFarFirst ? ~__float_as_uint(tn) : __float_as_uint(tn);
        return (tn <= tf && (uint32_t)kid != kEmptyChild4) ? ((bits & ~3u) | slot) : 0xFFFFFFFFu;
    }
    __device__ __forceinline__ static void sort2(uint32_t& a, uint32_t& b)
    {
        const uint32_t lo = min(a, b), hi = max(a, b);
        a = lo;
        b = hi;
    }
    __device__ __forceinline__ static uint32_t kid_of(const int4& k, uint32_t key)
    {
        const uint32_t s = key & 3u;
        return (uint32_t)(s == 0u ? k.x : s == 1u ? k.y : s == 2u ? k.z : k.w);
    }
    // The binary traversal's stack discipline: entry sp-1 lives in `top`, so
    // a pop hands the next node over at once and reloads the register from
    // memory for the pop after it.
    template <class Stk>
    __device__ __forceinline__ void push(Stk stack, uint32_t e)
    {
        stack[this->sp - 1] = this->top;
        this->top = e;
        ++this->sp;
    }

    template <class Stk>
    __device__ __forceinline__ void round4(const Bvh4Node* __restrict__ nodes, const float4* __restrict__ tris,
                                           Stk stack)
    {
        while (!(this->cur & kLeafFlag)) {
            // one 128-byte node in three 256-bit loads and one 128-bit load
            const float4* p = reinterpret_cast<const float4*>(nodes + this->cur);
            float4 lx, hx, ly, hy, lz, hz;
            ldg_v8(p + 0, lx, hx);
            ldg_v8(p + 2, ly, hy);
            ldg_v8(p + 4, lz, hz);
            const int4 k = __ldg(reinterpret_cast<const int4*>(p + 6));
            uint32_t k0 = slab_key(lx.x, hx.x, ly.x, hy.x, lz.x, hz.x, k.x, 0u);
            uint32_t k1 = slab_key(lx.y, hx.y, ly.y, hy.y, lz.y, hz.y, k.y, 1u);
            uint32_t k2 = slab_key(lx.z, hx.z, ly.z, hy.z, lz.z, hz.z, k.z, 2u);
            uint32_t k3 = slab_key(lx.w, hx.w, ly.w, hy.w, lz.w, hz.w, k.w, 3u);
            sort2(k0, k1);
            sort2(k2, k3);
            sort2(k0, k2);
            sort2(k1, k3);
            sort2(k1, k2);
            if (k0 == 0xFFFFFFFFu) {
                this->cur = this->pop(stack);
                continue;
            }
            this->cur = kid_of(k, k0);
            const int extra = (k1 != 0xFFFFFFFFu) + (k2 != 0xFFFFFFFFu) + (k3 != 0xFFFFFFFFu);
            if (this->sp + extra > kStack4) {
                this->overflow = true;
                continue;
            }
            if (k3 != 0xFFFFFFFFu) push(stack, kid_of(k, k3));
            if (k2 != 0xFFFFFFFFu) push(stack, kid_of(k, k2));
            if (k1 != 0xFFFFFFFFu) push(stack, kid_of(k, k1));
        }
        while (this->cur != kSentinel && (this->cur & kLeafFlag)) {
            const uint32_t leaf = this->cur;
            this->cur = this->pop(stack);
            if (this->test_leaf(tris, leaf)) {
                this->cur = kSentinel;
                return;
            }
        }
    }
};

// Whole traversal of one ray (host-API kernels).  Returns false (and sets
// *err_flag) only if the stack would overflow, which the build rules out by
// checking the tree depth.
template <class Tr>
__device__ __forceinline__ bool traverse_with(const DeviceScene& S, V3 o, V3 d, float tmin, float tmax,
                                              TraceResult& res, int* err_flag)
{
    Tr tr;
    typename Tr::Entry stack[Tr::kStack];
    tr.init(S, stack, o, d, tmin, tmax);
    while (!tr.done()) tr.round(S, stack);
    res = tr.res;
    if (tr.overflow) atomicOr(err_flag, 1);
    return !tr.overflow;
}

template <bool kAnyHit>
__device__ __forceinline__ bool traverse(const DeviceScene& S, V3 o, V3 d, float tmin, float tmax,
                                         TraceResult& res, int* err_flag)
{
    if (S.nodes4) return traverse_with<Traversal4<kAnyHit>>(S, o, d, tmin, tmax, res, err_flag);
    return traverse_with<Traversal<kAnyHit>>(S, o, d, tmin, tmax, res, err_flag);
}

}  // namespace wf
