// wf_bvh.cu — device BVH build (Morton order + Karras 2012 radix tree).
//
// Replaces EmbreeAccelerator::build (reference src/accelerator/Embree.cpp
// :66-119).  Steps, all on the GPU:
//   1. per-triangle box and 63-bit Morton code of its centroid (21 bits per
//      axis over the scene's vertex bounds)
//   2. stable radix sort of (code, triangle)
//   3. Karras, "Maximizing Parallelism in the Construction of BVHs, Octrees,
//      and k-d Trees" (HPG 2012): internal node i finds its key range and
//      split from common-prefix lengths; equal codes are told apart by index
//   4. boxes bottom-up (second child to arrive at a node merges)
//   5. emit the traversal layout: each node holds its two children's boxes;
//      a child whose subtree has <= kLeafMax triangles becomes a leaf over
//      its contiguous range of sorted triangles.  Boxes are padded by a small
//      relative margin so the float slab test is conservative.
//   6. triangles in leaf order as (v0, v1-v0, v2-v0) plus ids.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <utility>
#include <vector>

#include "wf_bvh.h"
#include "wf_sort.h"

namespace wf {

namespace {

constexpr uint32_t kKarrasLeaf = 0x80000000u;

__device__ __forceinline__ uint64_t spread21(uint32_t v)
{
    uint64_t x = v & 0x1FFFFFu;
    x = (x | x << 32) & 0x1F00000000FFFFull;
    x = (x | x << 16) & 0x1F0000FF0000FFull;
    x = (x | x << 8) & 0x100F00F00F00F00Full;
    x = (x | x << 4) & 0x10C30C30C30C30C3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__global__ void k_tri_prep(const float* __restrict__ px, const float* __restrict__ py,
                           const float* __restrict__ pz, const int32_t* __restrict__ idx, int n,
                           float3 smin, float3 sext, float* __restrict__ tri_box,
                           uint64_t* __restrict__ codes, uint32_t* __restrict__ ids)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
        float x0 = px[a], y0 = py[a], z0 = pz[a];
        float x1 = px[b], y1 = py[b], z1 = pz[b];
        float x2 = px[c], y2 = py[c], z2 = pz[c];
        float lx = fminf(x0, fminf(x1, x2)), ly = fminf(y0, fminf(y1, y2)), lz = fminf(z0, fminf(z1, z2));
        float hx = fmaxf(x0, fmaxf(x1, x2)), hy = fmaxf(y0, fmaxf(y1, y2)), hz = fmaxf(z0, fmaxf(z1, z2));
        float* bx = tri_box + 6 * (int64_t)t;
        bx[0] = lx; bx[1] = ly; bx[2] = lz; bx[3] = hx; bx[4] = hy; bx[5] = hz;
        float cx = 0.5f * (lx + hx), cy = 0.5f * (ly + hy), cz = 0.5f * (lz + hz);
        auto q = [](float v, float lo, float ex) {
            float u = ex > 0.0f ? (v - lo) / ex : 0.0f;
            u = fminf(fmaxf(u, 0.0f), 1.0f);
            return (uint32_t)(u * 2097151.0f);
        };
        codes[t] = spread21(q(cx, smin.x, sext.x)) | (spread21(q(cy, smin.y, sext.y)) << 1) |
                   (spread21(q(cz, smin.z, sext.z)) << 2);
        ids[t] = (uint32_t)t;
    }
}

__device__ __forceinline__ int delta(const uint64_t* __restrict__ codes, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    uint64_t a = codes[i], b = codes[j];
    if (a == b) return 64 + __clz((uint32_t)(i ^ j));
    return __clzll((long long)(a ^ b));
}

__global__ void k_karras(const uint64_t* __restrict__ codes, int n, uint32_t* __restrict__ kid_l,
                         uint32_t* __restrict__ kid_r, int* __restrict__ parent_int,
                         int* __restrict__ parent_leaf, int* __restrict__ range_first,
                         int* __restrict__ range_last)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        int d = (delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1)) > 0 ? 1 : -1;
        int dmin = delta(codes, n, i, i - d);
        int lmax = 2;
        while (delta(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
        int j = i + l * d;
        int dnode = delta(codes, n, i, j);
        int s = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        int gamma = i + s * d + min(d, 0);
        int first = min(i, j), last = max(i, j);
        uint32_t left = (first == gamma) ? (kKarrasLeaf | (uint32_t)gamma) : (uint32_t)gamma;
        uint32_t right = (last == gamma + 1) ? (kKarrasLeaf | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
        kid_l[i] = left;
        kid_r[i] = right;
        range_first[i] = first;
        range_last[i] = last;
        if (left & kKarrasLeaf) parent_leaf[gamma] = i; else parent_int[gamma] = i;
        if (right & kKarrasLeaf) parent_leaf[gamma + 1] = i; else parent_int[gamma + 1] = i;
        if (i == 0) parent_int[0] = -1;
    }
}

__global__ void k_leaf_boxes(const float* __restrict__ tri_box, const uint32_t* __restrict__ sorted,
                             int n, float* __restrict__ leaf_box)
{
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const float* s = tri_box + 6 * (int64_t)sorted[j];
        float* d = leaf_box + 6 * (int64_t)j;
#pragma unroll
        for (int k = 0; k < 6; ++k) d[k] = s[k];
    }
}

__device__ __forceinline__ void load_box(uint32_t kid, const float* leaf_box, const float* int_box,
                                         float b[6])
{
    const float* s = (kid & kKarrasLeaf) ? leaf_box + 6 * (int64_t)(kid & ~kKarrasLeaf)
                                         : int_box + 6 * (int64_t)kid;
#pragma unroll
    for (int k = 0; k < 6; ++k) b[k] = __ldcg(s + k);
}

__global__ void k_boxes_up(int n, const uint32_t* __restrict__ kid_l, const uint32_t* __restrict__ kid_r,
                           const int* __restrict__ parent_int, const int* __restrict__ parent_leaf,
                           const float* __restrict__ leaf_box, float* int_box, int* flags)
{
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        int p = parent_leaf[j];
        // A tree of n leaves is at most n-1 levels deep; the bound only
        // guards against a corrupt parent array.
        for (int guard = 0; p >= 0 && guard < n; ++guard) {
            __threadfence();
            if (atomicAdd(&flags[p], 1) == 0) break;
            float a[6], b[6];
            load_box(kid_l[p], leaf_box, int_box, a);
            load_box(kid_r[p], leaf_box, int_box, b);
            float* o = int_box + 6 * (int64_t)p;
            __stcg(o + 0, fminf(a[0], b[0]));
            __stcg(o + 1, fminf(a[1], b[1]));
            __stcg(o + 2, fminf(a[2], b[2]));
            __stcg(o + 3, fmaxf(a[3], b[3]));
            __stcg(o + 4, fmaxf(a[4], b[4]));
            __stcg(o + 5, fmaxf(a[5], b[5]));
            p = parent_int[p];
        }
    }
}

__device__ __forceinline__ void pad_box(float b[6])
{
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float mag = fmaxf(fabsf(b[k]), fabsf(b[k + 3]));
        float pad = mag * 1e-5f + 1e-6f;
        b[k] = b[k] - pad;
        b[k + 3] = b[k + 3] + pad;
    }
}

__device__ __forceinline__ uint32_t encode_child(uint32_t kid, const int* range_first,
                                                 const int* range_last)
{
    int first, cnt;
    if (kid & kKarrasLeaf) {
        first = (int)(kid & ~kKarrasLeaf);
        cnt = 1;
    } else {
        first = range_first[kid];
        cnt = range_last[kid] - first + 1;
    }
    if (cnt <= kLeafMax) return kLeafFlag | ((uint32_t)first << 3) | (uint32_t)(cnt - 1);
    return kid;
}

__global__ void k_emit_nodes(int n, const uint32_t* __restrict__ kid_l, const uint32_t* __restrict__ kid_r,
                             const int* __restrict__ range_first, const int* __restrict__ range_last,
                             const float* __restrict__ leaf_box, const float* __restrict__ int_box,
                             BvhNode* __restrict__ nodes)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        float a[6], b[6];
        load_box(kid_l[i], leaf_box, int_box, a);
        load_box(kid_r[i], leaf_box, int_box, b);
        pad_box(a);
        pad_box(b);
        BvhNode nd;
        nd.c0xy = make_float4(a[0], a[3], a[1], a[4]);
        nd.c1xy = make_float4(b[0], b[3], b[1], b[4]);
        nd.cz = make_float4(a[2], a[5], b[2], b[5]);
        nd.kids = make_int4((int)encode_child(kid_l[i], range_first, range_last),
                            (int)encode_child(kid_r[i], range_first, range_last), 0, 0);
        nodes[i] = nd;
    }
}

// A scene of one triangle: a root with the leaf and an unreachable child.
__global__ void k_emit_single(const float* __restrict__ leaf_box, BvhNode* nodes)
{
    float a[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) a[k] = leaf_box[k];
    pad_box(a);
    BvhNode nd;
    nd.c0xy = make_float4(a[0], a[3], a[1], a[4]);
    nd.c1xy = make_float4(1e30f, 1e30f, 1e30f, 1e30f);
    nd.cz = make_float4(a[2], a[5], 1e30f, 1e30f);
    nd.kids = make_int4((int)kLeafFlag, (int)kLeafFlag, 0, 0);
    nodes[0] = nd;
}

__global__ void k_emit_tris(const float* __restrict__ px, const float* __restrict__ py,
                            const float* __restrict__ pz, const int32_t* __restrict__ idx,
                            const int32_t* __restrict__ tri_geom, const int32_t* __restrict__ tri_prim,
                            const uint32_t* __restrict__ sorted, int n, float4* __restrict__ tris)
{
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        int t = (int)sorted[j];
        int a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
        float x0 = px[a], y0 = py[a], z0 = pz[a];
        tris[3 * (int64_t)j + 0] = make_float4(x0, y0, z0, __int_as_float(t));
        tris[3 * (int64_t)j + 1] = make_float4(px[b] - x0, py[b] - y0, pz[b] - z0, __int_as_float(tri_geom[t]));
        tris[3 * (int64_t)j + 2] = make_float4(px[c] - x0, py[c] - y0, pz[c] - z0, __int_as_float(tri_prim[t]));
    }
}

__global__ void k_depth(int n, const int* __restrict__ parent_int, int* max_depth)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        int d = 0, p = parent_int[i];
        while (p >= 0 && d < 4096) {
            ++d;
            p = parent_int[p];
        }
        atomicMax(max_depth, d);
    }
}

// ===========================================================================
// PLOC: Meister & Bittner, "Parallel Locally-Ordered Clustering for Bounding
// Volume Hierarchy Construction" (IEEE TVCG 2018).  Clusters start as the
// Morton-sorted triangles; every iteration each cluster finds, among the
// kPlocRadius clusters on either side, the one whose union box has the
// smallest surface area (ties: the lower position), mutual nearest
// neighbours merge into a new node at the lower position, and the cluster
// array is compacted in order.  Node ids: triangles 0..N-1 (sorted
// position), internal nodes N.. in creation order, so children are created
// before their parents and the root is created last.
// ===========================================================================

#ifndef WF_PLOC_RADIUS
#define WF_PLOC_RADIUS 32  // 16 -> 32: lattice +10%, dense mesh unchanged, build +15%
#endif
constexpr int kPlocRadius = WF_PLOC_RADIUS;
constexpr int kPlocBlock = 256;

__device__ __forceinline__ float union_half_area(const float* a, const float* b)
{
    const float dx = fmaxf(a[3], b[3]) - fminf(a[0], b[0]);
    const float dy = fmaxf(a[4], b[4]) - fminf(a[1], b[1]);
    const float dz = fmaxf(a[5], b[5]) - fminf(a[2], b[2]);
    return dx * dy + dy * dz + dz * dx;
}

__global__ void __launch_bounds__(kPlocBlock) k_ploc_nn(const int* __restrict__ cl, int n,
                                                       const float* __restrict__ nbox, int* __restrict__ nn)
{
    __shared__ float sb[(kPlocBlock + 2 * kPlocRadius) * 6];
    const int block0 = blockIdx.x * kPlocBlock;
    for (int k = threadIdx.x; k < kPlocBlock + 2 * kPlocRadius; k += kPlocBlock) {
        const int g = block0 - kPlocRadius + k;
        if (g >= 0 && g < n) {
            const float* b = nbox + 6 * (int64_t)cl[g];
#pragma unroll
            for (int c = 0; c < 6; ++c) sb[k * 6 + c] = b[c];
        }
    }
    __syncthreads();
    const int i = block0 + threadIdx.x;
    if (i >= n) return;
    const float* bi = sb + (threadIdx.x + kPlocRadius) * 6;
    float best = 3.0e38f;
    int bj = -1;
    const int lo = max(0, i - kPlocRadius), hi = min(n - 1, i + kPlocRadius);
    for (int j = lo; j <= hi; ++j) {
        if (j == i) continue;
        const float a = union_half_area(bi, sb + (j - block0 + kPlocRadius) * 6);
        if (a < best) {
            best = a;
            bj = j;
        }
    }
    nn[i] = bj;
}

__global__ void k_ploc_flags(const int* __restrict__ nn, int n, int* __restrict__ merge, int* __restrict__ valid)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int j = nn[i];
        const bool mutual = j >= 0 && nn[j] == i;
        merge[i] = (mutual && i < j) ? 1 : 0;
        valid[i] = (mutual && i > j) ? 0 : 1;
    }
}

__global__ void k_ploc_apply(const int* __restrict__ cl, const int* __restrict__ nn, int n,
                             const int* __restrict__ merge, const int* __restrict__ m_off,
                             const int* __restrict__ valid, const int* __restrict__ v_off, int node_base,
                             int num_tris, float* __restrict__ nbox, int* __restrict__ left,
                             int* __restrict__ right, int* __restrict__ cnt, int* __restrict__ cl_out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!valid[i]) continue;
        int id = cl[i];
        if (merge[i]) {
            const int a = cl[i], b = cl[nn[i]];
            id = node_base + m_off[i];
            left[id - num_tris] = a;
            right[id - num_tris] = b;
            const float* ba = nbox + 6 * (int64_t)a;
            const float* bb = nbox + 6 * (int64_t)b;
            float* o = nbox + 6 * (int64_t)id;
            o[0] = fminf(ba[0], bb[0]);
            o[1] = fminf(ba[1], bb[1]);
            o[2] = fminf(ba[2], bb[2]);
            o[3] = fmaxf(ba[3], bb[3]);
            o[4] = fmaxf(ba[4], bb[4]);
            o[5] = fmaxf(ba[5], bb[5]);
            cnt[id] = cnt[a] + cnt[b];
        }
        cl_out[v_off[i]] = id;
    }
}


// Top-down over one iteration's nodes: children's first triangle position
// (depth-first order, left subtree first) and depth.
__global__ void k_ploc_topdown(int first_id, int count, int num_tris, const int* __restrict__ left,
                               const int* __restrict__ right, const int* __restrict__ cnt, int* __restrict__ offset,
                               int* __restrict__ depth)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const int id = first_id + k;
        const int l = left[id - num_tris], r = right[id - num_tris];
        offset[l] = offset[id];
        offset[r] = offset[id] + cnt[l];
        depth[l] = depth[id] + 1;
        depth[r] = depth[id] + 1;
    }
}

__global__ void k_ploc_root(int root, int* offset, int* depth)
{
    offset[root] = 0;
    depth[root] = 0;
}

// Kept interior nodes (interior[], from k_bin_leaves / k_bin_interior) are
// numbered in reverse creation order, q = (last id) - id: the root gets 0 and
// the nodes of one clustering pass — one band of the tree's levels — stay
// together, so the top levels every ray visits share cache lines.  (A
// depth-first order measured ~10% slower on the dense-mesh and lattice
// workloads.)  A child that is not kept becomes a leaf over its depth-first
// triangle range.
__global__ void k_ploc_keep(int num_tris, int last_id, const uint8_t* __restrict__ interior, int* __restrict__ keep)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q <= last_id - num_tris; q += gridDim.x * blockDim.x)
        keep[q] = interior[last_id - q - num_tris];
}

// Interior nodes with more than kLeafMax triangles below them (the 4-wide
// builder's bound on its node count), in the same numbering.
__global__ void k_ploc_big(int num_tris, int last_id, const int* __restrict__ cnt, int* __restrict__ keep)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q <= last_id - num_tris; q += gridDim.x * blockDim.x)
        keep[q] = cnt[last_id - q] > kLeafMax ? 1 : 0;
}

__device__ __forceinline__ uint32_t ploc_child(int c, int num_tris, int last_id, const int* cnt, const int* offset,
                                               const int* newid, const uint8_t* interior)
{
    if (c < num_tris || !interior[c - num_tris])
        return kLeafFlag | ((uint32_t)offset[c] << 3) | (uint32_t)(cnt[c] - 1);
    return (uint32_t)newid[last_id - c];
}

__global__ void k_ploc_emit(int num_tris, int last_id, const int* __restrict__ left, const int* __restrict__ right,
                            const int* __restrict__ cnt, const int* __restrict__ offset,
                            const int* __restrict__ depth, const int* __restrict__ newid,
                            const uint8_t* __restrict__ interior, const float* __restrict__ nbox,
                            BvhNode* __restrict__ nodes, int* __restrict__ max_depth)
{
    for (int id = num_tris + blockIdx.x * blockDim.x + threadIdx.x; id <= last_id; id += gridDim.x * blockDim.x) {
        if (!interior[id - num_tris]) continue;
        const int l = left[id - num_tris], r = right[id - num_tris];
        float a[6], b[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            a[k] = nbox[6 * (int64_t)l + k];
            b[k] = nbox[6 * (int64_t)r + k];
        }
        pad_box(a);
        pad_box(b);
        BvhNode nd;
        nd.c0xy = make_float4(a[0], a[3], a[1], a[4]);
        nd.c1xy = make_float4(b[0], b[3], b[1], b[4]);
        nd.cz = make_float4(a[2], a[5], b[2], b[5]);
        nd.kids = make_int4((int)ploc_child(l, num_tris, last_id, cnt, offset, newid, interior),
                            (int)ploc_child(r, num_tris, last_id, cnt, offset, newid, interior), 0, 0);
        nodes[newid[last_id - id]] = nd;
        atomicMax(max_depth, depth[id]);
    }
}

// Whole tree in one leaf (N <= kLeafMax): a root with that leaf and an
// unreachable second child.
__global__ void k_ploc_single(int num_tris, int root, const float* __restrict__ nbox, BvhNode* nodes)
{
    float a[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) a[k] = nbox[6 * (int64_t)root + k];
    pad_box(a);
    BvhNode nd;
    nd.c0xy = make_float4(a[0], a[3], a[1], a[4]);
    nd.c1xy = make_float4(1e30f, 1e30f, 1e30f, 1e30f);
    nd.cz = make_float4(a[2], a[5], 1e30f, 1e30f);
    nd.kids = make_int4((int)(kLeafFlag | (uint32_t)(num_tris - 1)), (int)kLeafFlag, 0, 0);
    nodes[0] = nd;
}

// Triangle order of the tree: sorted position p goes to offset[p].
__global__ void k_ploc_order(int n, const int* __restrict__ offset, const uint32_t* __restrict__ sorted_ids,
                             uint32_t* __restrict__ final_ids)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        final_ids[offset[p]] = sorted_ids[p];
}

__global__ void k_ploc_init(int n, const float* __restrict__ leaf_box, float* __restrict__ nbox,
                            int* __restrict__ cnt, int* __restrict__ cl)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k < 6; ++k) nbox[6 * (int64_t)i + k] = leaf_box[6 * (int64_t)i + k];
        cnt[i] = 1;
        cl[i] = i;
    }
}

// ---------------------------------------------------------------------------
// Collapse of the PLOC tree into 4-wide nodes, one level of wide nodes per
// pass (items = binary node ids of the level's wide nodes).
// ---------------------------------------------------------------------------

// Children of each wide node (kWidth of them at most): open the binary
// subtree greedily, always the child of largest surface area among those with
// more than kLeafCnt triangles, until kWidth children or none left to open.
// kids has 8 entries per item; unused ones are -1.
template <int kWidth, int kLeafCnt>
__global__ void k_wide_gather(const int* __restrict__ items, int count, int num_tris, const int* __restrict__ left,
                              const int* __restrict__ right, const int* __restrict__ cnt,
                              const float* __restrict__ nbox, int* __restrict__ kids, int* __restrict__ n_int,
                              int* __restrict__ n_tri)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const int b = items[k];
        int ch[8];
        int m = 0;
        if (cnt[b] <= kLeafCnt) {  // a whole tree small enough for one leaf child
            ch[m++] = b;
        } else {
            ch[m++] = left[b - num_tris];
            ch[m++] = right[b - num_tris];
            while (m < kWidth) {
                int best = -1;
                float best_a = -1.0f;
                for (int i = 0; i < m; ++i) {
                    if (cnt[ch[i]] <= kLeafCnt) continue;
                    const float* x = nbox + 6 * (int64_t)ch[i];
                    const float dx = x[3] - x[0], dy = x[4] - x[1], dz = x[5] - x[2];
                    const float a = dx * dy + dy * dz + dz * dx;
                    if (a > best_a) {
                        best_a = a;
                        best = i;
                    }
                }
                if (best < 0) break;
                const int x = ch[best];
                ch[best] = left[x - num_tris];
                ch[m++] = right[x - num_tris];
            }
        }
        int ni = 0, nt = 0;
        for (int i = 0; i < 8; ++i) {
            kids[8 * (int64_t)k + i] = i < m ? ch[i] : -1;
            if (i < m) {
                if (cnt[ch[i]] > kLeafCnt)
                    ++ni;
                else
                    nt += cnt[ch[i]];
            }
        }
        n_int[k] = ni;
        n_tri[k] = nt;
    }
}

// SAH-optimal collapse (Ylitie, Karras & Laine, HPG 2017, section 4.1).  For
// every interior binary node n and i = 1 .. kWidth-1, cost[n][i-1] is the
// least SAH cost of representing n's subtree by at most i roots, each a wide
// node or a leaf child of at most kLeafCnt triangles:
//   C(n, 1) = min(leaf: A(n) c_prim N(n) if N(n) <= kLeafCnt,
//                 node: A(n) c_node + D(n, kWidth))
//   C(n, i) = min(C(n, i - 1), D(n, i)),   D(n, j) = min_a C(l, a) + C(r, j - a)
// (a single triangle costs A c_prim for every i).  choice[n][i-1] records the
// minimiser: kChoiceLeaf / kChoiceNode for i = 1, kChoiceFewer for C(n, i-1),
// else the number of roots given to the left child; choice[n][kWidth-1] is
// the split of D(n, kWidth), the children of n as a wide node.  The passes of
// the clustering create parents after their children, so one launch per pass
// in creation order sees its children's costs.
constexpr float kSahNode = 1.0f, kSahPrim = 0.3f;
constexpr uint8_t kChoiceLeaf = 0xF0, kChoiceNode = 0xF1, kChoiceFewer = 0xF2;

__device__ __forceinline__ float box_area(const float* x)
{
    const float dx = x[3] - x[0], dy = x[4] - x[1], dz = x[5] - x[2];
    return dx * dy + dy * dz + dz * dx;
}

// Leaves of the binary tree: a subtree of at most kLeafMax triangles is one
// leaf; with sah (wf_tuning::bvh_builder 4) only where testing its triangles
// is expected to cost no more than descending it (surface area heuristic: a
// node test and a triangle test cost 1 each, weighted by the area of the box
// that leads to them).  Measured against the fixed rule: Cornell box +4.6%
// (its wall triangles get leaves of their own), lattice +0.7%, batched
// Cornell variants +0.3%, dense mesh -1.4% (twice the nodes: its small
// leaves were cheaper to test than to split).  One launch per clustering
// pass in creation order (children first).
constexpr float kBinSahPrim = 1.0f;

__global__ void k_bin_leaves(int first_id, int count, int num_tris, const int* __restrict__ left,
                             const int* __restrict__ right, const int* __restrict__ cnt,
                             const float* __restrict__ nbox, int sah, float* __restrict__ cost,
                             uint8_t* __restrict__ leaf)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const int id = first_id + k;
        const int64_t in = id - num_tris;
        const int N = cnt[id];
        if (!sah) {
            leaf[in] = N <= kLeafMax ? 1 : 0;
            continue;
        }
        float below = 0.0f;
        for (int h = 0; h < 2; ++h) {
            const int c = h ? right[in] : left[in];
            below += c < num_tris ? box_area(nbox + 6 * (int64_t)c) * kBinSahPrim : cost[c - num_tris];
        }
        const float A = box_area(nbox + 6 * (int64_t)id);
        const float split = A + below;
        const float as_leaf = N <= kLeafMax ? A * kBinSahPrim * (float)N : INFINITY;
        const bool lf = as_leaf <= split;
        leaf[in] = lf ? 1 : 0;
        cost[in] = lf ? as_leaf : split;
    }
}

// Interior nodes top down (one launch per pass, the root's first): the root
// is interior; a child node is interior when its parent is and it is no leaf.
__global__ void k_bin_root(int root, int num_tris, uint8_t* interior) { interior[root - num_tris] = 1; }

__global__ void k_bin_interior(int first_id, int count, int num_tris, const int* __restrict__ left,
                               const int* __restrict__ right, const uint8_t* __restrict__ leaf,
                               uint8_t* __restrict__ interior)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const int64_t in = first_id + k - num_tris;
        if (!interior[in]) continue;
        for (int h = 0; h < 2; ++h) {
            const int c = h ? right[in] : left[in];
            if (c >= num_tris) interior[c - num_tris] = leaf[c - num_tris] ? 0 : 1;
        }
    }
}

template <int kWidth, int kLeafCnt>
__global__ void k_wide_sah(int first_id, int count, int num_tris, const int* __restrict__ left,
                           const int* __restrict__ right, const int* __restrict__ cnt,
                           const float* __restrict__ nbox, float* __restrict__ cost, uint8_t* __restrict__ choice)
{
    constexpr int kC = kWidth - 1;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const int id = first_id + k;
        const int64_t in = id - num_tris;
        const int kid[2] = {left[in], right[in]};
        float c[2][kC];
        for (int h = 0; h < 2; ++h) {
            if (kid[h] < num_tris) {
                const float a = box_area(nbox + 6 * (int64_t)kid[h]) * kSahPrim;
                for (int i = 0; i < kC; ++i) c[h][i] = a;
            } else {
                const float* src = cost + (int64_t)(kid[h] - num_tris) * kC;
                for (int i = 0; i < kC; ++i) c[h][i] = src[i];
            }
        }
        float D[kWidth + 1];
        uint8_t Dk[kWidth + 1];
        for (int j = 2; j <= kWidth; ++j) {
            float best = INFINITY;
            int bk = 1;
            for (int a = 1; a < j; ++a) {
                const float v = c[0][a - 1] + c[1][j - a - 1];
                if (v < best) {
                    best = v;
                    bk = a;
                }
            }
            D[j] = best;
            Dk[j] = (uint8_t)bk;
        }
        const float A = box_area(nbox + 6 * (int64_t)id);
        const int N = cnt[id];
        // a subtree of <= kLeafCnt triangles is always one leaf child when it
        // takes one slot (the emit kernels make it one)
        const float c_leaf = N <= kLeafCnt ? A * kSahPrim * (float)N : INFINITY;
        const float c_node = N <= kLeafCnt ? INFINITY : A * kSahNode + D[kWidth];
        float* dst = cost + in * kC;
        uint8_t* ch = choice + in * kWidth;
        float cur = fminf(c_leaf, c_node);
        dst[0] = cur;
        ch[0] = c_leaf <= c_node ? kChoiceLeaf : kChoiceNode;
        for (int i = 2; i <= kC; ++i) {
            if (D[i] < cur) {
                cur = D[i];
                ch[i - 1] = Dk[i];
            } else {
                ch[i - 1] = kChoiceFewer;
            }
            dst[i - 1] = cur;
        }
        ch[kWidth - 1] = Dk[kWidth];
    }
}

// Children of each wide node from the SAH choices: the node's kWidth slots
// are split between its binary children, recursively, down to roots of one
// slot (a subtree of <= kLeafCnt triangles becomes a leaf child, a larger one
// an interior child); same outputs as k_wide_gather.
template <int kWidth, int kLeafCnt>
__global__ void k_wide_gather_sah(const int* __restrict__ items, int count, int num_tris,
                                  const int* __restrict__ left, const int* __restrict__ right,
                                  const int* __restrict__ cnt, const uint8_t* __restrict__ choice,
                                  int* __restrict__ kids, int* __restrict__ n_int, int* __restrict__ n_tri)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const int b = items[k];
        int ch[8];
        int m = 0;
        if (b < num_tris || cnt[b] <= kLeafCnt) {
            ch[m++] = b;
        } else {
            int sn[2 * kWidth], ss[2 * kWidth];
            int sp = 0;
            const int64_t bi = b - num_tris;
            const int a = choice[bi * kWidth + kWidth - 1];
            sn[sp] = right[bi];
            ss[sp++] = kWidth - a;
            sn[sp] = left[bi];
            ss[sp++] = a;
            while (sp > 0 && m < kWidth) {
                --sp;
                const int x = sn[sp];
                int j = ss[sp];
                if (x < num_tris || j <= 1) {
                    ch[m++] = x;
                    continue;
                }
                const int64_t xi = x - num_tris;
                uint8_t c = choice[xi * kWidth + j - 1];
                while (c == kChoiceFewer && j > 1) {
                    --j;
                    c = choice[xi * kWidth + j - 1];
                }
                if (j <= 1 || c >= kChoiceLeaf || sp + 2 > 2 * kWidth) {
                    ch[m++] = x;
                    continue;
                }
                sn[sp] = right[xi];
                ss[sp++] = j - c;
                sn[sp] = left[xi];
                ss[sp++] = c;
            }
        }
        int ni = 0, nt = 0;
        for (int i = 0; i < 8; ++i) {
            kids[8 * (int64_t)k + i] = i < m ? ch[i] : -1;
            if (i < m) {
                if (cnt[ch[i]] > kLeafCnt)
                    ++ni;
                else
                    nt += cnt[ch[i]];
            }
        }
        n_int[k] = ni;
        n_tri[k] = nt;
    }
}


// One level of 4-wide nodes: padded child boxes at full precision, interior
// children numbered from next_base in the order of the level's items, leaf
// children over their depth-first triangle range of the PLOC order.
__global__ void k_four_emit(const int* __restrict__ items, int count, int level_base, int next_base,
                            const int* __restrict__ kids, const int* __restrict__ int_off, int num_tris,
                            const int* __restrict__ cnt, const float* __restrict__ nbox,
                            const int* __restrict__ offset, Bvh4Node* __restrict__ nodes,
                            int* __restrict__ next_items)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        float pl[6][4];
        int word[4];
        int irank = 0;
        for (int i = 0; i < 4; ++i) {
            const int c = kids[8 * (int64_t)k + i];
            float b[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            if (c < 0) {
                word[i] = (int)kEmptyChild4;
            } else {
                for (int a = 0; a < 6; ++a) b[a] = nbox[6 * (int64_t)c + a];
                pad_box(b);
                if (c < num_tris || cnt[c] <= kLeafMax) {
                    word[i] = (int)(kLeafFlag | ((uint32_t)offset[c] << 3) | (uint32_t)(cnt[c] - 1));
                } else {
                    const int slot = int_off[k] + irank++;
                    word[i] = next_base + slot;
                    next_items[slot] = c;
                }
            }
            // planes: lo x, hi x, lo y, hi y, lo z, hi z
            pl[0][i] = b[0];
            pl[1][i] = b[3];
            pl[2][i] = b[1];
            pl[3][i] = b[4];
            pl[4][i] = b[2];
            pl[5][i] = b[5];
        }
        Bvh4Node nd;
        nd.lox = make_float4(pl[0][0], pl[0][1], pl[0][2], pl[0][3]);
        nd.hix = make_float4(pl[1][0], pl[1][1], pl[1][2], pl[1][3]);
        nd.loy = make_float4(pl[2][0], pl[2][1], pl[2][2], pl[2][3]);
        nd.hiy = make_float4(pl[3][0], pl[3][1], pl[3][2], pl[3][3]);
        nd.loz = make_float4(pl[4][0], pl[4][1], pl[4][2], pl[4][3]);
        nd.hiz = make_float4(pl[5][0], pl[5][1], pl[5][2], pl[5][3]);
        nd.kids = make_int4(word[0], word[1], word[2], word[3]);
        nd.pad = make_int4(0, 0, 0, 0);
        nodes[level_base + k] = nd;
    }
}

// ---------------------------------------------------------------------------
// Structural checks of a finished tree before it is used: every child index
// and triangle range must lie inside the arrays (a failed check rejects the
// tree; the traversal kernels then never see it).
// ---------------------------------------------------------------------------

__global__ void k_validate_binary(const BvhNode* __restrict__ nodes, int num_nodes, int num_tris, int* __restrict__ bad)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num_nodes; i += gridDim.x * blockDim.x) {
        bool ok = true;
        const int kid[2] = {nodes[i].kids.x, nodes[i].kids.y};
        for (int c = 0; c < 2; ++c) {
            const uint32_t k = (uint32_t)kid[c];
            if (k & kLeafFlag) {
                const int64_t first = (int64_t)((k & ~kLeafFlag) >> 3), cnt = (int64_t)(k & 7u) + 1;
                // an unreachable empty child (inverted box) may carry count 1 at 0
                ok = ok && first + cnt <= (int64_t)num_tris;
            } else {
                ok = ok && (int)k >= 0 && (int)k < num_nodes && (int)k != i;
            }
        }
        if (!ok) atomicOr(bad, 1);
    }
}

// 4-wide nodes: interior children only after their parent (level order, so
// every walk down the tree ends), leaf ranges inside the triangle array, at
// least one child per node.
__global__ void k_validate_four(const Bvh4Node* __restrict__ nodes, int num_nodes, int num_tris, int* __restrict__ bad)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num_nodes; i += gridDim.x * blockDim.x) {
        const int kid[4] = {nodes[i].kids.x, nodes[i].kids.y, nodes[i].kids.z, nodes[i].kids.w};
        bool ok = true;
        int used = 0;
        for (int c = 0; c < 4; ++c) {
            const uint32_t k = (uint32_t)kid[c];
            if (k == kEmptyChild4) continue;
            ++used;
            if (k & kLeafFlag) {
                const int64_t first = (int64_t)((k & ~kLeafFlag) >> 3), cnt = (int64_t)(k & 7u) + 1;
                ok = ok && cnt <= kLeafMax && first + cnt <= (int64_t)num_tris;
            } else {
                ok = ok && (int)k > i && (int)k < num_nodes;
            }
        }
        if (!ok || used == 0) atomicOr(bad, 1);
    }
}

int validate_tree(const BvhBuildOutput& out, int num_tris, int num_sms, cudaStream_t s, std::string& err)
{
    int* d_bad = nullptr;
    int bad = 0;
    if (cudaMalloc(&d_bad, sizeof(int)) != cudaSuccess) {
        err = "validation buffer";
        return -1;
    }
    cudaMemsetAsync(d_bad, 0, sizeof(int), s);
    if (out.nodes4)
        k_validate_four<<<num_sms * 8, 256, 0, s>>>(out.nodes4, out.num_nodes, num_tris, d_bad);
    else if (out.nodes)
        k_validate_binary<<<num_sms * 8, 256, 0, s>>>(out.nodes, out.num_nodes, num_tris, d_bad);
    cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    cudaFree(d_bad);
    if (e != cudaSuccess) {
        err = std::string("tree validation: ") + cudaGetErrorString(e);
        return -1;
    }
    if (bad) {
        err = "tree failed its structural check";
        return -1;
    }
    return 0;
}

#define WF_TRY(x)                                                      \
    do {                                                               \
        cudaError_t e_ = (x);                                          \
        if (e_ != cudaSuccess) {                                       \
            err = std::string(#x) + ": " + cudaGetErrorString(e_);     \
            goto fail;                                                 \
        }                                                              \
    } while (0)

}  // namespace

int build_lbvh(const BvhBuildInput& in, BvhBuildOutput& out, int num_sms, cudaStream_t s,
               std::string& err)
{
    const int n = in.num_tris;
    out.tris = nullptr;
    out.nodes = nullptr;
    out.num_nodes = 0;
    out.max_depth = 0;
    if (n <= 0) return 0;
    float* tri_box = nullptr;
    float* leaf_box = nullptr;
    float* int_box = nullptr;
    uint64_t *codes = nullptr, *codes_tmp = nullptr;
    uint32_t *ids = nullptr, *ids_tmp = nullptr, *hist = nullptr;
    uint32_t *kid_l = nullptr, *kid_r = nullptr;
    int *parent_int = nullptr, *parent_leaf = nullptr, *range_first = nullptr, *range_last = nullptr;
    int* flags = nullptr;
    int* d_depth = nullptr;
    unsigned long long* d_n = nullptr;
    uint64_t* sorted_codes = nullptr;
    uint32_t* sorted_ids = nullptr;
    const int nint = n > 1 ? n - 1 : 1;
    const int grid = num_sms * 8;
    const int nb = radix_blocks_for(n, num_sms);
    float3 smin = make_float3(in.bmin[0], in.bmin[1], in.bmin[2]);
    float3 sext = make_float3(in.bmax[0] - in.bmin[0], in.bmax[1] - in.bmin[1], in.bmax[2] - in.bmin[2]);
    unsigned long long hn = (unsigned long long)n;
    int h_depth = 0;

    WF_TRY(cudaMalloc(&tri_box, 6 * sizeof(float) * (size_t)n));
    WF_TRY(cudaMalloc(&leaf_box, 6 * sizeof(float) * (size_t)n));
    WF_TRY(cudaMalloc(&int_box, 6 * sizeof(float) * (size_t)nint));
    WF_TRY(cudaMalloc(&codes, sizeof(uint64_t) * (size_t)n));
    WF_TRY(cudaMalloc(&codes_tmp, sizeof(uint64_t) * (size_t)n));
    WF_TRY(cudaMalloc(&ids, sizeof(uint32_t) * (size_t)n));
    WF_TRY(cudaMalloc(&ids_tmp, sizeof(uint32_t) * (size_t)n));
    WF_TRY(cudaMalloc(&hist, sizeof(uint32_t) * radix_hist_words(nb)));
    WF_TRY(cudaMalloc(&kid_l, sizeof(uint32_t) * (size_t)nint));
    WF_TRY(cudaMalloc(&kid_r, sizeof(uint32_t) * (size_t)nint));
    WF_TRY(cudaMalloc(&parent_int, sizeof(int) * (size_t)nint));
    WF_TRY(cudaMalloc(&parent_leaf, sizeof(int) * (size_t)n));
    WF_TRY(cudaMalloc(&range_first, sizeof(int) * (size_t)nint));
    WF_TRY(cudaMalloc(&range_last, sizeof(int) * (size_t)nint));
    WF_TRY(cudaMalloc(&flags, sizeof(int) * (size_t)nint));
    WF_TRY(cudaMalloc(&d_depth, sizeof(int)));
    WF_TRY(cudaMalloc(&d_n, sizeof(unsigned long long)));
    WF_TRY(cudaMalloc(&out.tris, 3 * sizeof(float4) * (size_t)n));
    WF_TRY(cudaMalloc(&out.nodes, sizeof(BvhNode) * (size_t)nint));
    WF_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * (size_t)nint, s));
    WF_TRY(cudaMemsetAsync(d_depth, 0, sizeof(int), s));
    WF_TRY(cudaMemsetAsync(parent_leaf, 0xFF, sizeof(int) * (size_t)n, s));
    WF_TRY(cudaMemsetAsync(parent_int, 0xFF, sizeof(int) * (size_t)nint, s));
    WF_TRY(cudaMemcpyAsync(d_n, &hn, sizeof(hn), cudaMemcpyHostToDevice, s));

    k_tri_prep<<<grid, 256, 0, s>>>(in.px, in.py, in.pz, in.idx, n, smin, sext, tri_box, codes, ids);
    {
        RadixSortArgs a{codes, ids, codes_tmp, ids_tmp, hist, d_n, nb, 0, 64, &sorted_codes, &sorted_ids};
        radix_sort_pairs(a, s);
    }
    k_leaf_boxes<<<grid, 256, 0, s>>>(tri_box, sorted_ids, n, leaf_box);
    if (n == 1) {
        k_emit_single<<<1, 1, 0, s>>>(leaf_box, out.nodes);
        out.num_nodes = 1;
        h_depth = 0;
    } else {
        k_karras<<<grid, 256, 0, s>>>(sorted_codes, n, kid_l, kid_r, parent_int, parent_leaf,
                                      range_first, range_last);
        k_boxes_up<<<grid, 256, 0, s>>>(n, kid_l, kid_r, parent_int, parent_leaf, leaf_box, int_box, flags);
        k_emit_nodes<<<grid, 256, 0, s>>>(n, kid_l, kid_r, range_first, range_last, leaf_box, int_box,
                                          out.nodes);
        k_depth<<<grid, 256, 0, s>>>(n, parent_int, d_depth);
        out.num_nodes = n - 1;
        WF_TRY(cudaMemcpyAsync(&h_depth, d_depth, sizeof(int), cudaMemcpyDeviceToHost, s));
    }
    k_emit_tris<<<grid, 256, 0, s>>>(in.px, in.py, in.pz, in.idx, in.tri_geom, in.tri_prim, sorted_ids,
                                     n, out.tris);
    WF_TRY(cudaGetLastError());
    WF_TRY(cudaStreamSynchronize(s));
    out.max_depth = h_depth;

    cudaFree(tri_box);
    cudaFree(leaf_box);
    cudaFree(int_box);
    cudaFree(codes);
    cudaFree(codes_tmp);
    cudaFree(ids);
    cudaFree(ids_tmp);
    cudaFree(hist);
    cudaFree(kid_l);
    cudaFree(kid_r);
    cudaFree(parent_int);
    cudaFree(parent_leaf);
    cudaFree(range_first);
    cudaFree(range_last);
    cudaFree(flags);
    cudaFree(d_depth);
    cudaFree(d_n);
    if (h_depth + 2 > kStackSize) {
        err = "BVH deeper than the traversal stack: depth " + std::to_string(h_depth);
        cudaFree(out.tris);
        cudaFree(out.nodes);
        out.tris = nullptr;
        out.nodes = nullptr;
        return -1;
    }
    return 0;
fail:
    cudaFree(tri_box);
    cudaFree(leaf_box);
    cudaFree(int_box);
    cudaFree(codes);
    cudaFree(codes_tmp);
    cudaFree(ids);
    cudaFree(ids_tmp);
    cudaFree(hist);
    cudaFree(kid_l);
    cudaFree(kid_r);
    cudaFree(parent_int);
    cudaFree(parent_leaf);
    cudaFree(range_first);
    cudaFree(range_last);
    cudaFree(flags);
    cudaFree(d_depth);
    cudaFree(d_n);
    cudaFree(out.tris);
    cudaFree(out.nodes);
    out.tris = nullptr;
    out.nodes = nullptr;
    return -1;
}


namespace {

// Device buffers of one build, freed together.
struct BuildScratch {
    std::vector<void*> ptrs;
    template <class T>
    cudaError_t alloc(T** p, size_t count)
    {
        *p = nullptr;
        cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
        if (e == cudaSuccess) ptrs.push_back((void*)*p);
        return e;
    }
    ~BuildScratch()
    {
        for (void* p : ptrs) cudaFree(p);
    }
};

// The binary PLOC tree: node ids 0..n-1 triangles (Morton position), n..
// interior nodes; boxes unpadded; offset = first triangle position of a
// node's subtree in depth-first order (final_ids maps positions to
// triangles); depth from the root.
struct PlocTree {
    int n = 0, root = 0;
    std::vector<std::pair<int, int>> iters;  // (first node id, nodes) of each clustering pass
    float* nbox = nullptr;
    int *cnt = nullptr, *left = nullptr, *right = nullptr, *offset = nullptr, *depth = nullptr;
    int *block_sums = nullptr, *d_total = nullptr;
    uint32_t* final_ids = nullptr;
};

int ploc_tree(const BvhBuildInput& in, int num_sms, cudaStream_t s, std::string& err, BuildScratch& B, PlocTree& T)
{
    const int n = in.num_tris;
    T.n = n;
    float *tri_box, *leaf_box;
    uint64_t *codes, *codes_tmp;
    uint32_t *ids, *ids_tmp, *hist;
    unsigned long long* d_n;
    int *cl, *cl2, *nn, *merge, *valid, *m_off, *v_off;
    uint64_t* sorted_codes = nullptr;
    uint32_t* sorted_ids = nullptr;
    const int64_t nn_all = 2 * (int64_t)n - 1;
    const int grid = num_sms * 8;
    const int nb = radix_blocks_for(n, num_sms);
    const float3 smin = make_float3(in.bmin[0], in.bmin[1], in.bmin[2]);
    const float3 sext = make_float3(in.bmax[0] - in.bmin[0], in.bmax[1] - in.bmin[1], in.bmax[2] - in.bmin[2]);
    const unsigned long long hn = (unsigned long long)n;
    std::vector<std::pair<int, int>> iters;  // (first node id, nodes) per iteration
    int cur_n = n, next_id = n;

    WF_TRY(B.alloc(&tri_box, 6 * (size_t)n));
    WF_TRY(B.alloc(&leaf_box, 6 * (size_t)n));
    WF_TRY(B.alloc(&T.nbox, 6 * (size_t)nn_all));
    WF_TRY(B.alloc(&codes, (size_t)n));
    WF_TRY(B.alloc(&codes_tmp, (size_t)n));
    WF_TRY(B.alloc(&ids, (size_t)n));
    WF_TRY(B.alloc(&ids_tmp, (size_t)n));
    WF_TRY(B.alloc(&hist, radix_hist_words(nb)));
    WF_TRY(B.alloc(&T.final_ids, (size_t)n));
    WF_TRY(B.alloc(&d_n, 1));
    WF_TRY(B.alloc(&T.cnt, (size_t)nn_all));
    WF_TRY(B.alloc(&T.left, (size_t)n));
    WF_TRY(B.alloc(&T.right, (size_t)n));
    WF_TRY(B.alloc(&cl, (size_t)n));
    WF_TRY(B.alloc(&cl2, (size_t)n));
    WF_TRY(B.alloc(&nn, (size_t)n));
    WF_TRY(B.alloc(&merge, (size_t)n));
    WF_TRY(B.alloc(&valid, (size_t)n));
    WF_TRY(B.alloc(&m_off, (size_t)n));
    WF_TRY(B.alloc(&v_off, (size_t)n));
    WF_TRY(B.alloc(&T.block_sums, (size_t)(n + 1023) / 1024 + 1));
    WF_TRY(B.alloc(&T.d_total, 2));
    WF_TRY(B.alloc(&T.offset, (size_t)nn_all));
    WF_TRY(B.alloc(&T.depth, (size_t)nn_all));
    WF_TRY(cudaMemcpyAsync(d_n, &hn, sizeof(hn), cudaMemcpyHostToDevice, s));

    k_tri_prep<<<grid, 256, 0, s>>>(in.px, in.py, in.pz, in.idx, n, smin, sext, tri_box, codes, ids);
    {
        RadixSortArgs a{codes, ids, codes_tmp, ids_tmp, hist, d_n, nb, 0, 64, &sorted_codes, &sorted_ids};
        radix_sort_pairs(a, s);
    }
    k_leaf_boxes<<<grid, 256, 0, s>>>(tri_box, sorted_ids, n, leaf_box);
    k_ploc_init<<<grid, 256, 0, s>>>(n, leaf_box, T.nbox, T.cnt, cl);
    while (cur_n > 1) {
        k_ploc_nn<<<(cur_n + kPlocBlock - 1) / kPlocBlock, kPlocBlock, 0, s>>>(cl, cur_n, T.nbox, nn);
        k_ploc_flags<<<grid, 256, 0, s>>>(nn, cur_n, merge, valid);
        exclusive_scan_i32(merge, cur_n, m_off, T.block_sums, T.d_total, s);
        exclusive_scan_i32(valid, cur_n, v_off, T.block_sums, T.d_total + 1, s);
        int tot[2] = {0, 0};
        WF_TRY(cudaMemcpyAsync(tot, T.d_total, sizeof(tot), cudaMemcpyDeviceToHost, s));
        WF_TRY(cudaStreamSynchronize(s));
        if (tot[0] <= 0 || tot[1] != cur_n - tot[0]) {
            err = "PLOC iteration merged no clusters";
            return -1;
        }
        k_ploc_apply<<<grid, 256, 0, s>>>(cl, nn, cur_n, merge, m_off, valid, v_off, next_id, n, T.nbox, T.left,
                                         T.right, T.cnt, cl2);
        iters.push_back({next_id, tot[0]});
        next_id += tot[0];
        std::swap(cl, cl2);
        cur_n = tot[1];
    }
    T.root = n == 1 ? 0 : next_id - 1;
    T.iters = iters;
    k_ploc_root<<<1, 1, 0, s>>>(T.root, T.offset, T.depth);
    for (auto it = iters.rbegin(); it != iters.rend(); ++it)
        k_ploc_topdown<<<std::max(1, std::min(grid, (it->second + 255) / 256)), 256, 0, s>>>(
            it->first, it->second, n, T.left, T.right, T.cnt, T.offset, T.depth);
    k_ploc_order<<<grid, 256, 0, s>>>(n, T.offset, sorted_ids, T.final_ids);
    WF_TRY(cudaGetLastError());
    return 0;
fail:
    return -1;
}

}  // namespace

int build_ploc(const BvhBuildInput& in, BvhBuildOutput& out, int num_sms, cudaStream_t s, std::string& err,
               bool sah_leaves)
{
    const int n = in.num_tris;
    out.tris = nullptr;
    out.nodes = nullptr;
    out.num_nodes = 0;
    out.max_depth = 0;
    if (n <= 0) return 0;
    BuildScratch B;
    PlocTree T;
    int *keep, *newid, *d_depth;
    float* bin_cost;
    uint8_t *leaf, *interior;
    const int grid = num_sms * 8;
    int h_depth = 0;
    if (ploc_tree(in, num_sms, s, err, B, T)) goto fail;
    WF_TRY(B.alloc(&keep, (size_t)n));
    WF_TRY(B.alloc(&newid, (size_t)n));
    WF_TRY(B.alloc(&d_depth, 1));
    WF_TRY(B.alloc(&bin_cost, (size_t)n));
    WF_TRY(B.alloc(&leaf, (size_t)n));
    WF_TRY(B.alloc(&interior, (size_t)n));
    WF_TRY(cudaMemsetAsync(d_depth, 0, sizeof(int), s));
    WF_TRY(cudaMemsetAsync(interior, 0, (size_t)n, s));
    if (n <= kLeafMax) {
        WF_TRY(cudaMalloc(&out.nodes, sizeof(BvhNode)));
        k_ploc_single<<<1, 1, 0, s>>>(n, T.root, T.nbox, out.nodes);
        out.num_nodes = 1;
    } else {
        const int ninternal = T.root - n + 1;
        for (const auto& it : T.iters)
            k_bin_leaves<<<std::max(1, std::min(grid, (it.second + 255) / 256)), 256, 0, s>>>(
                it.first, it.second, n, T.left, T.right, T.cnt, T.nbox, sah_leaves ? 1 : 0, bin_cost, leaf);
        k_bin_root<<<1, 1, 0, s>>>(T.root, n, interior);
        for (auto it = T.iters.rbegin(); it != T.iters.rend(); ++it)
            k_bin_interior<<<std::max(1, std::min(grid, (it->second + 255) / 256)), 256, 0, s>>>(
                it->first, it->second, n, T.left, T.right, leaf, interior);
        k_ploc_keep<<<grid, 256, 0, s>>>(n, T.root, interior, keep);
        exclusive_scan_i32(keep, ninternal, newid, T.block_sums, T.d_total, s);
        int kept = 0;
        WF_TRY(cudaMemcpyAsync(&kept, T.d_total, sizeof(int), cudaMemcpyDeviceToHost, s));
        WF_TRY(cudaStreamSynchronize(s));
        WF_TRY(cudaMalloc(&out.nodes, sizeof(BvhNode) * (size_t)std::max(kept, 1)));
        k_ploc_emit<<<grid, 256, 0, s>>>(n, T.root, T.left, T.right, T.cnt, T.offset, T.depth, newid, interior,
                                        T.nbox, out.nodes, d_depth);
        out.num_nodes = kept;
        WF_TRY(cudaMemcpyAsync(&h_depth, d_depth, sizeof(int), cudaMemcpyDeviceToHost, s));
    }
    WF_TRY(cudaMalloc(&out.tris, 3 * sizeof(float4) * (size_t)n));
    k_emit_tris<<<grid, 256, 0, s>>>(in.px, in.py, in.pz, in.idx, in.tri_geom, in.tri_prim, T.final_ids, n,
                                     out.tris);
    WF_TRY(cudaGetLastError());
    WF_TRY(cudaStreamSynchronize(s));
    out.max_depth = h_depth;
    if (h_depth + 2 > kStackSize) {
        err = "BVH deeper than the traversal stack: depth " + std::to_string(h_depth);
        goto fail;
    }
    if (validate_tree(out, n, num_sms, s, err)) goto fail;
    return 0;
fail:
    cudaFree(out.tris);
    cudaFree(out.nodes);
    out.tris = nullptr;
    out.nodes = nullptr;
    return -1;
}

int build_ploc4(const BvhBuildInput& in, BvhBuildOutput& out, int num_sms, cudaStream_t s, std::string& err)
{
    const int n = in.num_tris;
    out.tris = nullptr;
    out.nodes = nullptr;
    out.nodes4 = nullptr;
    out.num_nodes = 0;
    out.max_depth = 0;
    if (n <= 0) return 0;
    BuildScratch B;
    PlocTree T;
    const int grid = num_sms * 8;
    int *keep, *keep_off, *items, *next_items, *kids, *n_int, *n_tri, *int_off;
    float* sah_cost = nullptr;
    uint8_t* sah_choice = nullptr;
    int cap = 1, level_base = 0, count = 1, next_base = 1, levels = 0;
    if (ploc_tree(in, num_sms, s, err, B, T)) goto fail;
    if (n > 1) {  // SAH costs and choices for 4-wide nodes, pass by pass
        WF_TRY(B.alloc(&sah_cost, 3 * (size_t)(n - 1)));
        WF_TRY(B.alloc(&sah_choice, 4 * (size_t)(n - 1)));
        for (const auto& it : T.iters)
            k_wide_sah<4, kLeafMax><<<std::max(1, std::min(grid, (it.second + 127) / 128)), 128, 0, s>>>(
                it.first, it.second, n, T.left, T.right, T.cnt, T.nbox, sah_cost, sah_choice);
    }
    // Every 4-wide node stands for a distinct binary node of more than
    // kLeafMax triangles (or the root): that count bounds the node array.
    WF_TRY(B.alloc(&keep, (size_t)n));
    WF_TRY(B.alloc(&keep_off, (size_t)n));
    if (n > 1) {
        const int ninternal = T.root - n + 1;
        k_ploc_big<<<grid, 256, 0, s>>>(n, T.root, T.cnt, keep);
        exclusive_scan_i32(keep, ninternal, keep_off, T.block_sums, T.d_total, s);
        WF_TRY(cudaMemcpyAsync(&cap, T.d_total, sizeof(int), cudaMemcpyDeviceToHost, s));
        WF_TRY(cudaStreamSynchronize(s));
        cap = std::max(cap, 1);
    }
    WF_TRY(B.alloc(&items, (size_t)cap));
    WF_TRY(B.alloc(&next_items, (size_t)cap));
    WF_TRY(B.alloc(&kids, 8 * (size_t)cap));
    WF_TRY(B.alloc(&n_int, (size_t)cap));
    WF_TRY(B.alloc(&n_tri, (size_t)cap));
    WF_TRY(B.alloc(&int_off, (size_t)cap));
    WF_TRY(cudaMalloc(&out.nodes4, sizeof(Bvh4Node) * (size_t)cap));
    WF_TRY(cudaMemcpyAsync(items, &T.root, sizeof(int), cudaMemcpyHostToDevice, s));
    while (count > 0) {
        ++levels;
        if (1 + 3 * levels > kStack4) {
            err = "4-wide BVH deeper than the traversal stack";
            goto fail;
        }
        const int g = std::max(1, std::min(grid, (count + 127) / 128));
        if (n > 1)
            k_wide_gather_sah<4, kLeafMax><<<g, 128, 0, s>>>(items, count, n, T.left, T.right, T.cnt, sah_choice, kids,
                                                             n_int, n_tri);
        else
            k_wide_gather<4, kLeafMax><<<g, 128, 0, s>>>(items, count, n, T.left, T.right, T.cnt, T.nbox, kids, n_int,
                                                          n_tri);
        exclusive_scan_i32(n_int, count, int_off, T.block_sums, T.d_total, s);
        int next = 0;
        WF_TRY(cudaMemcpyAsync(&next, T.d_total, sizeof(int), cudaMemcpyDeviceToHost, s));
        WF_TRY(cudaStreamSynchronize(s));
        if ((int64_t)next_base + next > cap) {
            err = "4-wide BVH larger than its node bound";
            goto fail;
        }
        k_four_emit<<<g, 128, 0, s>>>(items, count, level_base, next_base, kids, int_off, n, T.cnt, T.nbox, T.offset,
                                      out.nodes4, next_items);
        std::swap(items, next_items);
        level_base = next_base;
        next_base += next;
        count = next;
    }
    WF_TRY(cudaMalloc(&out.tris, 3 * sizeof(float4) * (size_t)n));
    k_emit_tris<<<grid, 256, 0, s>>>(in.px, in.py, in.pz, in.idx, in.tri_geom, in.tri_prim, T.final_ids, n,
                                     out.tris);
    WF_TRY(cudaGetLastError());
    WF_TRY(cudaStreamSynchronize(s));
    out.num_nodes = level_base;  // every level written: total nodes
    out.max_depth = levels;
    if (validate_tree(out, n, num_sms, s, err)) goto fail;
    return 0;
fail:
    cudaFree(out.tris);
    cudaFree(out.nodes4);
    out.tris = nullptr;
    out.nodes4 = nullptr;
    return -1;
}

}  // namespace wf
