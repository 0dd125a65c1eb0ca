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

#include <string>

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

}  // namespace wf
