// wf_bvh.h — device BVH build (wf_bvh.cu).
#pragma once

#include <cstdint>
#include <string>

#include "wf_device.cuh"

namespace wf {

struct BvhBuildInput {
    const float* px;           // device vertex positions
    const float* py;
    const float* pz;
    const int32_t* idx;        // device indices, 3 per triangle (global)
    const int32_t* tri_geom;   // device, per global triangle: mesh index
    const int32_t* tri_prim;   // device, per global triangle: index in mesh
    int32_t num_tris;
    float bmin[3], bmax[3];    // vertex bounds (host values)
};

struct BvhBuildOutput {
    float4* tris;      // 3 * num_tris float4 (cudaMalloc'd; caller frees)
    BvhNode* nodes;    // num_nodes (cudaMalloc'd; caller frees), binary trees
    int num_nodes;
    int max_depth;
    Bvh4Node* nodes4 = nullptr;  // 4-wide tree instead of nodes
};

// Returns 0 on success, -1 with err set otherwise.
int build_lbvh(const BvhBuildInput& in, BvhBuildOutput& out, int num_sms, cudaStream_t s,
               std::string& err);

// PLOC (Meister & Bittner 2018) over the same Morton order: higher-quality
// trees (smaller surface-area cost) for the same traversal layout.  Leaves:
// every subtree of <= kLeafMax triangles, or with sah_leaves only those the
// surface area heuristic prefers to splitting.
int build_ploc(const BvhBuildInput& in, BvhBuildOutput& out, int num_sms, cudaStream_t s,
               std::string& err, bool sah_leaves = false);

// PLOC tree collapsed top-down into 4-wide nodes (Bvh4Node), level by
// level, with the SAH-optimal choice of each node's (up to four) children
// (dynamic programming over each binary subtree, Ylitie et al. 2017); subtrees of <= kLeafMax triangles stay leaves
// over the same triangle order as build_ploc.  out.nodes4 / out.num_nodes /
// out.max_depth (levels).
int build_ploc4(const BvhBuildInput& in, BvhBuildOutput& out, int num_sms, cudaStream_t s, std::string& err);

}  // namespace wf
