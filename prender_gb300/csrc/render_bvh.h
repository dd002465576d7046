// The render path's own 4-wide BVH over a mesh (no reference counterpart).
//
// The reference's SAH tree (BVH.cpp / QBVH.cpp) is kept for the exact
// first-hit path, where ids and distances must match it bit for bit.  The
// FP32 render traversal only needs the closest hit (or any hit below a
// distance), which does not depend on the tree, so it gets a tree built for
// GPU traversal: binned SAH, collapsed to 8-wide nodes with quantised
// child boxes, leaves of at most three triangles.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "pr_internal.h"

namespace pr {

// Appends the mesh's nodes to nodes (root first, child and triangle indices
// absolute) in WNode's compressed 8-wide layout, and its triangles to tris
// (three float4 vertices per slot, the face id in the first one's w).
// Returns the tree's depth in nodes (the root is depth 1).
int build_render_bvh(const float* vertices, const int32_t* faces, int32_t n_faces, std::vector<WNode>& nodes,
                     std::vector<float4>& tris);

// The binary tree the wide nodes are collapsed from: node 0 is the root; a
// leaf has left = right = -1 and holds faces order[first .. first + count).
struct BinNode {
  float mn[3], mx[3];
  int32_t left, right, first, count;
};

// The same binary tree built on the GPU (render_bvh_gpu.cu): the host
// builder's split decisions, made with the same float operations in the
// same order, so the tree is the host's (triangles within a leaf may come in
// another order, and so may the halves of a node whose centroids all
// coincide).  The vertices and faces are host arrays; s is the stream used.
cudaError_t build_render_bvh_binary_gpu(const float* vertices, int32_t n_vertices, const int32_t* faces,
                                        int32_t n_faces, cudaStream_t s, std::vector<BinNode>& tree,
                                        std::vector<int32_t>& order);

// Collapses such a binary tree to wide nodes exactly as build_render_bvh
// does (appending to nodes and tris); returns the depth.
int emit_render_bvh(const float* vertices, const int32_t* faces, const std::vector<BinNode>& tree,
                    const std::vector<int32_t>& order, std::vector<WNode>& nodes, std::vector<float4>& tris);

// Meshes of at least this many faces get their render tree from the GPU.
constexpr int32_t kGpuBuildMinFaces = 4096;

}  // namespace pr
