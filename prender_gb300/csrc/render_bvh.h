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

#include "pr_internal.h"

namespace pr {

// Appends the mesh's nodes to nodes (root first, child and triangle indices
// absolute) in WNode's compressed 8-wide layout, and its triangles to tris
// (three float4 vertices per slot, the face id in the first one's w).
// Returns the tree's depth in nodes (the root is depth 1).
int build_render_bvh(const float* vertices, const int32_t* faces, int32_t n_faces, std::vector<WNode>& nodes,
                     std::vector<float4>& tris);

}  // namespace pr
