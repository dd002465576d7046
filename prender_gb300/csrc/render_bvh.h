// The render path's own 4-wide BVH over a mesh (no reference counterpart).
//
// The reference's SAH tree (BVH.cpp / QBVH.cpp) is kept for the exact
// first-hit path, where ids and distances must match it bit for bit.  The
// FP32 render traversal only needs the closest hit (or any hit below a
// distance), which does not depend on the tree, so it gets a tree built for
// GPU traversal: binned SAH, small leaves, tight boxes.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "pr_internal.h"

namespace pr {

// Appends the mesh's nodes to nodes (root first, child indices absolute,
// leaves as kLeafBit | slot with a count) and its triangles to tris (three
// float4 vertices per slot, the face id in the first one's w), in GNode's
// layout: children 0-1 lie on the low side of axis_top, 2-3 on the high side,
// each pair ordered along its own split axis (the order the traversal uses).
void build_render_bvh(const float* vertices, const int32_t* faces, int32_t n_faces, std::vector<GNode>& nodes,
                      std::vector<float4>& tris);

}  // namespace pr
