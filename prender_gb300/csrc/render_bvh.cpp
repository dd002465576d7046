// Binned-SAH 4-wide BVH for the FP32 render traversal (see render_bvh.h).
//
// A binary tree is built top-down with 16 centroid bins on each axis and
// the surface-area cost Ct + Ci (A_L N_L + A_R N_R) / A against a leaf's
// Ci N; nodes of more than kMaxLeaf triangles are always split (at the
// median when every centroid falls in one bin).  Each binary node and its
// two children are then emitted as one 4-wide node (grandchildren in slots
// 0-3), which is the layout and child order the traversal expects.
#include "render_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace pr {
namespace {

constexpr int kBins = 16;
constexpr int kMaxLeaf = 8;
// a 4-wide node visit against one triangle test: measured on GB300 (mesh
// Cornell box, wavefront frame) over 1.2 / 3 / 6 / 12 with leaves of at most
// 8 or 16 triangles; 3 with 8 was fastest
constexpr float kCostNode = 3.0f;

struct Box {
  float mn[3] = {3.0e38f, 3.0e38f, 3.0e38f};
  float mx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  void grow(const Box& b) {
    for (int a = 0; a < 3; a++) {
      mn[a] = std::min(mn[a], b.mn[a]);
      mx[a] = std::max(mx[a], b.mx[a]);
    }
  }
  void grow(const float* p) {
    for (int a = 0; a < 3; a++) {
      mn[a] = std::min(mn[a], p[a]);
      mx[a] = std::max(mx[a], p[a]);
    }
  }
  bool empty() const { return mn[0] > mx[0]; }
  float area() const {
    if (empty()) return 0.0f;
    const float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
    return 2.0f * (dx * dy + dy * dz + dz * dx);
  }
};

struct Tri {
  Box box;
  float c[3];
  int32_t face;
};

struct BNode {
  Box box;
  int32_t left = -1, right = -1;  // children (both -1: leaf)
  int32_t first = 0, count = 0;   // leaf: range in the triangle order
  int32_t axis = 0;
};

class Builder {
 public:
  explicit Builder(std::vector<Tri>& t) : tris_(t) {}
  std::vector<BNode> nodes;

  int build(int first, int count) {
    const int id = (int)nodes.size();
    nodes.emplace_back();
    Box box, cb;
    for (int i = first; i < first + count; i++) {
      box.grow(tris_[i].box);
      cb.grow(tris_[i].c);
    }
    nodes[id].box = box;
    int axis = -1, split_bin = -1;
    float best = 3.0e38f;
    if (count > 1) {
      for (int a = 0; a < 3; a++) {
        const float ext = cb.mx[a] - cb.mn[a];
        if (!(ext > 0.0f)) continue;
        Box bb[kBins];
        int bn[kBins] = {};
        const float k = kBins * (1.0f - 1.0e-6f) / ext;
        for (int i = first; i < first + count; i++) {
          const int b = std::min(kBins - 1, (int)((tris_[i].c[a] - cb.mn[a]) * k));
          bb[b].grow(tris_[i].box);
          bn[b]++;
        }
        float rarea[kBins];
        int rcount[kBins];
        Box acc;
        int n = 0;
        for (int b = kBins - 1; b > 0; b--) {
          acc.grow(bb[b]);
          n += bn[b];
          rarea[b] = acc.area();
          rcount[b] = n;
        }
        Box lacc;
        int ln = 0;
        for (int b = 0; b < kBins - 1; b++) {
          lacc.grow(bb[b]);
          ln += bn[b];
          if (ln == 0 || rcount[b + 1] == 0) continue;
          const float c = lacc.area() * ln + rarea[b + 1] * rcount[b + 1];
          if (c < best) {
            best = c;
            axis = a;
            split_bin = b;
          }
        }
      }
    }
    const float area = box.area();
    const float split_cost = axis >= 0 && area > 0.0f ? kCostNode + best / area : 3.0e38f;
    if (count == 1 || (count <= kMaxLeaf && (float)count <= split_cost)) {
      nodes[id].first = first;
      nodes[id].count = count;
      return id;
    }
    int mid;
    int a = axis;
    if (a >= 0) {
      const float ext = cb.mx[a] - cb.mn[a];
      const float k = kBins * (1.0f - 1.0e-6f) / ext;
      const float lo = cb.mn[a];
      Tri* p = std::partition(tris_.data() + first, tris_.data() + first + count, [&](const Tri& t) {
        return std::min(kBins - 1, (int)((t.c[a] - lo) * k)) <= split_bin;
      });
      mid = (int)(p - tris_.data());
    } else {
      mid = first;
    }
    if (mid == first || mid == first + count) {  // no usable bin split: median of the widest axis
      a = 0;
      for (int q = 1; q < 3; q++)
        if (cb.mx[q] - cb.mn[q] > cb.mx[a] - cb.mn[a]) a = q;
      mid = first + count / 2;
      std::nth_element(tris_.data() + first, tris_.data() + mid, tris_.data() + first + count,
                       [&](const Tri& x, const Tri& y) { return x.c[a] < y.c[a]; });
    }
    nodes[id].axis = a;
    const int l = build(first, mid - first);
    const int r = build(mid, first + count - mid);
    nodes[id].left = l;
    nodes[id].right = r;
    return id;
  }

 private:
  std::vector<Tri>& tris_;
};

// outward by a few float ulps of the coordinates, so that the FP32 slab
// test (with its own rounding) never loses a box its triangle touches
Box padded(const Box& b) {
  Box o = b;
  for (int a = 0; a < 3; a++) {
    const float s = std::max(std::fabs(b.mn[a]), std::fabs(b.mx[a])) * 4.8e-7f + 1.0e-7f;
    o.mn[a] = b.mn[a] - s;
    o.mx[a] = b.mx[a] + s;
  }
  return o;
}

struct Emitter {
  const std::vector<BNode>& bn;
  const std::vector<Tri>& tris;
  const float* vertices;
  const int32_t* faces;
  std::vector<GNode>& out;
  std::vector<float4>& otris;

  int32_t leaf(const BNode& b, uint16_t& count) {
    const int32_t slot = (int32_t)(otris.size() / 3);
    for (int i = b.first; i < b.first + b.count; i++) {
      const int32_t f = tris[i].face;
      for (int k = 0; k < 3; k++) {
        const float* v = vertices + 3 * (size_t)faces[3 * (size_t)f + k];
        float4 q;
        q.x = v[0];
        q.y = v[1];
        q.z = v[2];
        int32_t w = (k == 0) ? f : 0;
        memcpy(&q.w, &w, 4);
        otris.push_back(q);
      }
    }
    count = (uint16_t)b.count;
    return (int32_t)(kLeafBit | (uint32_t)slot);
  }

  // one 4-wide node from binary node n (a leaf root becomes a node with one leaf child)
  int32_t emit(int n) {
    const int32_t idx = (int32_t)out.size();
    out.emplace_back();
    int slots[4] = {-1, -1, -1, -1};
    int at = 0, al = 0, ar = 0;
    const BNode& b = bn[n];
    if (b.left < 0) {
      slots[0] = n;
    } else {
      at = b.axis;
      const BNode& L = bn[b.left];
      const BNode& R = bn[b.right];
      if (L.left < 0) {
        slots[0] = b.left;
      } else {
        slots[0] = L.left;
        slots[1] = L.right;
        al = L.axis;
      }
      if (R.left < 0) {
        slots[2] = b.right;
      } else {
        slots[2] = R.left;
        slots[3] = R.right;
        ar = R.axis;
      }
    }
    GNode g;
    memset(&g, 0, sizeof(g));
    for (int s = 0; s < 4; s++) {
      if (slots[s] < 0) {
        g.child[s] = kChildInvalid;
        // an empty box no ray enters
        g.bmin_x[s] = g.bmin_y[s] = g.bmin_z[s] = 3.0e38f;
        g.bmax_x[s] = g.bmax_y[s] = g.bmax_z[s] = -3.0e38f;
        continue;
      }
      const BNode& c = bn[slots[s]];
      const Box pb = padded(c.box);
      g.bmin_x[s] = pb.mn[0];
      g.bmax_x[s] = pb.mx[0];
      g.bmin_y[s] = pb.mn[1];
      g.bmax_y[s] = pb.mx[1];
      g.bmin_z[s] = pb.mn[2];
      g.bmax_z[s] = pb.mx[2];
      if (c.left < 0) {
        uint16_t cnt = 0;
        g.child[s] = leaf(c, cnt);
        g.count[s] = cnt;
      } else {
        g.child[s] = emit(slots[s]);
      }
    }
    g.axes = at | (al << 2) | (ar << 4);
    out[idx] = g;
    return idx;
  }
};

}  // namespace

void build_render_bvh(const float* vertices, const int32_t* faces, int32_t n_faces, std::vector<GNode>& nodes,
                      std::vector<float4>& tris) {
  std::vector<Tri> t((size_t)n_faces);
  for (int32_t f = 0; f < n_faces; f++) {
    Tri& q = t[(size_t)f];
    q.face = f;
    for (int k = 0; k < 3; k++) q.box.grow(vertices + 3 * (size_t)faces[3 * (size_t)f + k]);
    for (int a = 0; a < 3; a++) q.c[a] = 0.5f * (q.box.mn[a] + q.box.mx[a]);
  }
  Builder b(t);
  b.nodes.reserve(2 * (size_t)n_faces);
  b.build(0, n_faces);
  Emitter e{b.nodes, t, vertices, faces, nodes, tris};
  e.emit(0);
}

}  // namespace pr
