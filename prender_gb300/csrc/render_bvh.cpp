// Binned-SAH BVH collapsed to compressed 8-wide nodes for the FP32 render
// traversal (see render_bvh.h and WNode in pr_internal.h).
//
// A binary tree is built top-down with 16 centroid bins on each axis and
// the surface-area cost Ct + Ci (A_L N_L + A_R N_R) / A against a leaf's
// Ci N; nodes of more than kMaxLeaf triangles are always split (at the
// median when every centroid falls in one bin).  Each wide node then takes
// a binary node's children and keeps opening the child of largest surface
// area until it holds eight (or only leaves remain).  Children go to slots
// by the octant of their centroid seen from the node's (greedy assignment
// of the eight corner directions), and their boxes are quantised outward on
// a grid of power-of-two spacing anchored at the node's padded minimum.
#include "render_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace pr {
namespace {

constexpr int kBins = 16;
constexpr int kMaxLeaf = 3;  // a wide node's meta byte holds at most three triangles per leaf
// a node visit against one triangle test in the binary SAH
constexpr float kCostNode = 3.0f;
constexpr int kWidth = 8;

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
  std::vector<WNode>& out;
  std::vector<float4>& otris;

  // children of binary node n for one wide node: open the largest inner child
  // until there are kWidth (a leaf root stays a single leaf child)
  void gather(int n, std::vector<int>& ch) const {
    ch.clear();
    if (bn[n].left < 0) {
      ch.push_back(n);
      return;
    }
    ch.push_back(bn[n].left);
    ch.push_back(bn[n].right);
    while ((int)ch.size() < kWidth) {
      int best = -1;
      float ba = -1.0f;
      for (int i = 0; i < (int)ch.size(); i++) {
        const BNode& c = bn[ch[i]];
        if (c.left < 0) continue;
        const float a = c.box.area();
        if (a > ba) {
          ba = a;
          best = i;
        }
      }
      if (best < 0) break;
      const int c = ch[best];
      ch[best] = bn[c].left;
      ch.push_back(bn[c].right);
    }
  }

  // slot of each child: greedy assignment of the octant corner directions
  // (slot s points to -/+ along axis a as bit a of s is 0/1) to the children
  // whose centroid, seen from the node's centre, lies furthest that way
  static void assign_slots(const Box& node, const std::vector<Box>& boxes, int slot_of[kWidth]) {
    const int n = (int)boxes.size();
    float cost[kWidth][kWidth];
    float nc[3];
    for (int a = 0; a < 3; a++) nc[a] = 0.5f * (node.mn[a] + node.mx[a]);
    for (int i = 0; i < n; i++) {
      float d[3];
      for (int a = 0; a < 3; a++) d[a] = 0.5f * (boxes[i].mn[a] + boxes[i].mx[a]) - nc[a];
      for (int s = 0; s < kWidth; s++)
        cost[i][s] = -((s & 1 ? d[0] : -d[0]) + (s & 2 ? d[1] : -d[1]) + (s & 4 ? d[2] : -d[2]));
    }
    bool child_done[kWidth] = {}, slot_used[kWidth] = {};
    for (int k = 0; k < n; k++) {
      int bi = -1, bs = -1;
      float bc = 3.0e38f;
      for (int i = 0; i < n; i++) {
        if (child_done[i]) continue;
        for (int s = 0; s < kWidth; s++)
          if (!slot_used[s] && cost[i][s] < bc) {
            bc = cost[i][s];
            bi = i;
            bs = s;
          }
      }
      child_done[bi] = true;
      slot_used[bs] = true;
      slot_of[bi] = bs;
    }
  }

  int max_depth = 0;

  // fills node idx from binary node n; returns after its subtree is emitted
  void emit(int idx, int n, int depth) {
    max_depth = std::max(max_depth, depth);
    std::vector<int> ch;
    gather(n, ch);
    const int nch = (int)ch.size();
    std::vector<Box> boxes(nch);
    Box nb;
    for (int i = 0; i < nch; i++) {
      boxes[i] = padded(bn[ch[i]].box);
      nb.grow(boxes[i]);
    }
    int slot_of[kWidth];
    assign_slots(nb, boxes, slot_of);
    int at_slot[kWidth];
    for (int s = 0; s < kWidth; s++) at_slot[s] = -1;
    for (int i = 0; i < nch; i++) at_slot[slot_of[i]] = i;

    WNode w;
    memset(&w, 0, sizeof(w));
    // grid of spacing 2^e >= extent / 253 with its origin one step below the
    // node's padded minimum
    uint32_t ebits[3];
    float scale[3];
    for (int a = 0; a < 3; a++) {
      const double ext = std::max((double)nb.mx[a] - (double)nb.mn[a], 1.0e-30);
      int e = (int)std::ceil(std::log2(ext / 253.0));
      e = std::max(-120, std::min(120, e));
      while (std::ldexp(253.0, e) < ext && e < 120) e++;
      ebits[a] = (uint32_t)(e + 127);
      scale[a] = std::ldexp(1.0f, e);
      w.p[a] = nb.mn[a] - scale[a];
    }
    uint8_t qlo[3][kWidth], qhi[3][kWidth], meta[kWidth] = {};
    uint32_t imask = 0;
    int n_inner = 0, n_tris = 0;
    for (int s = 0; s < kWidth; s++) {
      const int i = at_slot[s];
      if (i < 0) {  // empty: qlo > qhi, no ray enters
        for (int a = 0; a < 3; a++) {
          qlo[a][s] = 1;
          qhi[a][s] = 0;
        }
        continue;
      }
      for (int a = 0; a < 3; a++) {
        // outward to the grid, checked in float arithmetic
        int lo = (int)std::floor(((double)boxes[i].mn[a] - (double)w.p[a]) / scale[a]);
        int hi = (int)std::ceil(((double)boxes[i].mx[a] - (double)w.p[a]) / scale[a]);
        lo = std::max(0, std::min(255, lo));
        hi = std::max(0, std::min(255, hi));
        while (lo > 0 && w.p[a] + (float)lo * scale[a] > boxes[i].mn[a]) lo--;
        while (hi < 255 && w.p[a] + (float)hi * scale[a] < boxes[i].mx[a]) hi++;
        qlo[a][s] = (uint8_t)lo;
        qhi[a][s] = (uint8_t)hi;
      }
      const BNode& c = bn[ch[i]];
      if (c.left < 0) {
        meta[s] = (uint8_t)((((1u << c.count) - 1u) << 5) | (uint32_t)n_tris);
        n_tris += c.count;
      } else {
        imask |= 1u << s;
        n_inner++;
      }
    }
    w.e_imask = ebits[0] | ebits[1] << 8 | ebits[2] << 16 | imask << 24;
    for (int s = 0; s < kWidth; s++) {
      const int word = s >> 2, sh = 8 * (s & 3);
      w.meta[word] |= (uint32_t)meta[s] << sh;
      w.qlo_x[word] |= (uint32_t)qlo[0][s] << sh;
      w.qlo_y[word] |= (uint32_t)qlo[1][s] << sh;
      w.qlo_z[word] |= (uint32_t)qlo[2][s] << sh;
      w.qhi_x[word] |= (uint32_t)qhi[0][s] << sh;
      w.qhi_y[word] |= (uint32_t)qhi[1][s] << sh;
      w.qhi_z[word] |= (uint32_t)qhi[2][s] << sh;
    }
    // this node's leaf triangles, contiguous in slot order
    w.tri_base = (int32_t)(otris.size() / 3);
    for (int s = 0; s < kWidth; s++) {
      const int i = at_slot[s];
      if (i < 0 || bn[ch[i]].left >= 0) continue;
      const BNode& c = bn[ch[i]];
      for (int t = c.first; t < c.first + c.count; t++) {
        const int32_t f = tris[t].face;
        for (int k = 0; k < 3; k++) {
          const float* v = vertices + 3 * (size_t)faces[3 * (size_t)f + k];
          float4 q;
          q.x = v[0];
          q.y = v[1];
          q.z = v[2];
          int32_t wv = (k == 0) ? f : 0;
          memcpy(&q.w, &wv, 4);
          otris.push_back(q);
        }
      }
    }
    // inner children: a contiguous block, then each subtree
    w.child_base = (int32_t)out.size();
    out.resize(out.size() + (size_t)n_inner);
    out[(size_t)idx] = w;
    int k = 0;
    for (int s = 0; s < kWidth; s++) {
      const int i = at_slot[s];
      if (i < 0 || bn[ch[i]].left < 0) continue;
      emit(w.child_base + k, ch[i], depth + 1);
      k++;
    }
  }
};

}  // namespace

int build_render_bvh(const float* vertices, const int32_t* faces, int32_t n_faces, std::vector<WNode>& nodes,
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
  const int root = (int)nodes.size();
  nodes.emplace_back();
  e.emit(root, 0, 1);
  return e.max_depth;
}

int emit_render_bvh(const float* vertices, const int32_t* faces, const std::vector<BinNode>& tree,
                    const std::vector<int32_t>& order, std::vector<WNode>& nodes, std::vector<float4>& tris) {
  std::vector<BNode> bn(tree.size());
  for (size_t i = 0; i < tree.size(); i++) {
    const BinNode& q = tree[i];
    for (int a = 0; a < 3; a++) {
      bn[i].box.mn[a] = q.mn[a];
      bn[i].box.mx[a] = q.mx[a];
    }
    bn[i].left = q.left;
    bn[i].right = q.right;
    bn[i].first = q.first;
    bn[i].count = q.count;
  }
  std::vector<Tri> t(order.size());  // the emitter reads only the face of each position
  for (size_t i = 0; i < order.size(); i++) t[i].face = order[i];
  Emitter e{bn, t, vertices, faces, nodes, tris};
  const int root = (int)nodes.size();
  nodes.emplace_back();
  e.emit(root, 0, 1);
  return e.max_depth;
}

}  // namespace pr
