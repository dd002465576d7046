// Host-side scene import: pr_scene_desc -> flat GPU arrays.
//
// Restates the reference's scene set-up: entity geometry and areas
// (plane.h:146-177, sphere.h:23-27), light registration and ordering
// (scene_env.h:1567-1719, light.h:95-130), medium set-up
// (ParticipatingMediaPrm.h:133-160), face normals (ObjLoader.cpp:577-700),
// and the per-mesh QBVH: binary SAH build (BVH.cpp:194-348) flattened two
// levels at a time into 4-wide nodes (QBVH.cpp:161-302).  The build follows
// the reference's rules exactly (std::sort on centroids, the same cost
// bookkeeping, 0.01 box padding) so node and leaf order are identical.
//
// Compiled with -ffp-contract=off: the FP64 build must not depend on
// whether the host CPU fuses multiply-adds.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "pr_internal.h"
#include "scene_build.h"
#include "render_bvh.h"

namespace pr {
namespace {

constexpr double kInf = 1.0e128;  // constant.h:33

struct D3 {
  double x, y, z;
};
inline D3 add(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 scale(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
// the reference's SSE dot adds the x,z lanes first (vector3d.h dot/sqr)
inline double dot(D3 a, D3 b) { return (a.x * b.x + a.z * b.z) + a.y * b.y; }
inline double len(D3 a) { return std::sqrt(dot(a, a)); }
inline D3 unit(D3 a) { return scale(a, 1.0 / len(a)); }
inline D3 cross(D3 a, D3 b) {
  return {(a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)};
}
inline D3 mk(const double* p) { return {p[0], p[1], p[2]}; }

struct TriBox {
  double bmin[3], bmax[3], c[3];
};

struct BNode {
  double box[2][3];
  int children[2] = {-1, -1};
  int axis = 0;
  std::vector<int> objects;
};

// BoundingBox::CalcSurfaceArea, member and template forms (BoundingBox.h:29-39)
inline double area_member(const double* mn, const double* mx) {
  double dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
  return dx * dy + dx * dz + dy * dz;
}
inline double area_template(const double* mn, const double* mx) {
  double d0 = mx[0] - mn[0], d1 = mx[1] - mn[1], d2 = mx[2] - mn[2];
  return d0 * d1 + d1 * d2 + d0 * d2;
}

class SahBuilder {
 public:
  explicit SahBuilder(const std::vector<TriBox>& t) : tris_(t) {}
  std::vector<BNode> nodes;

  void run(int n) {
    nodes.clear();
    nodes.reserve(2 * (size_t)n);
    nodes.emplace_back();
    std::vector<int> all(n);
    for (int i = 0; i < n; i++) all[i] = i;
    build(all, 0);
  }

 private:
  const std::vector<TriBox>& tris_;

  void bounds(const std::vector<int>& objs, double* mn, double* mx) const {
    for (int k = 0; k < 3; k++) { mn[k] = tris_[objs[0]].bmin[k]; mx[k] = tris_[objs[0]].bmax[k]; }
    for (size_t i = 1; i < objs.size(); i++) {
      const TriBox& a = tris_[objs[i]];
      for (int k = 0; k < 3; k++) {
        if (a.bmin[k] < mn[k]) mn[k] = a.bmin[k];
        if (a.bmax[k] > mx[k]) mx[k] = a.bmax[k];
      }
    }
  }
  static void merge(double* mn, double* mx, const TriBox& b) {
    for (int k = 0; k < 3; k++) {
      mn[k] = std::min(mn[k], b.bmin[k]);
      mx[k] = std::max(mx[k], b.bmax[k]);
    }
  }
  void sort_axis(std::vector<int>& v, int axis) const {
    const std::vector<TriBox>& t = tris_;
    std::sort(v.begin(), v.end(), [&t, axis](int a, int b) { return t[a].c[axis] < t[b].c[axis]; });
  }
  void build(const std::vector<int>& targets, int index) {
    bounds(targets, nodes[index].box[0], nodes[index].box[1]);
    const double inv_surf = 1.0 / area_template(nodes[index].box[0], nodes[index].box[1]);
    const size_t n = targets.size();
    int best_axis = -1, best_index = -1;
    double best_cost = -1;
    std::vector<double> left_area(n), right_area(n);
    for (int axis = 0; axis < 3; axis++) {
      std::vector<int> L = targets, R;
      sort_axis(L, axis);
      right_area[n - 1] = kInf;
      R.push_back(L.back());
      L.pop_back();
      double mn[3], mx[3];
      bounds(R, mn, mx);
      for (int i = (int)L.size() - 1; i >= 0; i--) {
        right_area[i] = area_member(mn, mx);
        merge(mn, mx, tris_[L[i]]);
        R.push_back(L.back());
        L.pop_back();
      }
      L.push_back(R.back());
      R.pop_back();
      bounds(L, mn, mx);
      const double leaf_cost = (double)n;
      for (int i = (int)R.size() - 1, cut = 0; i >= 0; i--, cut++) {
        left_area[cut] = area_member(mn, mx);
        merge(mn, mx, tris_[R.back()]);
        L.push_back(R.back());
        R.pop_back();
        // sizes are taken after the move, as the reference does (BVH.cpp:288-292)
        const double cost = 2.0 + (left_area[cut] * (double)L.size() + right_area[cut] * (double)R.size()) * inv_surf;
        if ((cost < best_cost || best_cost == -1) && cost < leaf_cost) {
          best_cost = cost;
          best_index = cut;
          best_axis = axis;
        }
      }
    }
    if (best_axis == -1) {
      nodes[index].objects = targets;
      return;
    }
    std::vector<int> lefts = targets;
    sort_axis(lefts, best_axis);
    std::vector<int> rights(lefts.begin() + best_index + 1, lefts.end());
    lefts.resize(best_index + 1);
    const int c0 = (int)nodes.size();
    nodes[index].axis = best_axis;
    nodes[index].children[0] = c0;
    nodes[index].children[1] = c0 + 1;
    nodes.emplace_back();
    nodes.emplace_back();
    build(lefts, c0);
    build(rights, c0 + 1);
  }
};

inline bool is_leaf(const BNode& b) { return b.children[0] == -1; }

// Flattens a binary SAH tree into 4-wide nodes, the reference way
// (QBVH.cpp:202-302): grandchildren in slots 2i+j, a leaf child in slot 2i
// with slot 2i+1 invalid, new nodes numbered in depth-first order.
class Flattener {
 public:
  Flattener(const std::vector<BNode>& b, MeshQbvh& out) : bvh_(b), out_(out) {}
  void run() {
    out_.nodes.clear();
    out_.ref_leaf.clear();
    out_.leaf_tris.clear();
    out_.nodes.emplace_back();
    flatten(0, 0);
  }

 private:
  const std::vector<BNode>& bvh_;
  MeshQbvh& out_;

  void make_leaf(size_t index, const BNode& leaf, int slot) {
    RefNode& rn = out_.nodes[index];
    rn.ref_child[slot] = (int64_t)(((uint64_t)1 << 63) | (uint64_t)out_.ref_leaf.size());
    rn.leaf_first[slot] = (int32_t)out_.leaf_tris.size();
    rn.leaf_count[slot] = (int32_t)leaf.objects.size();
    for (int o : leaf.objects) {
      out_.ref_leaf.push_back(o);
      out_.leaf_tris.push_back(o);
    }
    out_.ref_leaf.push_back(-1);
  }
  void put_box(size_t index, const BNode& b, int slot) {
    for (int a = 0; a < 3; a++) {
      out_.nodes[index].box[0][a][slot] = (float)b.box[0][a];
      out_.nodes[index].box[1][a][slot] = (float)b.box[1][a];
    }
  }
  void flatten(size_t index, int target) {
    const BNode& nt = bvh_[target];
    {
      RefNode& rn = out_.nodes[index];
      rn.axis_top = nt.axis;
      rn.axis_left = is_leaf(bvh_[nt.children[0]]) ? 0 : bvh_[nt.children[0]].axis;
      rn.axis_right = is_leaf(bvh_[nt.children[1]]) ? 0 : bvh_[nt.children[1]].axis;
    }
    for (int i = 0; i < 2; i++) {
      const BNode& child = bvh_[nt.children[i]];
      if (is_leaf(child)) {
        const int slot = 2 * i;
        make_leaf(index, child, slot);
        out_.nodes[index].ref_child[slot + 1] = -1;
        put_box(index, child, slot);
      } else {
        for (int j = 0; j < 2; j++) {
          const int slot = 2 * i + j;
          const int gci = child.children[j];
          put_box(index, bvh_[gci], slot);
          if (is_leaf(bvh_[gci])) {
            make_leaf(index, bvh_[gci], slot);
          } else {
            const size_t nn = out_.nodes.size();
            out_.nodes.emplace_back();
            out_.nodes[index].ref_child[slot] = (int64_t)nn;
            flatten(nn, gci);
          }
        }
      }
    }
  }
};

}  // namespace

int build_mesh_qbvh(const float* vertices, const int32_t* faces, int n_faces, MeshQbvh& out, std::string& err) {
  // Triangle::CreateBoundingBox (polygon.h:686-703): 0.01 padding
  std::vector<TriBox> boxes((size_t)n_faces);
  for (int f = 0; f < n_faces; f++) {
    double mn[3] = {kInf, kInf, kInf}, mx[3] = {-kInf, -kInf, -kInf};
    for (int k = 0; k < 3; k++) {
      const float* v = vertices + 3 * (size_t)faces[3 * (size_t)f + k];
      for (int a = 0; a < 3; a++) {
        const double x = v[a];
        if (mn[a] > x) mn[a] = x;
        if (mx[a] < x) mx[a] = x;
      }
    }
    for (int a = 0; a < 3; a++) {
      boxes[f].bmin[a] = mn[a] - 0.01;
      boxes[f].bmax[a] = mx[a] + 0.01;
      // BoundingBox centre: (min + max) / 2.0 (BoundingBox.h:14-19)
      boxes[f].c[a] = (boxes[f].bmin[a] + boxes[f].bmax[a]) / 2.0;
    }
  }
  SahBuilder b(boxes);
  b.run(n_faces);
  if (is_leaf(b.nodes[0])) {
    err = "mesh too small: its SAH root is a leaf, so the reference would fall back to a binary BVH";
    return PR_E_BUILD;
  }
  Flattener fl(b.nodes, out);
  fl.run();
  for (const RefNode& rn : out.nodes)
    for (int s = 0; s < 4; s++)
      if (rn.leaf_count[s] > 0xFFFF) {
        err = "QBVH leaf larger than 65535 triangles";
        return PR_E_BUILD;
      }
  return PR_OK;
}

// Obj::CalcNormalVector for meshes without vertex normals (ObjLoader.cpp:582-598, :686-697)
void face_normals(const float* V, const int32_t* F, int n_faces, std::vector<float>& out) {
  out.resize(3 * (size_t)n_faces);
  for (int f = 0; f < n_faces; f++) {
    const int32_t* fc = F + 3 * (size_t)f;
    float dx1 = V[3 * fc[1]] - V[3 * fc[0]], dy1 = V[3 * fc[1] + 1] - V[3 * fc[0] + 1],
          dz1 = V[3 * fc[1] + 2] - V[3 * fc[0] + 2];
    float dx2 = V[3 * fc[2]] - V[3 * fc[0]], dy2 = V[3 * fc[2] + 1] - V[3 * fc[0] + 1],
          dz2 = V[3 * fc[2] + 2] - V[3 * fc[0] + 2];
    float nx = dy1 * dz2 - dz1 * dy2, ny = dz1 * dx2 - dx1 * dz2, nz = dx1 * dy2 - dy1 * dx2;
    float a = std::sqrt(nx * nx + ny * ny + nz * nz);
    if (a != 0.0f) {
      nx /= a;
      ny /= a;
      nz /= a;
    }
    out[3 * f] = nx;
    out[3 * f + 1] = ny;
    out[3 * f + 2] = nz;
  }
}

void vertex_normals(const float* V, const int32_t* F, int n_faces, int n_vertices, std::vector<float>& out) {
  out.assign(3 * (size_t)n_vertices, 0.0f);
  std::vector<int> count((size_t)n_vertices, 0);
  for (int f = 0; f < n_faces; f++) {
    const int32_t* fc = F + 3 * (size_t)f;
    const float dx1 = V[3 * fc[1]] - V[3 * fc[0]], dy1 = V[3 * fc[1] + 1] - V[3 * fc[0] + 1],
                dz1 = V[3 * fc[1] + 2] - V[3 * fc[0] + 2];
    const float dx2 = V[3 * fc[2]] - V[3 * fc[0]], dy2 = V[3 * fc[2] + 1] - V[3 * fc[0] + 1],
                dz2 = V[3 * fc[2] + 2] - V[3 * fc[0] + 2];
    const float n[3] = {dy1 * dz2 - dz1 * dy2, dz1 * dx2 - dx1 * dz2, dx1 * dy2 - dy1 * dx2};
    for (int k = 0; k < 3; k++) {
      for (int a = 0; a < 3; a++) out[3 * (size_t)fc[k] + a] += n[a];
      count[(size_t)fc[k]]++;
    }
  }
  for (int i = 0; i < n_vertices; i++) {
    if (count[(size_t)i] == 0) continue;
    float* n = &out[3 * (size_t)i];
    for (int a = 0; a < 3; a++) n[a] = (float)((double)n[a] / (double)count[(size_t)i]);
    const float a = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (a != 0.0f)
      for (int k = 0; k < 3; k++) n[k] /= a;
  }
}

void face_normals_vn(const float* VN, const int32_t* FVN, int n_faces, std::vector<float>& out) {
  out.resize(3 * (size_t)n_faces);
  for (int i = 0; i < n_faces; i++) {
    float c[3];
    for (int a = 0; a < 3; a++) {
      const float s = (VN[3 * (size_t)FVN[3 * i] + a] + VN[3 * (size_t)FVN[3 * i + 1] + a]) + VN[3 * (size_t)FVN[3 * i + 2] + a];
      c[a] = (float)(s / 3.0);
    }
    double ln = (double)((c[0] * c[0] + c[1] * c[1]) + c[2] * c[2]);
    if (ln > 1.0e-16) {
      ln = std::sqrt(ln);
      for (int a = 0; a < 3; a++) c[a] = (float)(c[a] / ln);
    }
    for (int a = 0; a < 3; a++) out[3 * (size_t)i + a] = c[a];
  }
}

static bool is_light(const pr_material& m) {  // Material::isLight (material.h)
  const D3 c = mk(m.color), e = mk(m.emission);
  return m.type == PR_MAT_DIFFUSE && len(c) < 0.001 && len(e) > 0.001;
}

// The material a face of OBJ material O shows (Triangle::intersect,
// polygon.h:228-400) on an entity of material B (pm / base): with a map_Kd
// texture the colour is B's times the texel, else O's Kd and Ks (Ks 0 for a
// diffuse B); a '#REFLECTION' type also takes its type, '#EMISSION' (times
// the texel with a texture), Ks (likewise), Ni and '#ROUGHNESS', and the
// type's own colours: Ks for mirrors and glass, Kd (times the texel) for
// Ward ('#WARD') and Phong (Ns).  Appended to hs.mats; out = its index.
static int derive_obj_material(HostScene& hs, const pr_material& pm, const GMaterial& base, const pr_obj_material& o,
                               int32_t& out, std::string& err) {
  if (o.alpha >= 0.0 && o.alpha < 1.0) {
    err = "OBJ materials with d < 1 (the reference's stochastic alpha test) are not rendered here";
    return PR_E_UNSUPPORTED;
  }
  if (o.reflection >= 0 && o.reflection != PR_MAT_DIFFUSE && o.reflection != PR_MAT_SPECULAR &&
      o.reflection != PR_MAT_REFRACTION && o.reflection != PR_MAT_WARD && o.reflection != PR_MAT_PHONG) {
    err = "OBJ material '#REFLECTION " + std::to_string(o.reflection) + "' is not on this path";
    return PR_E_UNSUPPORTED;
  }
  if (pm.type == PR_MAT_SSS_REFRACTION || base.sss) {
    err = "OBJ materials on subsurface entities are not on this path";
    return PR_E_UNSUPPORTED;
  }
  GMaterial g = base;
  double C[3], Sp[3], E[3];
  for (int k = 0; k < 3; k++) {
    C[k] = pm.color[k];
    Sp[k] = pm.specular[k];
    E[k] = pm.emission[k];
  }
  int mask = 0;
  double rough = pm.roughness, ior = pm.refractive_index, wx = pm.ward_alpha[0], wy = pm.ward_alpha[1];
  double pn = pm.phong_exponent;
  int type = pm.type;
  if (o.texture) {
    if (o.texture_width <= 0 || o.texture_height <= 0) { err = "map_Kd texture size must be positive"; return PR_E_ARG; }
    mask = 1;  // B's colour times the texel
    if (o.reflection >= 0) {
      for (int k = 0; k < 3; k++) {
        E[k] = o.emission[k];
        Sp[k] = o.specular[k];
      }
      mask |= 2 | 4;
    }
  } else {
    for (int k = 0; k < 3; k++) {
      C[k] = o.diffuse[k];
      Sp[k] = pm.type == PR_MAT_DIFFUSE ? 0.0 : o.specular[k];
    }
    if (o.reflection >= 0)
      for (int k = 0; k < 3; k++) {
        E[k] = o.emission[k];
        Sp[k] = o.specular[k];
      }
  }
  if (o.reflection >= 0) {
    type = o.reflection;
    ior = o.refraction_index;
    rough = o.roughness;
    if (type == PR_MAT_SPECULAR || type == PR_MAT_REFRACTION) {
      for (int k = 0; k < 3; k++) C[k] = o.specular[k];
      mask &= ~1;
    }
    if (type == PR_MAT_WARD) {
      wx = o.ward[0];
      wy = o.ward[1];
    }
    if (type == PR_MAT_PHONG) pn = o.shininess;
    if (type == PR_MAT_WARD || type == PR_MAT_PHONG) {
      for (int k = 0; k < 3; k++) C[k] = o.diffuse[k];
      if (o.texture) mask |= 1;
    }
    if (type == PR_MAT_REFRACTION && !(ior > 0.0)) { err = "OBJ glass needs Ni > 0"; return PR_E_ARG; }
    if (type == PR_MAT_WARD && !(wx > 0.0 && wy > 0.0)) { err = "OBJ Ward material needs '#WARD ax ay' > 0"; return PR_E_ARG; }
  }
  g.type = type;
  for (int k = 0; k < 3; k++) {
    g.color[k] = (float)C[k];
    g.color_d[k] = C[k];
    g.emission[k] = (float)E[k];
    g.emission_d[k] = E[k];
    g.specular[k] = (float)Sp[k];
  }
  g.roughness = (float)rough;
  g.roughness_d = rough;
  g.ior = (float)ior;
  g.ior_d = ior;
  g.ward_ax = (float)wx;
  g.ward_ay = (float)wy;
  g.phong_n = (float)pn;
  g.mtex_off = -1;
  g.mtex_mask = mask;
  g.mtex_repeat = o.repeat;
  g.mesh_smooth = o.smooth == 1 ? 1 : (o.smooth == 2 ? 2 : 0);
  if (o.texture) {
    g.mtex_off = (int32_t)hs.texels.size();
    g.mtex_w = o.texture_width;
    g.mtex_h = o.texture_height;
    const size_t n = (size_t)g.mtex_w * g.mtex_h;
    if (hs.texels.size() + n > (size_t)INT32_MAX) { err = "textures too large"; return PR_E_ARG; }
    for (size_t k = 0; k < n; k++)
      hs.texels.push_back(make_float4((float)(o.texture[3 * k] / 255.0), (float)(o.texture[3 * k + 1] / 255.0),
                                      (float)(o.texture[3 * k + 2] / 255.0), 0.0f));
  }
  out = (int32_t)hs.mats.size();
  hs.mats.push_back(g);
  return PR_OK;
}


// The reference-layout QBVH of one mesh (QBVH.cpp:161-302) into the exact
// path's arrays, and the entity's indexes into them.
static int append_exact_qbvh(HostScene& hs, GEntity& g, int entity, const float* vertices, const int32_t* faces,
                             int n_faces, std::string& err) {
  MeshQbvh q;
  int st = build_mesh_qbvh(vertices, faces, n_faces, q, err);
  if (st != PR_OK) {
    err = "mesh of entity " + std::to_string(entity) + ": " + err;
    return st;
  }
  g.node_base = (int32_t)hs.nodes.size();
  g.slot_base = (int32_t)(hs.tris.size() / 3);
  for (const RefNode& rn : q.nodes) {
    GNode gn;
    memset(&gn, 0, sizeof(gn));
    for (int s = 0; s < 4; s++) {
      gn.bmin_x[s] = rn.box[0][0][s]; gn.bmax_x[s] = rn.box[1][0][s];
      gn.bmin_y[s] = rn.box[0][1][s]; gn.bmax_y[s] = rn.box[1][1][s];
      gn.bmin_z[s] = rn.box[0][2][s]; gn.bmax_z[s] = rn.box[1][2][s];
      const int64_t c = rn.ref_child[s];
      if (c == -1) {
        gn.child[s] = kChildInvalid;
      } else if (c < 0) {  // leaf
        gn.child[s] = (int32_t)(kLeafBit | (uint32_t)(g.slot_base + rn.leaf_first[s]));
        gn.count[s] = (uint16_t)rn.leaf_count[s];
      } else {
        gn.child[s] = (int32_t)(g.node_base + c);
      }
    }
    gn.axes = rn.axis_top | (rn.axis_left << 2) | (rn.axis_right << 4);
    hs.nodes.push_back(gn);
  }
  for (int t : q.leaf_tris) {
    for (int k = 0; k < 3; k++) {
      const float* v = vertices + 3 * (size_t)faces[3 * (size_t)t + k];
      float4 f4;
      f4.x = v[0];
      f4.y = v[1];
      f4.z = v[2];
      int32_t w = (k == 0) ? t : 0;
      memcpy(&f4.w, &w, 4);
      hs.tris.push_back(f4);
    }
  }
  hs.mesh_qbvh.push_back(std::move(q));
  hs.mesh_entity.push_back(entity);
  return PR_OK;
}

int complete_exact_qbvh(HostScene& hs, std::string& err) {
  for (const HostScene::DeferredMesh& m : hs.deferred_exact) {
    int st = append_exact_qbvh(hs, hs.ents[(size_t)m.entity], m.entity, m.vertices.data(), m.faces.data(),
                               (int)(m.faces.size() / 3), err);
    if (st != PR_OK) return st;
  }
  hs.deferred_exact.clear();
  return PR_OK;
}

// WormHole as SceneEnv builds it (scene_env.h:2100-2145, WormHole.h:126-170)
// and the two frames Setup makes (WormHole.h:321-395): a ray starting at
// mouth m (the 'in' mouth unless it starts more than 1e6 from the origin)
// turns into the basis whose rows are X = the unit vector from the mouth to
// the camera, Y = unit(z x X) (y x X when that vanishes), Z = unit(X x Y);
// its inverse is InvertMatrix_'s cofactor inverse, whose terms for a matrix
// without translation reduce to the 3 x 3 cofactors below (a determinant
// below 1e-16 leaves the identity, as the class does).
static int build_wormhole(const pr_scene_desc* d, HostScene& hs, std::string& err) {
  hs.worm = GWorm{};
  for (auto& t : hs.worm_tex) t.clear();
  const pr_wormhole& pw = d->wormhole;
  if (!pw.enabled) return PR_OK;
  if (d->kerr.enabled) { err = "a scene holds a black hole or a wormhole, not both"; return PR_E_UNSUPPORTED; }
  if (pw.max_steps <= 0 || pw.max_steps > 10000000) {
    err = "geodesics_max_length must be in 1..1e7 (an unbounded trace is not run on the GPU)";
    return PR_E_ARG;
  }
  if (!(pw.rho > 0.0) || !(pw.w > 0.0) || !std::isfinite(pw.a)) {
    err = "the wormhole needs Rho > 0, W > 0 and a finite a";
    return PR_E_ARG;
  }
  GWorm& w = hs.worm;
  w.enabled = 1;
  w.max_steps = pw.max_steps;
  for (int k = 0; k < 3; k++) {
    w.pos[0][k] = pw.in[k];
    w.pos[1][k] = pw.out[k];
  }
  w.Rho = pw.rho;
  w.a = std::fabs(pw.a);
  w.M = pw.w / 1.42953;
  w.usr_sign = pw.sign;
  const D3 cam = mk(pw.camera);
  for (int m = 0; m < 2; m++) {
    const D3 X = unit(sub(cam, mk(w.pos[m])));
    D3 Y = unit(cross(D3{0.0, 0.0, 1.0}, X));
    if (len(Y) < 1.0e-16) Y = unit(cross(D3{0.0, 1.0, 0.0}, X));
    const D3 Z = unit(cross(X, Y));
    double* A = w.mat[m];
    double* B = w.inv[m];
    for (int i = 0; i < 16; i++) A[i] = B[i] = (i % 5 == 0) ? 1.0 : 0.0;
    const D3 rows[3] = {X, Y, Z};
    for (int r = 0; r < 3; r++) {
      A[4 * r] = rows[r].x;
      A[4 * r + 1] = rows[r].y;
      A[4 * r + 2] = rows[r].z;
    }
    double c[11];
    c[0] = A[5] * A[10] - A[9] * A[6];
    c[4] = A[8] * A[6] - A[4] * A[10];
    c[8] = A[4] * A[9] - A[8] * A[5];
    c[1] = A[9] * A[2] - A[1] * A[10];
    c[5] = A[0] * A[10] - A[8] * A[2];
    c[9] = A[8] * A[1] - A[0] * A[9];
    c[2] = A[1] * A[6] - A[5] * A[2];
    c[6] = A[4] * A[2] - A[0] * A[6];
    c[10] = A[0] * A[5] - A[4] * A[1];
    double det = (A[0] * c[0] + A[1] * c[4]) + A[2] * c[8];
    if (!(det < 1.0e-16)) {
      det = 1.0 / det;
      for (int i : {0, 1, 2, 4, 5, 6, 8, 9, 10}) B[i] = c[i] * det;
    }
  }
  for (int k = 0; k < 2; k++) {
    for (int q = 0; q < 4; q++) w.map_coef[k][q] = pw.map_coef[k][q];
    w.tex_coef[k] = pw.texture_coef[k];
    if (pw.texture[k]) {
      if (pw.texture_width[k] <= 0 || pw.texture_height[k] <= 0) {
        err = "wormhole background texture size must be positive";
        return PR_E_ARG;
      }
      hs.worm_tex[k].assign(pw.texture[k], pw.texture[k] + 3 * (size_t)pw.texture_width[k] * pw.texture_height[k]);
      w.tex_w[k] = pw.texture_width[k];
      w.tex_h[k] = pw.texture_height[k];
    }
  }
  return PR_OK;
}

int build_host_scene(const pr_scene_desc* d, HostScene& hs, std::string& err, const SceneBuildOptions& opt) {
  hs = HostScene();
  if (!d || d->n_entities < 0 || d->n_materials < 0 || d->n_meshes < 0) { err = "null or negative scene sizes"; return PR_E_ARG; }
  if (d->n_entities > kMaxEntities) { err = "too many entities"; return PR_E_ARG; }
  if ((d->n_materials > 0 && !d->materials) || (d->n_entities > 0 && !d->entities) ||
      (d->n_meshes > 0 && !d->meshes)) { err = "null scene array"; return PR_E_ARG; }
  for (int i = 0; i < d->n_materials; i++) {
    const pr_material& pm = d->materials[i];
    GMaterial g;
    memset(&g, 0, sizeof(g));
    g.type = pm.type;
    g.roughness = (float)pm.roughness;
    g.ior = (float)pm.refractive_index;
    for (int k = 0; k < 3; k++) {
      g.color[k] = (float)pm.color[k];
      g.emission[k] = (float)pm.emission[k];
      g.color_d[k] = pm.color[k];
      g.emission_d[k] = pm.emission[k];
    }
    g.roughness_d = pm.roughness;
    g.ior_d = pm.refractive_index;
    // texture and IBL images (material.h:176-236): texels as float RGB, a
    // bitmap's bytes / 255 (BitMap cell values), an HDR image's values
    g.tex_off = g.ibl_off = g.bump_off = g.mtex_off = -1;
    if (pm.bump) {
      if (pm.bump_width <= 0 || pm.bump_height <= 0) { err = "bump map size must be positive"; return PR_E_ARG; }
      if (pm.bump_width != pm.bump_height) {
        err = "bump maps are square here (the reference wraps the row above the first to W - 1)";
        return PR_E_UNSUPPORTED;
      }
      if (pm.type != PR_MAT_DIFFUSE && pm.type != PR_MAT_SPECULAR && pm.type != PR_MAT_WARD && pm.type != PR_MAT_PHONG) {
        err = "bump maps on glass and subsurface materials are not on this path";
        return PR_E_UNSUPPORTED;
      }
      g.bump_off = (int32_t)hs.bump_texels.size();
      g.bump_w = pm.bump_width;
      g.bump_h = pm.bump_height;
      const size_t n = (size_t)g.bump_w * g.bump_h;
      for (size_t k = 0; k < n; k++)
        hs.bump_texels.push_back((float)(0.299 * pm.bump[3 * k] + 0.587 * pm.bump[3 * k + 1] + 0.114 * pm.bump[3 * k + 2]));
    }
    g.repeat = pm.repeat;
    g.map_flags = pm.map_flags;
    g.ibl_coef = (float)pm.ibl_coef;
    if (pm.texture) {
      if (pm.texture_width <= 0 || pm.texture_height <= 0) { err = "texture size must be positive"; return PR_E_ARG; }
      g.tex_off = (int32_t)hs.texels.size();
      g.tex_w = pm.texture_width;
      g.tex_h = pm.texture_height;
      const size_t n = (size_t)g.tex_w * g.tex_h;
      if (hs.texels.size() + n > (size_t)INT32_MAX) { err = "textures too large"; return PR_E_ARG; }
      for (size_t k = 0; k < n; k++)
        hs.texels.push_back(make_float4((float)(pm.texture[3 * k] / 255.0), (float)(pm.texture[3 * k + 1] / 255.0),
                                        (float)(pm.texture[3 * k + 2] / 255.0), 0.0f));
    }
    if (pm.ibl_rgb8 || pm.ibl_rgbf) {
      if (pm.ibl_rgb8 && pm.ibl_rgbf) { err = "an IBL image is either a bitmap or an HDR image"; return PR_E_ARG; }
      if (pm.ibl_width <= 0 || pm.ibl_height <= 0) { err = "IBL image size must be positive"; return PR_E_ARG; }
      g.ibl_off = (int32_t)hs.ibl_texels.size();
      g.ibl_w = pm.ibl_width;
      g.ibl_h = pm.ibl_height;
      const size_t n = (size_t)g.ibl_w * g.ibl_h;
      if (hs.ibl_texels.size() + n > (size_t)INT32_MAX) { err = "IBL images too large"; return PR_E_ARG; }
      for (size_t k = 0; k < n; k++) {
        float c[3];
        for (int q = 0; q < 3; q++) c[q] = pm.ibl_rgb8 ? (float)(pm.ibl_rgb8[3 * k + q] / 255.0) : pm.ibl_rgbf[3 * k + q];
        hs.ibl_texels.push_back(make_float4(c[0], c[1], c[2], 0.0f));
      }
      if (is_light(pm)) {
        err = "an emitting material with an IBL image (a light whose emission the shadow ray's hit decides) is not "
              "on this path";
        return PR_E_UNSUPPORTED;
      }
    }
    if (pm.type == PR_MAT_SSS_REFRACTION || pm.type == PR_MAT_SSS_DIFFUSE || pm.type == PR_MAT_SSS_WARD) {
      const pr_medium& md = pm.medium;
      if (pm.type != PR_MAT_SSS_REFRACTION || (md.level != -2 && md.level != -1) || !md.use_bssrdf ||
          pm.roughness != 0.0) {
        err = "subsurface scattering: only the directional-dipole forms (reflection reflection + "
              "Subsurface_Scattering, level -2 or -1, roughness 0) are on this path";
        return PR_E_UNSUPPORTED;
      }
      // setup_Scattering (ParticipatingMediaPrm.h:133-160) when the SCATTERING line is > PS_EPS
      double ss[3], sa[3], tc[3] = {0, 0, 0};
      for (int k = 0; k < 3; k++) { ss[k] = md.sigma_s_rgb[k]; sa[k] = md.sigma_a_rgb[k]; }
      double sc = (ss[0] + ss[1] + ss[2]) / 3, ab = (sa[0] + sa[1] + sa[2]) / 3;
      bool tables = false;
      if (sc > 1.0e-6) {
        const double scale = md.scale > 0.0 ? md.scale : 1.0;
        for (int k = 0; k < 3; k++) { ss[k] *= scale; sa[k] *= scale; }
        sc = (ss[0] + ss[1] + ss[2]) / 3;
        ab = (sa[0] + sa[1] + sa[2]) / 3;
        if (sc + ab < 1.0e-12) {
          for (int k = 0; k < 3; k++) ss[k] = sa[k] = 1.0;
          sc = ab = 0.0;
        } else {
          for (int k = 0; k < 3; k++) tc[k] = ss[k] + sa[k];
        }
        tables = true;
      }
      // channel-sampling table of setup_Scattering for SAMPLE_ABSORBING
      // (ParticipatingMediaPrm.h:161-231): largest channel, smallest (of
      // absorbingColor, as the reference takes it for every table), middle
      g.sss_tsum = 0.0f;
      g.sss_idx = 0;
      g.sss_t[0] = g.sss_t[1] = g.sss_t[2] = (float)(1.0 / 3.0);
      if (tables) {
        double max_s = -9999999.0, min_s = 9999999.0;
        int max_i = -1, min_i = -1, mid_i = -1;
        for (int k = 0; k < 3; k++) {
          if (max_s < sa[k]) { max_s = sa[k]; max_i = k; }
          if (min_s > sa[k]) { min_s = sa[k]; min_i = k; }
        }
        for (int k = 0; k < 3; k++)
          if (max_s > sa[k] && min_s < sa[k]) { mid_i = k; break; }
        if (mid_i == -1) {
          const double av = (sa[0] + sa[1] + sa[2]) / 3;
          const double mx = std::max(std::max(sa[0], sa[1]), sa[2]), mn = std::min(std::min(sa[0], sa[1]), sa[2]);
          mid_i = (std::fabs(mx - av) < std::fabs(mn - av)) ? max_i : min_i;
        }
        const double sum = sa[0] + sa[1] + sa[2];
        if (sum > 1.0e-14) {
          g.sss_tsum = (float)sum;
          g.sss_t[0] = (float)(sa[min_i] / sum);
          g.sss_t[1] = (float)(sa[mid_i] / sum);
          g.sss_t[2] = (float)(sa[max_i] / sum);
        }
        g.sss_idx = min_i | (mid_i << 4) | (max_i << 8);
      }
      g.sss_level = md.level;
      for (int k = 0; k < 3; k++) {
        g.sss_ss[k] = (float)ss[k];
        g.sss_g[k] = (float)md.phase_g[k];
      }
      // DirectionalDipole (bssrdf.h:75-128)
      auto C1 = [](double n) {
        const double r = n > 1.0 ? -9.23372 + n * (22.2272 + n * (-20.9292 + n * (10.2291 + n * (-2.54396 + 0.254913 * n))))
                                 : 0.919317 + n * (-3.4793 + n * (6.75335 + n * (-7.80989 + n * (4.98554 - 1.36881 * n))));
        return r / 2.0;
      };
      auto C2 = [](double n) {
        double r = -1641.1 + n * (1213.67 + n * (-568.556 + n * (164.798 + n * (-27.0181 + 1.91826 * n))));
        r += (((135.926 / n) - 656.175) / n + 1376.53) / n;
        return r / 3.0;
      };
      const double eta = pm.r_refractive_index;
      double stp_min = 1e300;
      for (int k = 0; k < 3; k++) {
        const double ssp = ss[k] * (1.0 - md.phase_g[k]);
        const double stp = ssp + sa[k];
        const double albedo_p = ssp / stp;
        const double D = 1.0 / (3.0 * stp);
        g.sss_D[k] = (float)D;
        g.sss_sigma_tr[k] = (float)std::sqrt(sa[k] / D);
        g.sss_de[k] = (float)(2.131 * D / std::sqrt(albedo_p));
        g.sss_sigma_t[k] = (float)(ss[k] + sa[k]);
        g.sss_tr[k] = (float)tc[k];
        stp_min = std::min(stp_min, stp);
      }
      const double Cp = (1.0 - 2.0 * C1(eta)) / 4.0, Ce = (1.0 - 3.0 * C2(eta)) / 2.0;
      g.sss = 1;
      g.sss_eta = (float)eta;
      g.sss_Cp = (float)Cp;
      g.sss_Ce = (float)Ce;
      g.sss_A = (float)((1.0 - Ce) / (2.0 * Cp));
      g.sss_falloff = (float)(stp_min * 0.001);
      // probe-disk radius heuristic (Subsurface_Scattering.h:701-714)
      const double x = std::min({ss[0], ss[1], ss[2]});
      double y = 2.0 - 1.0 / (1.0 + std::exp(-4.0 * (x - 1.6)));
      if (ab < 0.001) y *= 1.3 - std::exp(std::min({sa[0], sa[1], sa[2]}) * 1000.0);
      g.sss_rmax0 = (float)(1.25 * std::sqrt(std::log(1.0e-4) / -stp_min) * y * md.r_max);
    } else if (pm.type != PR_MAT_DIFFUSE && pm.type != PR_MAT_SPECULAR && pm.type != PR_MAT_REFRACTION &&
               pm.type != PR_MAT_REFRACTION_FRESNEL && pm.type != PR_MAT_WARD && pm.type != PR_MAT_PHONG) {
      err = "material type " + std::to_string(pm.type) + " is not on this path yet";
      return PR_E_UNSUPPORTED;
    }
    for (int k = 0; k < 3; k++) g.specular[k] = (float)pm.specular[k];
    g.ward_ax = (float)pm.ward_alpha[0];
    g.ward_ay = (float)pm.ward_alpha[1];
    g.phong_n = (float)pm.phong_exponent;
    if (pm.type == PR_MAT_WARD && !(pm.ward_alpha[0] > 0.0 && pm.ward_alpha[1] > 0.0)) {
      err = "Ward roughness alpha_x and alpha_y must be positive";
      return PR_E_ARG;
    }
    if (pm.type == PR_MAT_PHONG && !(pm.phong_exponent > -1.0)) {
      err = "Phong exponent must be above -1";
      return PR_E_ARG;
    }
    hs.mats.push_back(g);
  }
  // global medium (scene_env.h:1892-1896 + setup_Scattering)
  {
    const pr_medium& m = d->medium;
    double ss[3], sa[3];
    for (int k = 0; k < 3; k++) { ss[k] = m.sigma_s_rgb[k]; sa[k] = m.sigma_a_rgb[k]; }
    double s_mean = (ss[0] + ss[1] + ss[2]) / 3, a_mean = (sa[0] + sa[1] + sa[2]) / 3;
    double t_mean = s_mean + a_mean;
    GMedium& g = hs.medium;
    memset(&g, 0, sizeof(g));
    if (t_mean < 1.0e-12) {
      g.on = 0;
      for (int k = 0; k < 3; k++) { g.sigma_s[k] = 1.0f; g.sigma_t[k] = 2.0f; }
    } else {
      g.on = d->participating_media ? 1 : 0;
      g.sigma_s_mean = (float)s_mean;
      g.sigma_t_mean = (float)t_mean;
      for (int k = 0; k < 3; k++) { g.sigma_s[k] = (float)ss[k]; g.sigma_t[k] = (float)(ss[k] + sa[k]); }
    }
    for (int k = 0; k < 3; k++) g.g[k] = (float)m.phase_g[k];
  }
  for (int k = 0; k < 3; k++) {
    hs.background[k] = d->background[k];
    hs.env_light[k] = d->environment_light[k];
  }
  double ext = 1.0;
  auto grow = [&ext](double x) { ext = std::max(ext, std::fabs(x)); };
  // meshes shaded with interpolated normals, and textured meshes: the
  // per-face vertex-normal and texture-coordinate records exist only then
  bool any_smooth = false, any_mesh_tex = false, any_obj_mat = false;
  for (int i = 0; i < d->n_entities; i++) {
    const pr_entity& pe = d->entities[i];
    if (pe.type != PR_ENT_POLYGON || pe.material < 0 || pe.material >= d->n_materials) continue;
    if (pe.mesh < 0 || pe.mesh >= d->n_meshes) continue;
    const pr_material& pm = d->materials[pe.material];
    const pr_mesh& pm_ = d->meshes[pe.mesh];
    any_smooth = any_smooth || pe.smooth != 0;
    any_mesh_tex = any_mesh_tex || pm.texture || pm.ibl_rgb8 || pm.ibl_rgbf;
    if (pm_.obj_materials && pm_.face_obj_material && pm_.n_obj_materials > 0) {
      any_obj_mat = true;
      for (int k = 0; k < pm_.n_obj_materials; k++) {
        any_smooth = any_smooth || pm_.obj_materials[k].smooth == 1;
        any_mesh_tex = any_mesh_tex || pm_.obj_materials[k].texture;
      }
    }
  }
  for (int i = 0; i < d->n_entities; i++) {
    const pr_entity& pe = d->entities[i];
    if (pe.material < 0 || pe.material >= d->n_materials) { err = "entity material out of range"; return PR_E_SCENE; }
    GEntity g;
    memset(&g, 0, sizeof(g));
    g.type = pe.type;
    g.material = pe.material;
    g.normal_inverse = pe.normal_inverse < 0 ? -1 : 1;
    const pr_material& pm = d->materials[pe.material];
    const bool textured = pm.texture || pm.ibl_rgb8 || pm.ibl_rgbf || pm.bump;
    if (textured && pe.type != PR_ENT_SPHERE && pe.type != PR_ENT_UVPLANE && pe.type != PR_ENT_POLYGON) {
      err = "textures and IBL images are read on spheres, hemispheres, uvplanes and meshes only";
      return PR_E_UNSUPPORTED;
    }
    if (textured && (hs.mats[pe.material].sss || d->kerr.enabled || d->wormhole.enabled)) {
      err = "textures on subsurface materials or in a black hole or wormhole scene are not on this path";
      return PR_E_UNSUPPORTED;
    }
    if (pe.type == PR_ENT_SPHERE) {
      for (int k = 0; k < 3; k++) g.p[k] = pe.p[k];
      g.radius = pe.radius;
      g.hemisphere = pe.hemisphere ? 1 : 0;
      if (g.hemisphere && (is_light(pm) || d->kerr.enabled || d->wormhole.enabled)) {
        err = "hemispheres that emit, or in a black hole or wormhole scene, are not on this path";
        return PR_E_UNSUPPORTED;
      }
      g.area = 12.5663706143591729538505735331180115 * pe.radius * pe.radius;  // PS_FORPI r^2
      if (g.hemisphere) g.area *= 0.5;
      for (int k = 0; k < 3; k++) {  // Sphere::CreateBoundingBox (sphere.h:58-63)
        g.bb_min[k] = pe.p[k] - pe.radius - 0.01;
        g.bb_max[k] = pe.p[k] + pe.radius + 0.01;
      }
      if (pe.radius < 1.0e4)
        for (int k = 0; k < 3; k++) { grow(pe.p[k] - pe.radius); grow(pe.p[k] + pe.radius); }
    } else if (pe.type == PR_ENT_UVPLANE) {  // UVPlane ctor + CalcArea (plane.h:146-177)
      const D3 U = mk(pe.u), V = mk(pe.v);
      g.u_length = len(U);
      g.v_length = len(V);
      const D3 u = unit(U), v = unit(V), n = unit(cross(u, v));
      for (int k = 0; k < 3; k++) {
        g.p[k] = pe.p[k];
        g.u_axis[k] = (&u.x)[k];
        g.v_axis[k] = (&v.x)[k];
        g.normal[k] = (&n.x)[k];
      }
      g.area = len(scale(u, g.u_length)) * len(scale(v, g.v_length)) * (1.0 - std::pow(dot(u, v), 2.0));
      {  // UVPlane::CreateBoundingBox (plane.h:191-215)
        const D3 o = mk(pe.p), Uu = scale(u, g.u_length), Vv = scale(v, g.v_length);
        const D3 q[4] = {o, add(o, Vv), add(o, Uu), add(add(o, Uu), Vv)};
        for (int k = 0; k < 3; k++) { g.bb_min[k] = 1e300; g.bb_max[k] = -1e300; }
        for (const D3& c : q)
          for (int k = 0; k < 3; k++) {
            g.bb_min[k] = std::min(g.bb_min[k], (&c.x)[k]);
            g.bb_max[k] = std::max(g.bb_max[k], (&c.x)[k]);
          }
      }
      for (int k = 0; k < 3; k++) grow(pe.p[k]);
    } else if (pe.type == PR_ENT_CIRCLE) {
      // Circle ctor (circle.h:117-134): a UVPlane(o, r u, r v) with u, v from
      // OrthonormalBasis(n); its plane normal is never inverted (the base
      // UVPlane keeps the default normal_vector_inverse) and CalcArea = pi r^2
      if (!(pe.radius > 0.0) || pe.radius_inner < 0.0) { err = "disk radius must be positive"; return PR_E_SCENE; }
      const D3 w = mk(pe.normal);
      const D3 u = std::fabs(w.x) > 1.0e-6 ? unit(cross(D3{0.0, 1.0, 0.0}, w)) : unit(cross(D3{1.0, 0.0, 0.0}, w));
      const D3 v = unit(cross(w, u));
      const D3 U = scale(u, pe.radius), V = scale(v, pe.radius);
      const D3 n = unit(cross(unit(U), unit(V)));
      g.normal_inverse = 1;
      for (int k = 0; k < 3; k++) {
        g.p[k] = pe.p[k];
        g.u_axis[k] = (&u.x)[k];
        g.v_axis[k] = (&v.x)[k];
        g.normal[k] = (&n.x)[k];
      }
      g.radius = pe.radius;
      g.radius_inner = pe.radius_inner;
      g.u_length = pe.radius;
      g.v_length = pe.radius_inner;
      g.area = pe.radius * pe.radius * 3.14159265358979323846;
      // the base UVPlane's own axes and lengths (plane.h:146-157): the disk
      // texture reads its (u, v) through them
      const D3 Uu = unit(U), Vu = unit(V);
      for (int k = 0; k < 3; k++) {
        g.du_axis[k] = (&Uu.x)[k];
        g.dv_axis[k] = (&Vu.x)[k];
      }
      g.du_len = len(U);
      g.dv_len = len(V);
      for (int k = 0; k < 3; k++) g.disk_em[k] = pm.emission[k];
      for (int k = 0; k < 3; k++) { grow(pe.p[k] - pe.radius); grow(pe.p[k] + pe.radius); }
    } else if (pe.type == PR_ENT_POLYGON) {
      if (pe.mesh < 0 || pe.mesh >= d->n_meshes) { err = "entity mesh out of range"; return PR_E_SCENE; }
      const pr_mesh& pm_ = d->meshes[pe.mesh];
      if (pm_.n_faces <= 0 || !pm_.vertices || !pm_.faces) { err = "empty mesh"; return PR_E_SCENE; }
      for (int64_t f = 0; f < 3 * (int64_t)pm_.n_faces; f++)
        if (pm_.faces[f] < 0 || pm_.faces[f] >= pm_.n_vertices) { err = "face index out of range"; return PR_E_SCENE; }
      if (is_light(pm)) { err = "mesh lights are not sampled by the reference's next-event estimation"; return PR_E_UNSUPPORTED; }
      const bool big = pm_.n_faces >= kGpuBuildMinFaces;
      const int64_t n3 = 3 * (int64_t)pm_.n_faces;
      if (pm_.vertex_normals || pm_.face_vn) {
        if (!pm_.vertex_normals || !pm_.face_vn || pm_.n_vertex_normals <= 0) {
          err = "vertex normals need the normals and their face ids";
          return PR_E_SCENE;
        }
        for (int64_t f = 0; f < n3; f++)
          if (pm_.face_vn[f] < 0 || pm_.face_vn[f] >= pm_.n_vertex_normals) {
            err = "vertex-normal id out of range";
            return PR_E_SCENE;
          }
      }
      if (pm_.uv || pm_.face_uv) {
        if (!pm_.uv || !pm_.face_uv || pm_.n_uv <= 0) { err = "texture coordinates need the values and their face ids"; return PR_E_SCENE; }
        for (int64_t f = 0; f < n3; f++)
          if (pm_.face_uv[f] < 0 || pm_.face_uv[f] >= pm_.n_uv) { err = "texture-coordinate id out of range"; return PR_E_SCENE; }
      }
      // OBJ materials (usemtl): one derived material per material the faces use
      const bool obj_mats = pm_.obj_materials && pm_.face_obj_material && pm_.n_obj_materials > 0;
      bool obj_tex = false, obj_smooth = false;
      std::vector<int32_t> derived;
      if (obj_mats) {
        if (d->kerr.enabled || d->wormhole.enabled) {
          err = "OBJ materials in a black hole or wormhole scene are not on this path";
          return PR_E_UNSUPPORTED;
        }
        derived.assign((size_t)pm_.n_obj_materials, -2);
        for (int64_t f = 0; f < (int64_t)pm_.n_faces; f++) {
          const int32_t k = pm_.face_obj_material[f];
          if (k < -1 || k >= pm_.n_obj_materials) { err = "face OBJ-material index out of range"; return PR_E_SCENE; }
          if (k >= 0 && derived[(size_t)k] == -2) {
            int st = derive_obj_material(hs, pm, hs.mats[(size_t)pe.material], pm_.obj_materials[k], derived[(size_t)k], err);
            if (st != PR_OK) return st;
            obj_tex = obj_tex || pm_.obj_materials[k].texture;
            obj_smooth = obj_smooth || pm_.obj_materials[k].smooth == 1;
          }
        }
      }
      const bool mesh_tex = pm.texture || pm.ibl_rgb8 || pm.ibl_rgbf || obj_tex;
      if (mesh_tex || pm.bump) {
        // the reference indexes the image with (W - 1) u, (H - 1) v of the
        // interpolated coordinates, with no wrap (polygon.h:507-618); a bump
        // map's lookup runs too, though its normal does not reach the hit
        if (!pm_.uv) { err = "a texture, IBL image or bump map on a mesh needs texture coordinates (vt)"; return PR_E_UNSUPPORTED; }
        for (int64_t k = 0; k < 2 * (int64_t)pm_.n_uv; k++)
          if (!(pm_.uv[k] >= 0.0f && pm_.uv[k] <= 1.0f)) {
            err = "texture coordinates of a textured mesh must lie in [0, 1] (the reference reads no wrap there)";
            return PR_E_UNSUPPORTED;
          }
      }
      if ((pe.smooth || obj_smooth) && (d->kerr.enabled || d->wormhole.enabled)) {
        err = "smooth meshes in a black hole or wormhole scene are not on this path";
        return PR_E_UNSUPPORTED;
      }
      std::vector<float> fn;
      if (pm_.face_normals) fn.assign(pm_.face_normals, pm_.face_normals + 3 * (size_t)pm_.n_faces);
      else if (pm_.vertex_normals) face_normals_vn(pm_.vertex_normals, pm_.face_vn, pm_.n_faces, fn);
      else face_normals(pm_.vertices, pm_.faces, pm_.n_faces, fn);
      const bool needs_vn = pe.smooth || obj_smooth;
      g.mesh_flags = (pe.smooth ? 1 : 0) | (mesh_tex ? 2 : 0) | (obj_mats ? 4 : 0) | (needs_vn ? 8 : 0);
      if (any_smooth) {
        std::vector<float> vn;
        const float* VN = pm_.vertex_normals;
        const int32_t* FVN = pm_.face_vn ? pm_.face_vn : pm_.faces;
        if (needs_vn && !VN) {
          vertex_normals(pm_.vertices, pm_.faces, pm_.n_faces, pm_.n_vertices, vn);
          VN = vn.data();
        }
        for (int64_t f = 0; f < n3; f++)
          for (int a = 0; a < 3; a++) hs.fvn.push_back(needs_vn ? VN[3 * (size_t)FVN[f] + a] : 0.0f);
      }
      if (any_obj_mat)
        for (int64_t f = 0; f < (int64_t)pm_.n_faces; f++) {
          const int32_t k = obj_mats ? pm_.face_obj_material[f] : -1;
          hs.fmat.push_back(k >= 0 ? derived[(size_t)k] : -1);
        }
      if (any_mesh_tex)
        for (int64_t f = 0; f < n3; f++)
          for (int a = 0; a < 2; a++) hs.fuv.push_back(mesh_tex ? pm_.uv[2 * (size_t)pm_.face_uv[f] + a] : 0.0f);
      g.face_base = (int32_t)(hs.fnorm.size() / 3);
      g.n_faces = pm_.n_faces;
      if (big && opt.defer_exact && !d->kerr.enabled && !d->wormhole.enabled) {
        g.node_base = -1;
        g.slot_base = -1;
        HostScene::DeferredMesh dm;
        dm.entity = i;
        dm.vertices.assign(pm_.vertices, pm_.vertices + 3 * (size_t)pm_.n_vertices);
        dm.faces.assign(pm_.faces, pm_.faces + 3 * (size_t)pm_.n_faces);
        hs.deferred_exact.push_back(std::move(dm));
      } else {
        int st = append_exact_qbvh(hs, g, i, pm_.vertices, pm_.faces, pm_.n_faces, err);
        if (st != PR_OK) return st;
      }
      for (int a = 0; a < 3; a++) {
        g.bmin[a] = 3.0e38f;
        g.bmax[a] = -3.0e38f;
      }
      for (int64_t f = 0; f < 3 * (int64_t)pm_.n_faces; f++) {
        const float* v = pm_.vertices + 3 * (size_t)pm_.faces[f];
        for (int a = 0; a < 3; a++) {
          g.bmin[a] = std::min(g.bmin[a], v[a]);
          g.bmax[a] = std::max(g.bmax[a], v[a]);
          grow(v[a]);
        }
      }
      // Polygon::CreateBoundingBox over every vertex of the mesh (polygon.h:875-889)
      for (int a = 0; a < 3; a++) { g.bb_min[a] = 1e300; g.bb_max[a] = -1e300; }
      for (int64_t k = 0; k < (int64_t)pm_.n_vertices; k++)
        for (int a = 0; a < 3; a++) {
          g.bb_min[a] = std::min(g.bb_min[a], (double)pm_.vertices[3 * k + a]);
          g.bb_max[a] = std::max(g.bb_max[a], (double)pm_.vertices[3 * k + a]);
        }
      for (int a = 0; a < 3; a++) { g.bb_min[a] -= 0.01; g.bb_max[a] += 0.01; }
      hs.fnorm.insert(hs.fnorm.end(), fn.begin(), fn.end());
      // the render traversal's own tree (same closest hits, fewer tests)
      if (big && opt.gpu_render_trees) {
        g.rnode_base = -1;
        hs.pending_trees.push_back({i, &pm_});
      } else {
        g.rnode_base = (int32_t)hs.rnodes.size();
        const int rdepth = build_render_bvh(pm_.vertices, pm_.faces, pm_.n_faces, hs.rnodes, hs.rtris);
        if (rdepth > kWStack) {
          err = "mesh " + std::to_string(i) + ": render tree of depth " + std::to_string(rdepth) +
                " exceeds the traversal stack (" + std::to_string(kWStack) + ")";
          return PR_E_BUILD;
        }
      }
    } else if (pe.type == PR_ENT_INF_LIGHT) {
      // no geometry: the traversals skip type 0, only the light list keeps it
      // (scene_env.h:1525-1541)
    } else {
      err = "entity type " + std::to_string(pe.type) + " is not on this path yet";
      return PR_E_UNSUPPORTED;
    }
    // subsurface probe-disk radius, clamped by the object's size (Subsurface_Scattering.h:716-718)
    const GMaterial& gm = hs.mats[pe.material];
    if (gm.sss) {
      if (pe.type == PR_ENT_CIRCLE) { err = "subsurface scattering on a disk is not on this path"; return PR_E_UNSUPPORTED; }
      const D3 ext = {g.bb_max[0] - g.bb_min[0], g.bb_max[1] - g.bb_min[1], g.bb_max[2] - g.bb_min[2]};
      const double ln = len(ext);
      g.sss_rmax = gm.sss_rmax0 > ln ? ln * 0.3 : gm.sss_rmax0;
    }
    hs.ents.push_back(g);
  }
  // lights: registration order (scene_env.h:1525-1541, :1567-1586,
  // :1645-1663, :1692-1719), then LightList::random_light_setup's sort by
  // power, descending (light.h:97).  Power: area * |emission|; a spot light
  // SpotLightPower(|emission|) of the default cone (the reference computes
  // it before it sets the entity's angles); an infinity light |emission|.
  struct L {
    double power;
    GLight g;
  };
  std::vector<L> lights;
  hs.light_id.assign(hs.ents.size(), -1);
  const double PI = 3.14159265358979323846, RAD = PI / 180.0;
  for (int i = 0; i < (int)hs.ents.size(); i++) {
    const pr_entity& pe = d->entities[i];
    const pr_material& pm = d->materials[hs.ents[i].material];
    const int ty = hs.ents[i].type;
    if (pe.parallel_light && pe.spot_light) {
      err = "an entity is either a parallel or a spot light";
      return PR_E_UNSUPPORTED;
    }
    if ((pe.parallel_light || pe.spot_light) && (ty == PR_ENT_INF_LIGHT || ty == PR_ENT_POLYGON)) {
      err = "parallel and spot lights are uvplanes or spheres";
      return PR_E_UNSUPPORTED;
    }
    if (!is_light(pm)) continue;
    const double elen = len(mk(pm.emission));
    L l;
    memset(&l.g, 0, sizeof(l.g));
    l.g.ent = i;
    l.g.mat = hs.ents[i].material;
    l.g.kind = PR_LIGHT_AREA;
    l.g.att[2] = 1.0f;
    l.power = hs.ents[i].area * elen;
    D3 dir = mk(pe.light_dir);
    if (ty == PR_ENT_INF_LIGHT) {
      if (!(len(dir) > 0.0)) { err = "an infinity light needs a direction"; return PR_E_SCENE; }
      l.g.kind = PR_LIGHT_INFINITY;
      l.power = elen;
    } else if (pe.parallel_light) {
      if (ty == PR_ENT_CIRCLE) {
        err = "a parallel disk light samples the disk the way the reference leaves undefined (circle.h:110-134)";
        return PR_E_UNSUPPORTED;
      }
      if (ty == PR_ENT_UVPLANE && len(dir) < 1.0e-16) {  // the plane's own normal (scene_env.h:1575-1578)
        const GEntity& g = hs.ents[i];
        dir = D3{g.normal[0] * g.normal_inverse, g.normal[1] * g.normal_inverse, g.normal[2] * g.normal_inverse};
      }
      if (!(len(dir) > 0.0)) { err = "a parallel sphere light needs parallel_light_dir"; return PR_E_SCENE; }
      l.g.kind = PR_LIGHT_PARALLEL;
    } else if (pe.spot_light) {
      if (ty != PR_ENT_SPHERE) {
        err = "spot lights are spheres (the reference reads every spot light's centre as a sphere's)";
        return PR_E_UNSUPPORTED;
      }
      l.g.kind = PR_LIGHT_SPOT;
      const double c0 = std::cos(30.0 * RAD), c1 = std::cos(25.0 * RAD);  // Light() defaults (light.h:41-43)
      l.power = elen * 2.0 * PI * (1.0 - .5 * (c1 + c0));
      l.g.cos_total = (float)std::cos(pe.spot_angle[0] * RAD);
      l.g.cos_start = (float)std::cos((pe.spot_angle[0] - pe.spot_angle[1]) * RAD);
      l.g.falloff = (float)pe.spot_falloff;
      for (int k = 0; k < 3; k++) {
        l.g.att[k] = (float)pe.spot_attenuation[k];
        l.g.center[k] = (float)pe.p[k];
      }
    }
    for (int k = 0; k < 3; k++) l.g.dir[k] = (float)(&dir.x)[k];
    l.g.dir_len = (float)len(dir);
    hs.ents[i].is_light = 1;
    if (ty == PR_ENT_CIRCLE) hs.disk_light = true;
    hs.light_id[i] = (int32_t)lights.size();
    lights.push_back(l);
  }
  std::sort(lights.begin(), lights.end(), [](const L& a, const L& b) { return a.power > b.power; });
  if ((int)lights.size() > kMaxLights) { err = "too many lights"; return PR_E_ARG; }
  for (const L& l : lights) hs.lights.push_back(l.g);
  if (d->kerr.enabled || d->wormhole.enabled)
    for (const GLight& g : hs.lights)
      if (g.kind != PR_LIGHT_AREA) {
        err = "parallel, spot and infinity lights are sampled along straight rays only (no black hole or wormhole)";
        return PR_E_UNSUPPORTED;
      }
  hs.scene_scale = (float)ext;
  // black hole (scene_env.h:701-766, :2056-2098; KerrBlackHole ctor :86-151)
  hs.kerr = GKerr{};
  hs.kerr_texture.clear();
  const pr_kerr& pk = d->kerr;
  if (pk.enabled) {
    if (!(pk.a * pk.a < 1.0)) { err = "Kerr spin must satisfy |a| < M = 1"; return PR_E_SCENE; }
    if (pk.max_steps <= 0 || pk.max_steps > 10000000) {
      err = "geodesics_max_length must be in 1..1e7 (an unbounded trace is not run on the GPU)";
      return PR_E_ARG;
    }
    if (pk.escape_radius < 0.0) { err = "escape_radius must be >= 0"; return PR_E_ARG; }
    GKerr& k = hs.kerr;
    k.enabled = 1;
    k.max_steps = pk.max_steps;
    for (int q = 0; q < 3; q++) k.pos[q] = pk.position[q];
    k.a = pk.a;
    k.a2 = pk.a * pk.a;
    k.M = 1.0;
    k.Rhor = k.M + std::sqrt(k.M * k.M - k.a2) + 1e-10;
    for (int q = 0; q < 4; q++) k.map_coef[q] = pk.map_coef[q];
    k.escape_radius = pk.escape_radius;
    if (pk.precision != PR_KERR_FP64 && pk.precision != PR_KERR_FP32) { err = "unknown Kerr precision"; return PR_E_ARG; }
    k.precision = pk.precision;
    // farthest and nearest scene surface from the hole (Cartesian, conservative)
    const D3 P = mk(k.pos);
    double far = 0.0, near = 1.0e300;
    for (const GEntity& e : hs.ents) {
      double f = 0.0, n = 0.0;
      if (e.type == PR_ENT_SPHERE || e.type == PR_ENT_CIRCLE) {
        const double dc = len(sub(mk(e.p), P));
        f = dc + e.radius;
        n = e.type == PR_ENT_SPHERE ? std::fabs(dc - e.radius)                      // a sphere is its surface
                                    : std::max({0.0, e.radius_inner - dc, dc - e.radius});  // the annulus
      } else if (e.type == PR_ENT_UVPLANE) {
        const D3 o = mk(e.p), U = scale(mk(e.u_axis), e.u_length), V = scale(mk(e.v_axis), e.v_length);
        const D3 corner[4] = {o, add(o, U), add(o, V), add(add(o, U), V)};
        for (const D3& q : corner) f = std::max(f, len(sub(q, P)));
        const D3 ctr = add(o, scale(add(U, V), 0.5));
        n = std::max(0.0, len(sub(ctr, P)) - 0.5 * len(add(U, V)) - 0.5 * len(sub(U, V)));
      } else {  // mesh: its bounding box
        double dn2 = 0.0, df2 = 0.0;
        for (int a = 0; a < 3; a++) {
          const double pa = (&P.x)[a], lo = e.bmin[a], hi = e.bmax[a];
          const double dn = pa < lo ? lo - pa : (pa > hi ? pa - hi : 0.0);
          const double dfa = std::max(std::fabs(pa - lo), std::fabs(pa - hi));
          dn2 += dn * dn;
          df2 += dfa * dfa;
        }
        f = std::sqrt(df2);
        n = std::sqrt(dn2);
      }
      far = std::max(far, f);
      near = std::min(near, n);
    }
    if (hs.ents.empty()) near = 0.0;
    k.scene_radius = far;
    // in Boyer-Lindquist r: a point at Cartesian distance d has r <= d <= sqrt(r^2 + a^2)
    k.scene_inner = near * near > k.a2 ? std::sqrt(near * near - k.a2) : 0.0;
    k.texture_coef = pk.texture_coef;
    if (pk.texture) {
      if (pk.texture_width <= 0 || pk.texture_height <= 0) { err = "background texture size must be positive"; return PR_E_ARG; }
      hs.kerr_texture.assign(pk.texture, pk.texture + 3 * (size_t)pk.texture_width * pk.texture_height);
      k.tex_w = pk.texture_width;
      k.tex_h = pk.texture_height;
    }
    // accretion disk: inner_orbit (KerrBlackHole.h:215-240) with M = 1 and
    // the class's cbrt(x) = pow(x, 1/3)
    {
      const double M = k.M, a = k.a, a2 = k.a2, m2 = M * M;
      auto cbrt_r = [](double x) { return std::pow(x, 1.0 / 3.0); };
      const double z1 = 1 + cbrt_r(1 - a2 / m2) * (cbrt_r(1 + a / M) + cbrt_r(1 - a / M));
      const double z2 = std::sqrt(3 * a2 / m2 + z1 * z1);
      k.Rmstable = M * (3 + z2 - std::sqrt((3 - z1) * (3 + z1 + 2 * z2)));
    }
    k.use_temp = pk.use_accretion_disk_temperature ? 1 : 0;
    k.doppler_effect = pk.color_doppler_factor_effect;
    for (int q = 0; q < 3; q++) k.observer[q] = pk.observer[q];
    k.disk_seed = pk.disk_seed;
    hs.kerr_disk_texture.clear();
    if (pk.disk_texture) {
      if (pk.disk_texture_width <= 0 || pk.disk_texture_height <= 0) {
        err = "accretion disk texture size must be positive";
        return PR_E_ARG;
      }
      hs.kerr_disk_texture.assign(pk.disk_texture,
                                  pk.disk_texture + 4 * (size_t)pk.disk_texture_width * pk.disk_texture_height);
      k.disk_w = pk.disk_texture_width;
      k.disk_h = pk.disk_texture_height;
    }
    for (size_t i = 0; i < hs.ents.size(); i++) {
      GEntity& e = hs.ents[i];
      const pr_entity& pe = d->entities[i];
      const pr_material& pm = d->materials[pe.material];
      if (e.type != PR_ENT_CIRCLE || pe.blackhole_disk < 0 || !pm.disk_map) continue;
      // the reference indexes its disk-texture list with blackhole_disk (circle.h:240-242)
      if (hs.kerr_disk_texture.empty() || pe.blackhole_disk != 0) {
        err = "a disk_map disk under the black hole needs accretion-disk texture 0";
        return PR_E_SCENE;
      }
      if (!(e.radius > k.Rmstable)) { err = "the accretion disk must reach beyond the ISCO"; return PR_E_SCENE; }
      e.kerr_disk = 1;
    }
  }
  return build_wormhole(d, hs, err);
}

}  // namespace pr
