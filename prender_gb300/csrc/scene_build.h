// Host scene built from a pr_scene_desc (see scene_build.cpp).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "pr_internal.h"

namespace pr {

// One 4-wide node in the reference's own terms (QBVH.h:53-61), kept on the
// host for export and for the GPU node encoding.
struct RefNode {
  float box[2][3][4] = {};     // [min/max][xyz][child]
  int64_t ref_child[4] = {0, 0, 0, 0};  // QBVH child word: leaf = top bit | ref leaf start
  int32_t leaf_first[4] = {0, 0, 0, 0};  // first slot in leaf_tris (leaf children)
  int32_t leaf_count[4] = {0, 0, 0, 0};
  int32_t axis_top = 0, axis_left = 0, axis_right = 0;
};

struct MeshQbvh {
  std::vector<RefNode> nodes;
  std::vector<int32_t> ref_leaf;   // face ids with -1 terminators (m_leafObjectArray)
  std::vector<int32_t> leaf_tris;  // face ids, leaves contiguous, no terminators
};

struct HostScene {
  std::vector<GMaterial> mats;
  std::vector<GEntity> ents;
  std::vector<GNode> nodes;
  std::vector<float4> tris;
  std::vector<WNode> rnodes;   // render-path trees
  std::vector<float4> rtris;
  std::vector<float> fnorm;
  // per face (indexed like fnorm): the three vertex normals of smooth meshes
  // (9 floats; empty when no mesh is smooth) and the three texture
  // coordinates of meshes with them (6 floats; empty when no textured mesh)
  std::vector<float> fvn, fuv;
  std::vector<int32_t> fmat;  // per face (like fnorm): derived OBJ-material index, -1 none
  std::vector<float4> texels;           // material textures, RGB / 255
  std::vector<float4> ibl_texels;       // material IBL images
  std::vector<float> bump_texels;       // material bump maps (luminance)
  std::vector<GLight> lights;           // in the reference's sorted order
  std::vector<int32_t> light_id;        // per entity: registration index (-1: not a light)
  std::vector<MeshQbvh> mesh_qbvh;
  std::vector<int32_t> mesh_entity;  // entity index of each mesh_qbvh
  GMedium medium{};
  double background[3] = {0, 0, 0};
  double env_light[3] = {0, 0, 0};
  float scene_scale = 1.0f;
  GKerr kerr{};
  std::vector<unsigned char> kerr_texture;
  std::vector<unsigned char> kerr_disk_texture;  // RGBA8
  GWorm worm{};
  std::vector<unsigned char> worm_tex[2];  // wormhole backgrounds (RGB8)
  bool disk_light = false;  // an emitting disk is registered as a light
  // meshes whose render tree the caller builds (pointers into the scene
  // description: valid during the upload call only)
  struct PendingTree {
    int entity;
    const pr_mesh* mesh;
  };
  std::vector<PendingTree> pending_trees;
  // meshes whose reference-layout QBVH is built on first use (copies)
  struct DeferredMesh {
    int entity;
    std::vector<float> vertices;
    std::vector<int32_t> faces;
  };
  std::vector<DeferredMesh> deferred_exact;
};

// How build_host_scene treats meshes of at least kGpuBuildMinFaces faces.
struct SceneBuildOptions {
  bool gpu_render_trees = false;  // leave their render trees to the caller (pending_trees)
  bool defer_exact = false;       // leave their reference-layout QBVH for later (deferred_exact),
                                  // except in scenes with a black hole, whose rays use it
};

int build_host_scene(const pr_scene_desc* d, HostScene& hs, std::string& err,
                     const SceneBuildOptions& opt = SceneBuildOptions());
// Builds the deferred reference-layout QBVHs of hs (appending nodes and
// triangles, setting their entities' node_base / slot_base).
int complete_exact_qbvh(HostScene& hs, std::string& err);
int build_mesh_qbvh(const float* vertices, const int32_t* faces, int n_faces, MeshQbvh& out, std::string& err);
void face_normals(const float* V, const int32_t* F, int n_faces, std::vector<float>& out);
// Obj::CalcNormalVector without vn lines (ObjLoader.cpp:577-700): each
// vertex's normal is the mean of the unnormalised face normals around it,
// normalised, in float; out holds 3 per vertex
void vertex_normals(const float* V, const int32_t* F, int n_faces, int n_vertices, std::vector<float>& out);
// the same with vn lines (ObjLoader.cpp:617-641): a face's normal is the
// normalised mean of its three vertex normals
void face_normals_vn(const float* VN, const int32_t* FVN, int n_faces, std::vector<float>& out);

}  // namespace pr
