// C ABI (include/prender_gpu.h): context, scene upload, closest-hit hook and
// the plain renderer.  Host buffers are staged through device copies owned
// by the context; every error becomes a status code plus pr_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/prender_gpu.h"
#include "adjoint.h"
#include "kerr.h"
#include "wormhole.h"
#include "mlt.h"
#include "pr_internal.h"
#include "render_kernels.h"
#include "scene_build.h"
#include "wavefront.h"

using namespace pr;

#include "ctx_internal.h"
#include "render_bvh.h"

namespace {

int fail(pr_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(pr_ctx* c, cudaError_t e, const char* what) {
  return fail(c, PR_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define PR_CUDA(ctx, call)                                   \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

int check_device_errors(pr_ctx* c) {
  uint32_t bits = 0;
  PR_CUDA(c, cudaMemcpyAsync(&bits, c->errword.p, 4, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  if (!bits) return PR_OK;
  return fail(c, PR_E_DEVICE, pr::device_error_message(bits));
}

template <class T>
cudaError_t upload(DevBuf& b, const std::vector<T>& v, cudaStream_t s) {
  cudaError_t e = b.ensure(sizeof(T) * std::max<size_t>(v.size(), 1));
  if (e != cudaSuccess || v.empty()) return e;
  return cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s);
}

}  // namespace

int pr::ctx_fail(pr_ctx* c, int code, const std::string& msg) { return fail(c, code, msg); }

std::string pr::device_error_message(uint32_t bits) {
  std::string m = "device check fired:";
  if (bits & PR_DEV_STACK_OVERFLOW) m += " traversal-stack-overflow";
  if (bits & PR_DEV_LOOP_CAP) m += " loop-cap";
  if (bits & PR_DEV_BAD_INDEX) m += " bad-index";
  if (bits & PR_DEV_QUEUE_OVERFLOW) m += " queue-overflow";
  if (bits & PR_DEV_NONFINITE) m += " non-finite-radiance";
  const uint32_t known = PR_DEV_STACK_OVERFLOW | PR_DEV_LOOP_CAP | PR_DEV_BAD_INDEX | PR_DEV_QUEUE_OVERFLOW | PR_DEV_NONFINITE;
  if (bits & ~known) m += " other (bits " + std::to_string(bits & ~known) + ")";
  return m;
}

extern "C" {

int pr_abi_version(void) { return PR_ABI_VERSION; }

pr_ctx* pr_create(int device, int* status) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0 || device < 0 || device >= n) {
    if (status) *status = (e != cudaSuccess || n == 0) ? PR_E_CUDA : PR_E_ARG;
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    if (status) *status = PR_E_CUDA;
    return nullptr;
  }
  pr_ctx* c = new pr_ctx();
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      c->errword.ensure(16) != cudaSuccess || c->counters.ensure(128) != cudaSuccess) {
    if (status) *status = PR_E_CUDA;
    delete c;
    return nullptr;
  }
  if (status) *status = PR_OK;
  return c;
}

void pr_destroy(pr_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->cur.release();
  for (DevBuf* b : {&c->k_status, &c->k_bl, &c->k_dir, &c->k_steps, &c->k_ent, &c->k_t,
                    &c->adj_scratch, &c->adj_grad, &c->k_sens})
    b->release();
  for (DevBuf* b : {&c->errword, &c->counters, &c->partial,
                    &c->out, &c->rays, &c->ires, &c->jres, &c->dres, &c->wf_o, &c->wf_d, &c->wf_beta, &c->wf_dpw,
                    &c->wf_L, &c->wf_sample, &c->wf_hit, &c->wf_hitv, &c->wf_nee, &c->wf_sho, &c->wf_shd, &c->wf_extq,
                    &c->wf_shq, &c->wf_spo, &c->wf_spd, &c->wf_spb, &c->wf_spw, &c->wf_sps, &c->wf_samp, &c->wf_live,
                    &c->wf_pix, &c->wf_ctl, &c->wf_frc, &c->wf_fre, &c->wf_frs, &c->wf_frl, &c->wf_spf,
                    &c->wf_neef})
    b->release();
  if (c->wf_graph) cudaGraphExecDestroy(c->wf_graph);
  if (c->batch_exec) cudaGraphExecDestroy(c->batch_exec);
  for (cudaStream_t st : c->batch_streams) cudaStreamDestroy(st);
  for (cudaEvent_t ev : c->batch_events) cudaEventDestroy(ev);
  c->batch_partial.release();
  if (c->wf_host_ctl) cudaFreeHost(c->wf_host_ctl);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  cudaGetLastError();  // teardown errors are not reported to later calls
  delete c;
}

const char* pr_last_error(const pr_ctx* c) { return c ? c->err.c_str() : "null context"; }

// render trees of the large meshes: binary tree on the GPU, wide nodes on the host
static int build_pending_trees(pr_ctx* c, HostScene& h) {
  for (const HostScene::PendingTree& pt : h.pending_trees) {
    std::vector<BinNode> tree;
    std::vector<int32_t> order;
    const pr_mesh& m = *pt.mesh;
    PR_CUDA(c, build_render_bvh_binary_gpu(m.vertices, m.n_vertices, m.faces, m.n_faces, c->stream, tree, order));
    h.ents[(size_t)pt.entity].rnode_base = (int32_t)h.rnodes.size();
    const int depth = emit_render_bvh(m.vertices, m.faces, tree, order, h.rnodes, h.rtris);
    if (depth > kWStack)
      return fail(c, PR_E_BUILD, "mesh of entity " + std::to_string(pt.entity) + ": render tree of depth " +
                                     std::to_string(depth) + " exceeds the traversal stack");
  }
  h.pending_trees.clear();  // they pointed into the caller's scene description
  return PR_OK;
}

// the reference-layout QBVHs that large meshes left for their first use
// (the exact first-hit path and the QBVH export)
static int ensure_exact(pr_ctx* c, SceneObjData& o) {
  if (o.host.deferred_exact.empty()) return PR_OK;
  std::string err;
  int st = complete_exact_qbvh(o.host, err);
  if (st != PR_OK) return fail(c, st, err);
  PR_CUDA(c, cudaSetDevice(c->device));
  PR_CUDA(c, upload(o.ents, o.host.ents, c->stream));
  PR_CUDA(c, upload(o.nodes, o.host.nodes, c->stream));
  PR_CUDA(c, upload(o.tris, o.host.tris, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  o.dev.ents = (const GEntity*)o.ents.p;
  o.dev.nodes = (const GNode*)o.nodes.p;
  o.dev.tris = (const float4*)o.tris.p;
  return PR_OK;
}

// host build + device copies of one scene (SceneEnv::Load + CreateEntList)
static int build_device_scene(pr_ctx* c, const pr_scene_desc* d, SceneObjData& o) {
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  std::string err;
  SceneBuildOptions opt;
  opt.gpu_render_trees = true;
  opt.defer_exact = true;
  int st = build_host_scene(d, o.host, err, opt);
  if (st != PR_OK) return fail(c, st, err);
  HostScene& h = o.host;
  st = build_pending_trees(c, h);
  if (st != PR_OK) return st;
  PR_CUDA(c, upload(o.ents, h.ents, c->stream));
  PR_CUDA(c, upload(o.mats, h.mats, c->stream));
  // the exact path's arrays get their space now, as an eager build would
  // take it, and are filled on first use: measured on GB300, letting the
  // wavefront pool take that space instead slows wf_shade by 15 % (the
  // pool's placement in memory matters to it; the cause is not known)
  size_t res_nodes = h.nodes.size(), res_tris = h.tris.size();
  for (const HostScene::DeferredMesh& m : h.deferred_exact) {
    const size_t nf = m.faces.size() / 3;
    res_tris += 3 * nf;
    res_nodes += (size_t)std::ceil((double)nf / 5.6);  // the reference's SAH: about 5.6 faces per 4-wide node
  }
  PR_CUDA(c, o.nodes.ensure(sizeof(GNode) * std::max<size_t>(res_nodes, 1)));
  PR_CUDA(c, o.tris.ensure(sizeof(float4) * std::max<size_t>(res_tris, 1)));
  PR_CUDA(c, upload(o.nodes, h.nodes, c->stream));
  PR_CUDA(c, upload(o.tris, h.tris, c->stream));
  PR_CUDA(c, upload(o.rnodes, h.rnodes, c->stream));
  PR_CUDA(c, upload(o.rtris, h.rtris, c->stream));
  PR_CUDA(c, upload(o.fnorm, h.fnorm, c->stream));
  // texel pools only for scenes with images (an allocation more or less
  // moves the wavefront pool, whose placement wf_shade is sensitive to)
  if (!h.texels.empty()) PR_CUDA(c, upload(o.texels, h.texels, c->stream));
  if (!h.ibl_texels.empty()) PR_CUDA(c, upload(o.ibl_texels, h.ibl_texels, c->stream));
  if (!h.bump_texels.empty()) PR_CUDA(c, upload(o.bump_texels, h.bump_texels, c->stream));
  if (!h.fvn.empty()) PR_CUDA(c, upload(o.fvn, h.fvn, c->stream));
  if (!h.fuv.empty()) PR_CUDA(c, upload(o.fuv, h.fuv, c->stream));
  if (!h.fmat.empty()) PR_CUDA(c, upload(o.fmat, h.fmat, c->stream));
  PR_CUDA(c, upload(o.kerr_tex, h.kerr_texture, c->stream));
  PR_CUDA(c, upload(o.kerr_disk_tex, h.kerr_disk_texture, c->stream));
  for (int k = 0; k < 2; k++)
    if (!h.worm_tex[k].empty()) PR_CUDA(c, upload(o.worm_tex[k], h.worm_tex[k], c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  o.worm = h.worm;
  for (int k = 0; k < 2; k++) o.worm.tex[k] = h.worm_tex[k].empty() ? nullptr : (const unsigned char*)o.worm_tex[k].p;
  o.kerr = h.kerr;
  o.kerr.texture = h.kerr_texture.empty() ? nullptr : (const unsigned char*)o.kerr_tex.p;
  o.kerr.disk_tex = h.kerr_disk_texture.empty() ? nullptr : (const uchar4*)o.kerr_disk_tex.p;
  DevScene& S = o.dev;
  memset(&S, 0, sizeof(S));
  S.ents = (const GEntity*)o.ents.p;
  S.mats = (const GMaterial*)o.mats.p;
  S.nodes = (const GNode*)o.nodes.p;
  S.tris = (const float4*)o.tris.p;
  S.rnodes = (const WNode*)o.rnodes.p;
  S.rtris = (const float4*)o.rtris.p;
  S.fnorm = (const float*)o.fnorm.p;
  S.texels = (const float4*)o.texels.p;
  S.ibl_texels = (const float4*)o.ibl_texels.p;
  S.bump_texels = (const float*)o.bump_texels.p;
  S.n_ents = (int)h.ents.size();
  S.n_lights = (int)h.lights.size();
  S.n_point_lights = 0;
  for (int i = 0; i < S.n_lights; i++) {
    S.lights[i] = h.lights[i];
    S.n_point_lights += h.lights[i].kind != PR_LIGHT_AREA ? 1 : 0;
  }
  for (int k = 0; k < 3; k++) {
    S.background[k] = h.background[k];
    S.env_light[k] = h.env_light[k];
  }
  S.medium = h.medium;
  S.scene_scale = h.scene_scale;
  S.has_sss = 0;
  S.has_glossy = 0;
  S.has_tex = 0;
  for (const GMaterial& gm : h.mats) {
    S.has_sss |= gm.sss;
    S.has_glossy |= (gm.type == PR_MAT_WARD || gm.type == PR_MAT_PHONG) ? 1 : 0;
    S.has_tex |= (gm.tex_off >= 0 || gm.ibl_off >= 0 || gm.bump_off >= 0) ? 1 : 0;
  }
  if (!h.fvn.empty()) S.has_tex |= 2;
  S.fvn = h.fvn.empty() ? nullptr : (const float*)o.fvn.p;
  S.fuv = h.fuv.empty() ? nullptr : (const float*)o.fuv.p;
  S.fmat = h.fmat.empty() ? nullptr : (const int32_t*)o.fmat.p;
  if (!h.fmat.empty()) S.has_tex |= 2;
  for (int k = 0; k < 3; k++) {
    S.bg[k] = (float)h.background[k];
    S.env[k] = (float)h.env_light[k];
  }
  for (int i = 0; i < S.n_ents; i++) {
    const GEntity& e = h.ents[i];
    GEntF& f = S.entf[i];
    f.type = e.type;
    f.material = e.material;
    f.normal_inverse = e.normal_inverse;
    f.is_light = e.is_light;
    f.light_id = i < (int)h.light_id.size() ? h.light_id[i] : -1;
    for (int k = 0; k < 3; k++) {
      f.p[k] = (float)e.p[k];
      f.u[k] = (float)e.u_axis[k];
      f.v[k] = (float)e.v_axis[k];
      f.n[k] = (float)e.normal[k];
    }
    f.radius_eps = (float)(e.radius + 1.0e-6);
    f.u_length = (float)e.u_length;
    f.v_length = (float)e.v_length;
    f.area = (float)e.area;
    f.face_base = e.face_base;
    f.node_base = e.rnode_base;
    f.sss_rmax = (float)e.sss_rmax;
  }
  return PR_OK;
}

int pr_scene_upload(pr_ctx* c, const pr_scene_desc* d) {
  if (!c) return PR_E_ARG;
  c->scene_ready = false;
  int st = build_device_scene(c, d, c->cur);
  if (st != PR_OK) return st;
  c->scene_ready = true;
  return PR_OK;
}

int pr_scene_check(const pr_scene_desc* d, char* msg, int msg_len) {
  HostScene hs;
  std::string err;
  SceneBuildOptions opt;
  opt.gpu_render_trees = true;  // big meshes' trees are left pending (not built here)
  opt.defer_exact = true;
  int st = PR_E_NOMEM;
  try {
    st = build_host_scene(d, hs, err, opt);
  } catch (const std::exception& ex) {  // allocation failures of the host build
    err = ex.what();
  }
  if (st != PR_OK && msg && msg_len > 0) {
    strncpy(msg, err.c_str(), (size_t)msg_len - 1);
    msg[msg_len - 1] = 0;
  }
  return st;
}

pr_scene_obj* pr_scene_create(pr_ctx* c, const pr_scene_desc* d, int* status) {
  if (!c) {
    if (status) *status = PR_E_ARG;
    return nullptr;
  }
  pr_scene_obj* o = new pr_scene_obj();
  int st = build_device_scene(c, d, o->data);
  if (status) *status = st;
  if (st != PR_OK) {
    o->data.release();
    delete o;
    return nullptr;
  }
  return o;
}

void pr_scene_release(pr_ctx* c, pr_scene_obj* o) {
  if (!o) return;
  if (c) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
  }
  o->data.release();
  delete o;
}

static void export_qbvh(const MeshQbvh& q, float* boxes, int64_t* children, int32_t* axes, int32_t* leaf_faces);

int pr_render_bvh_export(pr_ctx* c, const pr_mesh* m, int on_gpu, void* nodes, int64_t nodes_cap,
                         int32_t* tri_faces, int64_t tris_cap, int64_t* n_nodes, int64_t* n_tris) {
  if (!c) return PR_E_ARG;
  if (!m || m->n_faces <= 0 || m->n_vertices <= 0 || !m->vertices || !m->faces) return fail(c, PR_E_ARG, "empty mesh");
  for (int64_t f = 0; f < 3 * (int64_t)m->n_faces; f++)
    if (m->faces[f] < 0 || m->faces[f] >= m->n_vertices) return fail(c, PR_E_ARG, "face index out of range");
  std::vector<WNode> wn;
  std::vector<float4> wt;
  if (on_gpu) {
    PR_CUDA(c, cudaSetDevice(c->device));
    cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
    std::vector<BinNode> tree;
    std::vector<int32_t> order;
    PR_CUDA(c, build_render_bvh_binary_gpu(m->vertices, m->n_vertices, m->faces, m->n_faces, c->stream, tree, order));
    emit_render_bvh(m->vertices, m->faces, tree, order, wn, wt);
  } else {
    build_render_bvh(m->vertices, m->faces, m->n_faces, wn, wt);
  }
  const int64_t nn = (int64_t)wn.size(), nt = (int64_t)(wt.size() / 3);
  if (n_nodes) *n_nodes = nn;
  if (n_tris) *n_tris = nt;
  if ((nodes && nodes_cap < nn) || (tri_faces && tris_cap < nt)) return fail(c, PR_E_ARG, "output capacity too small");
  if (nodes) memcpy(nodes, wn.data(), sizeof(WNode) * wn.size());
  if (tri_faces)
    for (int64_t i = 0; i < nt; i++) memcpy(&tri_faces[i], &wt[(size_t)(3 * i)].w, 4);
  return PR_OK;
}

int pr_qbvh_info(pr_ctx* c, int entity, int64_t* n_nodes, int64_t* n_leaf_slots) {
  if (!c || !c->scene_ready) return fail(c, PR_E_SCENE, "no scene uploaded");
  const int st = ensure_exact(c, c->cur);
  if (st != PR_OK) return st;
  for (size_t m = 0; m < c->cur.host.mesh_entity.size(); m++)
    if (c->cur.host.mesh_entity[m] == entity) {
      if (n_nodes) *n_nodes = (int64_t)c->cur.host.mesh_qbvh[m].nodes.size();
      if (n_leaf_slots) *n_leaf_slots = (int64_t)c->cur.host.mesh_qbvh[m].ref_leaf.size();
      return PR_OK;
    }
  return fail(c, PR_E_ARG, "entity is not a mesh");
}

int pr_qbvh_export(pr_ctx* c, int entity, float* boxes, int64_t* children, int32_t* axes, int32_t* leaf_faces) {
  if (!c || !c->scene_ready) return fail(c, PR_E_SCENE, "no scene uploaded");
  const int st = ensure_exact(c, c->cur);
  if (st != PR_OK) return st;
  for (size_t m = 0; m < c->cur.host.mesh_entity.size(); m++)
    if (c->cur.host.mesh_entity[m] == entity) {
      export_qbvh(c->cur.host.mesh_qbvh[m], boxes, children, axes, leaf_faces);
      return PR_OK;
    }
  return fail(c, PR_E_ARG, "entity is not a mesh");
}

static void export_qbvh(const MeshQbvh& q, float* boxes, int64_t* children, int32_t* axes, int32_t* leaf_faces) {
  for (size_t i = 0; i < q.nodes.size(); i++) {
    const RefNode& rn = q.nodes[i];
    if (boxes) memcpy(boxes + 24 * i, rn.box, 24 * sizeof(float));
    if (children)
      for (int s = 0; s < 4; s++) children[4 * i + s] = rn.ref_child[s];
    if (axes) {
      axes[3 * i] = rn.axis_top;
      axes[3 * i + 1] = rn.axis_left;
      axes[3 * i + 2] = rn.axis_right;
    }
  }
  if (leaf_faces) memcpy(leaf_faces, q.ref_leaf.data(), q.ref_leaf.size() * sizeof(int32_t));
}

int pr_qbvh_build_host(const float* vertices, int32_t n_vertices, const int32_t* faces, int32_t n_faces,
                       int64_t* n_nodes, int64_t* n_leaf_slots, float* boxes, int64_t* children, int32_t* axes,
                       int32_t* leaf_faces) {
  if (!vertices || !faces || n_vertices <= 0 || n_faces <= 0) return PR_E_ARG;
  for (int64_t f = 0; f < 3 * (int64_t)n_faces; f++)
    if (faces[f] < 0 || faces[f] >= n_vertices) return PR_E_ARG;
  MeshQbvh q;
  std::string err;
  int st = build_mesh_qbvh(vertices, faces, n_faces, q, err);
  if (st != PR_OK) return st;
  if (n_nodes) *n_nodes = (int64_t)q.nodes.size();
  if (n_leaf_slots) *n_leaf_slots = (int64_t)q.ref_leaf.size();
  export_qbvh(q, boxes, children, axes, leaf_faces);
  return PR_OK;
}

int pr_first_hit_dev(pr_ctx* c, const double* rays, int64_t n, int32_t* entity, int32_t* prim, double* t) {
  if (!c) return PR_E_ARG;
  if (!c->scene_ready) return fail(c, PR_E_SCENE, "no scene uploaded");
  if (n < 0 || (n > 0 && (!rays || !entity || !prim || !t))) return fail(c, PR_E_ARG, "bad first-hit arguments");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  const int se = ensure_exact(c, c->cur);
  if (se != PR_OK) return se;
  PR_CUDA(c, cudaMemsetAsync(c->errword.p, 0, 4, c->stream));
  PR_CUDA(c, cudaMemsetAsync(c->counters.p, 0, 128, c->stream));
  PR_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  PR_CUDA(c, launch_first_hit(c->cur.dev, rays, n, entity, prim, t, (uint32_t*)c->errword.p,
                              (unsigned long long*)c->counters.p, c->stream));
  PR_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  unsigned long long cnt[4];
  PR_CUDA(c, cudaMemcpyAsync(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  int st = check_device_errors(c);
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->stats = pr_render_stats{0, (uint64_t)n, cnt[2], cnt[3], ms, 1};
  return st;
}

int pr_first_hit(pr_ctx* c, const double* rays, int64_t n, int32_t* entity, int32_t* prim, double* t) {
  if (!c) return PR_E_ARG;
  if (n < 0 || (n > 0 && (!rays || !entity || !prim || !t))) return fail(c, PR_E_ARG, "bad first-hit arguments");
  if (n == 0) return PR_OK;
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  PR_CUDA(c, c->rays.ensure(sizeof(double) * 6 * (size_t)n));
  PR_CUDA(c, c->ires.ensure(sizeof(int32_t) * (size_t)n));
  PR_CUDA(c, c->jres.ensure(sizeof(int32_t) * (size_t)n));
  PR_CUDA(c, c->dres.ensure(sizeof(double) * (size_t)n));
  PR_CUDA(c, cudaMemcpyAsync(c->rays.p, rays, sizeof(double) * 6 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  int st = pr_first_hit_dev(c, (const double*)c->rays.p, n, (int32_t*)c->ires.p, (int32_t*)c->jres.p, (double*)c->dres.p);
  if (st != PR_OK) return st;
  PR_CUDA(c, cudaMemcpyAsync(entity, c->ires.p, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaMemcpyAsync(prim, c->jres.p, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaMemcpyAsync(t, c->dres.p, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  return PR_OK;
}

int pr_trace_fast(pr_ctx* c, const double* rays, int64_t n, int32_t* entity, int32_t* prim, double* t) {
  if (!c) return PR_E_ARG;
  if (!c->scene_ready) return fail(c, PR_E_SCENE, "no scene uploaded");
  if (n < 0 || (n > 0 && (!rays || !entity || !prim || !t))) return fail(c, PR_E_ARG, "bad trace arguments");
  if (n == 0) return PR_OK;
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  PR_CUDA(c, c->rays.ensure(sizeof(double) * 6 * (size_t)n));
  PR_CUDA(c, c->ires.ensure(sizeof(int32_t) * (size_t)n));
  PR_CUDA(c, c->jres.ensure(sizeof(int32_t) * (size_t)n));
  PR_CUDA(c, c->dres.ensure(sizeof(double) * (size_t)n));
  PR_CUDA(c, cudaMemcpyAsync(c->rays.p, rays, sizeof(double) * 6 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  PR_CUDA(c, cudaMemsetAsync(c->errword.p, 0, 4, c->stream));
  PR_CUDA(c, launch_trace_fast(c->cur.dev, (const double*)c->rays.p, n, (int32_t*)c->ires.p, (int32_t*)c->jres.p,
                               (double*)c->dres.p, (uint32_t*)c->errword.p, c->stream));
  int st = check_device_errors(c);
  if (st != PR_OK) return st;
  PR_CUDA(c, cudaMemcpyAsync(entity, c->ires.p, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaMemcpyAsync(prim, c->jres.p, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaMemcpyAsync(t, c->dres.p, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  return PR_OK;
}

}  // extern "C"

// CameraScreenPram (render.h:105-150) and the Run() sample set-up (:1129-1139)
int pr::prepare_render(pr_ctx* c, const pr_camera* cam, const pr_render_params* p, uint64_t sample_offset,
                          RenderCfg& g, const SceneObjData* scene) {
  const SceneObjData& sc = scene ? *scene : c->cur;
  if (!cam || !p) return fail(c, PR_E_ARG, "null camera or parameters");
  if (cam->width <= 0 || cam->height <= 0 || cam->width > 32768 || cam->height > 32768)
    return fail(c, PR_E_ARG, "image size out of range");
  if (p->samples <= 0 || p->supersamples <= 0) return fail(c, PR_E_ARG, "samples and supersamples must be positive");
  if (p->nee && sc.host.disk_light)
    return fail(c, PR_E_UNSUPPORTED,
                "an emitting disk is a light whose sampling the reference leaves undefined (Circle does not set the "
                "UVPlane axes randomPoint reads, circle.h:110-134); render it without next-event estimation");
  if (sc.kerr.enabled && (p->nee || (p->media && sc.host.medium.on)))
    return fail(c, PR_E_UNSUPPORTED, "Kerr scenes render without next-event estimation and media");
  if (sc.worm.enabled && (p->nee || (p->media && sc.host.medium.on)))
    return fail(c, PR_E_UNSUPPORTED, "wormhole scenes render without next-event estimation and media");
  if (sc.dev.has_sss && (sc.kerr.enabled || sc.worm.enabled))
    return fail(c, PR_E_UNSUPPORTED, "subsurface (dipole) materials render in straight-ray scenes only");
  if (p->mode == PR_MODE_MLT) {
    if (sc.kerr.enabled || sc.worm.enabled)
      return fail(c, PR_E_UNSUPPORTED, "Metropolis light transport traces straight rays only");
    if (sc.dev.has_sss) return fail(c, PR_E_UNSUPPORTED, "Metropolis light transport does not cover subsurface materials");
    if (!(p->mlt_mutation > 0.0) || !(p->mlt_pre_sample > 0.0) || p->mlt_chains < 0 || p->mlt_chains > (1 << 24))
      return fail(c, PR_E_ARG, "Metropolis parameters: mutation and pre_sample must be positive, chains in 0..2^24");
  }
  memset(&g, 0, sizeof(g));
  double dir[3] = {cam->dir[0], cam->dir[1], cam->dir[2]};
  double phi = std::atan2(dir[1], dir[0]);
  const double PI = 3.14159265358979323846264338327950288;
  if (phi < 0.0) phi += 2.0 * PI;
  if (std::fabs(phi - PI) < 1.0e-6 || phi < 1.0e-6 || std::fabs(phi - 2.0 * PI) < 1.0e-6) {
    dir[1] += 1.0e-6;
    const double len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    for (double& x : dir) x /= len;
  }
  auto crs = [](const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  };
  auto nrm = [](double* a) {
    const double l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    for (int k = 0; k < 3; k++) a[k] /= l;
  };
  const double sw = cam->screen_width * cam->width / cam->height, sh = cam->screen_height;
  double sx[3], sy[3];
  crs(dir, cam->up, sx);
  nrm(sx);
  for (double& x : sx) x *= sw;
  crs(sx, dir, sy);
  nrm(sy);
  for (double& x : sy) x *= sh;
  double ctr[3];
  for (int k = 0; k < 3; k++) ctr[k] = cam->position[k] + dir[k] * cam->screen_dist;
  g.cam_pos = make_float3((float)cam->position[0], (float)cam->position[1], (float)cam->position[2]);
  g.center = make_float3((float)ctr[0], (float)ctr[1], (float)ctr[2]);
  g.screen_x = make_float3((float)sx[0], (float)sx[1], (float)sx[2]);
  g.screen_y = make_float3((float)sy[0], (float)sy[1], (float)sy[2]);
  g.width = cam->width;
  g.height = cam->height;
  g.iw = (float)(1.0 / cam->width);
  g.ih = (float)(1.0 / cam->height);
  int samples = p->samples, ss = p->supersamples;
  double rate = 1.0 / ss;
  if (p->tent_filter) {
    samples = samples * ss * ss;
    ss = 1;
    rate = 0.5;
  }
  g.spp = samples * ss * ss;
  g.ss = ss;
  g.rate = (float)rate;
  if (p->total_spp < 0) return fail(c, PR_E_ARG, "total_spp must be >= 0");
  // smp = 1 / samples / ss^2 (render.h:1139), over the whole frame when sharded
  g.smp = p->total_spp > 0 ? (float)(1.0 / p->total_spp) : (float)(1.0 / samples / (ss * ss));
  g.tent = p->tent_filter ? 1 : 0;
  g.cutoff = (float)p->luminance_cutoff;
  g.sensor = (float)p->sensor_response;
  g.depth = p->depth;
  g.depth_limit = p->depth_limit;
  g.nee = p->nee;
  g.media = p->media;
  g.flags = p->flags;
  g.max_vertices = p->max_path_vertices > 0 ? p->max_path_vertices : 512;
  g.seed = p->seed;
  g.sample_offset = sample_offset;
  g.tiles_x = (uint32_t)((cam->width + 7) / 8);
  g.tiles_y = (uint32_t)((cam->height + 3) / 4);
  // enough sample chunks to keep ~1.2M threads in flight
  const double pixels = (double)cam->width * cam->height;
  int chunks = (int)std::ceil(1.2e6 / pixels);
  chunks = std::max(1, std::min(chunks, g.spp));
  g.chunks = chunks;
  return PR_OK;
}

extern "C" {

// paths in flight (slots of the wavefront pool); PR_WF_SLOTS overrides
static unsigned int wavefront_slots() {
  const char* e = getenv("PR_WF_SLOTS");
  long v = e ? strtol(e, nullptr, 10) : 0;
  if (v < 1024 || v > (1L << 24)) v = 1L << 21;
  return (unsigned int)v;
}

// PR_MODE_MLT (Render::RunMLT's estimator as parallel chains, mlt.cu): the
// bootstrap of samples x (int)(W H pre_sample) paths on the GPU, their
// luminances read back for b and for the chains' starts (systematic
// resampling in proportion to luminance), then samples x (int)(W H
// mutation) mutations spread over the chains in launches of a few
// iterations; the image is the chains' mean times the sensor response / 4.
static int render_mlt(pr_ctx* c, const RenderCfg& g0, const pr_render_params* p, float* rgb_dev, int accumulate,
                      uint64_t& paths_out, uint64_t& launches_out) {
  RenderCfg g = g0;
  g.tent = 1;
  const int64_t size = (int64_t)g.width * g.height;
  const int64_t seeds64 = (int64_t)p->samples * (int64_t)(size * p->mlt_pre_sample);
  const int64_t total = (int64_t)p->samples * (int64_t)(size * p->mlt_mutation);
  if (seeds64 < 1 || total < 1) return fail(c, PR_E_ARG, "Metropolis: no seed paths or no mutations at this size");
  if (seeds64 > ((int64_t)1 << 28)) return fail(c, PR_E_ARG, "Metropolis: at most 2^28 seed paths");
  MltCfg m;
  memset(&m, 0, sizeof(m));
  m.seeds = (int)seeds64;
  int64_t chains = p->mlt_chains > 0 ? p->mlt_chains : 65536;
  chains = std::max<int64_t>(1, std::min<int64_t>(chains, total));
  m.chains = (int)chains;
  m.mutations = (total + chains - 1) / chains;
  m.p_large = 0.5f;
  m.pdf = (float)(4.0 * (double)size);
  m.chain_scale = (float)(1.0 / (double)m.mutations);
  m.seed = g.seed + g.sample_offset * 0x9E3779B97F4A7C15ull;
  g.seed = m.seed;
  const size_t n3 = (size_t)size * 3;
  PR_CUDA(c, c->mlt_lum.ensure(sizeof(float) * (size_t)m.seeds));
  PR_CUDA(c, c->mlt_path.ensure(sizeof(float4) * (size_t)m.seeds));
  PR_CUDA(c, c->mlt_start.ensure(sizeof(int32_t) * (size_t)m.chains));
  PR_CUDA(c, c->mlt_u.ensure(sizeof(float) * (size_t)m.chains * kMltDims));
  PR_CUDA(c, c->mlt_cur.ensure(sizeof(float4) * (size_t)m.chains));
  PR_CUDA(c, c->mlt_acc.ensure(sizeof(float) * n3));
  PR_CUDA(c, cudaMemsetAsync(c->mlt_acc.p, 0, sizeof(float) * n3, c->stream));
  const DevScene& S = c->cur.dev;
  uint32_t* err = (uint32_t*)c->errword.p;
  unsigned long long* cnt = (unsigned long long*)c->counters.p;
  PR_CUDA(c, launch_mlt_seeds(S, g, m, (float*)c->mlt_lum.p, (float4*)c->mlt_path.p, err, cnt, c->stream));
  std::vector<float> lum((size_t)m.seeds);
  PR_CUDA(c, cudaMemcpyAsync(lum.data(), c->mlt_lum.p, sizeof(float) * lum.size(), cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  double sum = 0.0;
  for (float v : lum) sum += (double)v;
  paths_out = (uint64_t)m.seeds;
  launches_out = 2;  // bootstrap, resolve
  if (sum >= 1.0e-14) {  // a black bootstrap leaves the image black (render.h:528-531)
    m.b = (float)(sum / m.seeds);
    std::vector<int32_t> start((size_t)m.chains);
    double acc = 0.0;
    size_t i = 0;
    for (int k = 0; k < m.chains; k++) {
      const double target = (k + 0.5) / m.chains * sum;
      while (i + 1 < lum.size() && acc + (double)lum[i] < target) acc += (double)lum[i++];
      start[(size_t)k] = (int32_t)i;
    }
    PR_CUDA(c, cudaMemcpyAsync(c->mlt_start.p, start.data(), sizeof(int32_t) * start.size(), cudaMemcpyHostToDevice,
                               c->stream));
    PR_CUDA(c, launch_mlt_init(m, (const int32_t*)c->mlt_start.p, (const float4*)c->mlt_path.p,
                               (const float*)c->mlt_lum.p, (float*)c->mlt_u.p, (float4*)c->mlt_cur.p, c->stream));
    const int64_t per_launch = 8;
    for (int64_t it = 0; it < m.mutations; it += per_launch)
      PR_CUDA(c, launch_mlt_chains(S, g, m, it, std::min<int64_t>(m.mutations, it + per_launch), (float*)c->mlt_u.p,
                                   (float4*)c->mlt_cur.p, (float*)c->mlt_acc.p, err, cnt, c->stream));
    paths_out += (uint64_t)m.chains * (uint64_t)m.mutations;
    launches_out += 1 + (uint64_t)((m.mutations + per_launch - 1) / per_launch);
  }
  const float scale = (float)(0.25 * p->sensor_response / (double)m.chains);
  PR_CUDA(c, launch_mlt_resolve((const float*)c->mlt_acc.p, rgb_dev, (int)n3, scale, accumulate, c->stream));
  return PR_OK;
}

static int render_wavefront(pr_ctx* c, const RenderCfg& g, float* rgb_dev, int accumulate,
                            const SceneObjData* scene = nullptr) {
  const SceneObjData& sc = scene ? *scene : c->cur;
  const unsigned int P = c->tuned_slots ? c->tuned_slots : wavefront_slots();
  const uint64_t wh = (uint64_t)g.width * g.height;
  // camera samples per pass (sample table 28 B each); subsurface scenes take
  // smaller passes, whose frames (72 B each) come from a per-pass pool
  const bool sss = sc.dev.has_sss != 0;
  const uint64_t max_pass = sss ? (4ull << 20) : (64ull << 20);
  uint64_t layers = std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)g.spp, max_pass / wh));
  const uint64_t pass_cap = layers * wh;
  const uint64_t frame_cap = sss ? std::min<uint64_t>(8 * pass_cap, 1ull << 30) : 0;
  const size_t f4 = sizeof(float4);
  PR_CUDA(c, c->wf_o.ensure(f4 * P));
  PR_CUDA(c, c->wf_d.ensure(f4 * P));
  PR_CUDA(c, c->wf_beta.ensure(f4 * P));
  PR_CUDA(c, c->wf_dpw.ensure(f4 * P));
  PR_CUDA(c, c->wf_L.ensure(f4 * P));
  PR_CUDA(c, c->wf_sample.ensure(8ull * P));
  PR_CUDA(c, c->wf_hit.ensure(f4 * P));
  PR_CUDA(c, c->wf_hitv.ensure(4ull * P));
  PR_CUDA(c, c->wf_nee.ensure(f4 * 3 * P));
  PR_CUDA(c, c->wf_sho.ensure(f4 * 3 * P));
  PR_CUDA(c, c->wf_shd.ensure(f4 * 3 * P));
  PR_CUDA(c, c->wf_extq.ensure(4ull * P));
  PR_CUDA(c, c->wf_shq.ensure(4ull * 3 * P));
  const unsigned int spawn_cap = 2 * P;
  PR_CUDA(c, c->wf_spo.ensure(f4 * spawn_cap));
  PR_CUDA(c, c->wf_spd.ensure(f4 * spawn_cap));
  PR_CUDA(c, c->wf_spb.ensure(f4 * spawn_cap));
  PR_CUDA(c, c->wf_spw.ensure(f4 * spawn_cap));
  PR_CUDA(c, c->wf_sps.ensure(8ull * spawn_cap));
  PR_CUDA(c, c->wf_samp.ensure(24ull * pass_cap));
  PR_CUDA(c, c->wf_live.ensure(4ull * pass_cap));
  PR_CUDA(c, c->wf_pix.ensure(24ull * wh));
  PR_CUDA(c, c->wf_ctl.ensure(sizeof(WfCtl)));
  if (sss) {
    PR_CUDA(c, c->wf_frc.ensure(24ull * frame_cap));
    PR_CUDA(c, c->wf_fre.ensure(24ull * frame_cap));
    PR_CUDA(c, c->wf_frs.ensure(f4 * frame_cap));
    PR_CUDA(c, c->wf_frl.ensure(8ull * frame_cap));
    PR_CUDA(c, c->wf_spf.ensure(4ull * spawn_cap));
    PR_CUDA(c, c->wf_neef.ensure(4ull * P));
  }
  if (!c->wf_host_ctl) PR_CUDA(c, cudaMallocHost((void**)&c->wf_host_ctl, sizeof(WfCtl)));
  WfBufs B{};
  B.o = (float4*)c->wf_o.p;
  B.d = (float4*)c->wf_d.p;
  B.beta = (float4*)c->wf_beta.p;
  B.dpw = (float4*)c->wf_dpw.p;
  B.L = (float4*)c->wf_L.p;
  B.sample = (uint64_t*)c->wf_sample.p;
  B.hit = (float4*)c->wf_hit.p;
  B.hitv = (float*)c->wf_hitv.p;
  B.nee = (float4*)c->wf_nee.p;
  B.sh_o = (float4*)c->wf_sho.p;
  B.sh_d = (float4*)c->wf_shd.p;
  B.extq = (int*)c->wf_extq.p;
  B.shq = (int*)c->wf_shq.p;
  B.sp_o = (float4*)c->wf_spo.p;
  B.sp_d = (float4*)c->wf_spd.p;
  B.sp_beta = (float4*)c->wf_spb.p;
  B.sp_dpw = (float4*)c->wf_spw.p;
  B.sp_sample = (uint64_t*)c->wf_sps.p;
  B.samp = (long long*)c->wf_samp.p;
  B.live = (int*)c->wf_live.p;
  B.pix = (long long*)c->wf_pix.p;
  B.ctl = (WfCtl*)c->wf_ctl.p;
  B.fr_c = sss ? (long long*)c->wf_frc.p : nullptr;
  B.fr_e = sss ? (long long*)c->wf_fre.p : nullptr;
  B.fr_scale = sss ? (float4*)c->wf_frs.p : nullptr;
  B.fr_link = sss ? (int2*)c->wf_frl.p : nullptr;
  B.sp_frame = sss ? (int*)c->wf_spf.p : nullptr;
  B.neef = sss ? (int*)c->wf_neef.p : nullptr;
  B.frame_cap = (unsigned int)frame_cap;
  B.err = (uint32_t*)c->errword.p;
  B.counters = (unsigned long long*)c->counters.p;
  B.n_slots = P;
  B.spawn_cap = spawn_cap;
  B.max_iterations = 20000u;  // bounded device loop; a frame needs a few hundred
  WfLaunch L;
  L.shade_blocks = (P + 127) / 128;
  L.sss = sss ? 1 : 0;
  L.ext = (sc.dev.n_point_lights > 0 || sc.dev.has_tex) ? 1 : 0;
  // persistent traversal: one resident wave of blocks (more waves only queue
  // behind it and find the rays taken)
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || sms <= 0) sms = 152;
  const unsigned int bps = c->tuned_trace_bps ? c->tuned_trace_bps : kTraceBlocksPerSM;
  L.trace_blocks = std::min<unsigned int>((P + 127) / 128, (unsigned int)sms * bps);
  PR_CUDA(c, cudaMemsetAsync(c->wf_nee.p, 0, f4 * 3 * P, c->stream));
  PR_CUDA(c, cudaMemsetAsync(B.pix, 0, 24ull * wh, c->stream));
  if (sss) {
    PR_CUDA(c, cudaMemsetAsync(B.neef, 0xFF, 4ull * P, c->stream));  // -1: no frame takes shadow terms
    PR_CUDA(c, cudaMemsetAsync(c->wf_L.p, 0, f4 * P, c->stream));   // the frame lane of every slot: none
  }
  // PR_WF_HOST_LOOP=1 drives the iterations from the host instead of the
  // graph's device-side while loop: profilers that cannot see kernels inside
  // conditional graph nodes see every launch this way (same kernels, same work)
  const char* host_loop = getenv("PR_WF_HOST_LOOP");
  const bool use_graph = !(host_loop && host_loop[0] == '1') && !c->force_host_loop;
  if (use_graph && !c->wf_graph_failed &&
      (!c->wf_graph || c->wf_graph_slots != P || c->wf_graph_trace_blocks != L.trace_blocks ||
       c->wf_graph_variant != L.sss + 2 * L.ext)) {
    if (c->wf_graph) {
      cudaStreamSynchronize(c->stream);  // the previous render's launch has finished with it
      cudaGraphExecDestroy(c->wf_graph);
    }
    c->wf_graph = nullptr;
    cudaError_t e = wf_build_graph(L, c->stream, &c->wf_graph);
    if (e != cudaSuccess) {
      cudaGetLastError();
      c->wf_graph = nullptr;
      c->wf_graph_failed = true;  // fall back to the host-driven loop
    } else {
      c->wf_graph_slots = P;
      c->wf_graph_trace_blocks = L.trace_blocks;
      c->wf_graph_variant = L.sss + 2 * L.ext;
    }
  }
  c->wf_passes = 0;
  for (double& t : c->kernel_ms) t = 0.0;
  for (uint64_t first = 0; first < (uint64_t)g.spp; first += layers) {
    c->wf_passes++;
    const uint64_t n_layers = std::min<uint64_t>(layers, (uint64_t)g.spp - first);
    B.pass_first = first;
    B.pass_samples = n_layers * wh;
    PR_CUDA(c, cudaMemsetAsync(B.samp, 0, 24ull * B.pass_samples, c->stream));
    PR_CUDA(c, wf_set_constants(sc.dev, g, B, c->stream));
    PR_CUDA(c, wf_reset_launch(P, c->stream));
    if (use_graph && c->wf_graph) PR_CUDA(c, cudaGraphLaunch(c->wf_graph, c->stream));
    else PR_CUDA(c, wf_run_host_loop(L, c->wf_host_ctl, (const WfCtl*)B.ctl, c->stream, c->kernel_ms));
  }
  PR_CUDA(c, wf_resolve_launch(rgb_dev, (int)(3 * wh), accumulate, g.sensor, c->stream));
  return PR_OK;
}

int pr_render_dev(pr_ctx* c, const pr_camera* cam, const pr_render_params* p, float* rgb_dev, uint64_t sample_offset,
                  int accumulate) {
  if (!c) return PR_E_ARG;
  if (!c->scene_ready) return fail(c, PR_E_SCENE, "no scene uploaded");
  if (!rgb_dev) return fail(c, PR_E_ARG, "null output");
  if (p && p->mode != PR_MODE_MEGAKERNEL && p->mode != PR_MODE_WAVEFRONT && p->mode != PR_MODE_MLT)
    return fail(c, PR_E_ARG, "unknown render mode");
  RenderCfg g;
  int st = prepare_render(c, cam, p, sample_offset, g);
  if (st != PR_OK) return st;
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  const size_t n3 = (size_t)g.width * g.height * 3;
  PR_CUDA(c, cudaMemsetAsync(c->errword.p, 0, 4, c->stream));
  PR_CUDA(c, cudaMemsetAsync(c->counters.p, 0, 128, c->stream));
  PR_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  const bool kerr = c->cur.kerr.enabled != 0, worm = c->cur.worm.enabled != 0;
  uint64_t mlt_paths = 0, mlt_launches = 0;
  if (kerr || worm) {
    // every scene query of a Kerr or wormhole scene is a geodesic trace: one form only
    PR_CUDA(c, c->partial.ensure(sizeof(float) * n3 * (size_t)g.chunks));
    if (kerr)
      PR_CUDA(c, launch_kerr_render(c->cur.dev, c->cur.kerr, g, (float*)c->partial.p, (uint32_t*)c->errword.p,
                                    (unsigned long long*)c->counters.p, c->stream));
    else
      PR_CUDA(c, launch_worm_render(c->cur.dev, c->cur.worm, g, (float*)c->partial.p, (uint32_t*)c->errword.p,
                                    (unsigned long long*)c->counters.p, c->stream));
    PR_CUDA(c, launch_reduce((const float*)c->partial.p, rgb_dev, (int)n3, g.chunks, accumulate, c->stream));
  } else if (p->mode == PR_MODE_MLT) {
    st = render_mlt(c, g, p, rgb_dev, accumulate, mlt_paths, mlt_launches);
    if (st != PR_OK) return st;
  } else if (p->mode == PR_MODE_WAVEFRONT) {
    st = render_wavefront(c, g, rgb_dev, accumulate);
    if (st != PR_OK) return st;
  } else {
    PR_CUDA(c, c->partial.ensure(sizeof(float) * n3 * (size_t)g.chunks));
    PR_CUDA(c, launch_megakernel(c->cur.dev, g, (float*)c->partial.p, (uint32_t*)c->errword.p,
                                 (unsigned long long*)c->counters.p, c->stream));
    PR_CUDA(c, launch_reduce((const float*)c->partial.p, rgb_dev, (int)n3, g.chunks, accumulate, c->stream));
  }
  PR_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  unsigned long long cnt[16];
  PR_CUDA(c, cudaMemcpyAsync(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  st = check_device_errors(c);
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  const bool wf = p->mode == PR_MODE_WAVEFRONT && !kerr && !worm;
  const bool mlt = p->mode == PR_MODE_MLT && !kerr && !worm;
  // MLT: paths = bootstrap paths + proposals
  const uint64_t paths = wf ? (uint64_t)g.spp * g.width * g.height : mlt ? mlt_paths : cnt[0];
  // wavefront: reset per pass + 4 per iteration + resolve; megakernel: kernel + reduce;
  // MLT: bootstrap, chain start, the chains' launches, resolve
  const uint64_t launches = wf ? 4 * cnt[5] + c->wf_passes + 1 : mlt ? mlt_launches : 2;
  // Kerr counters: [1] accepted RK steps, [2] RK attempts, [3] segment scene
  // tests, reported as pr_kerr_trace does (segments, nodes_visited, tri_tests)
  c->stats = kerr ? pr_render_stats{paths, cnt[3], cnt[1], cnt[2], ms, launches}
                  : pr_render_stats{paths, cnt[1], cnt[2], cnt[3], ms, launches};
  for (int k = 0; k < 3; k++) c->shadow_counts[k] = wf ? cnt[6 + k] : 0;
  return st;
}

int pr_render(pr_ctx* c, const pr_camera* cam, const pr_render_params* p, float* rgb, uint64_t sample_offset,
              int accumulate) {
  if (!c) return PR_E_ARG;
  if (!cam || !rgb) return fail(c, PR_E_ARG, "null camera or output");
  if (cam->width <= 0 || cam->height <= 0 || cam->width > 32768 || cam->height > 32768)
    return fail(c, PR_E_ARG, "image size out of range");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  const size_t bytes = sizeof(float) * 3 * (size_t)cam->width * cam->height;
  PR_CUDA(c, c->out.ensure(bytes));
  if (accumulate) PR_CUDA(c, cudaMemcpyAsync(c->out.p, rgb, bytes, cudaMemcpyHostToDevice, c->stream));
  int st = pr_render_dev(c, cam, p, (float*)c->out.p, sample_offset, accumulate);
  if (st != PR_OK) return st;
  PR_CUDA(c, cudaMemcpyAsync(rgb, c->out.p, bytes, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  return PR_OK;
}

static int adjoint_checks(pr_ctx* c, const pr_render_params* p) {
  if (!c->scene_ready) return fail(c, PR_E_SCENE, "no scene uploaded");
  if (c->cur.kerr.enabled || c->cur.worm.enabled)
    return fail(c, PR_E_UNSUPPORTED, "the adjoint pass traces straight rays only");
  if (p && p->media && c->cur.host.medium.on) return fail(c, PR_E_UNSUPPORTED, "the adjoint pass does not cover media");
  if (c->cur.dev.has_sss) return fail(c, PR_E_UNSUPPORTED, "the adjoint pass does not cover subsurface materials");
  if (c->cur.dev.n_point_lights > 0)
    return fail(c, PR_E_UNSUPPORTED, "the adjoint pass covers area lights only (no parallel, spot or infinity lights)");
  if (c->cur.dev.has_tex & 1)
    return fail(c, PR_E_UNSUPPORTED, "the adjoint pass differentiates material colours, not textures");
  if (c->cur.dev.has_tex & 2)
    return fail(c, PR_E_UNSUPPORTED, "the adjoint pass shades with face normals only (no smooth meshes)");
  for (const GMaterial& m : c->cur.host.mats)
    if (m.type == PR_MAT_WARD || m.type == PR_MAT_PHONG)
      return fail(c, PR_E_UNSUPPORTED, "the adjoint pass does not cover Ward or Phong materials (their lobes scale "
                                       "with the specular colour, not the colour it differentiates)");
  if ((int)c->cur.host.mats.size() > kAdjMaterials)
    return fail(c, PR_E_UNSUPPORTED, "the adjoint pass tracks at most " + std::to_string(kAdjMaterials) + " materials");
  return PR_OK;
}

int pr_render_adjoint_dev(pr_ctx* c, const pr_camera* cam, const pr_render_params* p, const float* dl_drgb,
                          uint64_t sample_offset, double* d_color, double* d_emission) {
  if (!c) return PR_E_ARG;
  int st = adjoint_checks(c, p);
  if (st != PR_OK) return st;
  if (!dl_drgb) return fail(c, PR_E_ARG, "null dL/d(image)");
  RenderCfg g;
  st = prepare_render(c, cam, p, sample_offset, g);
  if (st != PR_OK) return st;
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  const int n_mat = (int)c->cur.host.mats.size();
  // scratch for outputs the caller does not want
  PR_CUDA(c, c->adj_scratch.ensure(2 * 3 * sizeof(double) * (size_t)std::max(n_mat, 1)));
  double* dc = d_color ? d_color : (double*)c->adj_scratch.p;
  double* de = d_emission ? d_emission : (double*)c->adj_scratch.p + 3 * std::max(n_mat, 1);
  if (!d_color) PR_CUDA(c, cudaMemsetAsync(dc, 0, 3 * sizeof(double) * n_mat, c->stream));
  if (!d_emission) PR_CUDA(c, cudaMemsetAsync(de, 0, 3 * sizeof(double) * n_mat, c->stream));
  PR_CUDA(c, cudaMemsetAsync(c->errword.p, 0, 4, c->stream));
  PR_CUDA(c, cudaMemsetAsync(c->counters.p, 0, 128, c->stream));
  PR_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  PR_CUDA(c, launch_adjoint(c->cur.dev, g, dl_drgb, n_mat, dc, de, (uint32_t*)c->errword.p,
                            (unsigned long long*)c->counters.p, c->stream));
  PR_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  unsigned long long cnt[16];
  PR_CUDA(c, cudaMemcpyAsync(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  st = check_device_errors(c);
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->stats = pr_render_stats{cnt[0], cnt[1], cnt[2], cnt[3], ms, 1};
  return st;
}

int pr_render_adjoint(pr_ctx* c, const pr_camera* cam, const pr_render_params* p, const float* dl_drgb,
                      uint64_t sample_offset, double* d_color, double* d_emission, double* d_emission_scale) {
  if (!c) return PR_E_ARG;
  int st = adjoint_checks(c, p);
  if (st != PR_OK) return st;
  if (!cam || !dl_drgb) return fail(c, PR_E_ARG, "null camera or dL/d(image)");
  if (cam->width <= 0 || cam->height <= 0 || cam->width > 32768 || cam->height > 32768)
    return fail(c, PR_E_ARG, "image size out of range");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  const size_t bytes = sizeof(float) * 3 * (size_t)cam->width * cam->height;
  const int n_mat = (int)c->cur.host.mats.size();
  const size_t gb = 3 * sizeof(double) * (size_t)std::max(n_mat, 1);
  PR_CUDA(c, c->out.ensure(bytes));
  PR_CUDA(c, c->adj_grad.ensure(2 * gb));
  PR_CUDA(c, cudaMemcpyAsync(c->out.p, dl_drgb, bytes, cudaMemcpyHostToDevice, c->stream));
  PR_CUDA(c, cudaMemsetAsync(c->adj_grad.p, 0, 2 * gb, c->stream));
  double* dc = (double*)c->adj_grad.p;
  double* de = dc + 3 * std::max(n_mat, 1);
  st = pr_render_adjoint_dev(c, cam, p, (const float*)c->out.p, sample_offset, dc, de);
  if (st != PR_OK) return st;
  std::vector<double> h(6 * (size_t)std::max(n_mat, 1));
  PR_CUDA(c, cudaMemcpyAsync(h.data(), c->adj_grad.p, 2 * gb, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  const double* hc = h.data();
  const double* he = h.data() + 3 * std::max(n_mat, 1);
  double scale = 0.0;
  for (int m = 0; m < n_mat; m++)
    for (int k = 0; k < 3; k++) {
      if (d_color) d_color[3 * m + k] += hc[3 * m + k];
      if (d_emission) d_emission[3 * m + k] += he[3 * m + k];
      scale += he[3 * m + k] * c->cur.host.mats[m].emission_d[k];
    }
  if (d_emission_scale) *d_emission_scale = scale;
  return PR_OK;
}

// Autotuner: times one short frame (the caller's camera and parameters,
// one camera sample per pixel) for each candidate wavefront pool size and
// traversal grid, keeps the fastest for this context.  The image does not
// depend on either (per-branch streams, order-independent fixed-point sums).
int pr_autotune_wavefront(pr_ctx* c, const pr_camera* cam, const pr_render_params* p, int32_t* slots_out,
                          int32_t* trace_blocks_per_sm_out, double* ms_out) {
  if (!c) return PR_E_ARG;
  if (!c->scene_ready) return fail(c, PR_E_SCENE, "no scene uploaded");
  if (!cam || !p) return fail(c, PR_E_ARG, "null camera or parameters");
  if (c->cur.kerr.enabled || c->cur.worm.enabled)
    return fail(c, PR_E_UNSUPPORTED, "Kerr and wormhole scenes do not use the wavefront form");
  const unsigned int cand_slots[] = {1u << 19, 1u << 20, 1u << 21, 1u << 22};
  const unsigned int cand_bps[] = {kTraceBlocksPerSM / 2, kTraceBlocksPerSM, 2 * kTraceBlocksPerSM};
  // a tuning frame of the caller's scene with enough camera samples to keep
  // the largest pool full for a while (twice its slots, at least one per pixel)
  pr_render_params q = *p;
  q.mode = PR_MODE_WAVEFRONT;
  const double pixels = std::max(1.0, (double)cam->width * (double)cam->height);
  q.samples = (int32_t)std::max(1.0, std::ceil(2.0 * (double)cand_slots[3] / pixels));
  q.supersamples = 1;
  q.tent_filter = 0;
  q.total_spp = 0;
  const size_t bytes = sizeof(float) * 3 * (size_t)cam->width * cam->height;
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  PR_CUDA(c, c->out.ensure(bytes));
  double best = 1e300;
  unsigned int best_s = 0, best_b = 0;
  // candidates run the host-driven loop (no graph is rebuilt per candidate);
  // the figure compared is the sum of the kernels' own device times
  c->force_host_loop = true;
  int st = PR_OK;
  for (unsigned int sl : cand_slots) {
    for (unsigned int b : cand_bps) {
      c->tuned_slots = sl;
      c->tuned_trace_bps = b;
      double t = 0.0;
      for (int rep = 0; rep < 2 && st == PR_OK; rep++) {  // the first run grows the pool
        st = pr_render_dev(c, cam, &q, (float*)c->out.p, 0, 0);
        t = c->kernel_ms[0] + c->kernel_ms[1] + c->kernel_ms[2] + c->kernel_ms[3];
      }
      if (st != PR_OK) break;
      if (t < best) {
        best = t;
        best_s = sl;
        best_b = b;
      }
    }
    if (st != PR_OK) break;
  }
  c->force_host_loop = false;
  c->tuned_slots = best_s;
  c->tuned_trace_bps = best_b;
  if (st != PR_OK) return st;
  if (slots_out) *slots_out = (int32_t)best_s;
  if (trace_blocks_per_sm_out) *trace_blocks_per_sm_out = (int32_t)best_b;
  if (ms_out) *ms_out = best;
  return PR_OK;
}

int pr_last_kernel_times(pr_ctx* c, double* ms, unsigned long long* shadow_counts, int n) {
  if (!c || !ms || n < 0) return PR_E_ARG;
  for (int k = 0; k < n && k < 4; k++) ms[k] = c->kernel_ms[k];
  if (shadow_counts)
    for (int k = 0; k < 3; k++) shadow_counts[k] = c->shadow_counts[k];
  return PR_OK;
}

int pr_last_render_stats(pr_ctx* c, pr_render_stats* s) {
  if (!c || !s) return PR_E_ARG;
  *s = c->stats;
  return PR_OK;
}

int pr_kerr_trace_dev(pr_ctx* c, const double* rays, int64_t n, int32_t* status, double* final_bl, double* exit_dir,
                      int32_t* steps, int32_t* hit_entity, double* hit_t) {
  if (!c) return PR_E_ARG;
  if (!c->scene_ready) return fail(c, PR_E_SCENE, "no scene uploaded");
  if (!c->cur.kerr.enabled) return fail(c, PR_E_SCENE, "the scene has no black hole");
  if (n < 0 || (n > 0 && !rays)) return fail(c, PR_E_ARG, "bad ray buffer");
  if (n > (int64_t)1 << 31) return fail(c, PR_E_ARG, "at most 2^31 rays per call");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  PR_CUDA(c, cudaMemsetAsync(c->errword.p, 0, 4, c->stream));
  PR_CUDA(c, cudaMemsetAsync(c->counters.p, 0, 128, c->stream));
  PR_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  KerrOut o{status, final_bl, exit_dir, steps, hit_entity, hit_t};
  PR_CUDA(c, launch_kerr_trace(c->cur.dev, c->cur.kerr, rays, n, o, (uint32_t*)c->errword.p,
                               (unsigned long long*)c->counters.p, c->stream));
  PR_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  unsigned long long cnt[16];
  PR_CUDA(c, cudaMemcpyAsync(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  int st = check_device_errors(c);
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  // paths = rays, segments = segment scene tests, nodes_visited = accepted
  // steps, tri_tests = RK45 attempts (5 geodesic evaluations each)
  c->stats = pr_render_stats{cnt[0], cnt[3], cnt[1], cnt[2], ms, n > 0 ? 1ull : 0ull};
  return st;
}

int pr_kerr_trace(pr_ctx* c, const double* rays, int64_t n, int32_t* status, double* final_bl, double* exit_dir,
                  int32_t* steps, int32_t* hit_entity, double* hit_t) {
  if (!c) return PR_E_ARG;
  if (n < 0 || (n > 0 && !rays)) return fail(c, PR_E_ARG, "bad ray buffer");
  if (n > (int64_t)1 << 31) return fail(c, PR_E_ARG, "at most 2^31 rays per call");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  const size_t un = (size_t)std::max<int64_t>(n, 1);
  PR_CUDA(c, c->rays.ensure(48 * un));
  PR_CUDA(c, c->k_status.ensure(4 * un));
  PR_CUDA(c, c->k_bl.ensure(24 * un));
  PR_CUDA(c, c->k_dir.ensure(24 * un));
  PR_CUDA(c, c->k_steps.ensure(4 * un));
  PR_CUDA(c, c->k_ent.ensure(4 * un));
  PR_CUDA(c, c->k_t.ensure(8 * un));
  if (n > 0) PR_CUDA(c, cudaMemcpyAsync(c->rays.p, rays, 48 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  int st = pr_kerr_trace_dev(c, (const double*)c->rays.p, n, status ? (int32_t*)c->k_status.p : nullptr,
                             final_bl ? (double*)c->k_bl.p : nullptr, exit_dir ? (double*)c->k_dir.p : nullptr,
                             steps ? (int32_t*)c->k_steps.p : nullptr, hit_entity ? (int32_t*)c->k_ent.p : nullptr,
                             hit_t ? (double*)c->k_t.p : nullptr);
  if (st != PR_OK || n == 0) return st;
  const size_t sn = (size_t)n;
  if (status) PR_CUDA(c, cudaMemcpyAsync(status, c->k_status.p, 4 * sn, cudaMemcpyDeviceToHost, c->stream));
  if (final_bl) PR_CUDA(c, cudaMemcpyAsync(final_bl, c->k_bl.p, 24 * sn, cudaMemcpyDeviceToHost, c->stream));
  if (exit_dir) PR_CUDA(c, cudaMemcpyAsync(exit_dir, c->k_dir.p, 24 * sn, cudaMemcpyDeviceToHost, c->stream));
  if (steps) PR_CUDA(c, cudaMemcpyAsync(steps, c->k_steps.p, 4 * sn, cudaMemcpyDeviceToHost, c->stream));
  if (hit_entity) PR_CUDA(c, cudaMemcpyAsync(hit_entity, c->k_ent.p, 4 * sn, cudaMemcpyDeviceToHost, c->stream));
  if (hit_t) PR_CUDA(c, cudaMemcpyAsync(hit_t, c->k_t.p, 8 * sn, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  return PR_OK;
}

int pr_wormhole_trace_dev(pr_ctx* c, const double* rays, int64_t n, int32_t* status, double* final_y,
                          double* exit_dir, int32_t* steps, int32_t* hit_entity) {
  if (!c) return PR_E_ARG;
  if (!c->scene_ready) return fail(c, PR_E_SCENE, "no scene uploaded");
  if (!c->cur.worm.enabled) return fail(c, PR_E_SCENE, "the scene has no wormhole");
  if (n < 0 || (n > 0 && !rays)) return fail(c, PR_E_ARG, "bad ray buffer");
  if (n > (int64_t)1 << 31) return fail(c, PR_E_ARG, "at most 2^31 rays per call");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  PR_CUDA(c, cudaMemsetAsync(c->errword.p, 0, 4, c->stream));
  PR_CUDA(c, cudaMemsetAsync(c->counters.p, 0, 128, c->stream));
  PR_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  WormOut o{status, final_y, exit_dir, steps, hit_entity};
  PR_CUDA(c, launch_worm_trace(c->cur.dev, c->cur.worm, rays, n, o, (uint32_t*)c->errword.p,
                               (unsigned long long*)c->counters.p, c->stream));
  PR_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  unsigned long long cnt[16];
  PR_CUDA(c, cudaMemcpyAsync(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  int st = check_device_errors(c);
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  // as pr_kerr_trace: paths = rays, segments = segment scene tests,
  // nodes_visited = accepted steps, tri_tests = RK45 attempts
  c->stats = pr_render_stats{cnt[0], cnt[3], cnt[1], cnt[2], ms, n > 0 ? 1ull : 0ull};
  return st;
}

int pr_wormhole_trace(pr_ctx* c, const double* rays, int64_t n, int32_t* status, double* final_y, double* exit_dir,
                      int32_t* steps, int32_t* hit_entity) {
  if (!c) return PR_E_ARG;
  if (n < 0 || (n > 0 && !rays)) return fail(c, PR_E_ARG, "bad ray buffer");
  if (n > (int64_t)1 << 31) return fail(c, PR_E_ARG, "at most 2^31 rays per call");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  const size_t un = (size_t)std::max<int64_t>(n, 1);
  PR_CUDA(c, c->rays.ensure(48 * un));
  PR_CUDA(c, c->k_status.ensure(4 * un));
  PR_CUDA(c, c->k_bl.ensure(24 * un));
  PR_CUDA(c, c->k_dir.ensure(24 * un));
  PR_CUDA(c, c->k_steps.ensure(4 * un));
  PR_CUDA(c, c->k_ent.ensure(4 * un));
  if (n > 0) PR_CUDA(c, cudaMemcpyAsync(c->rays.p, rays, 48 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  int st = pr_wormhole_trace_dev(c, (const double*)c->rays.p, n, status ? (int32_t*)c->k_status.p : nullptr,
                                 final_y ? (double*)c->k_bl.p : nullptr, exit_dir ? (double*)c->k_dir.p : nullptr,
                                 steps ? (int32_t*)c->k_steps.p : nullptr, hit_entity ? (int32_t*)c->k_ent.p : nullptr);
  if (st != PR_OK || n == 0) return st;
  const size_t sn = (size_t)n;
  if (status) PR_CUDA(c, cudaMemcpyAsync(status, c->k_status.p, 4 * sn, cudaMemcpyDeviceToHost, c->stream));
  if (final_y) PR_CUDA(c, cudaMemcpyAsync(final_y, c->k_bl.p, 24 * sn, cudaMemcpyDeviceToHost, c->stream));
  if (exit_dir) PR_CUDA(c, cudaMemcpyAsync(exit_dir, c->k_dir.p, 24 * sn, cudaMemcpyDeviceToHost, c->stream));
  if (steps) PR_CUDA(c, cudaMemcpyAsync(steps, c->k_steps.p, 4 * sn, cudaMemcpyDeviceToHost, c->stream));
  if (hit_entity) PR_CUDA(c, cudaMemcpyAsync(hit_entity, c->k_ent.p, 4 * sn, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  return PR_OK;
}

int pr_image_to_rgb8_dev(pr_ctx* c, const float* rgb_dev, int32_t width, int32_t height, double gamma_offset,
                         uint8_t* out_dev) {
  if (!c) return PR_E_ARG;
  if (width <= 0 || height <= 0 || (int64_t)width * height > ((int64_t)1 << 30)) return fail(c, PR_E_ARG, "bad image size");
  if (!rgb_dev || !out_dev) return fail(c, PR_E_ARG, "null image buffer");
  if (gamma_offset < -0.01) return fail(c, PR_E_ARG, "negative gamma_offset");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  PR_CUDA(c, launch_to_rgb8(rgb_dev, width, height, gamma_offset, out_dev, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  return PR_OK;
}

int pr_image_to_rgb8(pr_ctx* c, const float* rgb, int32_t width, int32_t height, double gamma_offset, uint8_t* out) {
  if (!c) return PR_E_ARG;
  if (width <= 0 || height <= 0 || (int64_t)width * height > ((int64_t)1 << 30)) return fail(c, PR_E_ARG, "bad image size");
  if (!rgb || !out) return fail(c, PR_E_ARG, "null image buffer");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();
  const size_t n3 = (size_t)width * height * 3;
  // staging in the context's ray buffer: the float image, then the bytes
  PR_CUDA(c, c->rays.ensure(n3 * sizeof(float) + n3));
  float* d_in = (float*)c->rays.p;
  uint8_t* d_out = (uint8_t*)(d_in + n3);
  PR_CUDA(c, cudaMemcpyAsync(d_in, rgb, n3 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  const int st = pr_image_to_rgb8_dev(c, d_in, width, height, gamma_offset, d_out);
  if (st != PR_OK) return st;
  PR_CUDA(c, cudaMemcpyAsync(out, d_out, n3, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  return PR_OK;
}

int pr_image_to_rgbe_dev(pr_ctx* c, const float* rgb_dev, int32_t width, int32_t height, uint8_t* out_dev) {
  if (!c) return PR_E_ARG;
  if (width <= 0 || height <= 0 || (int64_t)width * height > ((int64_t)1 << 30)) return fail(c, PR_E_ARG, "bad image size");
  if (!rgb_dev || !out_dev) return fail(c, PR_E_ARG, "null image buffer");
  if (((uintptr_t)out_dev & 3) != 0) return fail(c, PR_E_ARG, "the RGBE buffer must be 4-byte aligned");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  PR_CUDA(c, launch_to_rgbe(rgb_dev, width, height, out_dev, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  return PR_OK;
}

int pr_image_to_rgbe(pr_ctx* c, const float* rgb, int32_t width, int32_t height, uint8_t* out) {
  if (!c) return PR_E_ARG;
  if (width <= 0 || height <= 0 || (int64_t)width * height > ((int64_t)1 << 30)) return fail(c, PR_E_ARG, "bad image size");
  if (!rgb || !out) return fail(c, PR_E_ARG, "null image buffer");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();
  const size_t n = (size_t)width * height;
  // staging in the context's ray buffer: the float image, then the RGBE pixels
  PR_CUDA(c, c->rays.ensure(n * 3 * sizeof(float) + n * 4));
  float* d_in = (float*)c->rays.p;
  uint8_t* d_out = (uint8_t*)(d_in + 3 * n);
  PR_CUDA(c, cudaMemcpyAsync(d_in, rgb, n * 3 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  const int st = pr_image_to_rgbe_dev(c, d_in, width, height, d_out);
  if (st != PR_OK) return st;
  PR_CUDA(c, cudaMemcpyAsync(out, d_out, n * 4, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  return PR_OK;
}

// the scene has a disk_map disk under its black hole (shaded from the disk texture)
static bool has_kerr_disk(const SceneObjData& o) {
  for (const GEntity& e : o.host.ents)
    if (e.kerr_disk) return true;
  return false;
}

int pr_kerr_disk_shade(pr_ctx* c, int entity, const double* points, int64_t n, int32_t* valid, double* color,
                       double* emission, double* alpha) {
  if (!c) return PR_E_ARG;
  if (!c->scene_ready) return fail(c, PR_E_SCENE, "no scene uploaded");
  if (!c->cur.kerr.enabled || !c->cur.kerr.disk_tex) return fail(c, PR_E_SCENE, "the scene has no accretion-disk texture");
  if (entity < 0 || entity >= (int)c->cur.host.ents.size() || c->cur.host.ents[entity].type != PR_ENT_CIRCLE)
    return fail(c, PR_E_ARG, "entity is not a disk");
  if (n < 0 || (n > 0 && (!points || !valid || !color || !emission || !alpha))) return fail(c, PR_E_ARG, "bad buffers");
  if (n > (int64_t)1 << 28) return fail(c, PR_E_ARG, "at most 2^28 points per call");
  if (n == 0) return PR_OK;
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  const size_t un = (size_t)n;
  // staging: points 3, colour 3, emission 3, alpha 1 doubles + valid per point
  PR_CUDA(c, c->k_sens.ensure(un * (10 * sizeof(double) + sizeof(int32_t))));
  double* d_pts = (double*)c->k_sens.p;
  double* d_col = d_pts + 3 * un;
  double* d_em = d_col + 3 * un;
  double* d_a = d_em + 3 * un;
  int32_t* d_v = (int32_t*)(d_a + un);
  PR_CUDA(c, cudaMemcpyAsync(d_pts, points, 24 * un, cudaMemcpyHostToDevice, c->stream));
  PR_CUDA(c, launch_kerr_disk_shade(c->cur.dev, c->cur.kerr, entity, d_pts, n, d_v, d_col, d_em, d_a, c->stream));
  PR_CUDA(c, cudaMemcpyAsync(valid, d_v, 4 * un, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaMemcpyAsync(color, d_col, 24 * un, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaMemcpyAsync(emission, d_em, 24 * un, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaMemcpyAsync(alpha, d_a, 8 * un, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  return PR_OK;
}

static int kerr_sens_common(pr_ctx* c, const double* rays, int64_t n, const double* basis, const double* cot,
                            int32_t* status, double* jac_dir, double* jac_bl, double* grad) {
  if (!c) return PR_E_ARG;
  if (!c->scene_ready) return fail(c, PR_E_SCENE, "no scene uploaded");
  if (!c->cur.kerr.enabled) return fail(c, PR_E_SCENE, "the scene has no black hole");
  if (has_kerr_disk(c->cur))
    return fail(c, PR_E_UNSUPPORTED, "the ray-bundle Jacobian does not differentiate the accretion disk's alpha test");
  if (n < 0 || (n > 0 && !rays)) return fail(c, PR_E_ARG, "bad ray buffer");
  if (n > (int64_t)1 << 28) return fail(c, PR_E_ARG, "at most 2^28 rays per call");
  if (n == 0) return PR_OK;
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  const size_t un = (size_t)n;
  // one staging buffer: rays 6, basis 6, cotangent 3, jac_dir 6, jac_bl 4, grad 2 doubles + status per ray
  PR_CUDA(c, c->k_sens.ensure(un * (27 * sizeof(double) + sizeof(int32_t))));
  double* d_rays = (double*)c->k_sens.p;
  double* d_basis = d_rays + 6 * un;
  double* d_cot = d_basis + 6 * un;
  double* d_jd = d_cot + 3 * un;
  double* d_jb = d_jd + 6 * un;
  double* d_g = d_jb + 4 * un;
  int32_t* d_st = (int32_t*)(d_g + 2 * un);
  PR_CUDA(c, cudaMemcpyAsync(d_rays, rays, 48 * un, cudaMemcpyHostToDevice, c->stream));
  if (basis) PR_CUDA(c, cudaMemcpyAsync(d_basis, basis, 48 * un, cudaMemcpyHostToDevice, c->stream));
  if (cot) PR_CUDA(c, cudaMemcpyAsync(d_cot, cot, 24 * un, cudaMemcpyHostToDevice, c->stream));
  PR_CUDA(c, cudaMemsetAsync(c->errword.p, 0, 4, c->stream));
  PR_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  PR_CUDA(c, launch_kerr_sensitivity(c->cur.dev, c->cur.kerr, d_rays, basis ? d_basis : nullptr, n, cot ? d_cot : nullptr,
                                     d_st, d_jd, d_jb, grad ? d_g : nullptr, (uint32_t*)c->errword.p, c->stream));
  PR_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  int st = check_device_errors(c);
  if (st != PR_OK) return st;
  if (status) PR_CUDA(c, cudaMemcpyAsync(status, d_st, 4 * un, cudaMemcpyDeviceToHost, c->stream));
  if (jac_dir) PR_CUDA(c, cudaMemcpyAsync(jac_dir, d_jd, 48 * un, cudaMemcpyDeviceToHost, c->stream));
  if (jac_bl) PR_CUDA(c, cudaMemcpyAsync(jac_bl, d_jb, 32 * un, cudaMemcpyDeviceToHost, c->stream));
  if (grad) PR_CUDA(c, cudaMemcpyAsync(grad, d_g, 16 * un, cudaMemcpyDeviceToHost, c->stream));
  PR_CUDA(c, cudaStreamSynchronize(c->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->stats = pr_render_stats{(unsigned long long)n, 0, 0, 0, ms, 1};
  return PR_OK;
}

int pr_kerr_sensitivity(pr_ctx* c, const double* rays, int64_t n, const double* basis, int32_t* status,
                        double* jac_dir, double* jac_bl) {
  return kerr_sens_common(c, rays, n, basis, nullptr, status, jac_dir, jac_bl, nullptr);
}

int pr_kerr_sensitivity_adjoint(pr_ctx* c, const double* rays, int64_t n, const double* basis,
                                const double* cotangent, double* grad) {
  if (c && n > 0 && (!cotangent || !grad)) return fail(c, PR_E_ARG, "null cotangent or gradient");
  return kerr_sens_common(c, rays, n, basis, cotangent, nullptr, nullptr, nullptr, grad);
}

// Many jobs (scene object, camera, parameters, output) as one captured CUDA
// graph: each job is the megakernel form (one render kernel + the ordered
// chunk reduction) on its own branch of the graph, so small and large
// frames overlap on the GPU; the graph is re-captured per call and updated
// in place when its shape is unchanged.
int pr_render_batch(pr_ctx* c, int n, const pr_job* jobs) {
  if (!c) return PR_E_ARG;
  if (n <= 0 || !jobs) return fail(c, PR_E_ARG, "empty batch");
  if (n > 4096) return fail(c, PR_E_ARG, "at most 4096 jobs per batch");
  PR_CUDA(c, cudaSetDevice(c->device));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  std::vector<RenderCfg> cfg((size_t)n);
  std::vector<size_t> off((size_t)n + 1, 0);
  uint64_t paths = 0;
  bool all_kerr = true;
  for (int j = 0; j < n; j++) {
    const pr_job& J = jobs[j];
    if (!J.scene) return fail(c, PR_E_ARG, "job " + std::to_string(j) + ": null scene");
    all_kerr = all_kerr && J.scene->data.kerr.enabled;
    if (!J.rgb_dev) return fail(c, PR_E_ARG, "job " + std::to_string(j) + ": null output");
    if (J.params.mode == PR_MODE_MLT)
      return fail(c, PR_E_UNSUPPORTED, "job " + std::to_string(j) + ": Metropolis renders run through pr_render");
    int st = prepare_render(c, &J.camera, &J.params, J.sample_offset, cfg[j], &J.scene->data);
    if (st != PR_OK) return fail(c, st, "job " + std::to_string(j) + ": " + c->err);
    // the batch fills the GPU with many jobs: fewer sample chunks per job
    cfg[j].chunks = std::max(1, std::min(cfg[j].chunks, (int)std::ceil(2.0e5 / ((double)cfg[j].width * cfg[j].height))));
    cfg[j].chunks = std::min(cfg[j].chunks, cfg[j].spp);
    off[j + 1] = off[j] + (size_t)cfg[j].width * cfg[j].height * 3 * (size_t)cfg[j].chunks;
    paths += (uint64_t)cfg[j].spp * cfg[j].width * cfg[j].height;
  }
  // jobs in the wavefront form share the context's path pool: they run one
  // after another on the context's stream, after the graph of the others
  std::vector<char> wf_job((size_t)n, 0);
  for (int j = 0; j < n; j++)
    wf_job[j] = jobs[j].params.mode == PR_MODE_WAVEFRONT && !jobs[j].scene->data.kerr.enabled &&
                !jobs[j].scene->data.worm.enabled;
  PR_CUDA(c, c->batch_partial.ensure(sizeof(float) * std::max<size_t>(off[n], 1)));
  const int n_streams = std::min(n, 16);
  while ((int)c->batch_streams.size() < n_streams) {
    cudaStream_t st;
    PR_CUDA(c, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    c->batch_streams.push_back(st);
  }
  while ((int)c->batch_events.size() < n_streams + 1) {
    cudaEvent_t ev;
    PR_CUDA(c, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    c->batch_events.push_back(ev);
  }
  PR_CUDA(c, cudaMemsetAsync(c->errword.p, 0, 4, c->stream));
  PR_CUDA(c, cudaMemsetAsync(c->counters.p, 0, 128, c->stream));
  // capture: fork to the branch streams, one megakernel + reduce per job, join
  cudaGraph_t graph = nullptr;
  PR_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaEventRecord(c->batch_events[n_streams], c->stream);
  for (int k = 0; k < n_streams && e == cudaSuccess; k++)
    e = cudaStreamWaitEvent(c->batch_streams[k], c->batch_events[n_streams], 0);
  float* part = (float*)c->batch_partial.p;
  for (int j = 0; j < n && e == cudaSuccess; j++) {
    if (wf_job[j]) continue;
    const pr_job& J = jobs[j];
    cudaStream_t st = c->batch_streams[j % n_streams];
    const SceneObjData& sc = J.scene->data;
    const int n3 = cfg[j].width * cfg[j].height * 3;
    if (sc.kerr.enabled)
      e = launch_kerr_render(sc.dev, sc.kerr, cfg[j], part + off[j], (uint32_t*)c->errword.p,
                             (unsigned long long*)c->counters.p, st);
    else if (sc.worm.enabled)
      e = launch_worm_render(sc.dev, sc.worm, cfg[j], part + off[j], (uint32_t*)c->errword.p,
                             (unsigned long long*)c->counters.p, st);
    else
      e = launch_megakernel(sc.dev, cfg[j], part + off[j], (uint32_t*)c->errword.p,
                            (unsigned long long*)c->counters.p, st);
    if (e == cudaSuccess) e = launch_reduce(part + off[j], J.rgb_dev, n3, cfg[j].chunks, J.accumulate, st);
  }
  for (int k = 0; k < n_streams && e == cudaSuccess; k++) {
    e = cudaEventRecord(c->batch_events[k], c->batch_streams[k]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->batch_events[k], 0);
  }
  cudaError_t e2 = cudaStreamEndCapture(c->stream, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return cuda_fail(c, e != cudaSuccess ? e : e2, "batch capture");
  }
  bool updated = false;
  if (c->batch_exec) {
    cudaGraphExecUpdateResultInfo info;
    updated = cudaGraphExecUpdate(c->batch_exec, graph, &info) == cudaSuccess;
    if (!updated) {
      cudaGetLastError();
      cudaGraphExecDestroy(c->batch_exec);
      c->batch_exec = nullptr;
    }
  }
  if (!updated) {
    e = cudaGraphInstantiate(&c->batch_exec, graph, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(graph);
      c->batch_exec = nullptr;
      return cuda_fail(c, e, "batch graph instantiate");
    }
  }
  cudaGraphDestroy(graph);
  PR_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  PR_CUDA(c, cudaGraphLaunch(c->batch_exec, c->stream));
  uint64_t launches = 0, wf_passes = 0;
  for (int j = 0; j < n; j++) {
    if (!wf_job[j]) {
      launches += 2;
      continue;
    }
    const int stw = render_wavefront(c, cfg[j], jobs[j].rgb_dev, jobs[j].accumulate, &jobs[j].scene->data);
    if (stw != PR_OK) return fail(c, stw, "job " + std::to_string(j) + ": " + c->err);
    wf_passes += c->wf_passes;
  }
  PR_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  unsigned long long cnt[16];
  PR_CUDA(c, cudaMemcpyAsync(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  int st = check_device_errors(c);
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  // wavefront jobs: 4 launches per iteration, a reset per pass and a resolve per job
  for (int j = 0; j < n; j++)
    if (wf_job[j]) launches += 1;
  launches += 4 * cnt[5] + wf_passes;
  // Kerr jobs' counters are reported as pr_kerr_trace reports them
  c->stats = all_kerr ? pr_render_stats{paths, cnt[3], cnt[1], cnt[2], ms, launches}
                      : pr_render_stats{paths, cnt[1], cnt[2], cnt[3], ms, launches};
  return st;
}

size_t pr_abi_sizeof(int which) {
  switch (which) {
    case 0: return sizeof(pr_medium);
    case 1: return sizeof(pr_material);
    case 2: return sizeof(pr_entity);
    case 3: return sizeof(pr_mesh);
    case 4: return sizeof(pr_kerr);
    case 5: return sizeof(pr_scene_desc);
    case 9: return sizeof(pr_job);
    case 6: return sizeof(pr_camera);
    case 7: return sizeof(pr_render_params);
    case 8: return sizeof(pr_render_stats);
    default: return 0;
  }
}

}  // extern "C"
