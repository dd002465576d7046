// Context object behind pr_ctx* (internal to the library).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/prender_gpu.h"
#include "pr_internal.h"
#include "render_kernels.h"
#include "scene_build.h"
#include "wavefront.h"

namespace pr {

struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e == cudaSuccess) n = bytes;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// one uploaded scene: host build, device copies, device view
struct SceneObjData {
  HostScene host;
  DevBuf ents, mats, nodes, tris, rnodes, rtris, fnorm, kerr_tex, kerr_disk_tex, texels, ibl_texels, bump_texels;
  DevBuf worm_tex[2], fvn, fuv, fmat;
  DevScene dev{};
  GKerr kerr{};
  GWorm worm{};
  void release() {
    for (DevBuf* b : {&ents, &mats, &nodes, &tris, &rnodes, &rtris, &fnorm, &kerr_tex, &kerr_disk_tex, &texels, &ibl_texels,
                      &bump_texels, &worm_tex[0], &worm_tex[1], &fvn, &fuv, &fmat})
      b->release();
  }
};

}  // namespace pr

struct pr_scene_obj {
  pr::SceneObjData data;
};

struct pr_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  pr::SceneObjData cur;  // the scene of pr_scene_upload
  bool scene_ready = false;
  pr::DevBuf errword, counters;  // 4 bytes / 4 x u64
  pr::DevBuf partial, out, rays, ires, jres, dres;
  pr::DevBuf k_status, k_bl, k_dir, k_steps, k_ent, k_t;  // pr_kerr_trace staging
  pr::DevBuf k_sens;                                        // pr_kerr_sensitivity staging
  pr::DevBuf mlt_lum, mlt_path, mlt_start, mlt_u, mlt_cur, mlt_acc;  // PR_MODE_MLT state
  pr::DevBuf adj_scratch, adj_grad;                         // adjoint outputs
  double kernel_ms[4] = {0, 0, 0, 0};        // wavefront shade / extend / shadow / control (host-driven loop)
  unsigned long long shadow_counts[3] = {0, 0, 0};  // shadow rays, nodes, triangles of the last wavefront frame
  pr_render_stats stats{};
  // wavefront pool
  pr::DevBuf wf_o, wf_d, wf_beta, wf_dpw, wf_L, wf_sample, wf_hit, wf_hitv, wf_nee, wf_sho, wf_shd, wf_extq, wf_shq;
  pr::DevBuf wf_spo, wf_spd, wf_spb, wf_spw, wf_sps, wf_samp, wf_live, wf_pix, wf_ctl;
  pr::DevBuf wf_frc, wf_fre, wf_frs, wf_frl, wf_spf, wf_neef;  // subsurface frames (wavefront form)
  unsigned int wf_slots = 0;
  cudaGraphExec_t wf_graph = nullptr;
  unsigned int wf_graph_slots = 0;
  unsigned int wf_graph_trace_blocks = 0;
  int wf_graph_variant = 0;          // shading kernel the graph launches: sss + 2 * ext
  unsigned int tuned_slots = 0;      // autotuner's wavefront pool size (0: default)
  unsigned int tuned_trace_bps = 0;  // autotuner's traversal blocks per SM (0: default)
  bool force_host_loop = false;      // the autotuner times candidates with the host-driven loop
  // pr_render_batch
  cudaGraphExec_t batch_exec = nullptr;
  std::vector<cudaStream_t> batch_streams;
  std::vector<cudaEvent_t> batch_events;
  pr::DevBuf batch_partial;
  bool wf_graph_failed = false;
  pr::WfCtl* wf_host_ctl = nullptr;
  uint64_t wf_passes = 0;
};


namespace pr {
// CameraScreenPram + Run() set-up for one render call (capi.cu)
int prepare_render(pr_ctx* c, const pr_camera* cam, const pr_render_params* p, uint64_t sample_offset, RenderCfg& g,
                   const SceneObjData* scene = nullptr);
int ctx_fail(pr_ctx* c, int code, const std::string& msg);
// names of the set bits of a device error word (PR_DEV_*), for pr_last_error
std::string device_error_message(uint32_t bits);
}  // namespace pr
