// Wavefront renderer buffers and launch interface (see wavefront.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "pr_internal.h"
#include "render_kernels.h"

namespace pr {

// device-side counters of one frame
// blocks of 128 resident per SM for the persistent traversal kernels
// (__launch_bounds__(128, 8): 64 registers a thread)
constexpr unsigned int kTraceBlocksPerSM = 8;

struct WfCtl {
  unsigned int ext_count;    // segments queued for wf_extend this iteration
  unsigned int sh_count;     // shadow rays queued for wf_shadow this iteration
  unsigned int spawn_head;   // glass branches taken from the ring (monotonic)
  unsigned int spawn_tail;   // glass branches put in the ring (monotonic)
  unsigned int spawn_ready;  // branches written before this iteration
  unsigned int iterations;
  unsigned int work;         // 1 while another iteration is needed
  unsigned int head_start;   // spawn_head when this iteration began (after correction)
  unsigned int ext_fetch;    // extension rays taken by wf_extend's lanes so far
  unsigned int sh_fetch;     // shadow rays taken by wf_shadow's lanes so far
  unsigned long long next_sample;
  unsigned int frame_next;   // subsurface frames handed out this pass
  unsigned int pad;
};

// structure-of-arrays path pool (P slots) and queues
struct WfBufs {
  float4 *o, *d, *beta, *dpw, *L;   // path state (w lanes carry depth / flags / branch / draws)
  uint64_t* sample;                 // camera sample (index within the pass) of each slot
  float4* hit;                      // t, entity, leaf slot, u
  float* hitv;                      // v
  float4 *nee, *sh_o, *sh_d;        // 3 per slot: pending shadow contribution, ray origin + tmax, direction
  int *extq, *shq;                  // compacted queues
  float4 *sp_o, *sp_d, *sp_beta, *sp_dpw;  // spawn ring (glass branches waiting for a slot)
  uint64_t* sp_sample;
  long long* samp;                  // 3 per camera sample: fixed-point radiance of split samples
  int* live;                        // branches still running per camera sample
  long long* pix;                   // 3 per pixel: fixed-point image
  WfCtl* ctl;
  // subsurface frames (scenes with dipole materials): a vertex whose radiance
  // the reference bounds (OVER_RADIANCE_CUT2 / 3 / 0) opens a frame; the
  // radiance of everything inside it collects in fr_c (fixed point), its own
  // terms in fr_e, and when its last branch or inner frame ends the frame
  // passes C + E to its parent unless |C / scale| > thr
  long long* fr_c;                  // 3 per frame
  long long* fr_e;                  // 3 per frame
  float4* fr_scale;                 // scale, thr
  int2* fr_link;                    // parent (-1: the camera sample), open branches and frames
  int* sp_frame;                    // frame of each waiting glass branch (-1: none)
  int* neef;                        // per slot: the frame whose E takes the pending shadow terms (-1: the path)
  unsigned int frame_cap;
  unsigned int frame_pad;
  uint32_t* err;
  unsigned long long* counters;     // paths, segments, nodes, triangle tests, extension segments,
                                    // iterations, shadow rays, shadow nodes, shadow triangle tests
  unsigned int n_slots;
  unsigned int spawn_cap;
  unsigned int max_iterations;
  unsigned int pad;
  uint64_t pass_first;              // first per-pixel sample index of this pass
  uint64_t pass_samples;            // camera samples in this pass (layers * W * H)
};

struct WfLaunch {
  unsigned int shade_blocks;
  unsigned int trace_blocks;
  int sss;    // the scene has subsurface materials: the fuller shading kernel with frames
  int ext;    // the scene has parallel, spot or infinity lights, textures or IBL images
};

cudaError_t wf_set_constants(const DevScene& S, const RenderCfg& cfg, const WfBufs& B, cudaStream_t s);
cudaError_t wf_reset_launch(unsigned int n_slots, cudaStream_t s);
cudaError_t wf_build_graph(const WfLaunch& L, cudaStream_t s, cudaGraphExec_t* exec);
// kernel_ms (4 entries, may be null) accumulates the device time of each
// kernel (shade, extend, shadow, control), measured with events
cudaError_t wf_run_host_loop(const WfLaunch& L, WfCtl* host_ctl_pinned, const WfCtl* dev_ctl, cudaStream_t s,
                             double* kernel_ms);
cudaError_t wf_resolve_launch(float* out, int n3, int accumulate, float sensor, cudaStream_t s);

}  // namespace pr
