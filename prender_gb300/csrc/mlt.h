// Primary-sample-space Metropolis light transport on the GPU (mlt.cu).
#pragma once
#include <cuda_runtime.h>

#include "pr_internal.h"
#include "render_kernels.h"

namespace pr {

// Primary samples kept per chain: the camera's six (pixel x, y, the
// sub-pixel halves, the tent filter) and the first draws of the path's
// first branch; later draws are independent in every proposal.
constexpr int kMltDims = 64;

struct MltCfg {
  int chains;            // independent Markov chains (one thread each)
  int seeds;             // bootstrap paths
  int64_t mutations;     // per chain
  float b;               // mean luminance of the bootstrap paths
  float p_large;         // large-step probability (0.5)
  float pdf;             // W H 4: the camera samples' inverse density
  float chain_scale;     // 1 / mutations
  uint64_t seed;
};

// bootstrap: seeds paths from fresh primary samples -> luminance, colour
// and pixel of each
cudaError_t launch_mlt_seeds(const DevScene& S, const RenderCfg& cfg, const MltCfg& m, float* lum, float4* path,
                             uint32_t* err, unsigned long long* counters, cudaStream_t stream);
// chains start from start[c] (a bootstrap index): primary samples and the
// current path's colour / pixel / luminance
cudaError_t launch_mlt_init(const MltCfg& m, const int32_t* start, const float4* seed_path, const float* seed_lum,
                            float* u, float4* cur, cudaStream_t stream);
// iterations [it0, it1) of every chain: propose, splat the current and the
// proposed path with Kelemen's weights into acc (3 floats per pixel),
// accept or keep
cudaError_t launch_mlt_chains(const DevScene& S, const RenderCfg& cfg, const MltCfg& m, int64_t it0, int64_t it1,
                              float* u, float4* cur, float* acc, uint32_t* err, unsigned long long* counters,
                              cudaStream_t stream);
// rgb (+)= acc * scale
cudaError_t launch_mlt_resolve(const float* acc, float* rgb, int n3, float scale, int accumulate, cudaStream_t stream);

}  // namespace pr
