// Launch interface of the wormhole geodesic tracer (wormhole.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "pr_internal.h"
#include "render_kernels.h"

namespace pr {

// per-ray results of pr_wormhole_trace (device buffers; any may be null)
struct WormOut {
  int32_t* status;    // 1 entity hit, 0 background 1 (l >= 0), 3 background 2
  double* final_y;    // 3 per ray: l, theta and phi of the last polyline direction
  double* exit_dir;   // 3 per ray
  int32_t* steps;
  int32_t* hit_entity;
};

// counters[0] rays, [1] accepted steps, [2] RK45 attempts, [3] segment tests
cudaError_t launch_worm_trace(const DevScene& S, const GWorm& W, const double* rays, int64_t n, WormOut out,
                              uint32_t* err, unsigned long long* counters, cudaStream_t stream);

// the renderer with every scene query traced through the wormhole; same
// output layout as launch_megakernel (per-chunk partial images)
cudaError_t launch_worm_render(const DevScene& S, const GWorm& W, const RenderCfg& cfg, float* partial, uint32_t* err,
                               unsigned long long* counters, cudaStream_t stream);

}  // namespace pr
