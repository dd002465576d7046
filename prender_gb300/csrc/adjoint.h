// Launch interface of the path-replay adjoint renderer (adjoint.cu).
#pragma once
#include <cuda_runtime.h>

#include "pr_internal.h"
#include "render_kernels.h"

namespace pr {

constexpr int kAdjMaterials = 16;  // materials the adjoint pass tracks

// adds dL/dC (3 per material) and dL/dE (3 per material) into d_color and
// d_emission (device, double); same launch geometry as the megakernel
cudaError_t launch_adjoint(const DevScene& S, const RenderCfg& cfg, const float* dl_drgb, int n_mat, double* d_color,
                           double* d_emission, uint32_t* err, unsigned long long* counters, cudaStream_t stream);

}  // namespace pr
