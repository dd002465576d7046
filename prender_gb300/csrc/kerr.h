// Launch interface of the Kerr geodesic tracer (kerr.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "pr_internal.h"
#include "render_kernels.h"
#include "../../include/prender_gpu.h"

namespace pr {

// per-ray results of pr_kerr_trace (device buffers; any may be null)
struct KerrOut {
  int32_t* status;
  double* final_bl;  // 3 per ray
  double* exit_dir;  // 3 per ray
  int32_t* steps;
  int32_t* hit_entity;
  double* hit_t;
};

// counters[0] rays, [1] accepted steps, [2] RK45 attempts, [3] segment tests
cudaError_t launch_kerr_trace_fp64(const DevScene& S, const GKerr& K, const double* rays, int64_t n, KerrOut out,
                                   uint32_t* err, unsigned long long* counters, cudaStream_t stream);
cudaError_t launch_kerr_trace_fp32(const DevScene& S, const GKerr& K, const double* rays, int64_t n, KerrOut out,
                                   uint32_t* err, unsigned long long* counters, cudaStream_t stream);

// the renderer with every scene query traced along a geodesic; same output
// layout as launch_megakernel (per-chunk partial images)
cudaError_t launch_kerr_render_fp64(const DevScene& S, const GKerr& K, const RenderCfg& cfg, float* partial,
                                    uint32_t* err, unsigned long long* counters, cudaStream_t stream);
cudaError_t launch_kerr_render_fp32(const DevScene& S, const GKerr& K, const RenderCfg& cfg, float* partial,
                                    uint32_t* err, unsigned long long* counters, cudaStream_t stream);

// forward-mode ray-bundle Jacobian (kerr_sens.cu); any output may be null
cudaError_t launch_kerr_sensitivity(const DevScene& S, const GKerr& K, const double* rays, const double* basis,
                                    int64_t n, const double* cot, int32_t* status, double* jac_dir, double* jac_bl,
                                    double* grad, uint32_t* err, cudaStream_t stream);

// accretion-disk shading at points of disk entity ent (kerr.cu)
cudaError_t launch_kerr_disk_shade(const DevScene& S, const GKerr& K, int ent, const double* pts, int64_t n,
                                   int32_t* valid, double* col, double* em, double* alpha, cudaStream_t stream);

inline cudaError_t launch_kerr_trace(const DevScene& S, const GKerr& K, const double* rays, int64_t n, KerrOut out,
                                     uint32_t* err, unsigned long long* counters, cudaStream_t stream) {
  return K.precision == PR_KERR_FP32 ? launch_kerr_trace_fp32(S, K, rays, n, out, err, counters, stream)
                                     : launch_kerr_trace_fp64(S, K, rays, n, out, err, counters, stream);
}
inline cudaError_t launch_kerr_render(const DevScene& S, const GKerr& K, const RenderCfg& cfg, float* partial,
                                      uint32_t* err, unsigned long long* counters, cudaStream_t stream) {
  return K.precision == PR_KERR_FP32 ? launch_kerr_render_fp32(S, K, cfg, partial, err, counters, stream)
                                     : launch_kerr_render_fp64(S, K, cfg, partial, err, counters, stream);
}

}  // namespace pr
