// Launch interfaces of the render / trace kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "pr_internal.h"

namespace pr {

// Render::Run state for one launch (render.h:1125-1269), prepared on the host.
struct RenderCfg {
  float3 cam_pos, center, screen_x, screen_y;
  float iw, ih, rate, smp;
  float cutoff, sensor;
  int width, height;
  int spp;          // camera samples per pixel in this launch (samples * ss^2)
  int ss;           // supersamples per axis after the tent-filter fold
  int tent;
  int depth, depth_limit;
  int nee, media;
  int flags;
  int max_vertices;
  int chunks;       // sample chunks per pixel (one thread each)
  uint32_t tiles_x, tiles_y;
  uint64_t seed;
  uint64_t sample_offset;
};

cudaError_t launch_megakernel(const DevScene& S, const RenderCfg& cfg, float* out, uint32_t* err,
                              unsigned long long* counters, cudaStream_t stream);
cudaError_t launch_reduce(const float* partial, float* dst, int n3, int chunks, int accumulate, cudaStream_t stream);
// 8-bit bitmap rows of a float image (output.cu)
cudaError_t launch_to_rgb8(const float* rgb, int width, int height, double gamma_offset, uint8_t* out,
                           cudaStream_t stream);
// Radiance RGBE pixels for the HDR writer (output.cu)
cudaError_t launch_to_rgbe(const float* rgb, int width, int height, uint8_t* out, cudaStream_t stream);
cudaError_t launch_trace_fast(const DevScene& S, const double* rays, int64_t n, int32_t* ent, int32_t* prim, double* t,
                              uint32_t* err, cudaStream_t stream);
cudaError_t launch_first_hit(const DevScene& S, const double* rays, int64_t n, int32_t* ent, int32_t* prim, double* t,
                             uint32_t* err, unsigned long long* counters, cudaStream_t stream);

}  // namespace pr
