// Kerr geodesics, mixed-precision form (PR_KERR_FP32; the templates are in
// kerr_math.cuh): the reference's FP64 Cash-Karp steps with its error
// control near the hole and among the scene geometry; FP32 increments of
// fixed h = 2 steps, added to the FP64 state, only for outbound rays beyond
// max(200 M, scene radius + 2) whose last FP64 error estimate is small; and
// an inbound ray with no radial turning point left reported as captured at
// once.  Compiled with FMA contraction (the FP64 form, kerr.cu, is not).
#include "kerr_math.cuh"

namespace pr {

cudaError_t launch_kerr_trace_fp32(const DevScene& S, const GKerr& K, const double* rays, int64_t n, KerrOut out,
                                   uint32_t* err, unsigned long long* counters, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = (n + 127) / 128;
  kerr_trace_kernel<true><<<(unsigned)blocks, 128, 0, stream>>>(S, K, rays, n, out, err, counters);
  return cudaGetLastError();
}

cudaError_t launch_kerr_render_fp32(const DevScene& S, const GKerr& K, const RenderCfg& cfg, float* partial,
                                    uint32_t* err, unsigned long long* counters, cudaStream_t stream) {
  const uint64_t threads = (uint64_t)cfg.tiles_x * cfg.tiles_y * 32ull * (uint64_t)cfg.chunks;
  const uint32_t blocks = (uint32_t)((threads + 127) / 128);
  kerr_render_kernel<true><<<blocks, 128, 0, stream>>>(S, K, cfg, partial, err, counters);
  return cudaGetLastError();
}

}  // namespace pr
