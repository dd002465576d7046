// Kerr geodesics, FP32 form (see kerr_math.cuh): FP32 integration with a
// float-pair state, FP64 only for the set-up, the pole steps and the exit
// direction.  Compiled with FMA contraction.
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
