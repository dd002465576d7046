// Kerr geodesics, FP64 form: the reference's arithmetic operation for
// operation.  This translation unit is compiled with -fmad=false, so every
// FP64 multiply and add rounds on its own in the order the reference writes
// them; with the same libm results a trace follows the reference's step
// sequence exactly (CUDA's sin / cos / acos / atan2 / pow may differ from
// the host libm in the last bit; the tests bound the effect on exit
// directions).
#include "kerr_math.cuh"

namespace pr {

cudaError_t launch_kerr_trace_fp64(const DevScene& S, const GKerr& K, const double* rays, int64_t n, KerrOut out,
                                   uint32_t* err, unsigned long long* counters, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = (n + 127) / 128;
  kerr_trace_kernel<false><<<(unsigned)blocks, 128, 0, stream>>>(S, K, rays, n, out, err, counters);
  return cudaGetLastError();
}

cudaError_t launch_kerr_render_fp64(const DevScene& S, const GKerr& K, const RenderCfg& cfg, float* partial,
                                    uint32_t* err, unsigned long long* counters, cudaStream_t stream) {
  const uint64_t threads = (uint64_t)cfg.tiles_x * cfg.tiles_y * 32ull * (uint64_t)cfg.chunks;
  const uint32_t blocks = (uint32_t)((threads + 127) / 128);
  kerr_render_kernel<false><<<blocks, 128, 0, stream>>>(S, K, cfg, partial, err, counters);
  return cudaGetLastError();
}

}  // namespace pr
