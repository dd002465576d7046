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

// the accretion disk's shading at given points (the test hook behind
// pr_kerr_disk_shade): valid, colour, emission, alpha per point
__global__ void __launch_bounds__(128) kerr_disk_shade_kernel(GKerr K, const GEntity* __restrict__ ents, int ent,
                                                              const double* __restrict__ pts, int64_t n,
                                                              int32_t* __restrict__ valid, double* __restrict__ col,
                                                              double* __restrict__ em, double* __restrict__ alpha) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double c[3] = {0, 0, 0}, e[3] = {0, 0, 0}, a = 0.0;
  const bool ok = kerr_disk_shade(K, ents[ent], {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, c, e, a);
  valid[i] = ok ? 1 : 0;
  for (int k = 0; k < 3; k++) {
    col[3 * i + k] = ok ? c[k] : 0.0;
    em[3 * i + k] = ok ? e[k] : 0.0;
  }
  alpha[i] = ok ? a : 0.0;
}

cudaError_t launch_kerr_disk_shade(const DevScene& S, const GKerr& K, int ent, const double* pts, int64_t n,
                                   int32_t* valid, double* col, double* em, double* alpha, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = (n + 127) / 128;
  kerr_disk_shade_kernel<<<(unsigned)blocks, 128, 0, stream>>>(K, S.ents, ent, pts, n, valid, col, em, alpha);
  return cudaGetLastError();
}

}  // namespace pr
