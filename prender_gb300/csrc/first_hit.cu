// Bit-exact closest hit: intersect_scene_ (scene.cpp:83-214) for a batch of
// FP64 rays, one thread per ray.  See device_common.cuh for how the FP64
// tests reproduce the reference's rounding.
#include "device_common.cuh"
#include "render_kernels.h"
#include "trace_fast.cuh"

namespace pr {

__global__ void __launch_bounds__(128) first_hit_kernel(DevScene S, const double* __restrict__ rays, int64_t n,
                                                        int32_t* __restrict__ ent, int32_t* __restrict__ prim,
                                                        double* __restrict__ tout, uint32_t* __restrict__ err,
                                                        unsigned long long* __restrict__ counters) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t nodes = 0, tris = 0;
  if (i < n) {
    const double* r = rays + 6 * i;
    const dv3 o = {r[0], r[1], r[2]}, d = {r[3], r[4], r[5]};
    double t;
    int e, p;
    const bool got = exact_closest(S, o, d, t, e, p, err, nodes, tris);
    ent[i] = got ? e : -1;
    prim[i] = got ? p : -1;
    tout[i] = got ? t : -1.0;
  }
  if (counters) {
    unsigned long long a = nodes, b = tris;
    for (int off = 16; off > 0; off >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, off);
      b += __shfl_down_sync(0xffffffffu, b, off);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(counters + 2, a);
      atomicAdd(counters + 3, b);
    }
  }
}

__global__ void __launch_bounds__(128) trace_fast_kernel(DevScene S, const double* __restrict__ rays, int64_t n,
                                                         int32_t* __restrict__ ent, int32_t* __restrict__ prim,
                                                         double* __restrict__ tout, uint32_t* __restrict__ err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* r = rays + 6 * i;
  const float3 o = f3((float)r[0], (float)r[1], (float)r[2]);
  const float3 d = f3((float)r[3], (float)r[4], (float)r[5]);
  FastHit h;
  TraceStats st{0, 0};
  const bool got = fast_closest(S, o, d, h, st, err);
  ent[i] = got ? h.ent : -1;
  prim[i] = (got && h.slot >= 0) ? __float_as_int(S.rtris[3 * (size_t)h.slot].w) : -1;
  tout[i] = got ? (double)h.t : -1.0;
}

cudaError_t launch_trace_fast(const DevScene& S, const double* rays, int64_t n, int32_t* ent, int32_t* prim, double* t,
                              uint32_t* err, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  trace_fast_kernel<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(S, rays, n, ent, prim, t, err);
  return cudaGetLastError();
}

cudaError_t launch_first_hit(const DevScene& S, const double* rays, int64_t n, int32_t* ent, int32_t* prim, double* t,
                             uint32_t* err, unsigned long long* counters, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = (n + 127) / 128;
  first_hit_kernel<<<(unsigned)blocks, 128, 0, stream>>>(S, rays, n, ent, prim, t, err, counters);
  return cudaGetLastError();
}

}  // namespace pr
