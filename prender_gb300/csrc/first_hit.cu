// Bit-exact closest hit: intersect_scene_ (scene.cpp:83-214) for a batch of
// FP64 rays, one thread per ray.  See device_common.cuh for how the FP64
// tests reproduce the reference's rounding.
#include "device_common.cuh"
#include "render_kernels.h"

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

cudaError_t launch_first_hit(const DevScene& S, const double* rays, int64_t n, int32_t* ent, int32_t* prim, double* t,
                             uint32_t* err, unsigned long long* counters, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = (n + 127) / 128;
  first_hit_kernel<<<(unsigned)blocks, 128, 0, stream>>>(S, rays, n, ent, prim, t, err, counters);
  return cudaGetLastError();
}

}  // namespace pr
