// Primary-sample-space Metropolis light transport (Render::RunMLT,
// render.h:363-785; Kelemen, Szirmay-Kalos, Antal and Csonka, "A Simple and
// Robust Mutation Strategy for the Metropolis Light Transport Algorithm",
// 2002) as many independent chains, one per thread.
//
// A path is a function of its primary samples: the camera takes the first
// six (pixel x, y, the sub-pixel halves, the tent filter's two), and the
// path's first branch the next ones, through the same shade() as the other
// renderers with a sampler that reads them (PssRng); draws past kMltDims
// and those of split branches are fresh in every proposal (an independent,
// symmetric proposal for those coordinates).  A proposal is a large step
// (every coordinate fresh, probability p_large) or a small step (Mutate0 of
// each coordinate, mlt.h:40-53); its values are derived from counter-based
// streams keyed by (chain, iteration, coordinate), so no proposal vector is
// stored: an accepted proposal is written back coordinate by coordinate.
// Each iteration splats the current and the proposed path with Kelemen's
// weights (a + large) / (L_new / b + p_large) and (1 - a) / (L_old / b +
// p_large), times the camera's inverse density W H 4, over the chain's
// length; b is the mean luminance of the bootstrap paths and the chains
// start from bootstrap paths drawn in proportion to their luminance.
#include "mlt.h"
#include "path_logic.cuh"

namespace pr {
namespace {

constexpr uint32_t kTagFresh = 0x4d4c5401u, kTagMutate = 0x4d4c5402u, kTagStep = 0x4d4c5403u;
constexpr uint32_t kTagExtra = 0x4d4c5500u;   // + branch
constexpr uint32_t kTagStream = 0x4d4c5600u;  // + branch
constexpr uint64_t kLargeBit = 1ull << 62, kSeedBit = 1ull << 63;

// the chains' primary samples (coordinate-major: u[k * chains + chain])
__constant__ float* c_mlt_u;
__constant__ int c_mlt_chains;

__device__ __forceinline__ float u01(uint32_t v) { return (float)(v >> 8) * (1.0f / 16777216.0f); }

__device__ __forceinline__ uint32_t phx(uint64_t seed, uint32_t tag, uint64_t stream, uint32_t k) {
  return philox4x32_10(make_uint4((uint32_t)stream, (uint32_t)(stream >> 32), k, tag),
                       make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)))
      .x;
}

// Mutate0 (mlt.h:40-53): an exponentially distributed step of 1/512 .. 1/16
__device__ __forceinline__ float mutate0(float x, float r) {
  const float s1 = 1.0f / 512.0f, s2 = 1.0f / 16.0f;
  const float dx = s1 / (s1 / s2 + fabsf(2.0f * r - 1.0f)) - s1 / (s1 / s2 + 1.0f);
  if (r < 0.5f) {
    const float x1 = x + dx;
    return x1 < 1.0f ? x1 : x1 - 1.0f;
  }
  const float x1 = x - dx;
  return x1 < 0.0f ? x1 + 1.0f : x1;
}

// coordinate k (< kMltDims) of the proposal (or bootstrap path) `sample`:
// bits 0..61 the stream (chain | iteration << 24, or the bootstrap index),
// bit 62 a large step, bit 63 a bootstrap path
__device__ __forceinline__ float pss_value(uint64_t seed, uint64_t sample, int k) {
  const uint64_t stream = sample & ~kLargeBit;
  if (sample & (kLargeBit | kSeedBit)) return u01(phx(seed, kTagFresh, stream, (uint32_t)k));
  const uint32_t chain = (uint32_t)(sample & 0xFFFFFFu);
  const float cur = c_mlt_u[(size_t)k * c_mlt_chains + chain];
  return mutate0(cur, u01(phx(seed, kTagMutate, stream, (uint32_t)k)));
}

}  // namespace

// shade()'s sampler under MLT: the first branch's draws are primary samples
// 6, 7, ...; the rest fresh per proposal
struct PssRng {
  uint64_t seed, sample;
  uint32_t branch, draws;
  uint32_t vstart, sdraws;  // the vertex's first draw; its stream draws so far
  __device__ __forceinline__ float next() {
    const uint32_t k = draws++;
    if (branch == 0 && k + 6u < (uint32_t)kMltDims) return pss_value(seed, sample, (int)k + 6);
    return u01(phx(seed, kTagExtra + (branch & 0xFFu), sample & ~kLargeBit, k));
  }
  // the light choice and surface NEE point: fresh in every proposal, as the
  // reference's Next01 draws them from its stream under MLT
  __device__ __forceinline__ float next_stream() {
    return u01(phx(seed, kTagStream + (branch & 0xFFu), sample & ~kLargeBit, (vstart << 6) + (sdraws++ & 63u)));
  }
};
__device__ __forceinline__ void rng_at(PssRng& r, uint64_t seed, uint64_t sample, uint32_t branch, uint32_t draws) {
  r.seed = seed;
  r.sample = sample;
  r.branch = branch;
  r.draws = draws;
  r.vstart = draws;
  r.sdraws = 0;
}
__device__ __forceinline__ float rng_stream(PssRng& r) { return r.next_stream(); }
__device__ __forceinline__ uint32_t rng_draws(const PssRng& r) { return r.draws; }

namespace {

struct MltPath {
  float3 F;
  int pix;  // (H - y - 1) W + x
};

__device__ __forceinline__ float luminance(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// generate_new_path (render.h:195-357): pixel and sub-pixel from the first
// six primary samples, the tent filter, radiance() over the stack of split
// branches (the plain renderer's loop with the primary-sample sampler)
__device__ MltPath mlt_path(const DevScene& S, const RenderCfg& cfg, uint64_t sample, uint32_t* err, TraceStats& st,
                            uint32_t& segs) {
  const uint64_t seed = cfg.seed;
  int x = (int)(pss_value(seed, sample, 0) * (float)cfg.width);
  int y = (int)(pss_value(seed, sample, 1) * (float)cfg.height);
  x = min(max(x, 0), cfg.width - 1);
  y = min(max(y, 0), cfg.height - 1);
  const int sxx = pss_value(seed, sample, 2) < 0.5f ? 0 : 1;
  const int syy = pss_value(seed, sample, 3) < 0.5f ? 0 : 1;
  const float rr1 = 2.0f * pss_value(seed, sample, 4), rr2 = 2.0f * pss_value(seed, sample, 5);
  const float dx = rr1 < 1.0f ? sqrtf(rr1) - 1.0f : 1.0f - sqrtf(2.0f - rr1);
  const float dy = rr2 < 1.0f ? sqrtf(rr2) - 1.0f : 1.0f - sqrtf(2.0f - rr2);
  const float r1 = (sxx + 0.5f + dx) * 0.5f, r2 = (syy + 0.5f + dy) * 0.5f;
  const float3 sp = cfg.center + cfg.screen_x * ((r1 + x) * cfg.iw - 0.5f) + cfg.screen_y * ((r2 + y) * cfg.ih - 0.5f);
  PathState stack[kSplitStack];
  int sp_ = 0;
  root_path(stack[sp_++], cfg.cam_pos, normalize(sp - cfg.cam_pos));
  float3 L = f3(0, 0, 0);
  while (sp_ > 0) {
    PathState ps = stack[--sp_];
    for (;;) {
      FastHit h;
      segs++;
      const bool hit = fast_closest(S, ps.o, ps.d, h, st, err);
      ShadowReq sh[3];
      int nsh = 0;
      PathState child;
      const int r = shade<false, true, true, PssRng>(S, cfg, ps, hit, h, sample, sh, nsh, child, err);
      for (int k = 0; k < nsh; k++) {
        segs++;
        if (!fast_occluded(S, sh[k].o, sh[k].d, sh[k].tmax, st, err)) ps.L += sh[k].contrib;
      }
      if (r == SHADE_SPLIT) {
        if (sp_ < kSplitStack) stack[sp_++] = child;
        else atomicOr(err, PR_DEV_LOOP_CAP);
      }
      if (r == SHADE_END) break;
    }
    L += ps.L;
  }
  if (!(isfinite(L.x) && isfinite(L.y) && isfinite(L.z))) {
    atomicOr(err, PR_DEV_NONFINITE);
    L = f3(0, 0, 0);
  }
  return MltPath{L, (cfg.height - y - 1) * cfg.width + x};
}

__device__ __forceinline__ void flush(unsigned long long* counters, uint32_t paths, uint32_t segs, const TraceStats& st) {
  if (!counters) return;
  unsigned long long a = paths, b = segs, c = st.nodes, d = st.tris;
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, off);
    b += __shfl_down_sync(0xffffffffu, b, off);
    c += __shfl_down_sync(0xffffffffu, c, off);
    d += __shfl_down_sync(0xffffffffu, d, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(counters + 0, a);
    atomicAdd(counters + 1, b);
    atomicAdd(counters + 2, c);
    atomicAdd(counters + 3, d);
  }
}

__global__ void __launch_bounds__(128, 3) mlt_seed_kernel(DevScene S, RenderCfg cfg, MltCfg m, float* __restrict__ lum,
                                                           float4* __restrict__ path, uint32_t* __restrict__ err,
                                                           unsigned long long* __restrict__ counters) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  TraceStats st{0, 0};
  uint32_t segs = 0, paths = 0;
  if (i < m.seeds) {
    const MltPath p = mlt_path(S, cfg, kSeedBit | (uint64_t)i, err, st, segs);
    lum[i] = luminance(p.F);
    path[i] = make_float4(p.F.x, p.F.y, p.F.z, __int_as_float(p.pix));
    paths = 1;
  }
  flush(counters, paths, segs, st);
}

__global__ void mlt_init_kernel(MltCfg m, const int32_t* __restrict__ start, const float4* __restrict__ seed_path,
                                const float* __restrict__ seed_lum, float* __restrict__ u, float4* __restrict__ cur) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.chains) return;
  const int s = start[c];
  for (int k = 0; k < kMltDims; k++)
    u[(size_t)k * m.chains + c] = u01(phx(m.seed, kTagFresh, kSeedBit | (uint64_t)s, (uint32_t)k));
  cur[c] = seed_path[s];
  (void)seed_lum;
}

__device__ __forceinline__ void splat(float* acc, int pix, float3 v) {
  atomicAdd(acc + 3 * (size_t)pix, v.x);
  atomicAdd(acc + 3 * (size_t)pix + 1, v.y);
  atomicAdd(acc + 3 * (size_t)pix + 2, v.z);
}

__global__ void __launch_bounds__(128, 3) mlt_chain_kernel(DevScene S, RenderCfg cfg, MltCfg m, int64_t it0, int64_t it1,
                                                            float* __restrict__ u, float4* __restrict__ cur,
                                                            float* __restrict__ acc, uint32_t* __restrict__ err,
                                                            unsigned long long* __restrict__ counters) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  TraceStats st{0, 0};
  uint32_t segs = 0, paths = 0;
  if (c < m.chains) {
    float4 co = cur[c];
    for (int64_t it = it0; it < it1; it++) {
      const uint64_t stream = ((uint64_t)it << 24) | (uint64_t)c;
      const float step_r = u01(phx(m.seed, kTagStep, stream, 0u));
      const float accept_r = u01(phx(m.seed, kTagStep, stream, 1u));
      const bool large = step_r < m.p_large;
      const uint64_t sample = stream | (large ? kLargeBit : 0ull);
      const MltPath np = mlt_path(S, cfg, sample, err, st, segs);
      paths++;
      const float3 Fo = f3(co.x, co.y, co.z);
      const float Lnew = luminance(np.F), Lold = luminance(Fo);
      const float a = Lold > 1.0e-16f ? fminf(1.0f, Lnew / Lold) : 1.0f;
      const float wn = (a + (large ? 1.0f : 0.0f)) / (Lnew / m.b + m.p_large) * m.chain_scale * m.pdf;
      const float wo = (1.0f - a) / (Lold / m.b + m.p_large) * m.chain_scale * m.pdf;
      if (wo > 0.0f && Lold > 0.0f) splat(acc, __float_as_int(co.w), Fo * wo);
      if (wn > 0.0f && Lnew > 0.0f) splat(acc, np.pix, np.F * wn);
      if (accept_r < a) {
        for (int k = 0; k < kMltDims; k++) {
          const float v = pss_value(m.seed, sample, k);
          u[(size_t)k * m.chains + c] = v;
        }
        co = make_float4(np.F.x, np.F.y, np.F.z, __int_as_float(np.pix));
      }
    }
    cur[c] = co;
  }
  flush(counters, paths, segs, st);
}

__global__ void mlt_resolve_kernel(const float* __restrict__ acc, float* __restrict__ rgb, int n3, float scale,
                                   int accumulate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  rgb[i] = (accumulate ? rgb[i] : 0.0f) + acc[i] * scale;
}

}  // namespace

cudaError_t launch_mlt_seeds(const DevScene& S, const RenderCfg& cfg, const MltCfg& m, float* lum, float4* path,
                             uint32_t* err, unsigned long long* counters, cudaStream_t stream) {
  if (m.seeds <= 0) return cudaSuccess;
  mlt_seed_kernel<<<(m.seeds + 127) / 128, 128, 0, stream>>>(S, cfg, m, lum, path, err, counters);
  return cudaGetLastError();
}

cudaError_t launch_mlt_init(const MltCfg& m, const int32_t* start, const float4* seed_path, const float* seed_lum,
                            float* u, float4* cur, cudaStream_t stream) {
  cudaError_t e = cudaMemcpyToSymbolAsync(c_mlt_u, &u, sizeof(float*), 0, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess)
    e = cudaMemcpyToSymbolAsync(c_mlt_chains, &m.chains, sizeof(int), 0, cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return e;
  mlt_init_kernel<<<(m.chains + 127) / 128, 128, 0, stream>>>(m, start, seed_path, seed_lum, u, cur);
  return cudaGetLastError();
}

cudaError_t launch_mlt_chains(const DevScene& S, const RenderCfg& cfg, const MltCfg& m, int64_t it0, int64_t it1,
                              float* u, float4* cur, float* acc, uint32_t* err, unsigned long long* counters,
                              cudaStream_t stream) {
  mlt_chain_kernel<<<(m.chains + 127) / 128, 128, 0, stream>>>(S, cfg, m, it0, it1, u, cur, acc, err, counters);
  return cudaGetLastError();
}

cudaError_t launch_mlt_resolve(const float* acc, float* rgb, int n3, float scale, int accumulate, cudaStream_t stream) {
  mlt_resolve_kernel<<<(n3 + 255) / 256, 256, 0, stream>>>(acc, rgb, n3, scale, accumulate);
  return cudaGetLastError();
}

}  // namespace pr
