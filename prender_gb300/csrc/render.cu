// Plain drop-in renderer (megakernel): one thread per (pixel, sample chunk)
// runs Render::Run's per-sample body (render.h:1203-1385) -- camera ray,
// the whole radiance() branch tree, luminance clamp -- with the per-vertex
// logic of path_logic.cuh.  Shadow rays and the next segment are traced in
// place; the refracted branch of a depth <= 2 glass split waits on a
// 4-entry stack (at most three splits are pending at once: depths 0, 1, 2).
//
// Each thread sums its samples in order and writes one partial image per
// sample chunk; reduce_chunks adds the chunks in order, so the image is
// deterministic.
#include <cuda_runtime.h>

#include "path_logic.cuh"

namespace pr {

// Subsurface continuations whose radiance the reference bounds
// (OVER_RADIANCE_CUT2 / 3): frame f collects its continuation's
// contributions C over all branches inside it; when its last branch ends,
// C (and the vertex's own emission and direct terms E) go to the parent
// unless |C / scale| exceeds the bound, in which case the vertex gave zero.
constexpr int kMaxSssFrames = 16;
struct SssFrames {
  float3 C[kMaxSssFrames], E[kMaxSssFrames], scale[kMaxSssFrames];
  float thr[kMaxSssFrames];
  int parent[kMaxSssFrames], open[kMaxSssFrames];
  int n;
};

__device__ __forceinline__ void frame_add(SssFrames& F, float3& root, int f, float3 x) {
  if (f < 0) root += x;
  else F.C[f] += x;
}

// a branch inside frame f ended (or a child frame closed): close every frame
// that has nothing open left
__device__ __forceinline__ void frame_release(SssFrames& F, float3& root, int f) {
  while (f >= 0) {
    if (--F.open[f] > 0) return;
    const float3 s = F.scale[f], c = F.C[f];
    const float3 q = f3(s.x != 0.0f ? c.x / s.x : 0.0f, s.y != 0.0f ? c.y / s.y : 0.0f, s.z != 0.0f ? c.z / s.z : 0.0f);
    const bool cut = sqrtf(dot(q, q)) > F.thr[f];
    const int p = F.parent[f];
    if (!cut) frame_add(F, root, p, c + F.E[f]);
    f = p;
  }
}

// One camera sample: the whole branch tree of radiance() for one root ray.
template <bool SSS>
__device__ float3 trace_sample(const DevScene& S, const RenderCfg& cfg, float3 o0, float3 d0, uint64_t sample_id,
                               TraceStats& st, uint32_t* err, uint32_t& segs) {
  PathState stack[kSplitStack];
  int sframe[kSplitStack];
  int sp = 0;
  root_path(stack[sp], o0, d0);
  sframe[sp++] = -1;
  float3 L = f3(0, 0, 0);
  SssFrames F;
  F.n = 0;
  while (sp > 0) {
    --sp;
    PathState ps = stack[sp];
    int fr = sframe[sp];
    for (;;) {
      FastHit h;
      segs++;
      const bool hit = fast_closest(S, ps.o, ps.d, h, st, err);
      ShadowReq sh[3];
      int nsh = 0;
      PathState child;
      SssFrameOut fo;
      fo.open = 0;
      const float3 Lb = ps.L;
      const int r = shade<SSS, SSS, SSS>(S, cfg, ps, hit, h, sample_id, sh, nsh, child, err, nullptr, nullptr,
                                         nullptr, SSS ? &fo : nullptr);
      const float3 Lown = ps.L - Lb;
      float3 Lnee = f3(0, 0, 0);
      for (int k = 0; k < nsh; k++) {
        segs++;
        if (!fast_occluded(S, sh[k].o, sh[k].d, sh[k].tmax, st, err)) Lnee += sh[k].contrib;
      }
      if (SSS && fo.open && F.n + fo.open <= kMaxSssFrames) {
        // the branch moves into a new frame (or two nested ones): what it
        // gathered before this vertex belongs outside, the vertex's own terms
        // to the frame, its continuation inside
        const int f = F.n++;
        F.E[f] = Lown + (fo.nee_inner ? f3(0, 0, 0) : Lnee);
        F.C[f] = f3(0, 0, 0);
        F.scale[f] = fo.scale;
        F.thr[f] = fo.thr;
        F.parent[f] = fr;
        F.open[f] = 1;
        frame_add(F, L, fr, Lb);
        int in = f;
        if (fo.open == 2) {
          in = F.n++;
          F.E[in] = f3(0, 0, 0);
          F.C[in] = f3(0, 0, 0);
          F.scale[in] = fo.scale2;
          F.thr[in] = fo.thr2;
          F.parent[in] = f;
          F.open[in] = 1;
        }
        F.C[in] += fo.inner + (fo.nee_inner ? Lnee : f3(0, 0, 0));
        ps.L = f3(0, 0, 0);
        fr = in;  // the parents keep their counts: the branch left, the child frame came
      } else {
        ps.L += Lnee;
        if (SSS && fo.open) ps.L += fo.inner;
      }
      if (r == SHADE_SPLIT) {
        if (sp < kSplitStack) {
          stack[sp] = child;
          sframe[sp++] = fr;
          if (SSS && fr >= 0) F.open[fr]++;
        } else {
          atomicOr(err, PR_DEV_LOOP_CAP);
        }
      }
      if (r == SHADE_END) break;
    }
    if (SSS) {
      frame_add(F, L, fr, ps.L);
      frame_release(F, L, fr);
    } else {
      L += ps.L;
    }
  }
  return L;
}

// the lean form (no subsurface or glossy lobes) at 8 blocks of 128 per SM
// (64 registers, spilling): plain mesh Cornell box 23.6 -> 24.8 Mpaths/s
// on GB300; the fuller form keeps 3 blocks per SM (168 registers)
template <bool SSS>
__global__ void __launch_bounds__(128, SSS ? 3 : 8) pt_megakernel(DevScene S, RenderCfg cfg, float* __restrict__ out,
                                                     uint32_t* __restrict__ err, unsigned long long* __restrict__ counters) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t warp = tid >> 5, lane = tid & 31;
  const uint32_t tiles_per_chunk = cfg.tiles_x * cfg.tiles_y;
  const uint32_t chunk = warp / tiles_per_chunk;
  if (chunk >= (uint32_t)cfg.chunks) return;
  const uint32_t tile = warp - chunk * tiles_per_chunk;
  const int x = (int)((tile % cfg.tiles_x) * 8 + (lane & 7));
  const int y = (int)((tile / cfg.tiles_x) * 4 + (lane >> 3));
  TraceStats st{0, 0};
  uint32_t segs = 0, paths = 0;
  if (x < cfg.width && y < cfg.height) {
    const int k0 = (int)(((int64_t)cfg.spp * chunk) / cfg.chunks);
    const int k1 = (int)(((int64_t)cfg.spp * (chunk + 1)) / cfg.chunks);
    float3 acc = f3(0, 0, 0);
    for (int k = k0; k < k1; k++) {
      float3 o, d;
      const uint64_t sample_id = camera_ray(cfg, x, y, cfg.sample_offset + (uint64_t)k, o, d);
      acc += finish_sample(cfg, trace_sample<SSS>(S, cfg, o, d, sample_id, st, err, segs), err);
      paths++;
    }
    acc = acc * cfg.sensor;
    float* o = out + 3 * ((size_t)chunk * cfg.width * cfg.height + (size_t)(cfg.height - y - 1) * cfg.width + x);
    o[0] = acc.x;
    o[1] = acc.y;
    o[2] = acc.z;
  }
  if (counters) {
    // warp-reduced statistics
    unsigned long long a = paths, b2 = segs, c = st.nodes, dd = st.tris;
    for (int off = 16; off > 0; off >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, off);
      b2 += __shfl_down_sync(0xffffffffu, b2, off);
      c += __shfl_down_sync(0xffffffffu, c, off);
      dd += __shfl_down_sync(0xffffffffu, dd, off);
    }
    if (lane == 0) {
      atomicAdd(counters + 0, a);
      atomicAdd(counters + 1, b2);
      atomicAdd(counters + 2, c);
      atomicAdd(counters + 3, dd);
    }
  }
}

// sums the per-chunk partial images in chunk order (deterministic) into
// dst; accumulate != 0 adds to what dst holds
__global__ void reduce_chunks(const float* __restrict__ partial, float* __restrict__ dst, int n3, int chunks,
                              int accumulate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  float s = accumulate ? dst[i] : 0.0f;
  for (int c = 0; c < chunks; c++) s += partial[(size_t)c * n3 + i];
  dst[i] = s;
}

cudaError_t launch_megakernel(const DevScene& S, const RenderCfg& cfg, float* out, uint32_t* err,
                              unsigned long long* counters, cudaStream_t stream) {
  const uint64_t threads = (uint64_t)cfg.tiles_x * cfg.tiles_y * 32ull * (uint64_t)cfg.chunks;
  const uint32_t blocks = (uint32_t)((threads + 127) / 128);
  // the fuller instantiation (subsurface frames, glossy lobes, parallel /
  // spot / infinity lights, textures) only where needed
  if (S.has_sss || S.has_glossy || S.n_point_lights > 0 || S.has_tex)
    pt_megakernel<true><<<blocks, 128, 0, stream>>>(S, cfg, out, err, counters);
  else pt_megakernel<false><<<blocks, 128, 0, stream>>>(S, cfg, out, err, counters);
  return cudaGetLastError();
}

cudaError_t launch_reduce(const float* partial, float* dst, int n3, int chunks, int accumulate, cudaStream_t stream) {
  reduce_chunks<<<(n3 + 255) / 256, 256, 0, stream>>>(partial, dst, n3, chunks, accumulate);
  return cudaGetLastError();
}

}  // namespace pr
