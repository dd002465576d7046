// Adjoint of the plain renderer by path replay: gradients of a scalar image
// loss with respect to every material's colour (albedo) and emission.
//
// The caller renders the image with pr_render, forms dL/d(pixel), and calls
// the adjoint with the same camera, parameters and sample range.  Each
// thread replays its camera samples with the same counter-based streams, so
// it walks exactly the paths of the forward render (Vicini, Speierer and
// Jakob, "Path Replay Backpropagation", SIGGRAPH 2021), and accumulates:
//
//  * colour: every term a branch adds to L after a non-terminal vertex j is
//    proportional to C_{m_j} once (BRDF_Diffuse / Specular / Refraction all
//    scale the continuation and the vertex's next-event terms by the
//    material colour, brdf.h:408-953).  With n_m the number of such
//    vertices of material m and S_m the sum of the branch radiance L
//    recorded right after each of them (before its next-event terms),
//    d L_branch / d C_m = (n_m L_branch - S_m) / C_m per channel.  A glass
//    branch handed back at a split inherits its ancestors' vertices.
//  * emission: shade() reports every emitted term as weight x emission
//    (EmissionTap); next-event terms carry their light's material.
//
// Sampling decisions (Russian roulette, light choice, glass branch choice)
// are held fixed and their probabilities are treated as constants, the
// usual estimator of the derivative of the expectation; the luminance clamp
// of a sample is differentiated exactly.  Scenes with media are
// not supported by this pass; materials are limited to kAdjMaterials.
#include <cuda_runtime.h>

#include "adjoint.h"
#include "path_logic.cuh"

namespace pr {
namespace {

struct Anc {
  int8_t m[3];  // materials of the vertices before the split (depth <= 2)
  int8_t n;
};

__device__ __forceinline__ float3 safe_div(float3 a, float3 c) {
  return f3(c.x != 0.0f ? a.x / c.x : 0.0f, c.y != 0.0f ? a.y / c.y : 0.0f, c.z != 0.0f ? a.z / c.z : 0.0f);
}

// one camera sample: returns the sample's radiance L (before the clamp) and
// adds d L / d C_m to g_col and d L / d E_m to g_em
__device__ float3 adjoint_sample(const DevScene& S, const RenderCfg& cfg, float3 o0, float3 d0, uint64_t sample_id,
                                 int n_mat, float3* g_col, float3* g_em, TraceStats& st, uint32_t* err,
                                 uint32_t& segs) {
  PathState stack[kSplitStack];
  Anc anc[kSplitStack];
  int sp = 0;
  root_path(stack[sp], o0, d0);
  anc[sp].n = 0;
  sp++;
  float3 L = f3(0, 0, 0);
  EmissionTap tap{g_em, n_mat};
  float cnt[kAdjMaterials];
  float3 Ssum[kAdjMaterials];
  while (sp > 0) {
    --sp;
    PathState ps = stack[sp];
    Anc mine = anc[sp];  // this branch's vertex materials so far (first three), ancestors included
    for (int m = 0; m < n_mat; m++) {
      cnt[m] = 0.0f;
      Ssum[m] = f3(0, 0, 0);
    }
    for (int k = 0; k < mine.n; k++) cnt[mine.m[k]] += 1.0f;  // the child's radiance all comes after them
    for (;;) {
      FastHit h;
      segs++;
      const bool hit = fast_closest(S, ps.o, ps.d, h, st, err);
      ShadowReq sh[3];
      int nsh = 0;
      PathState child;
      const int r = shade<false, false>(S, cfg, ps, hit, h, sample_id, sh, nsh, child, err, nullptr, nullptr, &tap);
      if (r != SHADE_END) {
        // a non-terminal vertex: everything this branch adds from here on scales with its colour
        const int m = S.entf[h.ent].material;
        cnt[m] += 1.0f;
        Ssum[m] += ps.L;
        if (mine.n < 3) mine.m[mine.n++] = (int8_t)m;
      }
      for (int k = 0; k < nsh; k++) {
        segs++;
        if (!fast_occluded(S, sh[k].o, sh[k].d, sh[k].tmax, st, err)) {
          ps.L += sh[k].contrib;
          tap.em(sh[k].lmat, sh[k].ew);
        }
      }
      if (r == SHADE_SPLIT) {
        if (sp < kSplitStack) {
          stack[sp] = child;
          anc[sp] = mine;
          sp++;
        } else {
          atomicOr(err, PR_DEV_LOOP_CAP);
        }
      }
      if (r == SHADE_END) break;
    }
    for (int m = 0; m < n_mat; m++)
      if (cnt[m] > 0.0f) g_col[m] += safe_div(ps.L * cnt[m] - Ssum[m], ld3(S.mats[m].color));
    L += ps.L;
  }
  return L;
}

}  // namespace

__global__ void __launch_bounds__(128) adjoint_kernel(DevScene S, RenderCfg cfg, const float* __restrict__ dl_drgb,
                                                      int n_mat, double* __restrict__ d_color,
                                                      double* __restrict__ d_emission, uint32_t* __restrict__ err,
                                                      unsigned long long* __restrict__ counters) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t warp = tid >> 5, lane = tid & 31;
  const uint32_t tiles_per_chunk = cfg.tiles_x * cfg.tiles_y;
  const uint32_t chunk = warp / tiles_per_chunk;
  if (chunk >= (uint32_t)cfg.chunks) return;  // whole warps leave together
  const uint32_t tile = warp - chunk * tiles_per_chunk;
  const int x = (int)((tile % cfg.tiles_x) * 8 + (lane & 7));
  const int y = (int)((tile / cfg.tiles_x) * 4 + (lane >> 3));
  float3 G_col[kAdjMaterials], G_em[kAdjMaterials];
  for (int m = 0; m < kAdjMaterials; m++) G_col[m] = G_em[m] = f3(0, 0, 0);
  TraceStats st{0, 0};
  uint32_t segs = 0, paths = 0;
  if (x < cfg.width && y < cfg.height) {
    const size_t pix = (size_t)(cfg.height - y - 1) * cfg.width + x;
    const float3 delta = f3(dl_drgb[3 * pix], dl_drgb[3 * pix + 1], dl_drgb[3 * pix + 2]) * cfg.sensor;
    const int k0 = (int)(((int64_t)cfg.spp * chunk) / cfg.chunks);
    const int k1 = (int)(((int64_t)cfg.spp * (chunk + 1)) / cfg.chunks);
    float3 g_col[kAdjMaterials], g_em[kAdjMaterials];
    for (int k = k0; k < k1; k++) {
      for (int m = 0; m < n_mat; m++) g_col[m] = g_em[m] = f3(0, 0, 0);
      float3 o, d;
      const uint64_t sample_id = camera_ray(cfg, x, y, cfg.sample_offset + (uint64_t)k, o, d);
      const float3 L = adjoint_sample(S, cfg, o, d, sample_id, n_mat, g_col, g_em, st, err, segs);
      // finish_sample: v = L * smp, and above the cutoff v_c = c v / lum(v),
      // whose derivative is (c / lum) (dv - v (W . dv) / lum) with W the
      // luminance weights: the adjoint of the clamp maps delta to
      // (c / lum) (delta - (delta . v / lum) W)
      const float3 v = L * cfg.smp;
      float3 w = delta * cfg.smp;
      if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z))) {
        w = f3(0, 0, 0);
      } else if (cfg.cutoff > 0.0f) {
        const float3 W = f3(0.2126f, 0.7152f, 0.0722f);
        const float lum = dot(W, v);
        if (lum > cfg.cutoff) w = (delta - W * (dot(delta, v) / lum)) * (cfg.cutoff / lum * cfg.smp);
      }
      for (int m = 0; m < n_mat; m++) {
        G_col[m] += w * g_col[m];
        G_em[m] += w * g_em[m];
      }
      paths++;
    }
  }
  // warp sums, then one double atomic per value and warp
  for (int m = 0; m < n_mat; m++) {
    float v[6] = {G_col[m].x, G_col[m].y, G_col[m].z, G_em[m].x, G_em[m].y, G_em[m].z};
#pragma unroll
    for (int q = 0; q < 6; q++) {
      float a = v[q];
      for (int off = 16; off > 0; off >>= 1) a += __shfl_down_sync(0xffffffffu, a, off);
      if (lane == 0 && a != 0.0f) atomicAdd((q < 3 ? d_color : d_emission) + 3 * m + (q % 3), (double)a);
    }
  }
  if (counters) {
    unsigned long long a = paths, b = segs, c = st.nodes, dd = st.tris;
    for (int off = 16; off > 0; off >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, off);
      b += __shfl_down_sync(0xffffffffu, b, off);
      c += __shfl_down_sync(0xffffffffu, c, off);
      dd += __shfl_down_sync(0xffffffffu, dd, off);
    }
    if (lane == 0) {
      atomicAdd(counters + 0, a);
      atomicAdd(counters + 1, b);
      atomicAdd(counters + 2, c);
      atomicAdd(counters + 3, dd);
    }
  }
}

cudaError_t launch_adjoint(const DevScene& S, const RenderCfg& cfg, const float* dl_drgb, int n_mat, double* d_color,
                           double* d_emission, uint32_t* err, unsigned long long* counters, cudaStream_t stream) {
  const uint64_t threads = (uint64_t)cfg.tiles_x * cfg.tiles_y * 32ull * (uint64_t)cfg.chunks;
  const uint32_t blocks = (uint32_t)((threads + 127) / 128);
  adjoint_kernel<<<blocks, 128, 0, stream>>>(S, cfg, dl_drgb, n_mat, d_color, d_emission, err, counters);
  return cudaGetLastError();
}

}  // namespace pr
