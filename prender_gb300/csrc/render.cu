// Plain drop-in renderer: one thread per (pixel, sample chunk), iterative
// form of the reference's recursive radiance() (radiance.h:25-556).
//
// The recursion  L = Env + E + D + W * L_child  becomes a loop that adds
// beta * (Env + E + D) at each vertex and multiplies beta by W.  The only
// place the reference's recursion branches -- ideal glass at depth <= 2
// traces both reflection and refraction (brdf.h:899-936) -- pushes the
// refracted branch on a 4-entry stack.  Each branch draws from its own
// counter-based stream, keyed by (seed, sample id, branch id).
//
// Estimator details follow the reference, including its quirks:
//   * Russian roulette after DEPTH with p = max(E + colour), halved per level
//     beyond DEPTH_LIMIT (radiance.h:79-126);
//   * DIFFUSE / SPECULAR split by roughness (radiance.h:514-545);
//   * lights picked with index (int)(u (N-1) + 0.5) and probability 1
//     (light.h:146-151), 3 shadow rays per diffuse vertex (def.h:10),
//     emission of a light hit counted only at depth 0 with NEE
//     (brdf.h:443-476), uvplane lights dark from behind (brdf.h:434-440);
//   * specular / glass NEE as a light hit along the mirror / refraction
//     direction, not Fresnel-weighted (brdf.h:731-737, :788-936);
//   * glass: Schlick Fresnel, P = 0.25 + 0.5 Re beyond depth 2 (brdf.h:841-898);
//   * homogeneous medium: scatter with p = clamp(1 - exp(-sigma_s t)),
//     truncated free flight with scalar sigma_t, RGB transmittance, HG
//     phase with the reference's cos-theta expression unless
//     PR_FLAG_HG_CORRECT, NEE through the medium (ParticipatingMedia.h:27-461);
//   * per-sample luminance clamp and sensor response (render.h:1375-1409).
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "render_kernels.h"
#include "trace_fast.cuh"

namespace pr {

struct Branch {
  float3 o, d;
  float3 beta;
  float3 dp_w;  // weight of the pending light-hit term (specular / glass NEE)
  int depth;
  uint32_t id;
  int dp;       // 1: add dp_w * emission if the next hit is a light
};

struct Vertex {
  float3 p, n;  // hit point and geometric normal (after the entity's normal inversion)
  int mat, ent;
  float t;
};

__device__ __forceinline__ float3 medium_tr(const GMedium& m, float d) {
  return f3(expf(-m.sigma_t[0] * d), expf(-m.sigma_t[1] * d), expf(-m.sigma_t[2] * d));
}

// OrthonormalBasis (vector3d.h:244-253)
__device__ __forceinline__ void onb(float3 w, float3& u, float3& v) {
  if (fabsf(w.x) > 1.0e-6f) u = normalize(cross(f3(0.0f, 1.0f, 0.0f), w));
  else u = normalize(cross(f3(1.0f, 0.0f, 0.0f), w));
  v = normalize(cross(w, u));
}

__device__ __forceinline__ void make_vertex(const DevScene& S, float3 o, float3 d, const FastHit& h, Vertex& v) {
  const GEntity& e = S.ents[h.ent];
  v.ent = h.ent;
  v.mat = e.material;
  v.t = h.t;
  if (e.type == PR_ENT_SPHERE) {
    // position and normal in FP64 from the FP64 distance (sphere.h:89-95)
    const double t = h.t;
    const double px = (double)o.x + t * (double)d.x, py = (double)o.y + t * (double)d.y, pz = (double)o.z + t * (double)d.z;
    const double nx = px - e.p[0], ny = py - e.p[1], nz = pz - e.p[2];
    const double il = 1.0 / sqrt(nx * nx + ny * ny + nz * nz);
    v.p = f3((float)px, (float)py, (float)pz);
    v.n = f3((float)(nx * il), (float)(ny * il), (float)(nz * il));
  } else if (e.type == PR_ENT_UVPLANE) {
    v.p = o + d * h.t;
    v.n = f3((float)e.normal[0], (float)e.normal[1], (float)e.normal[2]);
  } else {
    // the hit point from the barycentrics: its error is a few ulps of the
    // vertex coordinates, not of the ray length, which the ulp-scaled
    // origin offset (offset_ray) relies on
    const float4* T = S.tris + 3 * (size_t)h.slot;
    const float4 A = __ldg(T), B = __ldg(T + 1), C = __ldg(T + 2);
    const float w = 1.0f - h.u - h.v;
    v.p = f3(w * A.x + h.u * B.x + h.v * C.x, w * A.y + h.u * B.y + h.v * C.y, w * A.z + h.u * B.z + h.v * C.z);
    v.n = ld3(S.fnorm + 3 * (size_t)(e.face_base + __float_as_int(A.w)));
  }
  if (e.normal_inverse < 0) v.n = -v.n;
}

// a point on light entity le (direct_radiance_sample, directLight_radiance.h:326-377;
// the media variant omits the uvplane's normal * PS_EPS lift, ParticipatingMedia.h:213-224)
__device__ __forceinline__ float3 sample_light(const GEntity& le, Rng& rng, bool lift) {
  if (le.type == PR_ENT_SPHERE) {
    const float r1 = 6.28318530717958647692f * rng.next();
    const float r2 = 1.0f - 2.0f * rng.next();
    const float sq = sqrtf(fmaxf(0.0f, 1.0f - r2 * r2));
    float sn, cs;
    sincosf(r1, &sn, &cs);
    const float R = (float)(le.radius + kEps);
    return f3((float)le.p[0], (float)le.p[1], (float)le.p[2]) + f3(sq * cs, sq * sn, r2) * R;
  }
  const float t = (float)le.v_length * rng.next();  // v first, then u (directLight_radiance.h:359-360)
  const float s = (float)le.u_length * rng.next();
  float3 lp = f3((float)le.p[0], (float)le.p[1], (float)le.p[2]) +
              f3((float)le.u_axis[0], (float)le.u_axis[1], (float)le.u_axis[2]) * s +
              f3((float)le.v_axis[0], (float)le.v_axis[1], (float)le.v_axis[2]) * t;
  if (lift) lp = lp + f3((float)le.normal[0], (float)le.normal[1], (float)le.normal[2]) * (float)kEps;
  return lp;
}

__device__ __forceinline__ float3 light_normal(const GEntity& le, float3 lp, bool use_inverse) {
  float3 n;
  if (le.type == PR_ENT_SPHERE) n = normalize(lp - f3((float)le.p[0], (float)le.p[1], (float)le.p[2]));
  else n = f3((float)le.normal[0], (float)le.normal[1], (float)le.normal[2]);
  if (use_inverse && le.normal_inverse < 0) n = -n;
  return n;
}

__device__ __forceinline__ const GEntity& pick_light(const DevScene& S, Rng& rng) {
  int idx = (int)(rng.next() * (float)(S.n_lights - 1) + 0.5f);
  idx = min(max(idx, 0), S.n_lights - 1);
  return S.ents[S.light_ent[idx]];
}

// NEE at a diffuse vertex (eval_direct_radiance, directLight_radiance.h:19-313)
__device__ float3 nee_surface(const DevScene& S, const Vertex& v, float3 on, float3 colour, bool media, Rng& rng,
                              TraceStats& st, uint32_t* err, uint32_t& segs) {
  float3 acc = f3(0, 0, 0);
  const float3 origin = offset_ray(v.p, on);
  for (int i = 0; i < 3; i++) {
    const GEntity& le = pick_light(S, rng);
    const float3 lp = sample_light(le, rng, true);
    const float3 ln = light_normal(le, lp, true);
    const float3 dl = lp - v.p;
    const float dist2 = dot(dl, dl);
    const float dist = sqrtf(dist2);
    const float3 ldir = dl / dist;
    const float dot0 = dot(on, ldir), dot1 = -dot(ln, ldir);
    if (dot0 >= 0.0f && dot1 >= 0.0f) {
      segs++;
      // visible iff nothing is hit closer than the light point - 1e-3
      // (directLight_radiance.h:136-171); the distance is measured from the
      // shadow ray's own (offset) origin, which can sit ~1e-3 nearer to the
      // light than the hit point
      const float3 dlo = lp - origin;
      const float disto = sqrtf(dot(dlo, dlo));
      if (!fast_occluded(S, origin, dlo / disto, disto - 1.0e-3f, st, err)) {
        const float G = dot0 * dot1 / dist2;
        const GMaterial& lm = S.mats[le.material];
        float3 em = ld3(lm.emission);
        if (media) em = em * medium_tr(S.medium, dist);
        acc += em * colour * (0.31830988618379067154f * G * (float)le.area);
      }
    }
  }
  return acc * (1.0f / 3.0f);
}

// NEE from a point in the medium (eval_direct_radiance_media, ParticipatingMedia.h:27-268)
__device__ float3 nee_medium(const DevScene& S, float3 pos, Rng& rng, TraceStats& st, uint32_t* err, uint32_t& segs) {
  float3 acc = f3(0, 0, 0);
  for (int i = 0; i < 3; i++) {
    const GEntity& le = pick_light(S, rng);
    const float3 lp = sample_light(le, rng, false);
    const float3 ln = light_normal(le, lp, false);
    const float3 dl = lp - pos;
    const float dist2 = dot(dl, dl);
    const float dist = sqrtf(dist2);
    const float3 ldir = dl / dist;
    const float dot1 = -dot(ln, ldir);
    if (dot1 >= 0.0f) {
      segs++;
      if (!fast_occluded(S, pos, ldir, dist - 1.0e-3f, st, err)) {
        const GMaterial& lm = S.mats[le.material];
        const float G = dot1 / dist2;
        acc += ld3(lm.emission) * (0.31830988618379067154f * G * (float)le.area) * medium_tr(S.medium, dist);
      }
    }
  }
  return acc * (1.0f / 3.0f);
}

// sampleHG (sampler.h:24-93); the reference's cos expression is (g/2)(...)
__device__ __forceinline__ float3 sample_hg(float3 raydir, float g, Rng& rng, bool correct) {
  float3 u, v;
  onb(raydir, u, v);
  const float r1 = 6.28318530717958647692f * rng.next();
  const float r2 = rng.next();
  const float s = (1.0f - g * g) / (1.0f - g + 2.0f * g * r2);
  const float cost = correct ? (1.0f + g * g - s * s) / (2.0f * g) : 0.5f * g * (1.0f + g * g - s * s);
  const float sint = sqrtf(fmaxf(0.0f, 1.0f - cost * cost));
  float sn, cs;
  sincosf(r1, &sn, &cs);
  return normalize(u * (sint * cs) + v * (sint * sn) + raydir * cost);
}

__device__ __forceinline__ float3 sample_sphere_dir(Rng& rng) {
  const float r1 = 6.28318530717958647692f * rng.next();
  const float r2 = 1.0f - 2.0f * rng.next();
  const float sq = sqrtf(fmaxf(0.0f, 1.0f - r2 * r2));
  float sn, cs;
  sincosf(r1, &sn, &cs);
  return normalize(f3(sq * cs, sq * sn, r2));
}

__device__ __forceinline__ float phase_hg(float g, float c) {
  const float w = 1.0f + g * g - 2.0f * g * c;
  if (fabsf(w) < 1.0e-12f) return 0.0f;
  return 0.0795774715459476679f * (1.0f - g * g) / (w * sqrtf(w));
}

// One camera sample: the whole branch tree of radiance() for one root ray.
__device__ float3 trace_sample(const DevScene& S, const RenderCfg& cfg, float3 o0, float3 d0, uint64_t sample_id,
                               TraceStats& st, uint32_t* err, uint32_t& segs, uint32_t& verts) {
  Branch stack[kSplitStack];
  int sp = 0;
  stack[sp++] = Branch{o0, d0, f3(1, 1, 1), f3(0, 0, 0), 0, 0u, 0};
  uint32_t next_id = 1;
  float3 L = f3(0, 0, 0);
  const bool nee = cfg.nee != 0;
  const bool media = cfg.media != 0 && S.medium.on != 0;
  const float3 env = f3((float)S.env_light[0], (float)S.env_light[1], (float)S.env_light[2]);
  const float3 bg = f3((float)S.background[0], (float)S.background[1], (float)S.background[2]);
  while (sp > 0) {
    Branch b = stack[--sp];
    Rng rng;
    rng.init(cfg.seed, sample_id, b.id);
    float3 o = b.o, d = b.d, beta = b.beta;
    int depth = b.depth;
    for (;;) {
      if (++verts > (uint32_t)cfg.max_vertices) {
        atomicOr(err, PR_DEV_LOOP_CAP);
        break;
      }
      FastHit h;
      segs++;
      const bool hit = fast_closest(S, o, d, h, st, err);
      if (b.dp) {
        if (hit && S.ents[h.ent].is_light) {
          float3 em = ld3(S.mats[S.ents[h.ent].material].emission);
          if (media) em = em * medium_tr(S.medium, h.t);
          L += b.dp_w * em;
        }
        b.dp = 0;
      }
      if (!hit) {
        L += beta * bg;
        break;
      }
      Vertex v;
      make_vertex(S, o, d, h, v);
      const GMaterial& m = S.mats[v.mat];
      const GEntity& ent = S.ents[v.ent];
      const float3 E = ld3(m.emission), C = ld3(m.color);
      const float3 on = dot(v.n, d) < 0.0f ? v.n : -v.n;
      float p_rr = maxc(E + C);  // WARD / PHONG are not on this path
      if (depth > cfg.depth_limit) p_rr *= exp2f((float)(cfg.depth_limit - depth));
      const float3 trr = media ? medium_tr(S.medium, v.t) : f3(1, 1, 1);
      if (depth > cfg.depth) {
        if (rng.next() >= p_rr) {
          L += beta * trr * E;
          break;
        }
      } else {
        p_rr = 1.0f;
      }
      const bool entering = dot(on, v.n) > 0.0f;  // Entity::isInsideDir (entity.h:98-114)
      float p_scat = 0.0f;
      if (media && entering) {
        p_scat = fminf(fmaxf(1.0f - expf(-S.medium.sigma_s_mean * v.t), 0.01f), 0.99f);
        if (rng.next() < p_scat) {
          // ---- scattering in the medium before the surface
          const GMedium& md = S.medium;
          const int sel = min(2, (int)(3.0f * rng.next()));
          const float u = rng.next();
          const float et = expf(-md.sigma_t_mean * v.t);
          const float ds = -logf(1.0f + u * (et - 1.0f)) / md.sigma_t_mean;
          const float pdf = expf(-md.sigma_t_mean * ds) * (-md.sigma_t_mean / (et - 1.0f));
          const float g = md.g[sel];
          float3 nd;
          float phase;
          if (g == 0.0f || fabsf(g) > 1.0f) {
            nd = sample_sphere_dir(rng);
            phase = 0.0795774715459476679f;
          } else {
            nd = sample_hg(d, g, rng, (cfg.flags & PR_FLAG_HG_CORRECT) != 0);
            phase = phase_hg(g, dot(nd, d));
          }
          const float3 npos = o + d * ds;
          const float3 tr = medium_tr(md, ds);
          float3 direct = f3(0, 0, 0);
          if (!ent.is_light && S.n_lights > 0) direct = nee_medium(S, npos, rng, st, err, segs);
          if (!(pdf > 0.0f)) break;
          if (ent.is_light) {
            if (depth == 0) L += beta * tr * E;
            break;
          }
          // phase / dirPdf == 1 in the reference's weight
          const float3 f = tr * f3(md.sigma_s[0], md.sigma_s[1], md.sigma_s[2]) * (phase / pdf / phase / p_scat / p_rr);
          L += beta * f * direct;
          beta = beta * f;
          o = npos;
          d = nd;
          depth++;
          continue;
        }
      }
      const float inv_rr = 1.0f / p_rr / (1.0f - p_scat);
      int kind;  // 0 diffuse, 1 specular, 2 glass
      if (m.type == PR_MAT_DIFFUSE) kind = (rng.next() < m.roughness) ? 0 : 1;
      else if (m.type == PR_MAT_SPECULAR) kind = (rng.next() < 1.0f - m.roughness) ? 1 : 0;
      else kind = 2;
      const float3 tri = (media && entering) ? trr : f3(1, 1, 1);
      if (kind == 0) {
        // ---- BRDF_Diffuse (brdf.h:408-700)
        if (ent.is_light) {
          if (ent.type == PR_ENT_UVPLANE && dot(v.n, d) >= 0.0f) break;
          if (!nee || depth == 0) L += beta * trr * E * inv_rr;
          break;
        }
        float3 u, w2;
        onb(on, u, w2);
        const float r1 = 6.28318530717958647692f * rng.next();
        const float r2 = rng.next();
        const float r2s = sqrtf(r2);
        float sn, cs;
        sincosf(r1, &sn, &cs);
        const float3 nd = normalize(u * (cs * r2s) + w2 * (sn * r2s) + on * sqrtf(1.0f - r2));
        float3 direct = f3(0, 0, 0);
        if (S.n_lights > 0) {
          if (nee) direct = nee_surface(S, v, on, C, media, rng, st, err, segs) * inv_rr;
          else for (int i = 0; i < 3; i++) (void)rng.next();  // light picks without area lights
        }
        L += beta * (env + tri * E + tri * direct);
        beta = beta * C * tri * inv_rr;
        o = offset_ray(v.p, on);
        d = nd;
        depth++;
        continue;
      }
      if (kind == 1) {
        // ---- BRDF_Specular (brdf.h:702-761): mirror about the geometric normal
        const float3 nd = normalize(d - v.n * (2.0f * dot(v.n, d)));
        L += beta * (env + tri * E);
        beta = beta * C * tri * inv_rr;
        b.dp = nee;
        b.dp_w = beta;
        o = offset_ray(v.p, dot(nd, v.n) > 0.0f ? v.n : -v.n);
        d = nd;
        depth++;
        continue;
      }
      // ---- BRDF_Refraction (brdf.h:763-953)
      const float3 refl = normalize(d - v.n * (2.0f * dot(v.n, d)));
      const bool into = dot(v.n, on) > 0.0f;
      const float nt = m.ior;
      const float nnt = into ? 1.0f / nt : nt;
      const float ddn = dot(d, on);
      const float cos2t = 1.0f - nnt * nnt * (1.0f - ddn * ddn);
      L += beta * (env + tri * E);
      const float3 base = beta * C * tri;
      const float3 refl_o = offset_ray(v.p, dot(refl, v.n) > 0.0f ? v.n : -v.n);
      if (cos2t < 0.0f) {  // total internal reflection
        beta = base * inv_rr;
        b.dp = nee;
        b.dp_w = beta;
        o = refl_o;
        d = refl;
        depth++;
        continue;
      }
      const float3 tdir = normalize(d * nnt - v.n * ((into ? 1.0f : -1.0f) * (ddn * nnt + sqrtf(fabsf(cos2t)))));
      const float a = nt - 1.0f, bb = nt + 1.0f;
      const float R0 = (a * a) / (bb * bb);
      const float c = 1.0f - (into ? -ddn : dot(tdir, -on));
      const float c2 = c * c;
      float Re = R0 + (1.0f - R0) * (c2 * c2 * c);
      float Tr = (1.0f - Re) * (nnt * nnt);
      float P = 0.25f + 0.5f * Re;
      if (m.type == PR_MAT_REFRACTION_FRESNEL) {
        if (into) { P = 1.0f; Re = 1.0f; Tr = 0.0f; }
        else { P = 0.0f; Re = 0.0f; Tr = 1.0f; }
      }
      const float3 tdir_o = offset_ray(v.p, dot(tdir, v.n) > 0.0f ? v.n : -v.n);
      if (depth > 2) {
        if (rng.next() < P) {
          const float3 W = base * (1.0f / (P * p_rr) / (1.0f - p_scat));
          beta = W * Re;
          b.dp_w = W;
          o = refl_o;
          d = refl;
        } else {
          const float3 W = base * (1.0f / ((1.0f - P) * p_rr) / (1.0f - p_scat));
          beta = W * Tr;
          b.dp_w = W;
          o = tdir_o;
          d = tdir;
        }
        b.dp = nee;
        depth++;
        continue;
      }
      const float3 W = base * inv_rr;
      if (sp < kSplitStack) {
        stack[sp++] = Branch{tdir_o, tdir, W * Tr, W, depth + 1, next_id++, nee ? 1 : 0};
      } else {
        atomicOr(err, PR_DEV_LOOP_CAP);
      }
      beta = W * Re;
      b.dp = nee;
      b.dp_w = W;
      o = refl_o;
      d = refl;
      depth++;
    }
  }
  return L;
}

__global__ void __launch_bounds__(128) pt_megakernel(DevScene S, RenderCfg cfg, float* __restrict__ out,
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
  uint32_t segs = 0, verts = 0, paths = 0;
  if (x < cfg.width && y < cfg.height) {
    const int k0 = (int)(((int64_t)cfg.spp * chunk) / cfg.chunks);
    const int k1 = (int)(((int64_t)cfg.spp * (chunk + 1)) / cfg.chunks);
    const uint32_t pix = (uint32_t)y * cfg.width + x;
    float3 acc = f3(0, 0, 0);
    for (int k = k0; k < k1; k++) {
      const uint64_t kg = cfg.sample_offset + (uint64_t)k;
      // subpixel and pass of per-pixel sample k (render.h:1203-1258)
      const int ssq = cfg.ss * cfg.ss;
      const int sub = (int)(kg % (uint64_t)ssq);
      const int sxx = sub % cfg.ss, syy = sub / cfg.ss;
      const uint64_t sample_id = kg * (uint64_t)cfg.width * (uint64_t)cfg.height + pix;
      Rng cam;
      cam.init(cfg.seed, sample_id, 0x80000000u);
      float dx = 0.0f, dy = 0.0f;
      if (cfg.tent) {
        const float rr1 = 2.0f * cam.next(), rr2 = 2.0f * cam.next();
        dx = rr1 < 1.0f ? sqrtf(rr1) - 1.0f : 1.0f - sqrtf(2.0f - rr1);
        dy = rr2 < 1.0f ? sqrtf(rr2) - 1.0f : 1.0f - sqrtf(2.0f - rr2);
      }
      const float r1 = (sxx + 0.5f + dx) * cfg.rate, r2 = (syy + 0.5f + dy) * cfg.rate;
      const float3 sp = cfg.center + cfg.screen_x * ((r1 + x) * cfg.iw - 0.5f) + cfg.screen_y * ((r2 + y) * cfg.ih - 0.5f);
      const float3 dir = normalize(sp - cfg.cam_pos);
      float3 v = trace_sample(S, cfg, cfg.cam_pos, dir, sample_id, st, err, segs, verts) * cfg.smp;
      if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z))) {
        atomicOr(err, PR_DEV_NONFINITE);
        v = f3(0, 0, 0);
      }
      if (cfg.cutoff > 0.0f) {  // per-sample luminance clamp (render.h:1375-1384)
        const float lum = 0.2126f * v.x + 0.7152f * v.y + 0.0722f * v.z;
        if (lum > cfg.cutoff) v = v * (cfg.cutoff / lum);
      }
      acc += v;
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
  pt_megakernel<<<blocks, 128, 0, stream>>>(S, cfg, out, err, counters);
  return cudaGetLastError();
}

cudaError_t launch_reduce(const float* partial, float* dst, int n3, int chunks, int accumulate, cudaStream_t stream) {
  reduce_chunks<<<(n3 + 255) / 256, 256, 0, stream>>>(partial, dst, n3, chunks, accumulate);
  return cudaGetLastError();
}

}  // namespace pr
