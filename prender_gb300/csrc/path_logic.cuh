// Per-vertex shading shared by the two render forms.
//
// The reference's recursive radiance() (radiance.h:25-556) becomes a state
// machine over a PathState: shade() consumes one closest hit, adds the
// vertex's terms to L, prepares up to three NEE shadow rays (their
// contributions are final unless the ray is blocked) and either continues
// the path, ends it, or -- for ideal glass at depth <= 2, where the
// reference traces both reflection and refraction (brdf.h:899-936) --
// continues with one branch and hands back the other.
//
// The megakernel traces the shadow rays and the next segment in place; the
// wavefront queues them.  Both call this same function with the same
// per-branch counter-based streams (branch ids form a binary tree: the
// children of branch b are 2b+1 (refraction) and 2b+2 (reflection)), so
// both forms follow identical paths and produce the same image up to float
// summation order.
#pragma once
#include "device_common.cuh"
#include "render_kernels.h"
#include "trace_fast.cuh"

namespace pr {

struct PathState {
  float3 o, d;
  float3 beta;
  float3 dpw;      // weight of the pending light-hit term (specular / glass NEE)
  float3 L;        // radiance gathered by this branch
  int depth;
  uint32_t branch;
  uint32_t draws;  // uniforms drawn so far from this branch's stream
  int dp;          // 1: the next hit adds dpw * emission if it is a light
};

struct ShadowReq {
  float3 o, d;
  float tmax;
  float3 contrib;  // added to L if nothing is hit before tmax
  float3 ew;       // contrib / emission of the light's material (adjoint)
  int lmat;        // the light's material
};

// d L / d emission: shade() reports every term it adds to L as
// weight * emission(material m) here (adjoint renders only; null otherwise)
struct EmissionTap {
  float3* g;  // one entry per material
  int n;
  __device__ __forceinline__ void em(int m, float3 w) {
    if (m >= 0 && m < n) g[m] += w;
  }
};

enum { SHADE_END = 0, SHADE_CONTINUE = 1, SHADE_SPLIT = 2 };

constexpr uint32_t kCameraStream = 0x80000000u;

// stream positioned at an arbitrary draw index (resumable between launches)
__device__ __forceinline__ void rng_at(Rng& r, uint64_t seed, uint64_t sample, uint32_t branch, uint32_t draws) {
  r.init(seed, sample, branch);
  r.ctr.z = draws >> 2;
  r.idx = 4;
  if (draws & 3) {
    r.buf = philox4x32_10(r.ctr, r.key);
    r.ctr.z++;
    r.idx = (int)(draws & 3);
  }
}
__device__ __forceinline__ uint32_t rng_draws(const Rng& r) { return ((r.ctr.z - (r.idx == 4 ? 0u : 1u)) << 2) + (r.idx == 4 ? 0u : (uint32_t)r.idx); }

__device__ __forceinline__ float3 medium_tr(const GMedium& m, float d) {
  return f3(expf(-m.sigma_t[0] * d), expf(-m.sigma_t[1] * d), expf(-m.sigma_t[2] * d));
}

// OrthonormalBasis (vector3d.h:244-253)
__device__ __forceinline__ void onb(float3 w, float3& u, float3& v) {
  if (fabsf(w.x) > 1.0e-6f) u = normalize(cross(f3(0.0f, 1.0f, 0.0f), w));
  else u = normalize(cross(f3(1.0f, 0.0f, 0.0f), w));
  v = normalize(cross(w, u));
}

struct Vertex {
  float3 p, n;  // hit point and geometric normal (after the entity's normal inversion)
  int mat, ent;
  float t;
};

__device__ __forceinline__ void make_vertex(const DevScene& S, float3 o, float3 d, const FastHit& h, Vertex& v) {
  const GEntF& e = S.entf[h.ent];
  v.ent = h.ent;
  v.mat = e.material;
  v.t = h.t;
  if (e.type == PR_ENT_SPHERE) {
    // position and normal in FP64 from the FP64 distance (sphere.h:89-95):
    // the hit's t plus the remainder fast_sphere kept in u
    const GEntity& ed = S.ents[h.ent];
    const double t = (double)h.t + (double)h.u;
    const double px = (double)o.x + t * (double)d.x, py = (double)o.y + t * (double)d.y, pz = (double)o.z + t * (double)d.z;
    const double nx = px - ed.p[0], ny = py - ed.p[1], nz = pz - ed.p[2];
    const double il = 1.0 / sqrt(nx * nx + ny * ny + nz * nz);
    v.p = f3((float)px, (float)py, (float)pz);
    v.n = f3((float)(nx * il), (float)(ny * il), (float)(nz * il));
  } else if (e.type == PR_ENT_UVPLANE || e.type == PR_ENT_CIRCLE) {
    v.p = o + d * h.t;
    v.n = f3(e.n[0], e.n[1], e.n[2]);
  } else {
    // the hit point from the barycentrics: its error is a few ulps of the
    // vertex coordinates, not of the ray length, which the ulp-scaled
    // origin offset (offset_ray) relies on
    const float4* T = S.rtris + 3 * (size_t)h.slot;
    const float4 A = __ldg(T), B = __ldg(T + 1), C = __ldg(T + 2);
    const float w = 1.0f - h.u - h.v;
    v.p = f3(w * A.x + h.u * B.x + h.v * C.x, w * A.y + h.u * B.y + h.v * C.y, w * A.z + h.u * B.z + h.v * C.z);
    v.n = ld3(S.fnorm + 3 * (size_t)(e.face_base + __float_as_int(A.w)));
  }
  if (e.normal_inverse < 0) v.n = -v.n;
}

// The reference's light choice and surface NEE point draw with Next01,
// which under Metropolis light transport is the thread's stream rather than
// a primary sample (mlt.h:166, light.h:147, directLight_radiance.h:343-371):
// a sampler may route those draws elsewhere; the stream samplers do not.
__device__ __forceinline__ float rng_stream(Rng& r) { return r.next(); }

// a point on light entity le (direct_radiance_sample, directLight_radiance.h:326-377;
// the media variant omits the uvplane's normal * PS_EPS lift, ParticipatingMedia.h:213-224)
template <class R>
__device__ __forceinline__ float3 sample_light(const GEntF& le, R& rng, bool lift) {
  if (le.type == PR_ENT_SPHERE) {
    const float r1 = 6.28318530717958647692f * (lift ? rng_stream(rng) : rng.next());
    const float r2 = 1.0f - 2.0f * (lift ? rng_stream(rng) : rng.next());
    const float sq = sqrtf(fmaxf(0.0f, 1.0f - r2 * r2));
    float sn, cs;
    sincosf(r1, &sn, &cs);
    return f3(le.p[0], le.p[1], le.p[2]) + f3(sq * cs, sq * sn, r2) * le.radius_eps;
  }
  const float t = le.v_length * (lift ? rng_stream(rng) : rng.next());  // v first, then u (directLight_radiance.h:359-360)
  const float s = le.u_length * (lift ? rng_stream(rng) : rng.next());
  float3 lp = f3(le.p[0], le.p[1], le.p[2]) + f3(le.u[0], le.u[1], le.u[2]) * s + f3(le.v[0], le.v[1], le.v[2]) * t;
  if (lift) lp = lp + f3(le.n[0], le.n[1], le.n[2]) * 1.0e-6f;
  return lp;
}

__device__ __forceinline__ float3 light_normal(const GEntF& le, float3 lp, bool use_inverse) {
  float3 n;
  if (le.type == PR_ENT_SPHERE) n = normalize(lp - f3(le.p[0], le.p[1], le.p[2]));
  else n = f3(le.n[0], le.n[1], le.n[2]);
  if (use_inverse && le.normal_inverse < 0) n = -n;
  return n;
}

// LightList::randomLight (light.h:132-155): rounded index, probability 1
template <class R>
__device__ __forceinline__ const GLight& pick_light(const DevScene& S, R& rng) {
  int idx = (int)(rng_stream(rng) * (float)(S.n_lights - 1) + 0.5f);
  idx = min(max(idx, 0), S.n_lights - 1);
  return S.lights[idx];
}

// SpotLightEmission / |emission| (light.h:47-73): the cone falloff of the
// direction from the light's centre to p, over the distance attenuation
__device__ __forceinline__ float spot_factor(const GLight& L, float3 p) {
  const float3 dl = f3(L.center[0], L.center[1], L.center[2]) - p;
  const float dist = sqrtf(dot(dl, dl));
  const float3 wi = dl / dist;
  float inv_a = L.att[0] + dist * (L.att[1] + L.att[2] * dist);
  if (inv_a < 1.0e-3f) inv_a = 1.0f;
  const float ct = -dot(f3(L.dir[0], L.dir[1], L.dir[2]), wi);
  float f;
  if (ct < L.cos_total) f = 0.0f;
  else if (ct > L.cos_start) f = 1.0f;
  else f = powf((ct - L.cos_total) / (L.cos_start - L.cos_total), L.falloff);
  return f / inv_a;
}

// One next-event sample of light L seen from point p (direct_radiance_sample
// + eval_direct_radiance, directLight_radiance.h:19-387; a medium point,
// surface = false, has no cosine at the receiver, samples uvplanes without
// the normal * PS_EPS lift and ignores normal inversion,
// ParticipatingMedia.h:27-268).  Area lights: a point on the light, G =
// cos0 cos1 / d^2 over pdf = 1 / area, visible iff nothing is hit before
// the point.  Parallel lights: direction -dir, G = cos0, visible iff the
// first thing hit along it is the light itself.  Spot lights: direction to
// the centre, G = cos0 of the sampled surface point (the reference keeps
// that cosine), the emission scaled by the cone falloff and attenuation,
// visible iff the light is the first thing hit.  Infinity lights: direction
// -dir as given, G = cos0 with that vector, visible iff nothing is hit; no
// medium attenuation (the reference has no light entity to measure to).
struct LightSample {
  float3 ldir;  // light_dir of eval_direct_radiance (the BRDF is evaluated towards it)
  float3 k;     // G / pdf, times the spot factor and the medium's transmittance
  float3 so, sd;  // shadow ray
  float tmax;
  bool area;    // area light: a diffuse receiver takes colour / pi, the other kinds colour
};

// parallel, spot and infinity lights (compiled into the shading
// instantiations for scenes that have them)
template <class R>
__device__ __forceinline__ bool point_light_sample(const DevScene& S, const GLight& L, float3 p, float3 on,
                                                   float3 origin, bool surface, bool media, R& rng,
                                                   LightSample& ls) {
  ls.area = false;
  ls.so = origin;
  if (L.kind == PR_LIGHT_INFINITY) {  // draws nothing
    ls.ldir = -f3(L.dir[0], L.dir[1], L.dir[2]);
    const float dot0 = surface ? dot(on, ls.ldir) : 1.0f;
    if (!(dot0 >= 0.0f)) return false;
    ls.k = f3(dot0, dot0, dot0);
    ls.sd = ls.ldir / L.dir_len;
    ls.tmax = 1.0e30f;
    return true;
  }
  const GEntF& le = S.entf[L.ent];
  const float3 lp = sample_light(le, rng, surface);
  float trd;  // path length through the medium
  float g;
  if (L.kind == PR_LIGHT_PARALLEL) {
    ls.ldir = -f3(L.dir[0], L.dir[1], L.dir[2]);
    g = surface ? dot(on, ls.ldir) : 1.0f;
    ls.sd = ls.ldir;
    const float3 dl = lp - p;
    trd = sqrtf(dot(dl, dl));
  } else {
    const float3 c = f3(L.center[0], L.center[1], L.center[2]);
    const float3 dc = c - p;
    trd = sqrtf(dot(dc, dc));
    ls.ldir = dc / trd;
    const float3 dl = lp - p;
    g = surface ? dot(on, dl / sqrtf(dot(dl, dl))) : 1.0f;
    const float3 dco = c - origin;
    ls.sd = dco / sqrtf(dot(dco, dco));
  }
  if (!(g >= 0.0f)) return false;
  if (L.kind == PR_LIGHT_SPOT) g *= spot_factor(L, p);
  // the light must be the first thing the shadow ray meets
  float tl = 3.0e38f, rest;
  bool on_light;
  if (le.type == PR_ENT_SPHERE) on_light = fast_sphere(S.ents[L.ent], origin, ls.sd, 3.0e38f, tl, rest);
  else on_light = fast_uvplane(le, origin, ls.sd, 3.0e38f, tl);
  if (!on_light) return false;
  ls.k = f3(g, g, g);
  if (media) ls.k = ls.k * medium_tr(S.medium, trd);
  ls.tmax = tl - 1.0e-3f;
  return true;
}

__device__ __forceinline__ void push_shadow(const DevScene& S, const LightSample& ls, float3 ew, int lmat,
                                            ShadowReq* sh, int& nsh) {
  sh[nsh].o = ls.so;
  sh[nsh].d = ls.sd;
  sh[nsh].tmax = ls.tmax;
  sh[nsh].ew = ew;
  sh[nsh].contrib = ew * ld3(S.mats[lmat].emission);
  sh[nsh].lmat = lmat;
  nsh++;
}

// direct_light_perfect_refrection (directLight_radiance.h:516-556): what a
// specular or glass vertex at o sees of the lights straight along d, as a
// factor on the emission of material mat (-1: nothing).  A miss meets an
// infinity light within |dir . -d - 1| < 1e-3 (LightList::InfinityLight,
// light.h:157-173); a light entity gives its emission, scaled for a
// parallel or spot light by the cosine to the light direction and the spot
// factor (parallel_light_direct / spot_light_direct, :406-477), where the
// reference takes the light kind from its sorted list at the entity's
// registration index.
template <bool EXT>
__device__ __forceinline__ float perfect_direct(const DevScene& S, float3 o, float3 d, bool hit, const FastHit& h,
                                                int& mat) {
  mat = -1;
  if (!EXT) {
    if (hit && S.entf[h.ent].is_light) mat = S.entf[h.ent].material;
    return 1.0f;
  }
  if (!hit) {
    for (int i = 0; i < S.n_lights; i++) {
      const GLight& L = S.lights[i];
      if (L.kind == PR_LIGHT_INFINITY && fabsf(-dot(f3(L.dir[0], L.dir[1], L.dir[2]), d) - 1.0f) < 1.0e-3f) {
        mat = L.mat;
        return 1.0f;
      }
    }
    return 0.0f;
  }
  const GEntF& e = S.entf[h.ent];
  if (!e.is_light) return 0.0f;
  mat = e.material;
  const GLight& L = S.lights[e.light_id];
  if (L.kind == PR_LIGHT_PARALLEL) return fmaxf(-dot(d, f3(L.dir[0], L.dir[1], L.dir[2])), 0.0f);
  if (L.kind == PR_LIGHT_SPOT) {
    const float3 dc = f3(L.center[0], L.center[1], L.center[2]) - o;
    const float c = dot(d, dc / sqrtf(dot(dc, dc)));
    return c >= 0.0f ? c * spot_factor(L, o) : 0.0f;
  }
  return 1.0f;
}


// sampleHG (sampler.h:24-93); the reference's cos expression is (g/2)(...)
template <class R>
__device__ __forceinline__ float3 sample_hg(float3 raydir, float g, R& rng, bool correct) {
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

template <class R>
__device__ __forceinline__ float3 sample_sphere_dir(R& rng) {
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

// camera ray of per-pixel sample kg (render.h:1203-1269); returns the sample id
__device__ __forceinline__ uint64_t camera_ray(const RenderCfg& cfg, int x, int y, uint64_t kg, float3& o, float3& d) {
  const int ssq = cfg.ss * cfg.ss;
  const int sub = (int)(kg % (uint64_t)ssq);
  const int sxx = sub % cfg.ss, syy = sub / cfg.ss;
  const uint64_t sample_id = kg * (uint64_t)cfg.width * (uint64_t)cfg.height + (uint64_t)y * cfg.width + x;
  Rng cam;
  cam.init(cfg.seed, sample_id, kCameraStream);
  float dx = 0.0f, dy = 0.0f;
  if (cfg.tent) {
    const float rr1 = 2.0f * cam.next(), rr2 = 2.0f * cam.next();
    dx = rr1 < 1.0f ? sqrtf(rr1) - 1.0f : 1.0f - sqrtf(2.0f - rr1);
    dy = rr2 < 1.0f ? sqrtf(rr2) - 1.0f : 1.0f - sqrtf(2.0f - rr2);
  }
  const float r1 = (sxx + 0.5f + dx) * cfg.rate, r2 = (syy + 0.5f + dy) * cfg.rate;
  const float3 sp = cfg.center + cfg.screen_x * ((r1 + x) * cfg.iw - 0.5f) + cfg.screen_y * ((r2 + y) * cfg.ih - 0.5f);
  o = cfg.cam_pos;
  d = normalize(sp - cfg.cam_pos);
  return sample_id;
}

__device__ __forceinline__ void root_path(PathState& ps, float3 o, float3 d) {
  ps.o = o;
  ps.d = d;
  ps.beta = f3(1, 1, 1);
  ps.dpw = f3(0, 0, 0);
  ps.L = f3(0, 0, 0);
  ps.depth = 0;
  ps.branch = 0;
  ps.draws = 0;
  ps.dp = 0;
}

// A subsurface vertex whose continuation the reference drops when
// |weight * incoming| exceeds a bound (OVER_RADIANCE_CUT2 / 3,
// Subsurface_Scattering.h:19-22): the caller accumulates the continuation
// and applies the bound when the continuation (all its branches) is done.
struct SssFrameOut {
  int open;       // frames opened at this vertex: 0, 1, or 2 nested ones
  float3 scale;   // path contributions = scale * (weight * incoming)
  float thr;
  float3 scale2;  // the inner frame (the single-scattering walk's OVER_RADIANCE_CUT0)
  float thr2;
  int nee_inner;  // this vertex's next-event terms belong to the innermost frame
  float3 inner;   // radiance this vertex adds inside the innermost frame (besides those)
};

// ParticipatingMedia::sample(u, SAMPLE_ABSORBING, inv) (ParticipatingMediaPrm.h:251-279)
// over the subsurface material's table
__device__ __forceinline__ int sss_channel(const GMaterial& m, float u, bool inv) {
  if (m.sss_tsum < 1.0e-14f) return min(2, (int)(3.0f * u));
  const int mn = m.sss_idx & 15, md = (m.sss_idx >> 4) & 15, mx = (m.sss_idx >> 8) & 15;
  const float t0 = m.sss_t[0], t1 = m.sss_t[1], t2 = m.sss_t[2];
  int ii = inv ? mn : 0;
  if (u < t0) ii = mn;
  else if (u < t0 + t1) ii = md;
  else if (u < t0 + t1 + t2) ii = mx;
  if (inv) {
    if (-u < -t0) ii = mn;
    else if (-u < -t0 - t1) ii = md;
    else if (-u < -t0 - t1 - t2) ii = mx;
  }
  return ii;
}

// fresnel (bssrdf.h:239-247)
__device__ __forceinline__ float dd_fresnel(float cos_theta, float eta) {
  const float s2 = 1.0f / (eta * eta) * (1.0f - cos_theta * cos_theta);
  if (s2 >= 1.0f) return 1.0f;
  const float ct = sqrtf(1.0f - s2);
  const float rs = (cos_theta - eta * ct) / (cos_theta + eta * ct);
  const float rp = (eta * cos_theta - ct) / (eta * cos_theta + ct);
  return (rs * rs + rp * rp) * 0.5f;
}

// Sp_d (bssrdf.h:131-172), channel j
__device__ __forceinline__ float dd_sp(const GMaterial& m, float3 x, float3 w, float r, float3 n0, int j) {
  const float str = m.sss_sigma_tr[j] * r, one = 1.0f + str, xw = dot(x, w), r2 = r * r, D = m.sss_D[j];
  const float t0 = 1.0f / (4.0f * m.sss_Cp) * 0.025330295910584444f * expf(-str) / (r * r2);
  const float t1 = r2 / D + 3.0f * one * xw;
  const float t2 = 3.0f * D * one * dot(w, n0);
  const float t3 = (one + 3.0f * D * (3.0f * one + str * str) / r2 * xw) * dot(x, n0);
  return t0 * (m.sss_Cp * t1 - m.sss_Ce * (t2 - t3));
}

// bssrdf (bssrdf.h:188-236) of the directional dipole (Frisvad, Hachisuka and
// Kjeldsen, ACM TOG 2014), entry (xi, ni, wi), exit (xo, no), channel j
__device__ __forceinline__ float dd_bssrdf(const GMaterial& m, float3 xi, float3 ni, float3 wi, float3 xo, float3 no,
                                           int j) {
  const float3 xoxi = xo - xi;
  const float r = sqrtf(dot(xoxi, xoxi));
  float3 ni_s = r < 1.0e-8f ? ni : cross(xoxi / r, normalize(cross(ni, xoxi)));
  const float nnt = 1.0f / m.sss_eta, ddn = -dot(wi, ni);
  const float3 w12 = normalize(wi * -nnt - ni * (ddn * nnt + sqrtf(fmaxf(0.0f, 1.0f - nnt * nnt * (1.0f - ddn * ddn)))));
  const float3 wv = w12 - ni_s * (2.0f * dot(w12, ni_s));
  const float de = m.sss_de[j], D = m.sss_D[j];
  const float xw = dot(xoxi, w12);
  const float cos_beta = -sqrtf(fmaxf(0.0f, (r * r - xw * xw) / (r * r + de * de)));
  const float mu0 = -dot(no, w12);
  float dr;
  if (mu0 > 0.0f) dr = sqrtf(fmaxf(0.0f, (D * mu0) * ((D * mu0) - de * cos_beta * 2.0f) + r * r));
  else dr = sqrtf(fmaxf(0.0f, 1.0f / (3.0f * m.sss_sigma_t[j] * 3.0f * m.sss_sigma_t[j]) + r * r));
  const float3 xoxv = xo - (xi + ni_s * (2.0f * m.sss_A * de));
  const float dv = sqrtf(dot(xoxv, xoxv));
  const float res = dd_sp(m, xoxi, w12, dr, no, j) - dd_sp(m, xoxv, wv, dv, no, j);
  return res < 0.0f ? 0.0f : res;
}

// Leaving a subsurface object at the end of the single-scattering walk
// (radiance_through_media at sc_max, Subsurface_Scattering.h:409-541): the
// path continues from exit hit oh (vertex ov) with the medium's
// transmittance over the last segment; into another object straight on,
// across the object's own surface refracted (mirrored under total internal
// reflection) and weighted by the surface colour, with three next-event
// samples at the exit point (colour / pi, the unflipped surface normal as
// orienting normal).  The reference computes Fresnel factors here that it
// does not apply.
template <bool EXT, class R>
__device__ inline void sss_exit(const DevScene& S, const RenderCfg& cfg, const GMaterial& m, int in_ent,
                                const FastHit& oh, const Vertex& ov, float3 dir, float rr2, float3 beta, int depth,
                                R& rng, ShadowReq* sh, int& nsh, PathState& ps) {
  const float3 Tr = f3(expf(-m.sss_tr[0] * oh.t), expf(-m.sss_tr[1] * oh.t), expf(-m.sss_tr[2] * oh.t));
  ps.dp = 0;
  ps.depth = depth;
  if (oh.ent != in_ent) {
    ps.beta = beta * Tr * (1.0f / rr2);
    ps.o = offset_ray(ov.p, dot(dir, ov.n) > 0.0f ? ov.n : -ov.n);
    ps.d = dir;
    return;
  }
  const float3 n = ov.n;
  const bool into = dot(n, dir) < 0.0f;
  const float3 oon = into ? n : -n;
  const float nnt = into ? 1.0f / m.ior : m.ior;
  const float ddn = dot(dir, oon);
  const float cos2t = 1.0f - nnt * nnt * (1.0f - ddn * ddn);
  float3 nd = dir;
  if (cos2t > 0.0f) nd = normalize(dir * nnt - n * ((into ? 1.0f : -1.0f) * (ddn * nnt + sqrtf(fabsf(cos2t)))));
  if (cos2t < 0.0f) nd = normalize(dir - n * (2.0f * dot(n, dir)));
  const float3 C = ld3(m.color);
  const float3 bw = beta * Tr * C * (1.0f / rr2);
  const bool nee = cfg.nee != 0;
  if (S.n_lights > 0 && (nee || EXT)) {
    // without NEE only parallel, spot and infinity lights are sampled (:519-535)
    const float3 origin = offset_ray(ov.p, n);
    const float3 wn = bw * C * (0.31830988618379067154f / 3.0f);
    for (int i = 0; i < 3; i++) {
      const GLight& L = pick_light(S, rng);
      if (EXT && L.kind != PR_LIGHT_AREA) {  // colour, not colour / pi
        LightSample ls;
        if (point_light_sample(S, L, ov.p, n, origin, true, cfg.media != 0 && S.medium.on != 0, rng, ls))
          push_shadow(S, ls, wn * ls.k * 3.14159265358979323846f, L.mat, sh, nsh);
        continue;
      }
      if (!nee) continue;
      const GEntF& le = S.entf[L.ent];
      const float3 lp = sample_light(le, rng, true);
      const float3 ln = light_normal(le, lp, true);
      const float3 dl = lp - ov.p;
      const float dist2 = dot(dl, dl);
      const float3 ldir = dl / sqrtf(dist2);
      const float dot0 = dot(n, ldir), dot1 = -dot(ln, ldir);
      if (dot0 >= 0.0f && dot1 >= 0.0f) {
        const float3 dlo = lp - origin;
        const float disto = sqrtf(dot(dlo, dlo));
        const float3 em = ld3(S.mats[le.material].emission);
        float3 ew = wn * (dot0 * dot1 / dist2 * le.area);
        if (cfg.media != 0 && S.medium.on != 0) ew = ew * medium_tr(S.medium, sqrtf(dist2));
        sh[nsh].o = origin;
        sh[nsh].d = dlo / disto;
        sh[nsh].tmax = disto - 1.0e-3f;
        sh[nsh].contrib = ew * em;
        sh[nsh].ew = ew;
        sh[nsh].lmat = le.material;
        nsh++;
      }
    }
  }
  ps.beta = bw;
  ps.o = offset_ray(ov.p, dot(nd, n) > 0.0f ? n : -n);
  ps.d = nd;
}

// ---- textures and IBL images on hits (sphere.h:104-240, plane.h:241-273)

// the sphere's (u, v) of a mapping: the spherical angles, then the
// equirectangular, angular and panoramic maps, each replacing the last where
// set; swap: the IBL and bump blocks' order (u from theta, v from phi);
// clamp: the IBL block's clamp of the angular map's cosine
__device__ __forceinline__ void sphere_uv(int flags, float3 vv, bool swap, bool clamp, float& u, float& v) {
  const float kPi = 3.14159265358979323846f, kTwoPi = 6.28318530717958647692f;
  const float th = acosf(fminf(1.0f, fmaxf(-1.0f, vv.z)));  // SphericalTheta (vector3d.h:259-261)
  float ph = atan2f(vv.y, vv.x);                             // SphericalPhi (:262-267)
  if (ph < 0.0f) ph += kTwoPi;
  if (ph >= kTwoPi) ph = 0.0f;
  u = swap ? th / kPi : ph / kTwoPi;
  v = swap ? ph / kTwoPi : th / kPi;
  if (flags & PR_MAP_EQUIRECTANGULAR) {
    const float len = sqrtf(vv.x * vv.x + vv.y * vv.y + vv.z * vv.z);
    if (len == 0.0f) {
      u = 0.0f;
      v = 0.5f;
    } else {
      const float lambda = atan2f(vv.z / len, vv.x / len);
      const float phi = asinf(fmaxf(-1.0f, fminf(1.0f, vv.y / len)));
      u = (lambda + kPi) / kTwoPi;
      u = u - floorf(u);
      v = fminf(1.0f, fmaxf(0.0f, (0.5f * kPi - phi) / kPi));
    }
  }
  if (flags & PR_MAP_ANGULAR) {
    const float c = clamp ? fminf(1.0f, fmaxf(-1.0f, vv.z)) : vv.z;
    const float r = acosf(c) / kPi / sqrtf(vv.x * vv.x + vv.y * vv.y);
    u = 0.5f * (vv.x * r) + 0.5f;
    v = 0.5f * (vv.y * r) + 0.5f;
  }
  if (flags & PR_MAP_PANORAMIC) {
    const float c = fminf(1.0f, fmaxf(-1.0f, vv.y));
    u = 0.5f * (1.0f + atan2f(vv.x, -vv.z) / kPi);
    v = 1.0f - acosf(c) / kPi;
  }
}

// the repeat wrap (sphere.h:189-196): the fraction, negatives from 1
__device__ __forceinline__ float tex_wrap(float x) {
  if (x < 0.0f || x > 1.0f) x = x - truncf(x);
  if (x < 0.0f) x = 1.0f - fabsf(x);
  return x;
}

__device__ __forceinline__ int tex_clamp(int i, int n) { return min(max(i, 0), n - 1); }

// the bump map's tilted normal at texel (i, j): central luminance
// differences (the reference's wrap at the edges, which a square map keeps
// in range) times 0.5 * scale along the tangents (sphere.h:411-492,
// plane.h:290-360); n is the entity's own normal before its inversion
__device__ __forceinline__ float3 bump_tilt(const DevScene& S, const GMaterial& m, int i, int j, float3 n, float3 sdir,
                                            float3 tdir, float scale) {
  const int W = m.bump_w, H = m.bump_h;
  i = tex_clamp(i, H);
  j = tex_clamp(j, W);
  int u0 = j - 1, u1 = j + 1, v0 = i - 1, v1 = i + 1;
  if (u0 < 0) u0 = W - 1;
  if (v0 < 0) v0 = W - 1;
  if (u1 >= W) u1 = 0;
  if (v1 >= H) v1 = 0;
  const float* Y = S.bump_texels + m.bump_off;
  const float gx = scale * (__ldg(Y + (size_t)i * W + u1) - __ldg(Y + (size_t)i * W + u0)) * 0.5f;
  const float gy = scale * (__ldg(Y + (size_t)v1 * W + j) - __ldg(Y + (size_t)v0 * W + j)) * 0.5f;
  return n + cross(n, tdir) * gx - cross(n, sdir) * gy;
}

// The hit point's material where a texture or IBL image rewrites it: the
// texture gives colour and specular, the IBL image colour and emission
// (ibl_coef times the texel); a bump map gives the tilted normal bn (and
// bit 2 of the result).  Bit 1 of the result: the material has an IBL
// image, whose hit the caller ends with its emission (radiance.h:45-50).
// Triangle::intersect's smooth normal and texture coordinates (polygon.h:
// 186-212) at a mesh hit with barycentrics (u, v): the normal interpolated
// from the face's vertex normals (then the entity's inversion), and the
// material's texture or IBL image at (W - 1) u, (H - 1) v of the
// interpolated coordinates (polygon.h:507-528: the texel is the colour, the
// specular colour stays; an IBL texel is the colour and, scaled, the
// emission).  Bump maps on meshes do not reach the hit the reference
// returns (polygon.h:529-618 writes the caller's record, which the hit
// then overwrites), so none is read here.  True for an IBL hit.
__device__ inline bool mesh_hit(const DevScene& S, const GMaterial& m, const GEntF& e, int flags, const FastHit& h,
                                Vertex& v, float3& C, float3& E, float3& Sp) {
  const int face = e.face_base + __float_as_int(__ldg(S.rtris + 3 * (size_t)h.slot).w);
  const float w = 1.0f - h.u - h.v;
  // an OBJ material's '#SMOOTH' overrides the entity's 'smooth' (polygon.h:178-188)
  const bool smooth = (flags & 4) && m.mesh_smooth ? m.mesh_smooth == 1 : (flags & 1) != 0;
  if (smooth && (flags & 8)) {
    const float* n = S.fvn + 9 * (size_t)face;
    float3 ns = normalize(f3(n[0] * w + n[3] * h.u + n[6] * h.v, n[1] * w + n[4] * h.u + n[7] * h.v,
                             n[2] * w + n[5] * h.u + n[8] * h.v));
    v.n = e.normal_inverse < 0 ? -ns : ns;
  }
  if (!(flags & 2)) return false;
  const float* t = S.fuv + 6 * (size_t)face;
  const float tu = t[0] * w + t[2] * h.u + t[4] * h.v, tv = t[1] * w + t[3] * h.u + t[5] * h.v;
  if ((flags & 4) && m.mtex_off >= 0) {
    // map_Kd: the texel at the repeated, wrapped coordinates scales the
    // derived colours the mask names (polygon.h:236-305)
    const float uu = tex_wrap(tu * (float)m.mtex_repeat), vv = tex_wrap(tv * (float)m.mtex_repeat);
    const float4 x = __ldg(S.texels + m.mtex_off + (size_t)tex_clamp((int)((m.mtex_h - 1) * vv), m.mtex_h) * m.mtex_w +
                           tex_clamp((int)((m.mtex_w - 1) * uu), m.mtex_w));
    const float3 tx = f3(x.x, x.y, x.z);
    if (m.mtex_mask & 1) C = C * tx;
    if (m.mtex_mask & 2) Sp = Sp * tx;
    if (m.mtex_mask & 4) E = E * tx;
  }
  if (m.tex_off >= 0) {
    const float4 x = __ldg(S.texels + m.tex_off + (size_t)tex_clamp((int)((m.tex_h - 1) * tv), m.tex_h) * m.tex_w +
                           tex_clamp((int)((m.tex_w - 1) * tu), m.tex_w));
    C = f3(x.x, x.y, x.z);
  }
  if (m.ibl_off < 0) return false;
  const float4 x = __ldg(S.ibl_texels + m.ibl_off + (size_t)tex_clamp((int)((m.ibl_h - 1) * tv), m.ibl_h) * m.ibl_w +
                         tex_clamp((int)((m.ibl_w - 1) * tu), m.ibl_w));
  C = f3(x.x, x.y, x.z);
  E = C * m.ibl_coef;
  return true;
}

__device__ inline int hit_texture(const DevScene& S, const GMaterial& m, const GEntF& e, const GEntity& ed, float3 p,
                                  float3 n_hit, float3& C, float3& E, float3& Sp, float3& bn) {
  const bool has_ibl = m.ibl_off >= 0;
  int res = has_ibl ? 1 : 0;
  if (e.type == PR_ENT_UVPLANE) {
    const float3 rel = p - f3(e.p[0], e.p[1], e.p[2]);
    const float u = dot(rel, f3(e.u[0], e.u[1], e.u[2])) / e.u_length;
    const float v = dot(rel, f3(e.v[0], e.v[1], e.v[2])) / e.v_length;
    const float uu = tex_wrap(u * (float)m.repeat), vv = tex_wrap(v * (float)m.repeat);
    if (m.bump_off >= 0) {
      bn = bump_tilt(S, m, (int)((m.bump_h - 1) * vv), (int)((m.bump_w - 1) * uu), f3(e.n[0], e.n[1], e.n[2]),
                     f3(e.u[0], e.u[1], e.u[2]), f3(e.v[0], e.v[1], e.v[2]), 1.0f);
      res |= 2;
    }
    if (m.tex_off >= 0) {
      const float4 t = __ldg(S.texels + m.tex_off + (size_t)tex_clamp((int)((m.tex_h - 1) * vv), m.tex_h) * m.tex_w +
                             tex_clamp((int)((m.tex_w - 1) * uu), m.tex_w));
      C = Sp = f3(t.x, t.y, t.z);
    }
    if (has_ibl) {
      const float4 t = __ldg(S.ibl_texels + m.ibl_off +
                             (size_t)tex_clamp((int)((m.ibl_h - 1) * vv), m.ibl_h) * m.ibl_w +
                             tex_clamp((int)((m.ibl_w - 1) * uu), m.ibl_w));
      C = f3(t.x, t.y, t.z);
      E = C * m.ibl_coef;
    }
    return res;
  }
  // sphere / hemisphere: hemisphere_map looks along y (x, y, z -> z, x, y)
  const float r = (float)ed.radius;
  const float3 q = p - f3(e.p[0], e.p[1], e.p[2]);
  const bool hm = (m.map_flags & PR_MAP_HEMISPHERE) != 0;
  const float px = hm ? q.z : q.x, py = hm ? q.x : q.y, pz = hm ? q.y : q.z;
  const float3 vv = f3(px / r, py / r, pz / r);
  if (m.bump_off >= 0 && fabsf(q.z - r) > 1.0e-16f) {  // the bump block tests the unmapped z
    float u, v;
    sphere_uv(m.map_flags, vv, true, false, u, v);
    if (ed.hemisphere) u *= 2.0f;
    const int j = (int)((m.bump_w - 1) * tex_wrap(u * (float)m.repeat));
    const int i = (int)((m.bump_h - 1) * tex_wrap(v * (float)m.repeat));
    const float th = acosf(fminf(1.0f, fmaxf(-1.0f, vv.z)));
    float ph = atan2f(vv.y, vv.x);
    if (ph < 0.0f) ph += 6.28318530717958647692f;
    if (ph >= 6.28318530717958647692f) ph = 0.0f;
    float st, ct, sp, cp;
    sincosf(th, &st, &ct);
    sincosf(ph, &sp, &cp);
    bn = bump_tilt(S, m, i, j, e.normal_inverse < 0 ? -n_hit : n_hit, f3(ct * cp, ct * sp, -st), f3(-st * sp, st * cp, 0.0f),
                   0.1f);
    res |= 2;
  }
  if (!(fabsf(pz - r) > 1.0e-16f)) return res;  // at the pole the reference leaves the material
  if (m.tex_off >= 0) {
    float u, v;
    sphere_uv(m.map_flags, vv, false, false, u, v);
    if (ed.hemisphere) u *= 2.0f;
    int j = (int)((m.tex_w - 1) * tex_wrap(u * (float)m.repeat));
    int i = (int)((m.tex_h - 1) * tex_wrap(v * (float)m.repeat));
    if (hm) {
      j = (int)((float)((m.tex_w - 1) / 2) + (m.tex_w - 1) * 0.5f * px / r);
      i = (int)((float)((m.tex_h - 1) / 2) + (m.tex_h - 1) * 0.5f * py / r);
    }
    const float4 t = __ldg(S.texels + m.tex_off + (size_t)tex_clamp(i, m.tex_h) * m.tex_w + tex_clamp(j, m.tex_w));
    C = Sp = f3(t.x, t.y, t.z);
  }
  if (has_ibl) {
    float u, v;
    sphere_uv(m.map_flags, vv, true, true, u, v);
    if (ed.hemisphere) u *= 2.0f;
    int j = (int)((m.ibl_w - 1) * u);
    int i = (int)((m.ibl_h - 1) * v);
    if (hm) {
      j = (int)((float)((m.ibl_w - 1) / 2) + (m.ibl_w - 1) * 0.5f * px / r);
      i = (int)((float)((m.ibl_h - 1) / 2) + (m.ibl_h - 1) * 0.5f * py / r);
    }
    const float4 t = __ldg(S.ibl_texels + m.ibl_off + (size_t)tex_clamp(i, m.ibl_h) * m.ibl_w + tex_clamp(j, m.ibl_w));
    C = f3(t.x, t.y, t.z);
    E = C * m.ibl_coef;
  }
  return res;
}

// a bump map's scale of a next-event term towards ldir
// (directLight_radiance.h:303-310) and of a scattered weight along dir
// (brdf.h:102-108, :552-557, :740-745); n is the hit's normal
__device__ __forceinline__ float bump_nee(float3 bn, float3 n, float3 ldir) {
  return fmaxf(0.0f, dot(ldir, bn)) / dot(ldir, n);
}
__device__ __forceinline__ float bump_weight(float3 bn, float3 n, float3 dir) {
  return fmaxf(0.1f, dot(dir, bn)) / dot(dir, n);
}

// the Phong (kind 4) or Ward (kind 5) lobe towards ldir as the reference's
// next-event samples evaluate it (directLight_radiance.h:211-256), with the
// specular colour left to the caller; 0 where it gives nothing
__device__ __forceinline__ float glossy_lobe(int kind, const GMaterial& m, float3 refl, float3 in, float3 on, float3 a,
                                             float3 b, float3 ldir) {
  if (kind == 4) {
    const float c = dot(refl, ldir);
    if (c < 0.0f) return 0.0f;
    return (m.phong_n + 2.0f) * 0.15915494309189533577f * powf(c, m.phong_n);
  }
  const float3 h = normalize(in + ldir);
  const float ww0 = dot(h, on) * dot(h, on);
  if (fabsf(ww0) < 1.0e-16f) return 0.0f;
  const float hu = dot(h, a) / m.ward_ax, hv = dot(h, b) / m.ward_ay;
  const float ww2 = 4.0f * 3.14159265358979323846f * m.ward_ax * m.ward_ay * sqrtf(fmaxf(0.0f, dot(ldir, on) * dot(in, on)));
  if (fabsf(ww2) < 1.0e-16f) return 0.0f;
  return expf(-(hu * hu + hv * hv) / ww0) / ww2;
}

// Shades the vertex found by the last closest-hit query of ps (SSS: with the
// subsurface material case compiled in; GLOSSY: with the Ward and Phong
// lobes; EXT: with parallel, spot and infinity lights, textures and IBL
// images; the plain form keeps a leaner instantiation for scenes without
// them).  A tracer
// that builds the vertex itself (the Kerr geodesic tracer) passes it as pre,
// and the colour a miss returns as miss (radiance.h:30-43); straight-ray
// callers leave both null.  ovr (colour, emission) replaces the material's
// where the entity rewrote its hit point's copy (the accretion disk).
template <bool SSS = false, bool GLOSSY = true, bool EXT = false, class R = Rng>
__device__ inline int shade(const DevScene& S, const RenderCfg& cfg, PathState& ps, bool hit, const FastHit& h,
                     uint64_t sample_id, ShadowReq* sh, int& nsh, PathState& child, uint32_t* err,
                     const Vertex* pre = nullptr, const float3* miss = nullptr, EmissionTap* tap = nullptr,
                     SssFrameOut* frame = nullptr, const float3* ovr = nullptr) {
  nsh = 0;
  const bool nee = cfg.nee != 0;
  const bool media = cfg.media != 0 && S.medium.on != 0;
  if (ps.dp) {  // light along a specular / refraction direction (directLight_radiance.h:516-556)
    if (EXT) {
      int lm;
      const float fl = perfect_direct<EXT>(S, ps.o, ps.d, hit, h, lm);
      if (lm >= 0 && fl > 0.0f) {
        // the medium attenuates a light entity's term over the hit distance (:549-552)
        const float3 w = ps.dpw * ((hit && media) ? medium_tr(S.medium, h.t) : f3(1, 1, 1)) * fl;
        ps.L += w * ld3(S.mats[lm].emission);
        if (tap) tap->em(lm, w);
      }
    } else if (hit && S.entf[h.ent].is_light) {
      float3 em = ld3(S.mats[S.entf[h.ent].material].emission);
      const float3 tr = media ? medium_tr(S.medium, h.t) : f3(1, 1, 1);
      ps.L += ps.dpw * (em * tr);
      if (tap) tap->em(S.entf[h.ent].material, ps.dpw * tr);
    }
    ps.dp = 0;
  }
  if (!hit) {
    ps.L += ps.beta * (miss ? *miss : f3(S.bg[0], S.bg[1], S.bg[2]));
    return SHADE_END;
  }
  if (ps.depth >= cfg.max_vertices) {
    atomicOr(err, PR_DEV_LOOP_CAP);
    return SHADE_END;
  }
  R rng;
  rng_at(rng, cfg.seed, sample_id, ps.branch, ps.draws);
  Vertex v;
  if (pre) v = *pre;
  else make_vertex(S, ps.o, ps.d, h, v);
  if (EXT && !pre && S.fmat && S.entf[v.ent].type == PR_ENT_POLYGON) {
    // the face's OBJ material (usemtl) selects a derived material
    const int fm = S.fmat[S.entf[v.ent].face_base + __float_as_int(__ldg(S.rtris + 3 * (size_t)h.slot).w)];
    if (fm >= 0) v.mat = fm;
  }
  const GMaterial& m = S.mats[v.mat];
  const GEntF& ent = S.entf[v.ent];
  float3 E = ovr ? ovr[1] : ld3(m.emission), C = ovr ? ovr[0] : ld3(m.color);
  float3 Sp = ld3(m.specular);
  float3 bn = f3(0, 0, 0);  // bump-tilted normal
  bool bumped = false;
  if (EXT && !pre && ent.type == PR_ENT_POLYGON) {
    const int mf = S.ents[v.ent].mesh_flags;
    if (mf && mesh_hit(S, m, ent, mf, h, v, C, E, Sp)) {
      ps.L += ps.beta * E;  // an IBL image on the mesh (radiance.h:45-50)
      if (tap) tap->em(v.mat, ps.beta);
      return SHADE_END;
    }
  } else if (EXT && (m.tex_off >= 0 || m.ibl_off >= 0 || m.bump_off >= 0)) {
    const int tx = hit_texture(S, m, ent, S.ents[v.ent], v.p, v.n, C, E, Sp, bn);
    if (tx & 1) {
      // an object with an IBL image gives its hit point's emission and
      // nothing else (radiance.h:45-50)
      ps.L += ps.beta * E;
      if (tap) tap->em(v.mat, ps.beta);
      return SHADE_END;
    }
    bumped = (tx & 2) != 0;
  }
  const float3 d = ps.d;
  const float3 on = dot(v.n, d) < 0.0f ? v.n : -v.n;
  // RR weight: emission + the reflectances the type can scatter with (radiance.h:79-89)
  float p_rr = maxc(m.type == PR_MAT_WARD ? E + C + Sp : m.type == PR_MAT_PHONG ? E + Sp : E + C);
  if (ps.depth > cfg.depth_limit) p_rr *= exp2f((float)(cfg.depth_limit - ps.depth));
  const float3 trr = media ? medium_tr(S.medium, v.t) : f3(1, 1, 1);
  int result = SHADE_CONTINUE;
  if (ps.depth > cfg.depth) {
    if (rng.next() >= p_rr) {
      ps.L += ps.beta * trr * E;
      if (tap) tap->em(v.mat, ps.beta * trr);
      ps.draws = rng_draws(rng);
      return SHADE_END;
    }
  } else {
    p_rr = 1.0f;
  }
  const bool entering = dot(on, v.n) > 0.0f;  // Entity::isInsideDir (entity.h:98-114)
  float p_scat = 0.0f;
  if (media && entering) {
    p_scat = fminf(fmaxf(1.0f - expf(-S.medium.sigma_s_mean * v.t), 0.01f), 0.99f);
    if (rng.next() < p_scat) {
      // ---- scattering in the medium before the surface (ParticipatingMedia.h:300-461)
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
      const float3 npos = ps.o + d * ds;
      const float3 tr = medium_tr(md, ds);
      // phase / dirPdf == 1 in the reference's weight
      const float3 f = tr * f3(md.sigma_s[0], md.sigma_s[1], md.sigma_s[2]) * (phase / pdf / phase / p_scat / p_rr);
      if (!ent.is_light && S.n_lights > 0) {
        // NEE from the medium point (eval_direct_radiance_media, ParticipatingMedia.h:27-268):
        // emission / pi for area lights, emission for the other kinds
        for (int i = 0; i < 3; i++) {
          const GLight& L = pick_light(S, rng);
          if (EXT && L.kind != PR_LIGHT_AREA) {
            LightSample ls;
            if (point_light_sample(S, L, npos, f3(0, 0, 0), npos, false, true, rng, ls))
              push_shadow(S, ls, ps.beta * f * ls.k * (1.0f / 3.0f), L.mat, sh, nsh);
            continue;
          }
          const GEntF& le = S.entf[L.ent];
          const float3 lp = sample_light(le, rng, false);
          const float3 ln = light_normal(le, lp, false);
          const float3 dl = lp - npos;
          const float dist2 = dot(dl, dl);
          const float dist = sqrtf(dist2);
          const float3 ldir = dl / dist;
          const float dot1 = -dot(ln, ldir);
          if (dot1 >= 0.0f) {
            const float G = dot1 / dist2;
            const float3 em = ld3(S.mats[le.material].emission);
            sh[nsh].o = npos;
            sh[nsh].d = ldir;
            sh[nsh].tmax = dist - 1.0e-3f;
            sh[nsh].ew = ps.beta * f * medium_tr(md, dist) * (0.31830988618379067154f * G * le.area * (1.0f / 3.0f));
            sh[nsh].contrib = sh[nsh].ew * em;
            sh[nsh].lmat = le.material;
            nsh++;
          }
        }
      }
      ps.draws = rng_draws(rng);
      if (!(pdf > 0.0f)) { nsh = 0; return SHADE_END; }
      if (ent.is_light) {
        if (ps.depth == 0) {
          ps.L += ps.beta * tr * E;
          if (tap) tap->em(v.mat, ps.beta * tr);
        }
        return SHADE_END;
      }
      ps.beta = ps.beta * f;
      ps.o = npos;
      ps.d = nd;
      ps.depth++;
      return SHADE_CONTINUE;
    }
  }
  const float inv_rr = 1.0f / p_rr / (1.0f - p_scat);
  int kind;  // 0 diffuse, 1 specular, 2 glass, 3 subsurface (directional dipole), 4 Phong, 5 Ward
  if (SSS && m.sss) kind = 3;
  else if (m.type == PR_MAT_DIFFUSE) kind = (rng.next() < m.roughness) ? 0 : 1;
  else if (m.type == PR_MAT_SPECULAR) kind = (rng.next() < 1.0f - m.roughness) ? 1 : 0;
  else if (GLOSSY && m.type == PR_MAT_PHONG) kind = (rng.next() < m.roughness) ? 0 : 4;  // radiance.h:470-484
  else if (GLOSSY && m.type == PR_MAT_WARD) {  // radiance.h:493-509: diffuse with probability rd / (rd + rs)
    const float rd = (C.x + C.y + C.z) * (1.0f / 3.0f), rs = (Sp.x + Sp.y + Sp.z) * (1.0f / 3.0f);
    kind = (rng.next() < rd / (rs + rd)) ? 0 : 5;
  } else kind = 2;
  const float3 tri = (media && entering) ? trr : f3(1, 1, 1);
  const float3 env = f3(S.env[0], S.env[1], S.env[2]);
  if (kind == 0) {
    // ---- BRDF_Diffuse (brdf.h:408-700)
    if (ent.is_light) {
      if (!(ent.type == PR_ENT_UVPLANE && dot(v.n, d) >= 0.0f) && (!nee || ps.depth == 0)) {
        ps.L += ps.beta * trr * E * inv_rr;
        if (tap) tap->em(v.mat, ps.beta * trr * inv_rr);
      }
      ps.draws = rng_draws(rng);
      return SHADE_END;
    }
    float3 u, w2;
    onb(on, u, w2);
    const float r1 = 6.28318530717958647692f * rng.next();
    const float r2 = rng.next();
    const float r2s = sqrtf(r2);
    float sn, cs;
    sincosf(r1, &sn, &cs);
    const float3 nd = normalize(u * (cs * r2s) + w2 * (sn * r2s) + on * sqrtf(1.0f - r2));
    const float3 origin = offset_ray(v.p, on);
    if (S.n_lights > 0) {
      if (nee || EXT) {
        // eval_direct_radiance (directLight_radiance.h:19-313), 3 samples
        // averaged; without NEE only parallel, spot and infinity lights
        // (brdf.h:590-605), which take the colour, not colour / pi
        const float3 w = ps.beta * tri * C * (inv_rr * 0.31830988618379067154f * (1.0f / 3.0f));
        for (int i = 0; i < 3; i++) {
          const GLight& L = pick_light(S, rng);
          if (EXT && L.kind != PR_LIGHT_AREA) {
            LightSample ls;
            if (point_light_sample(S, L, v.p, on, origin, true, media, rng, ls))
              push_shadow(S, ls, w * ls.k * (3.14159265358979323846f * (bumped ? bump_nee(bn, v.n, ls.ldir) : 1.0f)),
                          L.mat, sh, nsh);
            continue;
          }
          if (!nee) continue;
          const GEntF& le = S.entf[L.ent];
          const float3 lp = sample_light(le, rng, true);
          const float3 ln = light_normal(le, lp, true);
          const float3 dl = lp - v.p;
          const float dist2 = dot(dl, dl);
          const float dist = sqrtf(dist2);
          const float3 ldir = dl / dist;
          const float dot0 = dot(on, ldir), dot1 = -dot(ln, ldir);
          if (dot0 >= 0.0f && dot1 >= 0.0f) {
            // visible iff nothing is hit closer than the light point - 1e-3
            // (directLight_radiance.h:136-171), measured from the shadow
            // ray's own offset origin
            const float3 dlo = lp - origin;
            const float disto = sqrtf(dot(dlo, dlo));
            float3 em = ld3(S.mats[le.material].emission);
            if (media) em = em * medium_tr(S.medium, dist);
            sh[nsh].o = origin;
            sh[nsh].d = dlo / disto;
            sh[nsh].tmax = disto - 1.0e-3f;
            float3 ew = w * (dot0 * dot1 / dist2 * le.area);
            if (EXT && bumped) ew = ew * bump_nee(bn, v.n, ldir);
            sh[nsh].contrib = ew * em;
            sh[nsh].ew = media ? ew * medium_tr(S.medium, dist) : ew;
            sh[nsh].lmat = le.material;
            nsh++;
          }
        }
      } else {
        for (int i = 0; i < 3; i++) (void)rng.next();  // light picks; only parallel/spot/infinity lights would add
      }
    }
    ps.L += ps.beta * (env + tri * E);
    if (tap) tap->em(v.mat, ps.beta * tri);
    ps.beta = ps.beta * C * tri * inv_rr;
    if (EXT && bumped) ps.beta = ps.beta * bump_weight(bn, v.n, nd);
    ps.o = origin;
    ps.d = nd;
    ps.depth++;
    ps.draws = rng_draws(rng);
    return SHADE_CONTINUE;
  }
  if (GLOSSY && (kind == 4 || kind == 5)) {
    // ---- BRDF_Phong (brdf.h:16-190) / BRDF_Ward (brdf.h:192-319): one
    // direction from the lobe, weighted by the specular colour; a direction
    // below the surface gives the whole vertex zero.  Next-event samples are
    // evaluated with the same lobe (directLight_radiance.h:211-256)
    float3 a, b, nd;
    float ww;
    const float3 in = -d;
    const float3 refl = normalize(d - on * (2.0f * dot(on, d)));
    if (kind == 4) {
      onb(refl, a, b);
      const float ph = 6.28318530717958647692f * rng.next();
      float cost = powf(rng.next(), 1.0f / (m.phong_n + 1.0f));
      cost = fminf(1.0f, fmaxf(-1.0f, cost));
      const float sint = sqrtf(fmaxf(0.0f, 1.0f - cost * cost));
      float sn, cs;
      sincosf(ph, &sn, &cs);
      nd = normalize(a * (cs * sint) + b * (sn * sint) + refl * cost);
      ww = (m.phong_n + 2.0f) / (m.phong_n + 1.0f);
    } else {
      onb(on, a, b);
      const float ax = m.ward_ax, ay = m.ward_ay;
      const float u1 = rng.next(), u2 = rng.next();
      // importance sampling of the half vector (Walter, "Notes on the Ward BRDF", 2005)
      float phi = atanf(ay / ax * tanf(6.28318530717958647692f * u2));
      if (0.25f <= u2 && u2 <= 0.75f) phi += 3.14159265358979323846f;
      else if (0.75f < u2) phi += 6.28318530717958647692f;
      float sp, cp;
      sincosf(phi, &sp, &cp);
      const float theta = atanf(sqrtf(-logf(fmaxf(u1, 1.0e-30f)) / (cp * cp / (ax * ax) + sp * sp / (ay * ay))));
      float st, ct;
      sincosf(theta, &st, &ct);
      const float3 h = normalize(a * (cp * st) + b * (sp * st) + on * ct);
      nd = normalize(h * (2.0f * dot(in, h)) - in);
      const float hn = dot(h, on);
      ww = dot(h, in) * hn * hn * hn * sqrtf(fmaxf(0.0f, dot(nd, on) / dot(in, on)));
    }
    if (dot(on, nd) < 0.0f) {  // the reference returns zero for the vertex
      ps.draws = rng_draws(rng);
      return SHADE_END;
    }
    const float3 origin = offset_ray(v.p, on);
    if (S.n_lights > 0 && (nee || EXT)) {
      // without NEE only parallel, spot and infinity lights (brdf.h:128-146)
      const float3 w = ps.beta * tri * Sp * (inv_rr * (1.0f / 3.0f));
      for (int i = 0; i < 3; i++) {
        const GLight& L = pick_light(S, rng);
        if (EXT && L.kind != PR_LIGHT_AREA) {
          LightSample ls;
          if (!point_light_sample(S, L, v.p, on, origin, true, media, rng, ls)) continue;
          const float f = glossy_lobe(kind, m, refl, in, on, a, b, ls.ldir);
          if (f > 0.0f) push_shadow(S, ls, w * ls.k * (f * (bumped ? bump_nee(bn, v.n, ls.ldir) : 1.0f)), L.mat, sh, nsh);
          continue;
        }
        if (!nee) continue;
        const GEntF& le = S.entf[L.ent];
        const float3 lp = sample_light(le, rng, true);
        const float3 ln = light_normal(le, lp, true);
        const float3 dl = lp - v.p;
        const float dist2 = dot(dl, dl);
        const float dist = sqrtf(dist2);
        const float3 ldir = dl / dist;
        const float dot0 = dot(on, ldir), dot1 = -dot(ln, ldir);
        if (!(dot0 >= 0.0f && dot1 >= 0.0f)) continue;
        float f;  // the lobe's value towards the light (times specular, applied in w)
        if (kind == 4) {
          const float c = dot(refl, ldir);
          if (c < 0.0f) continue;
          f = (m.phong_n + 2.0f) * 0.15915494309189533577f * powf(c, m.phong_n);
        } else {
          const float3 h = normalize(in + ldir);
          const float ww0 = dot(h, on) * dot(h, on);
          if (fabsf(ww0) < 1.0e-16f) continue;
          const float hu = dot(h, a) / m.ward_ax, hv = dot(h, b) / m.ward_ay;
          const float ww2 = 4.0f * 3.14159265358979323846f * m.ward_ax * m.ward_ay * sqrtf(fmaxf(0.0f, dot0 * dot(in, on)));
          if (fabsf(ww2) < 1.0e-16f) continue;
          f = expf(-(hu * hu + hv * hv) / ww0) / ww2;
        }
        if (!(f > 0.0f)) continue;
        const float3 dlo = lp - origin;
        const float disto = sqrtf(dot(dlo, dlo));
        float3 em = ld3(S.mats[le.material].emission);
        if (media) em = em * medium_tr(S.medium, dist);
        sh[nsh].o = origin;
        sh[nsh].d = dlo / disto;
        sh[nsh].tmax = disto - 1.0e-3f;
        float3 ew = w * (f * dot0 * dot1 / dist2 * le.area);
        if (EXT && bumped) ew = ew * bump_nee(bn, v.n, ldir);
        sh[nsh].contrib = ew * em;
        sh[nsh].ew = media ? ew * medium_tr(S.medium, dist) : ew;
        sh[nsh].lmat = le.material;
        nsh++;
      }
    }
    ps.L += ps.beta * (env + tri * E);
    if (tap) tap->em(v.mat, ps.beta * tri);
    ps.beta = ps.beta * Sp * (ww * inv_rr) * tri;
    if (EXT && bumped) ps.beta = ps.beta * bump_weight(bn, v.n, nd);
    ps.o = origin;
    ps.d = nd;
    ps.depth++;
    ps.draws = rng_draws(rng);
    return SHADE_CONTINUE;
  }
  if (kind == 1) {
    // ---- BRDF_Specular (brdf.h:702-761): mirror about the geometric normal
    const float3 nd = normalize(d - v.n * (2.0f * dot(v.n, d)));
    ps.L += ps.beta * (env + tri * E);
    if (tap) tap->em(v.mat, ps.beta * tri);
    ps.beta = ps.beta * C * tri * inv_rr;
    if (EXT && bumped) ps.beta = ps.beta * bump_weight(bn, v.n, nd);  // the mirror ray and its light term
    ps.dp = nee;
    ps.dpw = ps.beta;
    ps.o = offset_ray(v.p, dot(nd, v.n) > 0.0f ? v.n : -v.n);
    ps.d = nd;
    ps.depth++;
    ps.draws = rng_draws(rng);
    return SHADE_CONTINUE;
  }
  float3 dg = d;  // the direction BRDF_Refraction sees (the subsurface branch passes the refracted one)
  if (SSS && kind == 3) {
    // ---- subsurface scattering, level -2 (radiance.h:154-224): refract into
    // the object, then BRDF_SSS2_ (Subsurface_Scattering.h:630-1181) with the
    // refracted direction
    const bool into_s = dot(v.n, on) > 0.0f;
    const float nts = m.ior, nnts = into_s ? 1.0f / nts : nts;
    const float ddns = dot(d, on);
    const float cos2ts = 1.0f - nnts * nnts * (1.0f - ddns * ddns);
    const float3 ts = cos2ts < 0.0f
                          ? normalize(d - on * (2.0f * dot(on, d)))
                          : normalize(d * nnts - v.n * ((into_s ? 1.0f : -1.0f) * (ddns * nnts + sqrtf(fabsf(cos2ts)))));
    const float3 mtr = f3(expf(-m.sss_tr[0] * v.t), expf(-m.sss_tr[1] * v.t), expf(-m.sss_tr[2] * v.t));
    if (!into_s) ps.beta = ps.beta * mtr;  // leaving: attenuated over the segment inside
    // exit point: Gaussian-disk probes along the orienting normal, at most 40 (:729-806)
    float3 tu, tv;
    onb(on, tu, tv);
    const float rmax = ent.sss_rmax, fall = m.sss_falloff;
    const float norm = 1.0f - expf(-fall * rmax * rmax);
    const float step = 0.5f * rmax / 40.0f;
    bool found = false;
    float3 sp = v.p, on2 = on, sw = on;
    float pdf_s = 1.0f, pdf_d = 1.0f;
    int exit_mat = v.mat;
    for (int i = 40; i >= 1 && !found; i--) {
      const float u1 = rng.next(), u2 = rng.next();
      const float r = sqrtf(logf(1.0f - u1 * norm) / -fall);
      float sn, cs;
      sincosf(6.28318530717958647692f * u2, &sn, &cs);
      const float px = r * cs, py = r * sn;
      const float3 po = v.p + tu * px + tv * py - on * ((float)i * step);
      FastHit ph;
      TraceStats pst{0, 0};
      if (!fast_closest(S, po, on, ph, pst, err)) continue;
      Vertex pv;
      make_vertex(S, po, on, ph, pv);
      float3 n2 = pv.n;
      if (dot(v.n, on) < 0.0f) n2 = -n2;
      float3 a2, b2;
      onb(n2, a2, b2);
      const float r1 = 6.28318530717958647692f * rng.next();
      const float r2 = rng.next(), r2s = sqrtf(r2);
      float sn1, cs1;
      sincosf(r1, &sn1, &cs1);
      const float3 dir = normalize(a2 * (cs1 * r2s) + b2 * (sn1 * r2s) + n2 * sqrtf(1.0f - r2));
      const float sd = dot(n2, dir) * 0.31830988618379067154f;
      if (sd > 0.0f) {
        found = true;
        sp = pv.p;
        on2 = n2;
        sw = dir;
        exit_mat = pv.mat;
        pdf_s = fall * expf(-fall * (px * px + py * py)) * 0.31830988618379067154f / norm;
        pdf_d = sd;
      }
    }
    const float cos_wi_n = dot(on2, sw);
    if (!found || cos_wi_n < 0.0f) {  // BRDF_SSS2_ returns zero
      ps.draws = rng_draws(rng);
      return SHADE_END;
    }
    const float3 wi = -ts;
    const float T21 = fmaxf(1.0f - dd_fresnel(dot(wi, on), m.sss_eta), 0.0f);
    const float T12 = fmaxf(1.0f - dd_fresnel(cos_wi_n, m.sss_eta), 0.0f);
    const float accept = into_s ? 0.5f : 0.0f;
    ps.L += ps.beta * (env + tri * E);
    if (rng.next() < accept) {
      if (m.sss_level == -1 && rng.next() >= 0.5f) {
        // ---- single scattering (level -1): radiance_through_media
        // (Subsurface_Scattering.h:31-543) from just inside the entry point
        // along the refracted direction, at most one scattering event.  Its
        // result is bounded twice: |Li| <= 100 inside the walk
        // (OVER_RADIANCE_CUT0) and |weight * Li| <= 100 here (CUT2)
        const float3 b0 = ps.beta * tri;
        const float3 bw1 = b0 * C * (1.0f / (accept * p_rr * (1.0f - p_scat) * 0.5f));
        const int dl30 = cfg.depth_limit * 30;
        const int dw = ps.depth + 1;
        if (frame) {
          frame->open = 2;
          frame->scale = b0;
          frame->thr = 100.0f;
          frame->scale2 = bw1;
          frame->thr2 = 100.0f;
          frame->nee_inner = 1;
          frame->inner = f3(0, 0, 0);
        }
        float rr2a = 1.0f;
        if (dw > dl30) {
          rr2a = exp2f((float)(cfg.depth_limit - dw));
          if (rng.next() >= rr2a) {  // the walk returns the object's emission
            if (frame) {
              frame->open = 1;
              frame->inner = bw1 * E;
            }
            ps.draws = rng_draws(rng);
            return SHADE_END;
          }
        }
        const float3 org0 = v.p - v.n * 1.0e-4f;
        FastHit oh;
        TraceStats wst{0, 0};
        Vertex ov;
        if (!fast_closest(S, org0, ts, oh, wst, err)) {
          if (frame) frame->open = 0;
          ps.draws = rng_draws(rng);
          return SHADE_END;
        }
        if (oh.t < 1.0e-4f) {  // too thin to scatter: leave at once (no CUT0 on this result)
          make_vertex(S, org0, ts, oh, ov);
          if (frame) frame->open = 1;
          sss_exit<EXT>(S, cfg, m, v.ent, oh, ov, ts, rr2a, bw1, ps.depth + 2, rng, sh, nsh, ps);
          ps.draws = rng_draws(rng);
          return SHADE_CONTINUE;
        }
        // a scattering point towards the far side, and a phase-function
        // direction that leaves the object or enters another (145 tries)
        bool ok = false;
        float t = 0.0f, pdf = 1.0f, phase = 1.0f;
        float3 nd = ts;
        FastHit wh;
        const bool hgc = (cfg.flags & PR_FLAG_HG_CORRECT) != 0;
        for (int kk = 0; kk < 145 && !ok; kk++) {
          const float st = m.sss_tr[sss_channel(m, rng.next(), true)];
          const float eb = expf(-st * oh.t);
          t = -logf(1.0f + rng.next() * (eb - 1.0f)) / st;
          pdf = expf(-st * t) * (-st / (eb - 1.0f));
          if (oh.t < t && oh.ent == v.ent) continue;  // beyond the object's far side
          const float3 norg = org0 + ts * t;
          const float g = m.sss_g[sss_channel(m, rng.next(), false)];
          if (g == 0.0f || fabsf(g) > 1.0f) {
            nd = sample_sphere_dir(rng);
            phase = 0.0795774715459476679f;
          } else {
            nd = sample_hg(ts, g, rng, hgc);
            phase = phase_hg(g, dot(ts, nd));
          }
          if (!fast_closest(S, norg, nd, wh, wst, err)) continue;
          make_vertex(S, norg, nd, wh, ov);
          const bool entering = dot(ov.n, nd) < 0.0f;  // Entity::isInsideDir
          ok = (wh.ent == v.ent) ? !entering : entering;
        }
        if (!ok) {
          if (frame) frame->open = 0;
          ps.draws = rng_draws(rng);
          return SHADE_END;
        }
        const float dir_pdf = phase;
        const float3 bw2 = bw1 * f3(expf(-m.sss_tr[0] * t) * m.sss_ss[0], expf(-m.sss_tr[1] * t) * m.sss_ss[1],
                                    expf(-m.sss_tr[2] * t) * m.sss_ss[2]) *
                           (phase / pdf / dir_pdf / rr2a);
        // scattering depth 1 = sc_max: leave along nd
        float rr2b = 1.0f;
        if (dw + 1 > dl30) {
          rr2b = fminf(exp2f((float)(cfg.depth_limit - dw - 1)), 0.5f);
          if (rng.next() >= rr2b) {
            if (frame) frame->inner = bw2 * E;
            ps.draws = rng_draws(rng);
            return SHADE_END;
          }
        }
        sss_exit<EXT>(S, cfg, m, v.ent, wh, ov, nd, rr2b, bw2, ps.depth + 3, rng, sh, nsh, ps);
        ps.draws = rng_draws(rng);
        return SHADE_CONTINUE;
      }
      // multiple scattering through the dipole, exit at sp towards sw (level
      // -1 takes it with probability 1/2: the continuation is weighted by 2,
      // the next-event terms at the exit point are not)
      const float pms = m.sss_level == -1 ? 0.5f : 1.0f;
      const float3 res = f3(dd_bssrdf(m, sp, on2, sw, v.p, on, 0), dd_bssrdf(m, sp, on2, sw, v.p, on, 1),
                            dd_bssrdf(m, sp, on2, sw, v.p, on, 2));
      const float k = T12 * cos_wi_n * T21 / pdf_s / pdf_d / accept / p_rr / (1.0f - p_scat);
      const float3 origin_s = offset_ray(sp, on2);
      if (S.n_lights > 0 && (nee || EXT)) {
        // direct_radiance_sample, 3 samples averaged: with NEE at the exit
        // point (the exit object's colour / pi); without it only parallel,
        // spot and infinity lights, at the ENTRY point with its own colour
        // (Subsurface_Scattering.h:961-1010)
        const float3 wn = ps.beta * tri * res * (k * (1.0f / 3.0f)) * ld3(S.mats[exit_mat].color) *
                          0.31830988618379067154f;
        for (int i = 0; i < 3; i++) {
          const GLight& L = pick_light(S, rng);
          if (EXT && L.kind != PR_LIGHT_AREA) {
            const float3 rp = nee ? sp : v.p, rn = nee ? on2 : on;
            const float3 ro = nee ? origin_s : offset_ray(v.p, on);
            const float3 wp = ps.beta * tri * res * (k * (1.0f / 3.0f)) * ld3(S.mats[nee ? exit_mat : v.mat].color);
            LightSample ls;
            if (point_light_sample(S, L, rp, rn, ro, true, media, rng, ls)) push_shadow(S, ls, wp * ls.k, L.mat, sh, nsh);
            continue;
          }
          if (!nee) continue;
          const GEntF& le = S.entf[L.ent];
          const float3 lp = sample_light(le, rng, true);
          const float3 ln = light_normal(le, lp, true);
          const float3 dl = lp - sp;
          const float dist2 = dot(dl, dl);
          const float3 ldir = dl / sqrtf(dist2);
          const float dot0 = dot(on2, ldir), dot1 = -dot(ln, ldir);
          if (dot0 >= 0.0f && dot1 >= 0.0f) {
            const float3 dlo = lp - origin_s;
            const float disto = sqrtf(dot(dlo, dlo));
            const float3 em = ld3(S.mats[le.material].emission);
            float3 ew = wn * (dot0 * dot1 / dist2 * le.area);
            if (media) ew = ew * medium_tr(S.medium, sqrtf(dist2));
            sh[nsh].o = origin_s;
            sh[nsh].d = dlo / disto;
            sh[nsh].tmax = disto - 1.0e-3f;
            sh[nsh].contrib = ew * em;
            sh[nsh].ew = ew;
            sh[nsh].lmat = le.material;
            nsh++;
          }
        }
      }
      if (frame) {
        frame->open = 1;
        frame->scale = ps.beta * tri;
        frame->thr = 100.0f;  // OVER_RADIANCE_CUT2
        frame->nee_inner = 0;
        frame->inner = f3(0, 0, 0);
      }
      ps.beta = ps.beta * tri * C * res * (k / pms);
      ps.o = origin_s;
      ps.d = sw;
      ps.depth++;
      ps.draws = rng_draws(rng);
      return SHADE_CONTINUE;
    }
    // Fresnel-surface refraction at the same point along the refracted
    // direction (:1080-1160): BRDF_Refraction weighted Tr / (1 - accept)
    if (frame) {
      frame->open = 1;
      frame->scale = ps.beta * tri;
      frame->thr = 200.0f;  // OVER_RADIANCE_CUT3
      frame->nee_inner = 0;
      frame->inner = f3(0, 0, 0);
    }
    ps.beta = ps.beta * tri * (into_s ? f3(1, 1, 1) : mtr) * (1.0f / (1.0f - accept));
    dg = ts;
  }
  // ---- BRDF_Refraction (brdf.h:763-953)
  const float3 refl = normalize(dg - v.n * (2.0f * dot(v.n, dg)));
  const bool into = dot(v.n, on) > 0.0f;
  const float nt = m.ior;
  const float nnt = into ? 1.0f / nt : nt;
  const float ddn = dot(dg, on);
  const float cos2t = 1.0f - nnt * nnt * (1.0f - ddn * ddn);
  ps.L += ps.beta * (env + tri * E);
  if (tap) tap->em(v.mat, ps.beta * tri);
  const float3 base = ps.beta * C * tri;
  const float3 refl_o = offset_ray(v.p, dot(refl, v.n) > 0.0f ? v.n : -v.n);
  if (cos2t < 0.0f) {  // total internal reflection
    ps.beta = base * inv_rr;
    ps.dp = nee;
    ps.dpw = ps.beta;
    ps.o = refl_o;
    ps.d = refl;
    ps.depth++;
    ps.draws = rng_draws(rng);
    return SHADE_CONTINUE;
  }
  const float3 tdir = normalize(dg * nnt - v.n * ((into ? 1.0f : -1.0f) * (ddn * nnt + sqrtf(fabsf(cos2t)))));
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
  if (ps.depth > 2) {
    if (rng.next() < P) {
      const float3 W = base * (1.0f / (P * p_rr) / (1.0f - p_scat));
      ps.beta = W * Re;
      ps.dpw = W;
      ps.o = refl_o;
      ps.d = refl;
    } else {
      const float3 W = base * (1.0f / ((1.0f - P) * p_rr) / (1.0f - p_scat));
      ps.beta = W * Tr;
      ps.dpw = W;
      ps.o = tdir_o;
      ps.d = tdir;
    }
    ps.dp = nee;
    ps.depth++;
    ps.draws = rng_draws(rng);
    return SHADE_CONTINUE;
  }
  // depth <= 2: both branches; the refracted one is handed back
  const float3 W = base * inv_rr;
  child.o = tdir_o;
  child.d = tdir;
  child.beta = W * Tr;
  child.dpw = W;
  child.L = f3(0, 0, 0);
  child.depth = ps.depth + 1;
  child.branch = 2 * ps.branch + 1;
  child.draws = 0;
  child.dp = nee;
  ps.beta = W * Re;
  ps.dp = nee;
  ps.dpw = W;
  ps.o = refl_o;
  ps.d = refl;
  ps.depth++;
  ps.branch = 2 * ps.branch + 2;
  ps.draws = 0;
  result = SHADE_SPLIT;
  return result;
}

// per-sample value after the weight 1/spp and the luminance clamp (render.h:1353, :1375-1384)
__device__ __forceinline__ float3 finish_sample(const RenderCfg& cfg, float3 L, uint32_t* err) {
  float3 v = L * cfg.smp;
  if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z))) {
    atomicOr(err, PR_DEV_NONFINITE);
    v = f3(0, 0, 0);
  }
  if (cfg.cutoff > 0.0f) {
    const float lum = 0.2126f * v.x + 0.7152f * v.y + 0.0722f * v.z;
    if (lum > cfg.cutoff) v = v * (cfg.cutoff / lum);
  }
  return v;
}

}  // namespace pr
