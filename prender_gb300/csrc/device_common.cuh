// Device-side math, counter-based random streams and ray/primitive tests.
//
// Two families of intersection code share the uploaded scene:
//   * exact_*: FP64 in the reference's operation order with every multiply
//     and add rounded separately (no FMA contraction), so closest hits and
//     distances equal the reference's bit for bit (scene.cpp:83-214,
//     QBVH.cpp:17-159, polygon.h:78-173, sphere.h:68-96, plane.h:86-239).
//     The QBVH boxes are FP32 as in the reference; triangle tests are
//     filtered in FP32 with a conservative error margin and only the
//     candidates are re-tested in FP64.
//   * fast_*: FP32 traversal for rendering: near-first child order, culling
//     against the current closest hit, any-hit shadow queries, and ray
//     origins moved off the surface by a few float ulps along the normal.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pr_internal.h"

namespace pr {

// ------------------------------------------------------------------ float3
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
__device__ __forceinline__ float3& operator*=(float3& a, float3 b) { a = a * b; return a; }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 normalize(float3 a) { return a * rsqrtf(dot(a, a)); }
__device__ __forceinline__ float maxc(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
__device__ __forceinline__ float3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }

// ----------------------------------------------------- exact FP64 helpers
struct dv3 {
  double x, y, z;
};
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ dv3 dsub3(dv3 a, dv3 b) { return {ds(a.x, b.x), ds(a.y, b.y), ds(a.z, b.z)}; }
__device__ __forceinline__ dv3 dadd3(dv3 a, dv3 b) { return {da(a.x, b.x), da(a.y, b.y), da(a.z, b.z)}; }
__device__ __forceinline__ dv3 dscale3(dv3 a, double s) { return {dm(a.x, s), dm(a.y, s), dm(a.z, s)}; }
// vector3d.h dot(): SSE lanes (x,y)+(z,0) then horizontal add = (xx+zz)+yy
__device__ __forceinline__ double ddot(dv3 a, dv3 b) { return da(da(dm(a.x, b.x), dm(a.z, b.z)), dm(a.y, b.y)); }
__device__ __forceinline__ dv3 dcross(dv3 a, dv3 b) {
  return {ds(dm(a.y, b.z), dm(a.z, b.y)), ds(dm(a.z, b.x), dm(a.x, b.z)), ds(dm(a.x, b.y), dm(a.y, b.x))};
}
__device__ __forceinline__ dv3 ldd3(const double* p) { return {p[0], p[1], p[2]}; }

constexpr double kEps = 1.0e-6;     // PS_EPS (constant.h:36)
constexpr double kInfD = 1.0e128;   // PS_INF (constant.h:33)

// ----------------------------------------------------------- Philox4x32-10
// Counter-based generator of Salmon et al., "Parallel random numbers: as
// easy as 1, 2, 3" (SC 2011).  Counter = (sample lo, sample hi, block,
// branch), key = seed.  Every path and every glass branch owns a stream,
// so sample k of any pixel can be regenerated (resume, replay, sharding).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

struct Rng {
  uint4 ctr;
  uint2 key;
  uint4 buf;
  int idx;
  __device__ void init(uint64_t seed, uint64_t sample, uint32_t branch) {
    key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    ctr = make_uint4((uint32_t)sample, (uint32_t)(sample >> 32), 0u, branch);
    idx = 4;
  }
  // uniform in [0, 1) with 24 random bits
  __device__ __forceinline__ float next() {
    if (idx == 4) {
      buf = philox4x32_10(ctr, key);
      ctr.z++;
      idx = 0;
    }
    const uint32_t v = (idx == 0) ? buf.x : (idx == 1) ? buf.y : (idx == 2) ? buf.z : buf.w;
    idx++;
    return (float)(v >> 8) * (1.0f / 16777216.0f);
  }
};

// -------------------------------------------------------------- ray offset
// Moves a surface point off the surface along n by a few float ulps (scaled
// integer offset), or by an absolute amount near the origin; after
// Waechter & Binder, "A Fast and Robust Method for Avoiding
// Self-Intersection", Ray Tracing Gems (2019), ch. 6.
__device__ __forceinline__ float3 offset_ray(float3 p, float3 n) {
  const float kOrigin = 1.0f / 32.0f, kFloatScale = 1.0f / 65536.0f, kIntScale = 256.0f;
  const int ox = (int)(kIntScale * n.x), oy = (int)(kIntScale * n.y), oz = (int)(kIntScale * n.z);
  const float px = __int_as_float(__float_as_int(p.x) + (p.x < 0 ? -ox : ox));
  const float py = __int_as_float(__float_as_int(p.y) + (p.y < 0 ? -oy : oy));
  const float pz = __int_as_float(__float_as_int(p.z) + (p.z < 0 ? -oz : oz));
  return f3(fabsf(p.x) < kOrigin ? p.x + kFloatScale * n.x : px, fabsf(p.y) < kOrigin ? p.y + kFloatScale * n.y : py,
            fabsf(p.z) < kOrigin ? p.z + kFloatScale * n.z : pz);
}

// ---------------------------------------------------------- exact (FP64)
// Sphere::intersect (sphere.h:68-96)
__device__ __forceinline__ bool exact_sphere(const GEntity& e, dv3 o, dv3 d, double& t) {
  const dv3 p_o = dsub3(ldd3(e.p), o);
  const double b = ddot(p_o, d);
  const double D4 = da(ds(dm(b, b), ddot(p_o, p_o)), dm(e.radius, e.radius));
  if (D4 < 0.0) return false;
  const double s = __dsqrt_rn(D4);
  const double t1 = ds(b, s), t2 = da(b, s);
  if (t1 < kEps && t2 < kEps) return false;
  t = (t1 > kEps) ? t1 : t2;
  // a hemisphere keeps the hit only on its y >= y_centre half (sphere.h:98-103)
  if (e.hemisphere && ds(da(o.y, dm(t, d.y)), e.p[1]) < 0.0) return false;
  return true;
}

// UVPlane::intersect over Plane::intersect (plane.h:86-110, :220-239)
__device__ __forceinline__ bool exact_uvplane(const GEntity& e, dv3 o, dv3 d, double& t) {
  dv3 n2 = ldd3(e.normal);
  if (e.normal_inverse < 0) n2 = {dm(n2.x, -1.0), dm(n2.y, -1.0), dm(n2.z, -1.0)};
  const double dd = ddot(d, n2);
  if (fabs(dd) < 1.0e-14) return false;
  const double tt = __ddiv_rn(ddot(dsub3(ldd3(e.p), o), n2), dd);
  const dv3 pos = {da(dm(d.x, tt), o.x), da(dm(d.y, tt), o.y), da(dm(d.z, tt), o.z)};
  if (tt < kEps) return false;
  const dv3 rel = dsub3(pos, ldd3(e.p));
  const double u = __ddiv_rn(ddot(rel, ldd3(e.u_axis)), e.u_length);
  const double v = __ddiv_rn(ddot(rel, ldd3(e.v_axis)), e.v_length);
  if (u < 0 || u > e.u_length) return false;
  if (v < 0 || v > e.v_length) return false;
  t = tt;
  return true;
}

// Circle::intersect (circle.h:177-200): the base UVPlane's plane test with
// no extent (its normal never inverted), then the annulus r_in <= |p - o| <= r
__device__ __forceinline__ bool exact_circle(const GEntity& e, dv3 o, dv3 d, double& t) {
  const dv3 n2 = ldd3(e.normal);
  const double dd = ddot(d, n2);
  if (fabs(dd) < 1.0e-14) return false;
  const double tt = __ddiv_rn(ddot(dsub3(ldd3(e.p), o), n2), dd);
  const dv3 pos = {da(dm(d.x, tt), o.x), da(dm(d.y, tt), o.y), da(dm(d.z, tt), o.z)};
  if (tt < kEps) return false;
  const dv3 rel = dsub3(pos, ldd3(e.p));
  const double r2 = ddot(rel, rel);
  if (r2 > dm(e.radius, e.radius)) return false;
  if (r2 < dm(e.radius_inner, e.radius_inner)) return false;
  t = tt;
  return true;
}

// Triangle::CheckIntersection2 + Triangle::intersect's t > PS_EPS (polygon.h:78-173)
__device__ __forceinline__ bool exact_triangle(float4 a, float4 b, float4 c, dv3 o, dv3 d, double& t) {
  const dv3 v0 = {a.x, a.y, a.z};
  const dv3 e1 = dsub3({b.x, b.y, b.z}, v0);
  const dv3 e2 = dsub3({c.x, c.y, c.z}, v0);
  const dv3 p = dcross(d, e2);
  const double det = ddot(e1, p);
  const dv3 tv = dsub3(o, v0);
  const dv3 q = dcross(tv, e1);
  const double eps = dm(kEps, 0.1);
  double inv_det, u, v;
  if (det > eps) {
    inv_det = __ddiv_rn(1.0, det);
    u = ddot(tv, p);
    if (u < 0.0 || u > det) return false;
    v = ddot(d, q);
    if (v < 0.0 || da(u, v) > det) return false;
  } else if (det < -eps) {
    inv_det = __ddiv_rn(1.0, det);
    u = ddot(tv, p);
    if (u > 0.0 || u < det) return false;
    v = ddot(d, q);
    if (v > 0.0 || da(u, v) < det) return false;
  } else {
    return false;
  }
  const double tt = dm(ddot(e2, q), inv_det);
  if (!(tt > kEps)) return false;
  t = tt;
  return true;
}

// FP32 pre-test for exact_triangle: false only when the FP64 test is
// certain to reject (|error| <= 16 eps_f32 times the magnitude of each
// dot product's terms, origin rounding included).
__device__ __forceinline__ bool maybe_triangle(float4 a, float4 b, float4 c, float3 of, float3 oabs, float3 d) {
  const float3 v0 = f3(a.x, a.y, a.z);
  const float3 e1 = f3(b.x, b.y, b.z) - v0, e2 = f3(c.x, c.y, c.z) - v0;
  const float3 p = cross(d, e2);
  const float det = dot(e1, p);
  const float3 tv = of - v0;
  const float3 q = cross(tv, e1);
  const float u = dot(tv, p), v = dot(d, q);
  const float3 ad = f3(fabsf(d.x), fabsf(d.y), fabsf(d.z));
  const float3 ae1 = f3(fabsf(e1.x), fabsf(e1.y), fabsf(e1.z)), ae2 = f3(fabsf(e2.x), fabsf(e2.y), fabsf(e2.z));
  const float3 at = oabs + f3(fabsf(v0.x), fabsf(v0.y), fabsf(v0.z));
  const float3 pa = f3(ad.y * ae2.z + ad.z * ae2.y, ad.z * ae2.x + ad.x * ae2.z, ad.x * ae2.y + ad.y * ae2.x);
  const float3 qa = f3(at.y * ae1.z + at.z * ae1.y, at.z * ae1.x + at.x * ae1.z, at.x * ae1.y + at.y * ae1.x);
  const float k = 16.0f * 5.9604645e-8f;
  const float mdet = k * dot(ae1, pa), mu = k * dot(at, pa), mv = k * dot(ad, qa);
  if (fabsf(det) <= 1.0e-7f + mdet) return true;
  if (det > 0.0f) {
    if (u < -mu || u > det + mu + mdet) return false;
    if (v < -mv || u + v > det + mu + mv + mdet) return false;
  } else {
    if (u > mu || u < det - mu - mdet) return false;
    if (v > mv || u + v < det - mu - mv - mdet) return false;
  }
  return true;
}

// CheckIntersection4floatAABB (BoundingBox.h:137-178) with SSE max/min
// semantics: the second operand wins unless the comparison holds.
__device__ __forceinline__ float sse_max(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float sse_min(float a, float b) { return a < b ? a : b; }

struct ExactRay {
  dv3 o, d;
  float ro[3], rid[3];
  int sign[3];
  float3 of, oabs, df;
};

__device__ __forceinline__ ExactRay make_exact_ray(dv3 o, dv3 d) {
  ExactRay r;
  r.o = o;
  r.d = d;
  const double dd[3] = {d.x, d.y, d.z}, oo[3] = {o.x, o.y, o.z};
  for (int a = 0; a < 3; a++) {
    r.sign[a] = dd[a] >= 0 ? 0 : 1;
    r.ro[a] = __double2float_rn(oo[a]);
    // (float)(1.0f / dir) with the division in double (QBVH.cpp:44-49)
    r.rid[a] = dd[a] == 0 ? __int_as_float(0x7f800000) : __double2float_rn(__ddiv_rn(1.0, dd[a]));
  }
  r.of = f3(r.ro[0], r.ro[1], r.ro[2]);
  r.oabs = f3(fabsf(r.ro[0]), fabsf(r.ro[1]), fabsf(r.ro[2]));
  r.df = f3(__double2float_rn(d.x), __double2float_rn(d.y), __double2float_rn(d.z));
  return r;
}

// QBVH::CheckIntersection (QBVH.cpp:17-137): LIFO stack, children pushed in
// the reference's axis order, no distance culling, strict '<' everywhere,
// so ties resolve exactly as in the reference.  Returns false and sets
// *err on stack overflow or a bad index.
__device__ inline bool exact_qbvh(const DevScene& S, const GEntity& e, const ExactRay& r, double& best_t, int& best_face,
                           uint32_t* err, uint64_t& nodes_visited, uint64_t& tri_tests) {
  int32_t stack[kStackSize];
  int sp = 0;
  stack[sp++] = e.node_base;
  double dist = -1.0;
  int face = -1;
  int guard = 0;
  while (sp > 0) {
    if (++guard > (1 << 24)) { atomicOr(err, PR_DEV_LOOP_CAP); break; }
    const int32_t ni = stack[--sp];
    const GNode& nd = S.nodes[ni];
    nodes_visited++;
    const float* bx[2][3] = {{nd.bmin_x, nd.bmin_y, nd.bmin_z}, {nd.bmax_x, nd.bmax_y, nd.bmax_z}};
    bool res[4];
    bool any = false;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      float tmin = 0.0f, tmax = 3.402823466e+38f;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        tmin = sse_max(tmin, __fmul_rn(__fsub_rn(bx[r.sign[a]][a][c], r.ro[a]), r.rid[a]));
        tmax = sse_min(tmax, __fmul_rn(__fsub_rn(bx[1 - r.sign[a]][a][c], r.ro[a]), r.rid[a]));
      }
      res[c] = tmax >= tmin;
      any |= res[c];
    }
    if (!any) continue;
    const int at = nd.axes & 3, al = (nd.axes >> 2) & 3, ar = (nd.axes >> 4) & 3;
    int order[4];
    const int lf = (r.sign[at] == 0) ? 0 : 2, rf = (lf + 2) & 3;
    if (r.sign[al] == 0) { order[lf] = 0; order[lf + 1] = 1; } else { order[lf] = 1; order[lf + 1] = 0; }
    if (r.sign[ar] == 0) { order[rf] = 2; order[rf + 1] = 3; } else { order[rf] = 3; order[rf + 1] = 2; }
    for (int i = 0; i < 4; i++) {
      const int c = order[i];
      const int32_t ch = nd.child[c];
      if (!res[c] || ch == kChildInvalid) continue;
      if (ch < 0) {
        const int32_t first = (int32_t)((uint32_t)ch & ~kLeafBit);
        const int cnt = nd.count[c];
        double nearest = -1.0;
        int nface = -1;
        for (int k = 0; k < cnt; k++) {
          const float4* T = S.tris + 3 * (size_t)(first + k);
          const float4 A = T[0], B = T[1], C = T[2];
          tri_tests++;
          if (!maybe_triangle(A, B, C, r.of, r.oabs, r.df)) continue;
          double tt;
          if (exact_triangle(A, B, C, r.o, r.d, tt) && tt > 0 && (nearest < 0 || tt < nearest)) {
            nearest = tt;
            nface = __float_as_int(A.w);
          }
        }
        if (nface >= 0 && nearest > kEps) {
          if (dist < 0 || dist > nearest) {
            dist = nearest;
            face = nface;
          }
        }
      } else {
        if (sp >= kStackSize) { atomicOr(err, PR_DEV_STACK_OVERFLOW); return false; }
        stack[sp++] = ch;
      }
    }
  }
  if (dist > 0) {
    best_t = dist;
    best_face = face;
    return true;
  }
  return false;
}

// The default hit-shading hook of exact_closest: no entity rewrites its hit.
struct NoHitShading {
  __device__ __forceinline__ void begin() {}
  __device__ __forceinline__ bool circle(const GEntity&, dv3) { return true; }
  __device__ __forceinline__ void best(const GEntity&) {}
};

// intersect_scene_ (scene.cpp:83-173): push the origin 1e-6 along the
// direction, loop over entities, keep the strictly closest.  hs sees every
// disk hit (at its hit point) before it competes for the closest, as
// Circle::intersect's own texture branch does (circle.h:177-335), and is told
// which entity ends up closest.
template <class HS>
__device__ inline bool exact_closest_hs(const DevScene& S, dv3 org, dv3 dir, double& t_out, int& ent_out,
                                        int& prim_out, uint32_t* err, uint64_t& nodes, uint64_t& tris, HS& hs) {
  const dv3 o2 = dadd3(org, dscale3(dir, 0.000001));
  double best = kInfD;
  int ent = -1, prim = -1;
  ExactRay r;
  bool ray_ready = false;
  hs.begin();
  for (int i = 0; i < S.n_ents; i++) {
    const GEntity& e = S.ents[i];
    double t;
    int face = -1;
    bool got = false;
    if (e.type == PR_ENT_SPHERE) {
      got = exact_sphere(e, o2, dir, t);
    } else if (e.type == PR_ENT_UVPLANE) {
      got = exact_uvplane(e, o2, dir, t);
    } else if (e.type == PR_ENT_CIRCLE) {
      got = exact_circle(e, o2, dir, t);
      // the hit point exactly as exact_circle forms it
      if (got) got = hs.circle(e, {da(dm(dir.x, t), o2.x), da(dm(dir.y, t), o2.y), da(dm(dir.z, t), o2.z)});
    } else if (e.type == PR_ENT_POLYGON) {
      if (!ray_ready) {
        r = make_exact_ray(o2, dir);
        ray_ready = true;
      }
      got = exact_qbvh(S, e, r, t, face, err, nodes, tris);
    }
    if (got && t < best) {
      best = t;
      ent = i;
      prim = face;
      hs.best(e);
    }
  }
  t_out = best;
  ent_out = ent;
  prim_out = prim;
  return ent >= 0;
}

__device__ inline bool exact_closest(const DevScene& S, dv3 org, dv3 dir, double& t_out, int& ent_out, int& prim_out,
                                     uint32_t* err, uint64_t& nodes, uint64_t& tris) {
  NoHitShading hs;
  return exact_closest_hs(S, org, dir, t_out, ent_out, prim_out, err, nodes, tris, hs);
}

}  // namespace pr
