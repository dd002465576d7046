// FP32 closest-hit and any-hit queries used while rendering.
//
// Traversal of the render path's compressed 8-wide trees (WNode) per thread
// with a small local stack of node groups: children visited near to far by
// their octant slots, each child box culled against the current closest hit,
// leaves tested as soon as their node is visited.
// Spheres keep the reference's FP64 test (its 1e5-radius walls cancel
// catastrophically in FP32); planes and triangles are FP32.
#pragma once
#include "device_common.cuh"

namespace pr {

struct FastHit {
  float t;
  int ent;
  int slot;   // leaf slot of the triangle (meshes), -1 otherwise
  float u, v; // barycentrics of the triangle hit
};

struct TraceStats {
  uint32_t nodes;
  uint32_t tris;
};

__device__ __forceinline__ bool fast_tri(const float4* __restrict__ T, float3 o, float3 d, float tmax, float& t, float& bu,
                                         float& bv) {
  const float4 A = __ldg(T), B = __ldg(T + 1), C = __ldg(T + 2);
  const float3 v0 = f3(A.x, A.y, A.z);
  const float3 e1 = f3(B.x, B.y, B.z) - v0, e2 = f3(C.x, C.y, C.z) - v0;
  const float3 p = cross(d, e2);
  const float det = dot(e1, p);
  if (fabsf(det) <= 1.0e-7f) return false;  // det eps of CheckIntersection2 (polygon.h:98)
  const float inv = 1.0f / det;
  const float3 tv = o - v0;
  const float u = dot(tv, p) * inv;
  if (u < 0.0f || u > 1.0f) return false;
  const float3 q = cross(tv, e1);
  const float v = dot(d, q) * inv;
  if (v < 0.0f || u + v > 1.0f) return false;
  const float tt = dot(e2, q) * inv;
  if (!(tt > 0.0f) || !(tt < tmax)) return false;
  t = tt;
  bu = u;
  bv = v;
  return true;
}

// Ray data of the wide traversal
struct WRay {
  float3 o, d, inv;
  int oct;  // sign bits of d (bit a: negative along axis a)
};

__device__ __forceinline__ float3 safe_inv(float3 d) {
  const float big = 1.0e30f;
  return f3(d.x != 0.0f ? 1.0f / d.x : copysignf(big, d.x), d.y != 0.0f ? 1.0f / d.y : copysignf(big, d.y),
            d.z != 0.0f ? 1.0f / d.z : copysignf(big, d.z));
}

__device__ __forceinline__ WRay make_wray(float3 o, float3 d) {
  WRay r;
  r.o = o;
  r.d = d;
  r.inv = safe_inv(d);
  r.oct = (d.x < 0.0f ? 1 : 0) | (d.y < 0.0f ? 2 : 0) | (d.z < 0.0f ? 4 : 0);
  return r;
}

// byte k of w as an exact float (0x4B0000qq is 2^23 + qq)
__device__ __forceinline__ float qbyte(uint32_t w, int k) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u + (uint32_t)k)) - 8388608.0f;
}

// three-input minimum / maximum (one instruction on sm_100 and later)
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

// bit i of m moves to bit i ^ x (x in 0..7)
__device__ __forceinline__ uint32_t permute_xor8(uint32_t m, int x) {
  if (x & 1) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
  if (x & 2) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
  if (x & 4) m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
  return m;
}

// Node group of the wide traversal: the node index of the first inner child,
// the node's inner-child mask and the not yet visited inner children that the
// ray hit, in traversal order (bit i: slot i ^ oct)
struct WGroup {
  int base;
  uint32_t bits;  // hits | imask << 8
};

// One wide node against the ray (slab test of its eight quantised child
// boxes against [0, tmax)): the group of its hit inner children and the
// mask of its hit leaves' triangles (bit k: triangle slot tri_base + k).
__device__ __forceinline__ void wnode_visit(const WNode* __restrict__ n, const WRay& r, float tmax, WGroup& g,
                                            uint32_t& tri_mask, int& tri_base) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(n));
  const int4 b = __ldg(reinterpret_cast<const int4*>(n) + 1);
  const uint4 c = __ldg(reinterpret_cast<const uint4*>(n) + 2);  // qlo_x, qlo_y
  const uint4 d = __ldg(reinterpret_cast<const uint4*>(n) + 3);  // qlo_z, qhi_x
  const uint4 e = __ldg(reinterpret_cast<const uint4*>(n) + 4);  // qhi_y, qhi_z
  const uint32_t em = __float_as_uint(a.w);
  // plane q of axis x at distance (p + q 2^e - o) / d = q sx + bx.  (Folding
  // the bytes' 2^23 bias into bx saves the subtraction but rounds bx by up
  // to half a grid step, which needs a step of margin around every box:
  // measured on GB300, twice the triangle tests per shadow ray and no gain.)
  const float sx = __uint_as_float((em & 0xFFu) << 23) * r.inv.x;
  const float sy = __uint_as_float(((em >> 8) & 0xFFu) << 23) * r.inv.y;
  const float sz = __uint_as_float(((em >> 16) & 0xFFu) << 23) * r.inv.z;
  const float bx = (a.x - r.o.x) * r.inv.x;
  const float by = (a.y - r.o.y) * r.inv.y;
  const float bz = (a.z - r.o.z) * r.inv.z;
  // near and far planes per axis: the low planes are near for a positive direction
  const bool nx = r.oct & 1, ny = r.oct & 2, nz = r.oct & 4;
  const uint32_t nx0 = nx ? d.z : c.x, nx1 = nx ? d.w : c.y, fx0 = nx ? c.x : d.z, fx1 = nx ? c.y : d.w;
  const uint32_t ny0 = ny ? e.x : c.z, ny1 = ny ? e.y : c.w, fy0 = ny ? c.z : e.x, fy1 = ny ? c.w : e.y;
  const uint32_t nz0 = nz ? e.z : d.x, nz1 = nz ? e.w : d.y, fz0 = nz ? d.x : e.z, fz1 = nz ? d.y : e.w;
  uint32_t hits = 0;
#pragma unroll
  for (int s = 0; s < 8; s++) {
    const int k = s & 3;
    const float tnx = fmaf(qbyte(s < 4 ? nx0 : nx1, k), sx, bx);
    const float tfx = fmaf(qbyte(s < 4 ? fx0 : fx1, k), sx, bx);
    const float tny = fmaf(qbyte(s < 4 ? ny0 : ny1, k), sy, by);
    const float tfy = fmaf(qbyte(s < 4 ? fy0 : fy1, k), sy, by);
    const float tnz = fmaf(qbyte(s < 4 ? nz0 : nz1, k), sz, bz);
    const float tfz = fmaf(qbyte(s < 4 ? fz0 : fz1, k), sz, bz);
    const float tn = fmax3(tnx, tny, fmaxf(tnz, 0.0f));
    const float tf = fmin3(tfx, tfy, fminf(tfz, tmax));
    hits |= (tn <= tf) ? (1u << s) : 0u;
  }
  const uint32_t imask = em >> 24;
  uint32_t tm = 0;
  if (hits & ~imask) {
#pragma unroll
    for (int s = 0; s < 8; s++) {
      const uint32_t m = ((s < 4 ? (uint32_t)b.z : (uint32_t)b.w) >> (8 * (s & 3))) & 0xFFu;
      tm |= ((hits >> s) & 1u) ? ((m >> 5) << (m & 31u)) : 0u;
    }
  }
  g.base = b.x;
  g.bits = permute_xor8(hits & imask, r.oct) | imask << 8;
  tri_mask = tm;
  tri_base = b.y;
}

// the next child of a group (its lowest pending hit); clears it
__device__ __forceinline__ int wgroup_next(WGroup& g, int oct) {
  const int i = __ffs(g.bits & 0xFFu) - 1;
  g.bits &= ~(1u << i);
  const int s = i ^ oct;
  return g.base + __popc((g.bits >> 8) & ((1u << s) - 1u));
}

// the root of a mesh as a group with one pending child
__device__ __forceinline__ WGroup wgroup_root(int root, int oct) {
  WGroup g;
  g.base = root;
  g.bits = (1u << oct) | (1u << 8);  // pending bit oct is slot 0, the only inner child
  return g;
}

// Wide-BVH closest hit (ANY = false) or any hit below tmax (ANY = true):
// children are visited near to far by the slot order, each node's leaf
// triangles tested as soon as the node is visited.
template <bool ANY>
__device__ __forceinline__ bool fast_qbvh(const DevScene& S, const GEntF& e, const WRay& r, float& tbest, int& slot,
                                          float& bu, float& bv, TraceStats& st, uint32_t* err) {
  WGroup stack[kWStack];
  int sp = 0;
  WGroup g = wgroup_root(e.node_base, r.oct);
  bool hit = false;
  int guard = 0;
  while (true) {
    if ((g.bits & 0xFFu) == 0) {
      if (sp == 0) break;
      g = stack[--sp];
    }
    if (++guard > (1 << 22)) { atomicOr(err, PR_DEV_LOOP_CAP); break; }
    const int child = wgroup_next(g, r.oct);
    if (g.bits & 0xFFu) {
      if (sp >= kWStack) { atomicOr(err, PR_DEV_STACK_OVERFLOW); return hit; }
      stack[sp++] = g;
    }
    st.nodes++;
    uint32_t tm;
    int tb;
    wnode_visit(S.rnodes + child, r, tbest, g, tm, tb);
    while (tm) {
      const int k = __ffs(tm) - 1;
      tm &= tm - 1u;
      st.tris++;
      float t, uu, vv;
      if (fast_tri(S.rtris + 3 * (size_t)(tb + k), r.o, r.d, tbest, t, uu, vv)) {
        tbest = t;
        slot = tb + k;
        bu = uu;
        bv = vv;
        hit = true;
        if (ANY) return true;
      }
    }
  }
  return hit;
}

// FP64 sphere distance of an FP32 ray; threshold PS_EPS as in sphere.h:80-87
__device__ __forceinline__ bool sphere_t64(const GEntity& e, float3 o, float3 d, double& tt) {
  const double px = e.p[0] - (double)o.x, py = e.p[1] - (double)o.y, pz = e.p[2] - (double)o.z;
  const double b = px * (double)d.x + py * (double)d.y + pz * (double)d.z;
  const double D4 = b * b - (px * px + py * py + pz * pz) + e.radius * e.radius;
  if (D4 < 0.0) return false;
  const double s = sqrt(D4);
  const double t1 = b - s, t2 = b + s;
  if (t1 < kEps && t2 < kEps) return false;
  tt = (t1 > kEps) ? t1 : t2;
  return true;
}

// t is the FP32 distance, rest what it rounded off (t + rest is the FP64
// distance to ~2^-48: the hit point is rebuilt from it, since the FP32
// distance alone is up to half an ulp of t off -- 1.5e-5 beyond t = 256, as
// much as the origin offset of the next ray near a coordinate of zero)
__device__ __forceinline__ bool fast_sphere(const GEntity& e, float3 o, float3 d, float tmax, float& t, float& rest) {
  double tt;
  if (!sphere_t64(e, o, d, tt) || !(tt < (double)tmax)) return false;
  // a hemisphere keeps the hit only on its y >= y_centre half (sphere.h:98-103)
  if (e.hemisphere && (double)o.y + tt * (double)d.y - e.p[1] < 0.0) return false;
  t = (float)tt;
  rest = (float)(tt - (double)t);
  return true;
}

// UVPlane::intersect semantics in FP32 (plane.h:86-110, :220-239): the
// extent check compares u / |U| against |U| (the reference's own rule).
__device__ __forceinline__ bool fast_uvplane(const GEntF& e, float3 o, float3 d, float tmax, float& t) {
  const float s = e.normal_inverse < 0 ? -1.0f : 1.0f;
  const float3 n = f3(e.n[0] * s, e.n[1] * s, e.n[2] * s);
  const float dd = dot(d, n);
  if (fabsf(dd) < 1.0e-14f) return false;
  const float3 org = f3(e.p[0], e.p[1], e.p[2]);
  const float tt = dot(org - o, n) / dd;
  if (!(tt > 0.0f) || !(tt < tmax)) return false;
  const float3 rel = (o + d * tt) - org;
  const float ul = e.u_length, vl = e.v_length;
  const float u = dot(rel, f3(e.u[0], e.u[1], e.u[2])) / ul;
  const float v = dot(rel, f3(e.v[0], e.v[1], e.v[2])) / vl;
  if (u < 0.0f || u > ul || v < 0.0f || v > vl) return false;
  t = tt;
  return true;
}

// Circle::intersect in FP32 (circle.h:177-200): plane test, then the annulus
// (u_length = radius, v_length = inner radius)
__device__ __forceinline__ bool fast_circle(const GEntF& e, float3 o, float3 d, float tmax, float& t) {
  const float3 n = f3(e.n[0], e.n[1], e.n[2]);
  const float dd = dot(d, n);
  if (fabsf(dd) < 1.0e-14f) return false;
  const float3 org = f3(e.p[0], e.p[1], e.p[2]);
  const float tt = dot(org - o, n) / dd;
  if (!(tt > 0.0f) || !(tt < tmax)) return false;
  const float3 rel = (o + d * tt) - org;
  const float r2 = dot(rel, rel);
  if (r2 > e.u_length * e.u_length || r2 < e.v_length * e.v_length) return false;
  t = tt;
  return true;
}

// closest hit over the entity list (strict '<' in list order)
__device__ __forceinline__ bool fast_closest(const DevScene& S, float3 o, float3 d, FastHit& h, TraceStats& st,
                                             uint32_t* err) {
  h.t = 3.0e38f;
  h.ent = -1;
  h.slot = -1;
  h.u = h.v = 0.0f;
  const WRay r = make_wray(o, d);
  for (int i = 0; i < S.n_ents; i++) {
    const GEntF& e = S.entf[i];
    float t = h.t, bu = 0.0f, bv = 0.0f;
    int slot = -1;
    bool got = false;
    if (e.type == PR_ENT_SPHERE) got = fast_sphere(S.ents[i], o, d, h.t, t, bu);
    else if (e.type == PR_ENT_UVPLANE) got = fast_uvplane(e, o, d, h.t, t);
    else if (e.type == PR_ENT_CIRCLE) got = fast_circle(e, o, d, h.t, t);
    else if (e.type == PR_ENT_POLYGON) got = fast_qbvh<false>(S, e, r, t, slot, bu, bv, st, err);
    if (got && t < h.t) {
      h.t = t;
      h.ent = i;
      h.slot = slot;
      h.u = bu;
      h.v = bv;
    }
  }
  return h.ent >= 0;
}

// any hit with t < tmax
__device__ __forceinline__ bool fast_occluded(const DevScene& S, float3 o, float3 d, float tmax, TraceStats& st,
                                              uint32_t* err) {
  const WRay r = make_wray(o, d);
  for (int i = 0; i < S.n_ents; i++) {
    const GEntF& e = S.entf[i];
    float t = tmax, bu, bv;
    int slot;
    bool got = false;
    if (e.type == PR_ENT_SPHERE) got = fast_sphere(S.ents[i], o, d, tmax, t, bu);
    else if (e.type == PR_ENT_UVPLANE) got = fast_uvplane(e, o, d, tmax, t);
    else if (e.type == PR_ENT_CIRCLE) got = fast_circle(e, o, d, tmax, t);
    else if (e.type == PR_ENT_POLYGON) got = fast_qbvh<true>(S, e, r, t, slot, bu, bv, st, err);
    if (got) return true;
  }
  return false;
}

}  // namespace pr
