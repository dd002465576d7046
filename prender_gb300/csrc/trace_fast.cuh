// FP32 closest-hit and any-hit queries used while rendering.
//
// QBVH traversal per thread with a small local stack: children ordered near
// to far by the node's split axes and the ray signs (the reference's own
// ordering, QBVH.cpp:80-100, popped nearest-first), each child box culled
// against the current closest hit, leaves tested as soon as they are met.
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

// 4-wide slab test; returns a mask of children whose box overlaps [0, tmax)
// and their entry distances.
__device__ __forceinline__ int box4(const GNode* __restrict__ node, float3 inv, float3 oinv, float tmax, float tn[4]) {
  const float4* n4 = reinterpret_cast<const float4*>(node);
  const float4 mnx = __ldg(n4 + 0), mxx = __ldg(n4 + 1), mny = __ldg(n4 + 2), mxy = __ldg(n4 + 3);
  const float4 mnz = __ldg(n4 + 4), mxz = __ldg(n4 + 5);
  const float a0[4] = {mnx.x, mnx.y, mnx.z, mnx.w}, a1[4] = {mxx.x, mxx.y, mxx.z, mxx.w};
  const float b0[4] = {mny.x, mny.y, mny.z, mny.w}, b1[4] = {mxy.x, mxy.y, mxy.z, mxy.w};
  const float c0[4] = {mnz.x, mnz.y, mnz.z, mnz.w}, c1[4] = {mxz.x, mxz.y, mxz.z, mxz.w};
  int mask = 0;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const float tx0 = fmaf(a0[c], inv.x, -oinv.x), tx1 = fmaf(a1[c], inv.x, -oinv.x);
    const float ty0 = fmaf(b0[c], inv.y, -oinv.y), ty1 = fmaf(b1[c], inv.y, -oinv.y);
    const float tz0 = fmaf(c0[c], inv.z, -oinv.z), tz1 = fmaf(c1[c], inv.z, -oinv.z);
    const float tnear = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    const float tfar = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    tn[c] = tnear;
    mask |= (tnear <= tfar) ? (1 << c) : 0;
  }
  return mask;
}

// QBVH closest hit (ANY = false) or any hit below tmax (ANY = true).
template <bool ANY>
__device__ __forceinline__ bool fast_qbvh(const DevScene& S, const GEntF& e, float3 o, float3 d, float3 inv, float& tbest,
                                          int& slot, float& bu, float& bv, TraceStats& st, uint32_t* err) {
  int32_t stack[kStackSize];
  int sp = 0;
  stack[sp++] = e.node_base;
  const float3 oinv = o * inv;
  const int sx = d.x >= 0.0f ? 0 : 1, sy = d.y >= 0.0f ? 0 : 1, sz = d.z >= 0.0f ? 0 : 1;
  bool hit = false;
  int guard = 0;
  while (sp > 0) {
    if (++guard > (1 << 22)) { atomicOr(err, PR_DEV_LOOP_CAP); break; }
    const int32_t ni = stack[--sp];
    const GNode* node = S.rnodes + ni;
    st.nodes++;
    float tn[4];
    const int mask = box4(node, inv, oinv, tbest, tn);
    if (!mask) continue;
    const int4 ch = __ldg(reinterpret_cast<const int4*>(node) + 6);
    const int4 meta = __ldg(reinterpret_cast<const int4*>(node) + 7);
    const int axes = meta.x;
    const int child[4] = {ch.x, ch.y, ch.z, ch.w};
    const int cnt[4] = {meta.y & 0xFFFF, (int)((uint32_t)meta.y >> 16), meta.z & 0xFFFF, (int)((uint32_t)meta.z >> 16)};
    const int sg[3] = {sx, sy, sz};
    const int at = axes & 3, al = (axes >> 2) & 3, ar = (axes >> 4) & 3;
    int order[4];
    const int lf = (sg[at] == 0) ? 0 : 2, rf = (lf + 2) & 3;
    if (sg[al] == 0) { order[lf] = 0; order[lf + 1] = 1; } else { order[lf] = 1; order[lf + 1] = 0; }
    if (sg[ar] == 0) { order[rf] = 2; order[rf + 1] = 3; } else { order[rf] = 3; order[rf + 1] = 2; }
    // leaves near to far now, inner nodes pushed far to near.  The leaf
    // triangles are gathered into one run first, so that all lanes of a warp
    // test their triangles in the same loop (one code path, not one per
    // child position)
    int lfirst[4], lcnt[4];
    float ltn[4];
    int nl = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int c = order[i];
      if (!((mask >> c) & 1) || child[c] == kChildInvalid || child[c] >= 0) continue;
      lfirst[nl] = (int32_t)((uint32_t)child[c] & ~kLeafBit);
      lcnt[nl] = cnt[c];
      ltn[nl] = tn[c];
      nl++;
    }
    for (int l = 0; l < nl; l++) {
      if (ltn[l] > tbest) continue;
      const int32_t first = lfirst[l];
      for (int k = 0; k < lcnt[l]; k++) {
        st.tris++;
        float t, uu, vv;
        if (fast_tri(S.rtris + 3 * (size_t)(first + k), o, d, tbest, t, uu, vv)) {
          tbest = t;
          slot = first + k;
          bu = uu;
          bv = vv;
          hit = true;
          if (ANY) return true;
        }
      }
    }
#pragma unroll
    for (int i = 3; i >= 0; i--) {
      const int c = order[i];
      if (!((mask >> c) & 1) || child[c] < 0) continue;
      if (tn[c] > tbest) continue;
      if (sp >= kStackSize) { atomicOr(err, PR_DEV_STACK_OVERFLOW); return hit; }
      stack[sp++] = child[c];
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

__device__ __forceinline__ float3 safe_inv(float3 d) {
  const float big = 1.0e30f;
  return f3(d.x != 0.0f ? 1.0f / d.x : copysignf(big, d.x), d.y != 0.0f ? 1.0f / d.y : copysignf(big, d.y),
            d.z != 0.0f ? 1.0f / d.z : copysignf(big, d.z));
}

// closest hit over the entity list (strict '<' in list order)
__device__ __forceinline__ bool fast_closest(const DevScene& S, float3 o, float3 d, FastHit& h, TraceStats& st,
                                             uint32_t* err) {
  h.t = 3.0e38f;
  h.ent = -1;
  h.slot = -1;
  h.u = h.v = 0.0f;
  const float3 inv = safe_inv(d);
  for (int i = 0; i < S.n_ents; i++) {
    const GEntF& e = S.entf[i];
    float t = h.t, bu = 0.0f, bv = 0.0f;
    int slot = -1;
    bool got = false;
    if (e.type == PR_ENT_SPHERE) got = fast_sphere(S.ents[i], o, d, h.t, t, bu);
    else if (e.type == PR_ENT_UVPLANE) got = fast_uvplane(e, o, d, h.t, t);
    else if (e.type == PR_ENT_CIRCLE) got = fast_circle(e, o, d, h.t, t);
    else if (e.type == PR_ENT_POLYGON) got = fast_qbvh<false>(S, e, o, d, inv, t, slot, bu, bv, st, err);
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
  const float3 inv = safe_inv(d);
  for (int i = 0; i < S.n_ents; i++) {
    const GEntF& e = S.entf[i];
    float t = tmax, bu, bv;
    int slot;
    bool got = false;
    if (e.type == PR_ENT_SPHERE) got = fast_sphere(S.ents[i], o, d, tmax, t, bu);
    else if (e.type == PR_ENT_UVPLANE) got = fast_uvplane(e, o, d, tmax, t);
    else if (e.type == PR_ENT_CIRCLE) got = fast_circle(e, o, d, tmax, t);
    else if (e.type == PR_ENT_POLYGON) got = fast_qbvh<true>(S, e, o, d, inv, t, slot, bu, bv, st, err);
    if (got) return true;
  }
  return false;
}

}  // namespace pr
