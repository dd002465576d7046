// Wormhole geodesics in FP64 (WormHole.h, scene.cpp:735-925): the Dneg
// wormhole of James, von Tunzelmann, Franklin and Thorne ("Visualizing
// Interstellar's wormhole", Am. J. Phys. 83, 2015) -- radius r(l), the
// geodesic equations (A7) from the initial conditions (A9) in a frame whose
// x axis points from the ray's mouth to the camera, Cash-Karp RK45 with the
// reference's step control, and a straight-segment scene test per step.
// This translation unit is compiled with -fmad=false: every FP64 multiply
// and add rounds on its own in the reference's order (CUDA's sin / cos /
// atan / log / acos may differ from the host libm in the last bit; the
// tests bound the effect on exit directions).
#include "device_common.cuh"
#include "path_logic.cuh"
#include "wormhole.h"

namespace pr {
namespace {

constexpr double kWPi = 3.14159265358979323846264338327950288;

// Cartesian::ToSpherical (vector3d.h:913-939)
__device__ __forceinline__ void w_to_sph(double x, double y, double z, double& r, double& th, double& ph) {
  r = sqrt(x * x + y * y + z * z);
  if (!(r > 1.0e-16)) {
    th = 0;
    ph = 0;
    return;
  }
  const double xx = x / r, yy = y / r, zz = z / r;
  th = acos(zz < -1.0 ? -1.0 : (zz > 1.0 ? 1.0 : zz));
  double phi;
  if (fabs(xx) < 1.0e-6 && fabs(yy) < 1.0e-6) phi = 0.0;
  else phi = atan2(yy, xx);
  if (phi < 0.0) phi += 2.0 * kWPi;
  if (phi >= 2.0 * kWPi) phi = 0.0;
  ph = phi;
}

// Spherical::ToCartesian (vector3d.h:879-887)
__device__ __forceinline__ dv3 w_to_cart(double r, double th, double ph) {
  const double sint = sin(th);
  return {r * cos(ph) * sint, r * sin(ph) * sint, r * cos(th)};
}

// Matrix4D * Vector3d (vector3d.h:760-768): the upper 3x3 block
__device__ __forceinline__ dv3 w_mul(const double* m, dv3 v) {
  return {v.x * m[0] + v.y * m[1] + v.z * m[2], v.x * m[4] + v.y * m[5] + v.z * m[6],
          v.x * m[8] + v.y * m[9] + v.z * m[10]};
}

__device__ __forceinline__ dv3 w_normalize(dv3 v) {  // normalize (vector3d.h:162-165)
  const double il = 1.0 / sqrt((v.x * v.x + v.z * v.z) + v.y * v.y);
  return {v.x * il, v.y * il, v.z * il};
}

struct WormRay {
  const GWorm* W;
  const double* mat;  // the frame of the ray's mouth
  const double* inv;
  double l0, theta0, phi0, n_l, n_ph, n_th;

  __device__ __forceinline__ double r_wh(double l) const {  // WormHole.h:172-180
    const double x = 2.0 * (fabs(l) - W->a) / (kWPi * W->M);
    if (fabs(l) > W->a) return W->Rho + W->M * (x * atan(x) - 0.5 * log(1.0 + x * x));
    return W->Rho;
  }
  __device__ __forceinline__ double drdl(double l) const {  // :182-193
    double sg = 1;
    if (l < 0) sg = -1;
    if (l == 0.0) sg = 0.0;
    if (fabs(l) > W->a) return (2.0 * atan((2.0 * (-W->a + fabs(l))) / (W->M * kWPi)) * sg) / kWPi;
    return 0;
  }
  // :195-238: Newton's method on r(l) = r from the start point, then from a
  __device__ double rtol(double r, double linit) const {
    const double M = W->M, Rho = W->Rho;
    double x = 2.0 * (fabs(linit) - W->a) / (kWPi * M);
    int stat = -1;
    for (int i = 0; i < 30; i++) {
      const double xi = x;
      x = x - (Rho + M * (x * atan(x) - 0.5 * log(1.0 + x * x)) - r) / (M * atan(x));
      if (fabs(x - xi) < 1.0e-6) {
        stat = 0;
        break;
      }
      if (!isfinite(x)) break;
    }
    double l = x * kWPi * M * 0.5 + W->a;
    if (stat != 0) {
      x = W->a;
      for (int i = 0; i < 30; i++) {
        const double xi = x;
        x = x - (Rho + M * (x * atan(x) - 0.5 * log(1.0 + x * x)) - r) / (M * atan(x));
        if (fabs(x - xi) < 1.0e-6) {
          l = x * kWPi * M * 0.5 + W->a;
          break;
        }
        if (!isfinite(x)) break;
      }
    }
    return (linit < 0) ? -fabs(l) : fabs(l);
  }
  // Setup + initial (WormHole.h:321-428)
  __device__ void start(dv3 org, dv3 dir, double sgn, double* y) {
    const int m = sgn >= 0 ? 0 : 1;
    mat = W->mat[m];
    inv = W->inv[m];
    double pr, pth, pph;
    w_to_sph(org.x - W->pos[m][0], org.y - W->pos[m][1], org.z - W->pos[m][2], pr, pth, pph);
    const dv3 q = w_mul(mat, w_to_cart(pr, pth, pph));
    double qr;
    w_to_sph(q.x, q.y, q.z, qr, theta0, phi0);
    l0 = rtol(qr, sgn * W->a / 2);
    double dr, dth, dph;
    w_to_sph(dir.x, dir.y, dir.z, dr, dth, dph);
    const dv3 rc = w_mul(mat, w_to_cart(dr, dth, dph));
    double rr, th, ph;
    w_to_sph(rc.x, rc.y, rc.z, rr, th, ph);
    const double sint = sin(th);
    const double Nx = sint * cos(ph), Ny = sint * sin(ph), Nz = cos(th);
    n_l = -Nx;
    n_ph = -Ny;
    n_th = Nz;
    y[0] = l0;
    y[1] = theta0;
    y[2] = phi0;
    y[3] = n_l;
    y[4] = r_wh(l0) * n_th;
  }
  // geodesic (WormHole.h:462-488): (A7)
  __device__ __forceinline__ void geodesic(const double* y, double* dydx) const {
    const double r = r_wh(y[0]);
    const double r2 = r * r;
    double sint = sin(y[1]);
    if (fabs(sint) < 1.0e-8) sint = sint > 0.0 ? 1.0e-8 : -1.0e-8;
    const double sint2 = sint * sint;
    const double r_l0 = r_wh(l0);
    const double b = r_l0 * sin(theta0) * n_ph;
    const double B2 = r_l0 * r_l0 * (n_th * n_th + n_ph * n_ph);
    const double invr2 = 1.0 / r2;
    dydx[0] = y[3];
    dydx[1] = y[4] * invr2;
    dydx[2] = b * invr2 / sint2;
    dydx[3] = B2 * drdl(y[0]) * invr2 / r;
    dydx[4] = (b * b * invr2) * (cos(y[1]) / (sint * sint2));
  }
  // rkstep (WormHole.h:541-612): Cash-Karp, the step negated (traceDir 1)
  __device__ void rkstep(const double* y, const double* dydx, double h, double* yout, double* yerr) const {
    double ak[5], t1[5], t2[5], t3[5], t4[5], t5[5];
    h *= -1.0;
    for (int i = 0; i < 5; i++) {
      const double hd = h * dydx[i], yi = y[i];
      t1[i] = yi + 0.2 * hd;
      t2[i] = yi + (3.0 / 40.0) * hd;
      t3[i] = yi + 0.3 * hd;
      t4[i] = yi - (11.0 / 54.0) * hd;
      t5[i] = yi + (1631.0 / 55296.0) * hd;
      yout[i] = yi + (37.0 / 378.0) * hd;
      yerr[i] = ((37.0 / 378.0) - (2825.0 / 27648.0)) * hd;
    }
    geodesic(t1, ak);
    for (int i = 0; i < 5; i++) {
      const double yt = h * ak[i];
      t2[i] += (9.0 / 40.0) * yt;
      t3[i] -= 0.9 * yt;
      t4[i] += 2.5 * yt;
      t5[i] += (175.0 / 512.0) * yt;
    }
    geodesic(t2, ak);
    for (int i = 0; i < 5; i++) {
      const double yt = h * ak[i];
      t3[i] += 1.2 * yt;
      t4[i] -= (70.0 / 27.0) * yt;
      t5[i] += (575.0 / 13824.0) * yt;
      yout[i] += (250.0 / 621.0) * yt;
      yerr[i] += ((250.0 / 621.0) - (18575.0 / 48384.0)) * yt;
    }
    geodesic(t3, ak);
    for (int i = 0; i < 5; i++) {
      const double yt = h * ak[i];
      t4[i] += (35.0 / 27.0) * yt;
      t5[i] += (44275.0 / 110592.0) * yt;
      yout[i] += (125.0 / 594.0) * yt;
      yerr[i] += ((125.0 / 594.0) - (13525.0 / 55296.0)) * yt;
    }
    geodesic(t4, ak);
    for (int i = 0; i < 5; i++) {
      const double yt = h * ak[i];
      t5[i] += (253.0 / 4096.0) * yt;
      yerr[i] -= (277.0 / 14336.0) * yt;
    }
    geodesic(t5, ak);
    for (int i = 0; i < 5; i++) {
      const double yt = h * ak[i];
      yout[i] += (512.0 / 1771.0) * yt;
      yerr[i] += ((512.0 / 1771.0) - 0.25) * yt;
    }
  }
  // NextPosition + rkqs (WormHole.h:490-535, :618-683): at most 2000 shrinks
  __device__ double next_position(double* y, const double* dydx, double htry, uint32_t& attempts) const {
    const double escal = 1e11;
    double yscal[5], ytemp[5], yerr[5];
    for (int i = 0; i < 5; i++) yscal[i] = fabs(y[i]) + fabs(dydx[i] * htry) + 1.0e-3;
    double h = htry, errmax = 0.0;
    for (int loops = 0; loops < 2000; loops++) {
      attempts++;
      rkstep(y, dydx, h, ytemp, yerr);
      errmax = 0.0;
      for (int i = 0; i < 5; i++) {
        const double temp = fabs(yerr[i] / yscal[i]);
        if (temp > errmax) errmax = temp;
      }
      errmax *= escal;
      if (errmax <= 1.0) break;
      const double htemp = 0.9 * h / sqrt(sqrt(errmax));
      h *= 0.1;
      if (h >= 0.0) {
        if (htemp > h) h = htemp;
      } else {
        if (htemp < h) h = htemp;
      }
    }
    const double hnext = errmax > 1.89e-4 ? 0.9 * h * pow(errmax, -0.2) : 5.0 * h;
    for (int i = 0; i < 5; i++) y[i] = ytemp[i];
    return hnext;
  }
  __device__ __forceinline__ dv3 world(dv3 q, double sgn) const {  // WorldAxisSystem (WormHole.h:430-447)
    const dv3 p = w_mul(inv, q);
    const int m = sgn >= 0 ? 0 : 1;
    return {p.x + W->pos[m][0], p.y + W->pos[m][1], p.z + W->pos[m][2]};
  }
};

struct WormHit {
  int status;  // 1 entity hit, 0 background 1, 3 background 2
  int steps, ent, prim;
  double t;
  dv3 seg_o, dir2;
  double y[5];
};

struct WormCount {
  uint32_t steps, attempts, segments;
  uint64_t nodes, tris;
};

// intersect_scene__ (scene.cpp:735-925) for one ray
__device__ void worm_trace_ray(const DevScene& S, const GWorm& W, dv3 org, dv3 dir, WormHit& out, WormCount& cnt,
                               uint32_t* err) {
  WormRay k;
  k.W = &W;
  double* y = out.y;
  double dydx[5];
  const double sign = sqrt((org.x * org.x + org.z * org.z) + org.y * org.y) > 1000000 ? -1.0 : 1.0;
  k.start(org, dir, sign, y);
  out.ent = -1;
  out.prim = -1;
  out.t = -1.0;
  double h_dist = 0.5;
  if (fabs(y[0]) < W.a || k.r_wh(y[0]) <= W.Rho) h_dist = h_dist * 0.15;
  double h_step = h_dist;
  dv3 org1 = org, org2 = org, dir2 = dir;
  int c = 0;
  while (W.max_steps < 0 ? true : c < W.max_steps) {
    if (fabs(y[0]) > 1.0e10 || fabs(k.r_wh(y[0])) > 1.0e10 || !isfinite(y[0])) break;
    double t;
    int ent, prim;
    cnt.segments++;
    if (exact_closest(S, org1, dir2, t, ent, prim, err, cnt.nodes, cnt.tris) && t < h_dist) {
      out.status = 1;
      out.steps = c;
      out.ent = ent;
      out.prim = prim;
      out.t = t;
      out.seg_o = org1;
      out.dir2 = dir2;
      return;
    }
    k.geodesic(y, dydx);
    if (fabs(h_step) < 1.0e-14) h_step = 1.0e-14;
    h_step = k.next_position(y, dydx, h_step, cnt.attempts);
    if (h_step > h_dist) h_step = h_dist;
    org1 = org2;
    org2 = k.world(w_to_cart(k.r_wh(y[0]), y[1], y[2]), y[0]);
    dir2 = w_normalize({org2.x - org1.x, org2.y - org1.y, org2.z - org1.z});
    c++;
    cnt.steps++;
  }
  if (W.usr_sign) y[0] = W.usr_sign * y[0];
  double dr;
  w_to_sph(dir2.x, dir2.y, dir2.z, dr, y[1], y[2]);
  out.status = y[0] >= 0 ? 0 : 3;
  out.steps = c;
  out.seg_o = org2;
  out.dir2 = dir2;
}

// the colour of a ray that ended on a background (scene.cpp:860-920 +
// SphericalMapping::Map, circle.h:92-105)
__device__ float3 worm_background(const GWorm& W, int side, const double* yy, const float* bg) {
  if (!W.tex[side]) return f3(bg[0], bg[1], bg[2]);
  double y1 = yy[1] * W.map_coef[side][0] + W.map_coef[side][1];
  double y2 = yy[2] * W.map_coef[side][2] + W.map_coef[side][3];
  y1 = fmod(y1, kWPi);
  y2 = fmod(y2, 2.0 * kWPi);
  double phi = y2, theta = y1;
  if (phi < 0.0) phi += 2.0 * kWPi;
  if (theta < 0.0) theta = -theta;
  if (!(phi == phi) || !(theta == theta)) return f3(0, 0, 0);
  const int tw = W.tex_w[side], th = W.tex_h[side];
  int x = (int)(phi / (2.0 * kWPi) * tw);
  x = ((x % tw) + tw) % tw;  // in range for any input, NaN included
  int yv = (int)(theta / kWPi * th);
  yv = ((yv % th) + th) % th;
  const unsigned char* t = W.tex[side] + 3 * ((size_t)yv * tw + x);
  const double c = W.tex_coef[side];
  return f3((float)(c * t[0] / 255.0), (float)(c * t[1] / 255.0), (float)(c * t[2] / 255.0));
}

__global__ void __launch_bounds__(128) worm_trace_kernel(DevScene S, GWorm W, const double* __restrict__ rays,
                                                         int64_t n, WormOut out, uint32_t* __restrict__ err,
                                                         unsigned long long* __restrict__ counters) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  WormCount c{0, 0, 0, 0, 0};
  if (i < n) {
    const double* r = rays + 6 * i;
    WormHit h;
    worm_trace_ray(S, W, {r[0], r[1], r[2]}, {r[3], r[4], r[5]}, h, c, err);
    if (out.status) out.status[i] = h.status;
    if (out.steps) out.steps[i] = h.steps;
    if (out.hit_entity) out.hit_entity[i] = h.status == 1 ? h.ent : -1;
    if (out.final_y)
      for (int k = 0; k < 3; k++) out.final_y[3 * i + k] = h.y[k];
    if (out.exit_dir) {
      out.exit_dir[3 * i] = h.dir2.x;
      out.exit_dir[3 * i + 1] = h.dir2.y;
      out.exit_dir[3 * i + 2] = h.dir2.z;
    }
  }
  if (counters) {
    if (i < n) atomicAdd(counters + 0, 1ull);
    atomicAdd(counters + 1, (unsigned long long)c.steps);
    atomicAdd(counters + 2, (unsigned long long)c.attempts);
    atomicAdd(counters + 3, (unsigned long long)c.segments);
  }
}

// a scene query of radiance() through the wormhole from a world-space
// origin: the hit vertex (with its world position in pw), or the colour of
// the background the ray ends on
__device__ bool worm_closest(const DevScene& S, const GWorm& W, dv3 o, float3 d, FastHit& h, Vertex& v, dv3& pw,
                             float3& miss, WormCount& c, uint32_t* err) {
  WormHit k;
  worm_trace_ray(S, W, o, {d.x, d.y, d.z}, k, c, err);
  if (k.status != 1) {
    miss = worm_background(W, k.status == 0 ? 0 : 1, k.y, S.bg);
    return false;
  }
  const GEntity& e = S.ents[k.ent];
  const dv3 o2 = dadd3(k.seg_o, dscale3(k.dir2, 0.000001));
  const dv3 p = {o2.x + k.t * k.dir2.x, o2.y + k.t * k.dir2.y, o2.z + k.t * k.dir2.z};
  float3 n;
  if (e.type == PR_ENT_SPHERE) n = normalize(f3((float)(p.x - e.p[0]), (float)(p.y - e.p[1]), (float)(p.z - e.p[2])));
  else if (e.type == PR_ENT_POLYGON) n = ld3(S.fnorm + 3 * (size_t)(e.face_base + k.prim));
  else n = f3((float)e.normal[0], (float)e.normal[1], (float)e.normal[2]);
  if (e.normal_inverse < 0) n = -n;
  pw = p;
  v.p = f3(0, 0, 0);  // relative to pw
  v.n = n;
  v.ent = k.ent;
  v.mat = e.material;
  v.t = (float)k.t;
  h.t = (float)k.t;
  h.ent = k.ent;
  h.slot = -1;
  h.u = h.v = 0.0f;
  return true;
}

// one camera sample of radiance() in a wormhole scene (no next-event
// estimation, no media: every query goes through the wormhole).  Objects
// on the far side sit more than 1e6 from the origin (the trace picks the
// mouth by that distance), where a float has a spacing of 0.125 or more:
// the next ray starts at the hit's world position in FP64, as in the
// reference (hitpoint.position), which shade() sees as the local origin 0.
__device__ float3 worm_trace_sample(const DevScene& S, const GWorm& W, const RenderCfg& cfg, float3 o0, float3 d0,
                                    uint64_t sample_id, WormCount& c, uint32_t* err) {
  PathState stack[kSplitStack];
  dv3 sorg[kSplitStack];
  int sp = 0;
  root_path(stack[sp], o0, d0);
  sorg[sp++] = {o0.x, o0.y, o0.z};
  float3 L = f3(0, 0, 0);
  while (sp > 0) {
    --sp;
    PathState ps = stack[sp];
    dv3 org = sorg[sp];
    for (;;) {
      FastHit h;
      Vertex v;
      float3 miss;
      dv3 pw;
      const bool hit = worm_closest(S, W, org, ps.d, h, v, pw, miss, c, err);
      ShadowReq sh[3];
      int nsh = 0;
      PathState child;
      const int r = shade(S, cfg, ps, hit, h, sample_id, sh, nsh, child, err, &v, &miss);
      if (r == SHADE_SPLIT) {
        if (sp < kSplitStack) {
          stack[sp] = child;
          sorg[sp++] = pw;
        } else {
          atomicOr(err, PR_DEV_LOOP_CAP);
        }
      }
      if (r == SHADE_END) break;
      org = pw;
    }
    L += ps.L;
  }
  return L;
}

__global__ void __launch_bounds__(128) worm_render_kernel(DevScene S, GWorm W, RenderCfg cfg, float* __restrict__ out,
                                                          uint32_t* __restrict__ err,
                                                          unsigned long long* __restrict__ counters) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t warp = tid >> 5, lane = tid & 31;
  const uint32_t tiles_per_chunk = cfg.tiles_x * cfg.tiles_y;
  const uint32_t chunk = warp / tiles_per_chunk;
  if (chunk >= (uint32_t)cfg.chunks) return;
  const uint32_t tile = warp - chunk * tiles_per_chunk;
  const int x = (int)((tile % cfg.tiles_x) * 8 + (lane & 7));
  const int y = (int)((tile / cfg.tiles_x) * 4 + (lane >> 3));
  WormCount c{0, 0, 0, 0, 0};
  uint32_t paths = 0;
  if (x < cfg.width && y < cfg.height) {
    const int k0 = (int)(((int64_t)cfg.spp * chunk) / cfg.chunks);
    const int k1 = (int)(((int64_t)cfg.spp * (chunk + 1)) / cfg.chunks);
    float3 acc = f3(0, 0, 0);
    for (int k = k0; k < k1; k++) {
      float3 o, d;
      const uint64_t sample_id = camera_ray(cfg, x, y, cfg.sample_offset + (uint64_t)k, o, d);
      acc += finish_sample(cfg, worm_trace_sample(S, W, cfg, o, d, sample_id, c, err), err);
      paths++;
    }
    acc = acc * cfg.sensor;
    float* po = out + 3 * ((size_t)chunk * cfg.width * cfg.height + (size_t)(cfg.height - y - 1) * cfg.width + x);
    po[0] = acc.x;
    po[1] = acc.y;
    po[2] = acc.z;
  }
  if (counters) {
    unsigned long long a = paths, b = c.segments, nn = c.nodes, tt = c.tris;
    for (int off = 16; off > 0; off >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, off);
      b += __shfl_down_sync(0xffffffffu, b, off);
      nn += __shfl_down_sync(0xffffffffu, nn, off);
      tt += __shfl_down_sync(0xffffffffu, tt, off);
    }
    if (lane == 0) {
      atomicAdd(counters + 0, a);
      atomicAdd(counters + 1, b);
      atomicAdd(counters + 2, nn);
      atomicAdd(counters + 3, tt);
    }
  }
}

}  // namespace

cudaError_t launch_worm_trace(const DevScene& S, const GWorm& W, const double* rays, int64_t n, WormOut out,
                              uint32_t* err, unsigned long long* counters, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = (n + 127) / 128;
  worm_trace_kernel<<<(unsigned)blocks, 128, 0, stream>>>(S, W, rays, n, out, err, counters);
  return cudaGetLastError();
}

cudaError_t launch_worm_render(const DevScene& S, const GWorm& W, const RenderCfg& cfg, float* partial, uint32_t* err,
                               unsigned long long* counters, cudaStream_t stream) {
  const uint64_t threads = (uint64_t)cfg.tiles_x * cfg.tiles_y * 32ull * (uint64_t)cfg.chunks;
  const uint32_t blocks = (uint32_t)((threads + 127) / 128);
  worm_render_kernel<<<blocks, 128, 0, stream>>>(S, W, cfg, partial, err, counters);
  return cudaGetLastError();
}

}  // namespace pr
