// Kerr geodesic tracer shared by the FP64 form (kerr.cu, compiled without
// FMA contraction) and the FP32 form (kerr_fast.cu): the Kerr branch of
// intersect_scene (scene.cpp:448-732) with KerrBlackHole's set-up,
// closed-form initial momenta (initial_condition 0), geodesic equations and
// Cash-Karp RK45 step control (KerrBlackHole.h:86-151, :310-440, :471-522,
// :660-852, :1239-1431).
//
// One thread traces one ray.  Each accepted RK step is followed by a
// straight-segment scene test from the previous polyline vertex.  All loops
// are bounded: at most max_steps steps per ray and 40 step-size retries per
// step.
#pragma once
#include <cuda_runtime.h>

#include "kerr.h"
#include "path_logic.cuh"

namespace pr {
namespace {


constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 6.28318530717958647692;

__device__ __forceinline__ double kclamp(double v, double lo, double hi) {  // Clamp (vector3d.h:236)
  if (v < lo) return lo;
  else if (v > hi) return hi;
  else return v;
}

// Cartesian::ToBoyerLindquist (vector3d.h:941-951)
__device__ __forceinline__ void cart_to_bl(double x, double y, double z, double a, double& r, double& th, double& ph) {
  double r0 = x * x + y * y + z * z;
  const double u = r0 - a * a;
  const double zz = 2. * a * z;
  r0 = sqrt((u + sqrt(u * u + zz * zz)) / 2.);
  th = acos(kclamp(z / r0, -1.0, 1.0));
  double phi = atan2(y / r0, x / r0);
  if (phi < 0.0) phi += kTwoPi;
  if (phi >= kTwoPi) phi = 0.0;
  r = r0;
  ph = phi;
}

// Spherical::ToBoyerLindquist (vector3d.h:888-898): BL (r, theta, phi) -> Cartesian
__device__ __forceinline__ dv3 bl_to_cart(double r, double th, double ph, double a) {
  const double rr = sqrt(r * r + a * a);
  const double sint = sin(th);
  return {rr * cos(ph) * sint, rr * sin(ph) * sint, r * cos(th)};
}

// Cartesian::ToSpherical (vector3d.h:900-918), angles only
__device__ __forceinline__ void cart_to_sph(double x, double y, double z, double& th, double& ph) {
  const double r = sqrt(x * x + y * y + z * z);
  double xx, yy, zz;
  if (r > 1.0e-16) {
    xx = x / r;
    yy = y / r;
    zz = z / r;
  } else {
    th = 0;
    ph = 0;
    return;
  }
  th = acos(kclamp(zz, -1.0, 1.0));
  double phi;
  if (fabs(xx) < 1.0e-6 && fabs(yy) < 1.0e-6) phi = 0.0;
  else phi = atan2(yy, xx);
  if (phi < 0.0) phi += 2.0 * kPi;
  if (phi >= 2.0 * kPi) phi = 0.0;
  ph = phi;
}

__device__ __forceinline__ dv3 dnormalize(dv3 v) {  // normalize (vector3d.h): v * (1 / |v|)
  const double l = sqrt((v.x * v.x + v.z * v.z) + v.y * v.y);
  const double il = 1.0 / l;
  return {v.x * il, v.y * il, v.z * il};
}

struct KerrRay {
  double a, a2, M;
  double L, kappa;

  // geodesic (KerrBlackHole.h:1239-1281)
  __device__ __forceinline__ void geodesic(const double* y, double* dydx) const {
    const double r = y[0];
    const double theta = y[1];
    const double pr = y[4];
    const double ptheta = y[5];
    const double r2 = r * r;
    const double twor = 2.0 * M * r;
    const double sintheta = sin(theta);
    double sin2 = sintheta * sintheta;
    const double costheta = cos(theta);
    const double cos2 = costheta * costheta;
    const double sigma = r2 + a2 * cos2;
    const double delta = r2 - twor + a2;
    const double sd = sigma * delta;
    const double siginv = 1.0 / sigma;
    const double bot = 1.0 / sd;
    if (fabs(sin2) < 1.0e-16) {
      if (sin2 < 0.0) sin2 = -1.0e-16;
      else sin2 = 1.0e-16;
    }
    dydx[0] = -pr * delta * siginv;
    dydx[1] = -ptheta * siginv;
    dydx[2] = -(twor * a + (sigma - twor) * L / sin2) * bot;
    dydx[3] = -(1.0 + (twor * (r2 + a2) - twor * a * L) * bot);
    dydx[4] = -(((r - 1.0) * (-kappa) + twor * (r2 + a2) - 2.0 * a * L) * bot - 2.0 * pr * pr * (r - 1.0) * siginv);
    dydx[5] = -sintheta * costheta * (L * L / (sin2 * sin2) - a2) * siginv;
  }

  // rkstep (KerrBlackHole.h:1288-1361), traceDir = +1
  __device__ __forceinline__ void rkstep(const double* y, const double* dydx, double h, double* yout,
                                         double* yerr) const {
    double ak[6], t1[6], t2[6], t3[6], t4[6], t5[6];
    h *= 1.0;
#pragma unroll
    for (int i = 0; i < 6; i++) {
      const double hdydx = h * dydx[i];
      const double yi = y[i];
      t1[i] = yi + 0.2 * hdydx;
      t2[i] = yi + (3.0 / 40.0) * hdydx;
      t3[i] = yi + 0.3 * hdydx;
      t4[i] = yi - (11.0 / 54.0) * hdydx;
      t5[i] = yi + (1631.0 / 55296.0) * hdydx;
      yout[i] = yi + (37.0 / 378.0) * hdydx;
      yerr[i] = ((37.0 / 378.0) - (2825.0 / 27648.0)) * hdydx;
    }
    geodesic(t1, ak);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      const double yt = h * ak[i];
      t2[i] += (9.0 / 40.0) * yt;
      t3[i] -= 0.9 * yt;
      t4[i] += 2.5 * yt;
      t5[i] += (175.0 / 512.0) * yt;
    }
    geodesic(t2, ak);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      const double yt = h * ak[i];
      t3[i] += 1.2 * yt;
      t4[i] -= (70.0 / 27.0) * yt;
      t5[i] += (575.0 / 13824.0) * yt;
      yout[i] += (250.0 / 621.0) * yt;
      yerr[i] += ((250.0 / 621.0) - (18575.0 / 48384.0)) * yt;
    }
    geodesic(t3, ak);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      const double yt = h * ak[i];
      t4[i] += (35.0 / 27.0) * yt;
      t5[i] += (44275.0 / 110592.0) * yt;
      yout[i] += (125.0 / 594.0) * yt;
      yerr[i] += ((125.0 / 594.0) - (13525.0 / 55296.0)) * yt;
    }
    geodesic(t4, ak);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      const double yt = h * ak[i];
      t5[i] += (253.0 / 4096.0) * yt;
      yerr[i] -= (277.0 / 14336.0) * yt;
    }
    geodesic(t5, ak);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      const double yt = h * ak[i];
      yout[i] += (512.0 / 1771.0) * yt;
      yerr[i] += ((512.0 / 1771.0) - 0.25) * yt;
    }
  }

  // NextPosition + rkqs (KerrBlackHole.h:471-522, :1366-1431): one accepted
  // step from y (escal 1e11, at most 40 shrinking retries); returns hnext
  __device__ __forceinline__ double next_position(double* y, const double* dydx, double htry,
                                                  uint32_t& attempts, double* errmax_out = nullptr) const {
    double yscal[6];
#pragma unroll
    for (int i = 0; i < 6; i++) yscal[i] = fabs(y[i]) + fabs(dydx[i] * htry) + 1.0e-3;
    const double escal = 1e11;
    double errmax = 0.0, h = htry;
    double yerr[6], ytemp[6];
    for (int loop = 0; loop < 40; loop++) {
      rkstep(y, dydx, h, ytemp, yerr);
      attempts++;
      errmax = 0.0;
#pragma unroll
      for (int i = 0; i < 6; i++) {
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
    double hnext;
    if (errmax > 1.89e-4) hnext = 0.9 * h * pow(errmax, -0.2);
    else hnext = 5.0 * h;
    if (errmax_out) *errmax_out = errmax;
#pragma unroll
    for (int i = 0; i < 6; i++) y[i] = ytemp[i];
    return hnext;
  }

  // initial2 (KerrBlackHole.h:310-440): momenta, L and kappa from (rdot, thetadot, phidot)
  __device__ __forceinline__ void initial2(double* y0, double* ydot0, double r0, double theta0) {
    y0[3] = 0;
    y0[4] = 0;
    y0[5] = 0;
    double sintheta = sin(theta0);
    const double costheta = cos(theta0);
    const double cos2 = costheta * costheta;
    double sin2 = sintheta * sintheta;
    const double POLE_THRESHOLD = 1e-8;
    if (sin2 < POLE_THRESHOLD * POLE_THRESHOLD) {
      const double sigma = r0 * r0 + a2;
      const double delta = r0 * r0 - 2.0 * M * r0 + a2;
      const double vphi_sin = ydot0[2] * sintheta;
      const double rdot0 = ydot0[0];
      const double thetadot0 = ydot0[1];
      const double energy2 =
          (sigma - 2.0 * r0) * (rdot0 * rdot0 / delta + thetadot0 * thetadot0) + delta * vphi_sin * vphi_sin;
      const double energy = sqrt(fabs(energy2)) + 1e-10;
      y0[4] = rdot0 * sigma / delta / energy;
      y0[5] = thetadot0 * sigma / energy;
      L = 0.0;
      kappa = y0[5] * y0[5] + a2 * sin2;
    } else {
      if (sin2 < 1e-16) {
        sintheta = 1e-16;
        sin2 = 1e-32;
      }
      const double rdot0 = ydot0[0];
      const double thetadot0 = ydot0[1];
      const double r2 = r0 * r0;
      const double sigma = r2 + a2 * cos2;
      const double delta = r2 - 2.0 * M * r0 + a2;
      const double s1 = sigma - 2.0 * r0;
      y0[4] = rdot0 * sigma / delta;
      y0[5] = thetadot0 * sigma;
      const double phidot0 = ydot0[2];
      const double energy2 = s1 * (rdot0 * rdot0 / delta + thetadot0 * thetadot0) + delta * sin2 * phidot0 * phidot0;
      const double energy = sqrt(fabs(energy2)) + 1.0e-10;
      y0[4] = y0[4] / energy;
      y0[5] = y0[5] / energy;
      L = ((sigma * delta * phidot0 - 2.0 * a * r0 * energy) * sin2 / s1) / energy;
      kappa = y0[5] * y0[5] + a2 * sin2 + L * L / sin2;
    }
    geodesic(y0, ydot0);
  }

  // RayToOrdinaryDifferentialEquationInitial, initial_condition 0 (KerrBlackHole.h:720-852)
  __device__ __forceinline__ void initial(dv3 dir, double* y, double* dydx, double r0, double theta0) {
    y[3] = 0;
    y[4] = 0;
    y[5] = 0;
    const double r = y[0], theta = y[1], phi = y[2];
    double theta_obs, phi_obs;
    cart_to_sph(dir.x, dir.y, dir.z, theta_obs, phi_obs);
    const double Phi = phi - phi_obs;
    const double cost = cos(theta);
    const double sintobs = sin(theta_obs);
    const double rr = r * r;
    const double sigma = rr + (a * cost) * (a * cost);
    const double R = sqrt(a2 + rr);
    const double v = -sintobs * cos(Phi);
    const double zdot = 1.;
    const double inv_sigma = 1.0 / sigma;
    const double sint = sin(theta);
    const double rdot0 = zdot * (r * R * v * sint - R * R * cos(theta_obs) * cost) * inv_sigma;
    const double thetadot0 = zdot * (r * sint * cos(theta_obs) + R * v * cost) * inv_sigma;
    double phidot0;
    if (fabs(sint) < 1e-8) phidot0 = 0.0;
    else phidot0 = zdot * sintobs * sin(Phi) / (R * sint);
    dydx[0] = rdot0;
    dydx[1] = thetadot0;
    dydx[2] = phidot0;
    initial2(y, dydx, r0, theta0);
  }
};

// result of one geodesic trace
struct KerrHit {
  int status;      // 0 background, 1 entity hit, 2 event horizon, 4 step underflow, 5 entity ahead at the end
  int steps;
  int ent, prim;   // hit entity / mesh face (status 1 and 5)
  double t;        // hit distance along the last segment
  dv3 seg_o;       // origin of the segment the hit lies on (before the 1e-6 push)
  dv3 dir2;        // last polyline direction
  double y[6];     // final state
  bool ov;         // status 1 on the accretion disk: its rewritten colour / emission
  float3 ovc, ove;
};

struct KerrCount {
  uint32_t steps, attempts, segments;
  uint64_t nodes, tris;
};

// ---- accretion disk under the black hole (circle.h:240-335) --------------
// calculateLuminance (color.h:47-49)
__device__ __forceinline__ double disk_lum(double x, double y, double z) {
  return 0.2126 * x + 0.7152 * y + 0.0722 * z;
}

// temperatureToRGB (KerrBlackHole.h:1595-1646): the reference's piecewise
// blackbody fit, temperature clamped to 1000..40000 K
__device__ inline void disk_temp_rgb(double temp, double c[3]) {
  temp = kclamp(temp, 1000.0, 40000.0);
  temp /= 100.0;
  double r, g, b;
  if (temp <= 66) r = 255;
  else r = kclamp(329.698727446 * pow(temp - 60, -0.1332047592), 0.0, 255.0);
  if (temp <= 66) g = kclamp(99.4708025861 * log(temp) - 161.1195681661, 0.0, 255.0);
  else g = kclamp(288.1221695283 * pow(temp - 60, -0.0755148492), 0.0, 255.0);
  if (temp >= 66) b = 255;
  else if (temp <= 19) b = 0;
  else b = kclamp(138.5177312231 * log(temp - 10) - 305.0447927307, 0.0, 255.0);
  c[0] = r / 255.0;
  c[1] = g / 255.0;
  c[2] = b / 255.0;
}

// wavelengthToIntensity (relativistic.h:64-81)
__device__ __forceinline__ double disk_wl(double wl, double center) {
  const double diff = wl - center;
  double it = exp(-(diff * diff) / (2.0 * 100.0 * 100.0));
  if (wl < 380.0 || wl > 750.0) it *= (wl < 380.0) ? exp(-(380.0 - wl) / 50.0) : exp(-(wl - 750.0) / 50.0);
  return it;
}

// applyDopplerShiftFull (relativistic.h:84-170): beaming D^4 blended with a
// wavelength shift of the three channels by the effect strength, in [0, 1]
__device__ inline void disk_doppler(double c[3], double d, double effect) {
  const double lam[3] = {700.0, 546.1, 435.8};
  const double f = 1.0 + (d - 1.0) * effect;
  double wl[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int src = 0; src < 3; src++) {
    const double w = lam[src] / f;
#pragma unroll
    for (int dst = 0; dst < 3; dst++) wl[dst] += c[src] * disk_wl(w, lam[dst]);
  }
  const double it = d * d * d * d;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double sh = kclamp(wl[k], 0, 1) * effect + (c[k] * it) * (1.0 - effect);
    c[k] = kclamp(sh, 0, 1);
  }
}

// The deterministic part of the disk branch at world point p: false where
// the disk is not there (inside the horizon or the ISCO, beyond its radius,
// off the texture); else colour, emission and alpha (circle.h:244-322).
__device__ inline bool kerr_disk_shade(const GKerr& K, const GEntity& e, dv3 p, double col[3], double em[3],
                                       double& alp) {
  const double rx = p.x - K.pos[0], ry = p.y - K.pos[1], rz = p.z - K.pos[2];
  double sr, sth, sph;
  cart_to_bl(rx, ry, rz, K.a, sr, sth, sph);
  if (sr < K.Rhor || sr > e.radius || !(sr >= K.Rmstable)) return false;
  // the base UVPlane's (u, v) of the hit (plane.h:228-229)
  const dv3 rel = dsub3(p, ldd3(e.p));
  const double u = ddot(rel, ldd3(e.du_axis)) / e.du_len;
  const double v = ddot(rel, ldd3(e.dv_axis)) / e.dv_len;
  // DiscMapping::MapUV (circle.h:53-77), rMin = ISCO, disk_r = the disk radius
  const double theta = atan2(u / sr, v / sr);
  const double rn = (sr - K.Rmstable) / (e.radius - K.Rmstable);
  const double fx = K.disk_w * 0.5 + K.disk_w * rn * cos(theta);
  const double fy = K.disk_h * 0.5 + K.disk_h * rn * sin(theta);
  // the int conversion truncates toward zero: in range iff -1 < f < size
  if (!(fx > -1.0 && fx < (double)K.disk_w) || !(fy > -1.0 && fy < (double)K.disk_h)) return false;
  const uchar4 t = K.disk_tex[(size_t)(int)fy * K.disk_w + (int)fx];
  const double tmp_r = sqrt((rx * rx + rz * rz) + ry * ry);
  col[0] = t.x / 255.0;
  col[1] = t.y / 255.0;
  col[2] = t.z / 255.0;
  if (K.use_temp) {
    // accretionDiskTemperatureGeom (KerrBlackHole.h:1565-1593), then
    // adjustToSourceLuminance (color.h:51-74) to 0..255 integer levels
    double temp = 0.0;
    if (tmp_r > K.Rmstable) {
      const double mdot = 0.1 * ((4.0 * kPi * 1.67262192369e-27) / (0.1 * 6.6524587158e-29));
      double inner = 1.0 - sqrt(K.Rmstable / tmp_r);
      if (inner < 0) inner = 0;
      temp = pow(mdot / (tmp_r * tmp_r * tmp_r) * inner, 0.25);
    }
    double tc[3];
    disk_temp_rgb(temp, tc);
    const double want = disk_lum(col[0], col[1], col[2]);
    const double cur = disk_lum(tc[0], tc[1], tc[2]);
    if (cur == 0.0) {
      const double v0 = (double)(int)kclamp((double)(int)round(want / 0.2126), 0, 255);
      col[0] = col[1] = col[2] = v0;
    } else {
      const double sc = want / cur;
#pragma unroll
      for (int k = 0; k < 3; k++) col[k] = kclamp((double)(int)round(tc[k] * sc), 0, 255);
    }
  }
#pragma unroll
  for (int k = 0; k < 3; k++) em[k] = e.disk_em[k] * col[k];
  alp = t.w / 255.0;
  const double cl = sqrt((col[0] * col[0] + col[2] * col[2]) + col[1] * col[1]) / 3.0;
  if (cl < alp) alp = cl;  // std::min(alpha, |colour| / 3)
  // the disk's orbital velocity (getDiskVelocity about +z with sign -1,
  // KerrBlackHole.h:1507-1531) scaled to the circular-orbit speed seen by a
  // locally non-rotating observer (circle.h:292-302)
  double vx = 0.0, vy = 0.0, vz = 0.0;
  if (!(tmp_r < 1e-6)) {
    const double vm = sqrt(1.0 / tmp_r);
    double dx = 0.0 * rz - 1.0 * ry, dy = 1.0 * rx - 0.0 * rz, dz = 0.0 * ry - 0.0 * rx;
    const double il = 1.0 / sqrt((dx * dx + dz * dz) + dy * dy);
    dx *= il;
    dy *= il;
    dz *= il;
    const double sg = vm * -1.0;
    vx = dx * sg;
    vy = dy * sg;
    vz = dz * sg;
  }
  const double a = K.a;
  const double omg = 1.0 / (pow(tmp_r, 3.0 / 2.0) + a);
  const double delt = tmp_r * tmp_r - 2.0 * tmp_r + a * a;
  const double A = pow(tmp_r, 4.0) + a * a * tmp_r * tmp_r + 2.0 * a * a * tmp_r;
  const double o = 2.0 * a * tmp_r / A;
  {
    const double il = 1.0 / sqrt((vx * vx + vz * vz) + vy * vy);
    const double m = omg - o, den = tmp_r * tmp_r * sqrt(delt);
    vx = ((vx * il) * m) * A;
    vy = ((vy * il) * m) * A;
    vz = ((vz * il) * m) * A;
    if (den == 0.0) {  // Vector3d::operator/ by zero (vector3d.h:67-75)
      vx = vy = vz = 1.0;
    } else {
      vx /= den;
      vy /= den;
      vz /= den;
    }
  }
  // calculateDopplerFactorFromObserver (KerrBlackHole.h:1534-1562)
  double dop = 1.0;
  {
    double wx = p.x - K.observer[0], wy = p.y - K.observer[1], wz = p.z - K.observer[2];
    const double iw = 1.0 / sqrt((wx * wx + wz * wz) + wy * wy);
    wx *= iw;
    wy *= iw;
    wz *= iw;
    const double beta = sqrt((vx * vx + vz * vz) + vy * vy);
    if (!(beta < 1e-6)) {
      const double ib = 1.0 / beta;
      const double cos_t = (wx * (vx * ib) + wz * (vz * ib)) + wy * (vy * ib);
      const double gamma = 1.0 / sqrt(1.0 - beta * beta);
      dop = 1.0 / (gamma * (1.0 - beta * cos_t));
    }
  }
  disk_doppler(col, dop, K.doppler_effect);
  disk_doppler(em, dop, K.doppler_effect);
  return true;
}

// exact_closest hook of the Kerr tracer: a disk_map disk is there only where
// its texture is and its alpha test passes; the closest hit on it carries the
// rewritten colour and emission.  The alpha test draws from its own stream
// (the reference draws it from the scene's generator, scene_env.h:213, :306).
struct KerrDiskShading {
  const GKerr* K;
  Rng* rng;
  bool cand, ov;
  float3 cc, ce, oc, oe;
  __device__ __forceinline__ void begin() { ov = false; }
  __device__ __forceinline__ bool circle(const GEntity& e, dv3 p) {
    cand = false;
    if (!e.kerr_disk || !K->disk_tex) return true;
    double col[3], em[3], alp;
    if (!kerr_disk_shade(*K, e, p, col, em, alp)) return false;
    if (alp == 0.0) return false;
    if (alp < 0.99 && alp <= (double)rng->next()) return false;
    cand = true;
    cc = f3((float)col[0], (float)col[1], (float)col[2]);
    ce = f3((float)em[0], (float)em[1], (float)em[2]);
    return true;
  }
  __device__ __forceinline__ void best(const GEntity& e) {
    ov = e.type == PR_ENT_CIRCLE && cand;
    oc = cc;
    oe = ce;
  }
};

// the key of the alpha-test stream: the render seed mixed with the disk seed
__device__ __forceinline__ uint64_t disk_stream_key(uint64_t seed, const GKerr& K) {
  return seed ^ (K.disk_seed * 0x9E3779B97F4A7C15ull);
}
constexpr uint32_t kDiskBranch = 0xFFFFFFFFu;  // counter lane of the alpha-test stream

// the Kerr branch of intersect_scene for one ray (scene.cpp:448-732)
template <class HS>
__device__ void kerr_trace_ray(const DevScene& S, const GKerr& K, dv3 org, dv3 dir, KerrHit& out, KerrCount& cnt,
                               uint32_t* err, HS& hs) {
  KerrRay k{K.a, K.a2, K.M, 0.0, 0.0};
  double* y = out.y;
  double dydx[6];
  const dv3 rel = {org.x - K.pos[0], org.y - K.pos[1], org.z - K.pos[2]};  // Setup (KerrBlackHole.h:153-166)
  double r0, th0, ph0;
  cart_to_bl(rel.x, rel.y, rel.z, K.a, r0, th0, ph0);
  y[0] = r0;
  y[1] = th0;
  y[2] = ph0;
  y[3] = 0;
  y[4] = 0;
  y[5] = 0;
  out.steps = 0;
  out.ov = false;
  out.ent = -1;
  out.prim = -1;
  out.t = -1.0;
  out.dir2 = dir;
  out.seg_o = org;
  if (r0 < K.Rhor) {
    out.status = 2;
    return;
  }
  k.initial(dir, y, dydx, r0, th0);
  const double h_dist = 2.0;
  double h_step = h_dist;
  dv3 org1 = org, org2 = org, dir2 = dir;
  int c = 0;
  while (c < K.max_steps) {
    double t;
    int ent, prim;
    cnt.segments++;
    if (exact_closest_hs(S, org1, dir2, t, ent, prim, err, cnt.nodes, cnt.tris, hs)) {
      if (t < h_dist) {
        // hit point of intersect_scene_: (org1 + 1e-6 dir2) + t dir2
        const dv3 o2 = dadd3(org1, dscale3(dir2, 0.000001));
        const dv3 p = {o2.x + t * dir2.x, o2.y + t * dir2.y, o2.z + t * dir2.z};
        double sr, sth, sph;
        cart_to_bl(p.x - K.pos[0], p.y - K.pos[1], p.z - K.pos[2], K.a, sr, sth, sph);
        out.steps = c;
        out.dir2 = dir2;
        out.seg_o = org1;
        if (sr < K.Rhor) {
          out.status = 2;
        } else {
          out.status = 1;
          out.ent = ent;
          out.prim = prim;
          out.t = t;
          out.ov = hs.ov;
          out.ovc = hs.oc;
          out.ove = hs.oe;
        }
        return;
      }
    }
    k.geodesic(y, dydx);
    if (fabs(h_step) < 1.0e-10) {
      out.status = 4;
      out.steps = c;
      out.dir2 = dir2;
      return;
    }
    const double r_before = y[0];
    h_step = k.next_position(y, dydx, h_step, cnt.attempts);
    if (h_step > h_dist) h_step = h_dist;
    if (y[0] < K.Rhor) {
      out.status = 2;
      out.steps = c;
      out.dir2 = dir2;
      return;
    }
    org1 = org2;
    const dv3 q = bl_to_cart(y[0], y[1], y[2], K.a);
    org2 = {q.x + K.pos[0], q.y + K.pos[1], q.z + K.pos[2]};
    dir2 = dnormalize({org2.x - org1.x, org2.y - org1.y, org2.z - org1.z});
    c++;
    cnt.steps++;
    // optional early exit (not in the reference): far out and receding
    if (K.escape_radius > 0.0 && y[0] > K.escape_radius && y[0] > r_before) break;
  }
  out.steps = c;
  out.dir2 = dir2;
  out.seg_o = org2;
  double t;
  int ent, prim;
  cnt.segments++;
  if (exact_closest_hs(S, org2, dir2, t, ent, prim, err, cnt.nodes, cnt.tris, hs)) {
    out.status = 5;
    out.ent = ent;
    out.prim = prim;
    out.t = t;
  } else {
    out.status = 0;
  }
}

// background map lookup of an escaped ray (scene.cpp:711-727; SphericalMapping::Map, circle.h:92-105)
__device__ __forceinline__ float3 kerr_background(const GKerr& K, const double* yy, const float* bg) {
  if (!K.texture) return f3(bg[0], bg[1], bg[2]);
  double y1 = yy[1] * K.map_coef[0] + K.map_coef[1];
  double y2 = yy[2] * K.map_coef[2] + K.map_coef[3];
  y1 = fmod(y1, kPi);
  y2 = fmod(y2, 2.0 * kPi);
  double phi = y2, theta = y1;
  if (phi < 0.0) phi += 2.0 * kPi;
  if (theta < 0.0) theta = -theta;
  int x = (int)(phi / (2.0 * kPi) * K.tex_w);
  x = ((x % K.tex_w) + K.tex_w) % K.tex_w;  // in range for any input, NaN included
  int yv = (int)(theta / kPi * K.tex_h);
  yv = ((yv % K.tex_h) + K.tex_h) % K.tex_h;
  const unsigned char* t = K.texture + 3 * ((size_t)yv * K.tex_w + x);
  return f3((float)(K.texture_coef * t[0] / 255.0), (float)(K.texture_coef * t[1] / 255.0),
            (float)(K.texture_coef * t[2] / 255.0));
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;
}

__device__ __forceinline__ void flush_counts(const KerrCount& c, uint32_t rays, unsigned long long* counters) {
  if (!counters) return;
  const unsigned long long a = warp_sum<unsigned long long>(rays), b = warp_sum<unsigned long long>(c.steps),
                           d = warp_sum<unsigned long long>(c.attempts),
                           e = warp_sum<unsigned long long>(c.segments);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(counters + 0, a);
    atomicAdd(counters + 1, b);
    atomicAdd(counters + 2, d);
    atomicAdd(counters + 3, e);
  }
}


// ======================================================================
// Mixed-precision form (pr_kerr.precision = PR_KERR_FP32).  GB300 runs FP32
// at 64x its FP64 rate.  This form keeps the reference's FP64 step (the same
// step control, so the same step sequence and polyline) wherever the
// integration needs it -- near the hole, at polar and radial turning points
// -- and switches to FP32 only where the reference's step is known to be the
// capped h = 2 accepted at the first attempt:
//  * far field: once a ray is outbound (dr/dlambda > 0), beyond
//    max(kFarRadius, scene radius + 2), with the last FP64 step's error
//    estimate below kFarErrmax (the estimate only falls further out), every
//    further step is h = 2 computed in FP32 and added to the FP64 state (the
//    reference accepts exactly these steps: errmax << 0.59 keeps hnext above
//    the cap); no segment test is needed there, nothing of the scene is
//    ahead of an outbound ray beyond the scene radius;
//  * capture: a ray inbound inside the innermost scene geometry whose radial
//    potential R(r) = ((r^2 + a^2) - a L)^2 - Delta (kappa - 2 a L) stays
//    positive down to the horizon has no turning point left; the reference
//    steps it on until its step size underflows (status 4, "no hit"), this
//    form reports that outcome at once.
// Status, steps to the far field, hits and exit directions follow the FP64
// form; the FP32 far-field steps differ from the reference's in rounding only.
// ======================================================================
constexpr double kFarRadius = 200.0;  // M
constexpr double kFarErrmax = 1.0e-3;
constexpr double kPoleSin2 = 1.0e-4;

struct KerrRayF {
  float a, a2, M;
  float L, kappa;

  // geodesic (KerrBlackHole.h:1239-1281) in FP32
  __device__ __forceinline__ void geodesic(const float* y, float* dydx) const {
    const float r = y[0], pr = y[4], ptheta = y[5];
    const float r2 = r * r;
    const float twor = 2.0f * M * r;
    float sintheta, costheta;
    sincosf(y[1], &sintheta, &costheta);
    float sin2 = sintheta * sintheta;
    const float cos2 = costheta * costheta;
    const float sigma = r2 + a2 * cos2;
    const float delta = r2 - twor + a2;
    const float siginv = 1.0f / sigma;
    const float bot = 1.0f / (sigma * delta);
    if (fabsf(sin2) < 1.0e-16f) sin2 = 1.0e-16f;
    const float r2a2 = r2 + a2;
    dydx[0] = -pr * delta * siginv;
    dydx[1] = -ptheta * siginv;
    dydx[2] = -(twor * a + (sigma - twor) * L / sin2) * bot;
    dydx[3] = -(1.0f + (twor * r2a2 - twor * a * L) * bot);
    dydx[4] = -(((r - 1.0f) * (-kappa) + twor * r2a2 - 2.0f * a * L) * bot - 2.0f * pr * pr * (r - 1.0f) * siginv);
    dydx[5] = -sintheta * costheta * (L * L / (sin2 * sin2) - a2) * siginv;
  }

  // one Cash-Karp step of size h in FP32, as increments dy = y_out - y
  __device__ __forceinline__ void step(const float* y, const float* dydx, float h, float* dy) const {
    float ak[6], t[6], k1[6], k2[6], k3[6], k4[6], k6[6];
#pragma unroll
    for (int i = 0; i < 6; i++) {
      k1[i] = h * dydx[i];
      t[i] = y[i] + 0.2f * k1[i];
    }
    geodesic(t, ak);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      k2[i] = h * ak[i];
      t[i] = y[i] + (3.0f / 40.0f) * k1[i] + (9.0f / 40.0f) * k2[i];
    }
    geodesic(t, ak);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      k3[i] = h * ak[i];
      t[i] = y[i] + 0.3f * k1[i] - 0.9f * k2[i] + 1.2f * k3[i];
    }
    geodesic(t, ak);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      k4[i] = h * ak[i];
      t[i] = y[i] - (11.0f / 54.0f) * k1[i] + 2.5f * k2[i] - (70.0f / 27.0f) * k3[i] + (35.0f / 27.0f) * k4[i];
    }
    geodesic(t, ak);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      const float k5 = h * ak[i];
      t[i] = y[i] + (1631.0f / 55296.0f) * k1[i] + (175.0f / 512.0f) * k2[i] + (575.0f / 13824.0f) * k3[i] +
             (44275.0f / 110592.0f) * k4[i] + (253.0f / 4096.0f) * k5;
    }
    geodesic(t, ak);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      k6[i] = h * ak[i];
      dy[i] = (37.0f / 378.0f) * k1[i] + (250.0f / 621.0f) * k3[i] + (125.0f / 594.0f) * k4[i] +
              (512.0f / 1771.0f) * k6[i];
    }
  }
};

// R(r) of the radial motion (E = 1): ((r^2 + a^2) - a L)^2 - Delta (kappa - 2 a L),
// where the reference's kappa = p_theta^2 + a^2 sin^2 + L^2 / sin^2 = Q + L^2 + a^2
__device__ __forceinline__ double radial_potential(double r, double a, double L, double kappa) {
  const double w = r * r + a * a - a * L;
  const double delta = r * r - 2.0 * r + a * a;
  return w * w - delta * (kappa - 2.0 * a * L);
}

// no turning point between the horizon and r: R > 0 on a fine grid of [r+, r]
__device__ __forceinline__ bool no_turning_point(double r, double rplus, double a, double L, double kappa) {
  const int n = 64;
  for (int i = 0; i <= n; i++) {
    const double rr = rplus + (r - rplus) * (double)i / n;
    if (!(radial_potential(rr, a, L, kappa) > 0.0)) return false;
  }
  return true;
}

// the Kerr branch of intersect_scene, mixed precision (see above)
template <class HS>
__device__ void kerr_trace_ray_fast(const DevScene& S, const GKerr& K, dv3 org, dv3 dir, KerrHit& out, KerrCount& cnt,
                                    uint32_t* err, HS& hs, bool capture_shortcut) {
  KerrRay k{K.a, K.a2, K.M, 0.0, 0.0};
  double* y = out.y;
  double dydx[6];
  const dv3 rel = {org.x - K.pos[0], org.y - K.pos[1], org.z - K.pos[2]};
  double r0, th0, ph0;
  cart_to_bl(rel.x, rel.y, rel.z, K.a, r0, th0, ph0);
  y[0] = r0;
  y[1] = th0;
  y[2] = ph0;
  y[3] = 0;
  y[4] = 0;
  y[5] = 0;
  out.steps = 0;
  out.ov = false;
  out.ent = -1;
  out.prim = -1;
  out.t = -1.0;
  out.dir2 = dir;
  out.seg_o = org;
  if (r0 < K.Rhor) {
    out.status = 2;
    return;
  }
  k.initial(dir, y, dydx, r0, th0);
  const KerrRayF kf{(float)K.a, (float)K.a2, (float)K.M, (float)k.L, (float)k.kappa};
  const double far = fmax(kFarRadius, K.scene_radius + 2.0);
  const double rplus = K.M + sqrt(K.M * K.M - K.a2);
  bool capture_checked = false;
  const double h_dist = 2.0;
  double h_step = h_dist;
  double errmax = 1.0;
  dv3 org1 = org, org2 = org, dir2 = dir;
  double yprev[3] = {y[0], y[1], y[2]};
  bool far_mode = false;
  int c = 0;
  while (c < K.max_steps) {
    if (!far_mode) {
      double t;
      int ent, prim;
      cnt.segments++;
      if (exact_closest_hs(S, org1, dir2, t, ent, prim, err, cnt.nodes, cnt.tris, hs)) {
        if (t < h_dist) {
          const dv3 o2 = dadd3(org1, dscale3(dir2, 0.000001));
          const dv3 p = {o2.x + t * dir2.x, o2.y + t * dir2.y, o2.z + t * dir2.z};
          double sr, sth, sph;
          cart_to_bl(p.x - K.pos[0], p.y - K.pos[1], p.z - K.pos[2], K.a, sr, sth, sph);
          out.steps = c;
          out.dir2 = dir2;
          out.seg_o = org1;
          if (sr < K.Rhor) {
            out.status = 2;
          } else {
            out.status = 1;
            out.ent = ent;
            out.prim = prim;
            out.t = t;
            out.ov = hs.ov;
            out.ovc = hs.oc;
            out.ove = hs.oe;
          }
          return;
        }
      }
    }
    if (far_mode) {
      const float stf = sinf((float)y[1]);
      if (stf * stf < (float)kPoleSin2) far_mode = false;  // a pole ahead: the reference's steps again
    }
    if (!far_mode) {
      k.geodesic(y, dydx);
      if (fabs(h_step) < 1.0e-10) {
        out.status = 4;
        out.steps = c;
        out.dir2 = dir2;
        return;
      }
    }
    const double r_before = y[0];
    if (capture_shortcut && !far_mode && !capture_checked && dydx[0] < 0.0 && y[0] < K.scene_inner) {
      // inbound inside all scene geometry: captured if no turning point is
      // left.  The reference ends such a ray with a step underflow (status 4)
      // or inside the horizon (2); the shortcut reports 4, so it is taken only
      // where the two look alike
      capture_checked = true;
      if (no_turning_point(y[0], rplus, K.a, k.L, k.kappa)) {
        out.status = 4;
        out.steps = c;
        out.dir2 = dir2;
        return;
      }
    }
    for (int i = 0; i < 3; i++) yprev[i] = y[i];
    if (far_mode) {
      float yf[6], df[6], dy[6];
#pragma unroll
      for (int i = 0; i < 6; i++) yf[i] = (float)y[i];
      kf.geodesic(yf, df);
      kf.step(yf, df, (float)h_dist, dy);
#pragma unroll
      for (int i = 0; i < 6; i++) y[i] += (double)dy[i];
      cnt.attempts++;
      h_step = h_dist;
    } else {
      h_step = k.next_position(y, dydx, h_step, cnt.attempts, &errmax);
      if (h_step > h_dist) h_step = h_dist;
      if (y[0] < K.Rhor) {
        out.status = 2;
        out.steps = c;
        out.dir2 = dir2;
        return;
      }
      org1 = org2;
      const dv3 q = bl_to_cart(y[0], y[1], y[2], K.a);
      org2 = {q.x + K.pos[0], q.y + K.pos[1], q.z + K.pos[2]};
      dir2 = dnormalize({org2.x - org1.x, org2.y - org1.y, org2.z - org1.z});
      const double st = sin(y[1]);
      if (y[0] > far && y[0] > r_before && errmax < kFarErrmax && h_step == h_dist && st * st >= kPoleSin2)
        far_mode = true;
    }
    c++;
    cnt.steps++;
    if (K.escape_radius > 0.0 && y[0] > K.escape_radius && y[0] > r_before) break;
  }
  if (far_mode) {
    // the polyline's last vertex and chord, in FP64, from the last two states
    const dv3 q1 = bl_to_cart(yprev[0], yprev[1], yprev[2], K.a);
    const dv3 q2 = bl_to_cart(y[0], y[1], y[2], K.a);
    org2 = {q2.x + K.pos[0], q2.y + K.pos[1], q2.z + K.pos[2]};
    dir2 = dnormalize({q2.x - q1.x, q2.y - q1.y, q2.z - q1.z});
  }
  out.steps = c;
  out.dir2 = dir2;
  out.seg_o = org2;
  double t;
  int ent, prim;
  cnt.segments++;
  if (exact_closest_hs(S, org2, dir2, t, ent, prim, err, cnt.nodes, cnt.tris, hs)) {
    out.status = 5;
    out.ent = ent;
    out.prim = prim;
    out.t = t;
  } else {
    out.status = 0;
  }
}

template <bool FAST>
__global__ void __launch_bounds__(128) kerr_trace_kernel(DevScene S, GKerr K, const double* __restrict__ rays,
                                                         int64_t n, KerrOut out, uint32_t* __restrict__ err,
                                                         unsigned long long* __restrict__ counters) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  KerrCount c{0, 0, 0, 0, 0};
  uint32_t rays_done = 0;
  if (i < n) {
    const double* r = rays + 6 * i;
    KerrHit h;
    Rng drng;
    drng.init(disk_stream_key(0, K), (uint64_t)i, kDiskBranch);
    KerrDiskShading hs{&K, &drng};
    if (FAST) kerr_trace_ray_fast(S, K, {r[0], r[1], r[2]}, {r[3], r[4], r[5]}, h, c, err, hs, true);
    else kerr_trace_ray(S, K, {r[0], r[1], r[2]}, {r[3], r[4], r[5]}, h, c, err, hs);
    if (out.status) out.status[i] = h.status;
    if (out.steps) out.steps[i] = h.steps;
    if (out.final_bl) {
      out.final_bl[3 * i] = h.y[0];
      out.final_bl[3 * i + 1] = h.y[1];
      out.final_bl[3 * i + 2] = h.y[2];
    }
    if (out.exit_dir) {
      out.exit_dir[3 * i] = h.dir2.x;
      out.exit_dir[3 * i + 1] = h.dir2.y;
      out.exit_dir[3 * i + 2] = h.dir2.z;
    }
    if (out.hit_entity) out.hit_entity[i] = h.ent;
    if (out.hit_t) out.hit_t[i] = h.t;
    rays_done = 1;
  }
  flush_counts(c, rays_done, counters);
}

// A closest-hit query of the renderer along a geodesic: on a hit, the vertex
// the straight-ray tracer would build from the last segment; on a miss, the
// colour radiance() returns (horizon black, background map or BACKGROUND).
template <bool FAST>
__device__ bool kerr_closest(const DevScene& S, const GKerr& K, float3 o, float3 d, FastHit& h, Vertex& v,
                             float3& miss, float3 ovr[2], bool& has_ovr, KerrCount& c, uint32_t* err, Rng& drng) {
  KerrHit k;
  KerrDiskShading hs{&K, &drng};
  // a captured ray's colour: black (horizon) or BACKGROUND (step underflow)
  // are the same only on a black background
  const bool black_bg = S.bg[0] == 0.0f && S.bg[1] == 0.0f && S.bg[2] == 0.0f;
  if (FAST) kerr_trace_ray_fast(S, K, {o.x, o.y, o.z}, {d.x, d.y, d.z}, k, c, err, hs, black_bg);
  else kerr_trace_ray(S, K, {o.x, o.y, o.z}, {d.x, d.y, d.z}, k, c, err, hs);
  has_ovr = false;
  if (k.status != 1) {
    if (k.status == 2) miss = f3(0, 0, 0);
    else if (k.status == 0) miss = kerr_background(K, k.y, S.bg);
    else miss = f3(S.bg[0], S.bg[1], S.bg[2]);
    return false;
  }
  const GEntity& e = S.ents[k.ent];
  const dv3 o2 = dadd3(k.seg_o, dscale3(k.dir2, 0.000001));
  const dv3 p = {o2.x + k.t * k.dir2.x, o2.y + k.t * k.dir2.y, o2.z + k.t * k.dir2.z};
  float3 n;
  if (e.type == PR_ENT_SPHERE) {
    n = normalize(f3((float)(p.x - e.p[0]), (float)(p.y - e.p[1]), (float)(p.z - e.p[2])));
  } else if (e.type == PR_ENT_POLYGON) {
    n = ld3(S.fnorm + 3 * (size_t)(e.face_base + k.prim));
  } else {
    n = f3((float)e.normal[0], (float)e.normal[1], (float)e.normal[2]);
  }
  if (e.normal_inverse < 0) n = -n;
  v.p = f3((float)p.x, (float)p.y, (float)p.z);
  v.n = n;
  v.ent = k.ent;
  v.mat = e.material;
  v.t = (float)k.t;
  if (k.ov) {  // the accretion disk's own colour and emission at this point
    has_ovr = true;
    ovr[0] = k.ovc;
    ovr[1] = k.ove;
  }
  h.t = (float)k.t;
  h.ent = k.ent;
  h.slot = -1;
  h.u = h.v = 0.0f;
  return true;
}

// one camera sample of radiance() in a Kerr scene (no next-event estimation,
// no media: every query is a geodesic, as intersect_scene makes it)
template <bool FAST>
__device__ float3 kerr_trace_sample(const DevScene& S, const GKerr& K, const RenderCfg& cfg, float3 o0, float3 d0,
                                    uint64_t sample_id, KerrCount& c, uint32_t* err) {
  PathState stack[kSplitStack];
  int sp = 0;
  root_path(stack[sp++], o0, d0);
  float3 L = f3(0, 0, 0);
  Rng drng;  // the accretion disk's alpha tests of this camera sample
  drng.init(disk_stream_key(cfg.seed, K), sample_id, kDiskBranch);
  while (sp > 0) {
    PathState ps = stack[--sp];
    for (;;) {
      FastHit h;
      Vertex v;
      float3 miss, ovr[2];
      bool has_ovr;
      const bool hit = kerr_closest<FAST>(S, K, ps.o, ps.d, h, v, miss, ovr, has_ovr, c, err, drng);
      ShadowReq sh[3];
      int nsh = 0;
      PathState child;
      const int r = shade(S, cfg, ps, hit, h, sample_id, sh, nsh, child, err, &v, &miss, nullptr, nullptr,
                          has_ovr ? ovr : nullptr);
      if (r == SHADE_SPLIT) {
        if (sp < kSplitStack) stack[sp++] = child;
        else atomicOr(err, PR_DEV_LOOP_CAP);
      }
      if (r == SHADE_END) break;
    }
    L += ps.L;
  }
  return L;
}

template <bool FAST>
__global__ void __launch_bounds__(128) kerr_render_kernel(DevScene S, GKerr K, RenderCfg cfg, float* __restrict__ out,
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
  KerrCount c{0, 0, 0, 0, 0};
  uint32_t paths = 0;
  if (x < cfg.width && y < cfg.height) {
    const int k0 = (int)(((int64_t)cfg.spp * chunk) / cfg.chunks);
    const int k1 = (int)(((int64_t)cfg.spp * (chunk + 1)) / cfg.chunks);
    float3 acc = f3(0, 0, 0);
    for (int k = k0; k < k1; k++) {
      float3 o, d;
      const uint64_t sample_id = camera_ray(cfg, x, y, cfg.sample_offset + (uint64_t)k, o, d);
      acc += finish_sample(cfg, kerr_trace_sample<FAST>(S, K, cfg, o, d, sample_id, c, err), err);
      paths++;
    }
    acc = acc * cfg.sensor;
    float* po = out + 3 * ((size_t)chunk * cfg.width * cfg.height + (size_t)(cfg.height - y - 1) * cfg.width + x);
    po[0] = acc.x;
    po[1] = acc.y;
    po[2] = acc.z;
  }
  flush_counts(c, paths, counters);
}


}  // namespace
}  // namespace pr
