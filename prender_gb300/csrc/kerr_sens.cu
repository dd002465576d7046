// Ray-bundle Jacobian of the Kerr map (forward mode).
//
// The initial direction d of a ray is perturbed within its pixel footprint,
// d(s, t) = normalize(d + s e1 + t e2), and the FP64 tracer (the reference's
// set-up, initial momenta, geodesic equations and Cash-Karp steps, as in
// kerr_math.cuh) runs on dual numbers that carry d/ds and d/dt alongside
// every value.  The step sizes, step acceptance and the polyline's segment
// tests follow the primal trace (their dependence on s, t is the integrator's
// error, not the map's), so the tangents are the derivatives of the
// discretised map along the same steps.  For a ray that leaves the scene
// (status 0) the kernel returns d(exit direction)/d(s, t) (3 x 2) and
// d(final theta, phi)/d(s, t) (2 x 2); the adjoint form contracts the first
// with a cotangent per ray, w^T J.  Other statuses give NaN.
#include <cuda_runtime.h>

#include "kerr_math.cuh"

namespace pr {
namespace {

struct Dual {
  double v, a, b;  // value, d/ds, d/dt
};
__device__ __forceinline__ Dual mkd(double v) { return {v, 0.0, 0.0}; }
__device__ __forceinline__ Dual operator+(Dual x, Dual y) { return {x.v + y.v, x.a + y.a, x.b + y.b}; }
__device__ __forceinline__ Dual operator-(Dual x, Dual y) { return {x.v - y.v, x.a - y.a, x.b - y.b}; }
__device__ __forceinline__ Dual operator-(Dual x) { return {-x.v, -x.a, -x.b}; }
__device__ __forceinline__ Dual operator*(Dual x, Dual y) {
  return {x.v * y.v, x.a * y.v + x.v * y.a, x.b * y.v + x.v * y.b};
}
__device__ __forceinline__ Dual operator/(Dual x, Dual y) {
  const double iv = 1.0 / y.v, q = x.v * iv;
  return {q, (x.a - q * y.a) * iv, (x.b - q * y.b) * iv};
}
__device__ __forceinline__ Dual operator+(Dual x, double c) { return {x.v + c, x.a, x.b}; }
__device__ __forceinline__ Dual operator+(double c, Dual x) { return {x.v + c, x.a, x.b}; }
__device__ __forceinline__ Dual operator-(Dual x, double c) { return {x.v - c, x.a, x.b}; }
__device__ __forceinline__ Dual operator-(double c, Dual x) { return {c - x.v, -x.a, -x.b}; }
__device__ __forceinline__ Dual operator*(Dual x, double c) { return {x.v * c, x.a * c, x.b * c}; }
__device__ __forceinline__ Dual operator*(double c, Dual x) { return {x.v * c, x.a * c, x.b * c}; }
__device__ __forceinline__ Dual operator/(Dual x, double c) { return {x.v / c, x.a / c, x.b / c}; }
__device__ __forceinline__ Dual operator/(double c, Dual x) { return mkd(c) / x; }
__device__ __forceinline__ Dual& operator+=(Dual& x, Dual y) { return x = x + y; }
__device__ __forceinline__ Dual& operator-=(Dual& x, Dual y) { return x = x - y; }
__device__ __forceinline__ Dual dsin(Dual x) {
  double s, c;
  sincos(x.v, &s, &c);
  return {s, c * x.a, c * x.b};
}
__device__ __forceinline__ Dual dcos(Dual x) {
  double s, c;
  sincos(x.v, &s, &c);
  return {c, -s * x.a, -s * x.b};
}
__device__ __forceinline__ Dual dsqrt(Dual x) {
  const double r = sqrt(x.v), g = r > 0.0 ? 0.5 / r : 0.0;
  return {r, g * x.a, g * x.b};
}
__device__ __forceinline__ Dual dfabs(Dual x) { return x.v < 0.0 ? -x : x; }
__device__ __forceinline__ Dual dacos(Dual x) {
  const double g = -1.0 / sqrt(fmax(1e-300, 1.0 - x.v * x.v));
  return {acos(x.v), g * x.a, g * x.b};
}
__device__ __forceinline__ Dual datan2(Dual y, Dual x) {
  const double den = x.v * x.v + y.v * y.v, ix = den > 0.0 ? 1.0 / den : 0.0;
  return {atan2(y.v, x.v), (x.v * y.a - y.v * x.a) * ix, (x.v * y.b - y.v * x.b) * ix};
}

struct DV3 {
  Dual x, y, z;
};

// the FP64 tracer on duals (formulas of kerr_math.cuh / KerrBlackHole.h)
struct KerrRayD {
  double a, a2, M;
  Dual L, kappa;

  __device__ void geodesic(const Dual* y, Dual* dydx) const {
    const Dual r = y[0], pr = y[4], ptheta = y[5];
    const Dual r2 = r * r;
    const Dual twor = (2.0 * M) * r;
    const Dual sintheta = dsin(y[1]);
    Dual sin2 = sintheta * sintheta;
    const Dual costheta = dcos(y[1]);
    const Dual cos2 = costheta * costheta;
    const Dual sigma = r2 + a2 * cos2;
    const Dual delta = r2 - twor + a2;
    const Dual siginv = 1.0 / sigma;
    const Dual bot = 1.0 / (sigma * delta);
    if (fabs(sin2.v) < 1.0e-16) sin2 = mkd(sin2.v < 0.0 ? -1.0e-16 : 1.0e-16);
    dydx[0] = -pr * delta * siginv;
    dydx[1] = -ptheta * siginv;
    dydx[2] = -(twor * a + (sigma - twor) * L / sin2) * bot;
    dydx[3] = -(1.0 + (twor * (r2 + a2) - twor * a * L) * bot);
    dydx[4] = -(((r - 1.0) * (-kappa) + twor * (r2 + a2) - (2.0 * a) * L) * bot - 2.0 * pr * pr * (r - 1.0) * siginv);
    dydx[5] = -sintheta * costheta * (L * L / (sin2 * sin2) - a2) * siginv;
  }

  __device__ void rkstep(const Dual* y, const Dual* dydx, double h, Dual* yout, Dual* yerr) const {
    Dual ak[6], t1[6], t2[6], t3[6], t4[6], t5[6];
    for (int i = 0; i < 6; i++) {
      const Dual hd = h * dydx[i];
      t1[i] = y[i] + 0.2 * hd;
      t2[i] = y[i] + (3.0 / 40.0) * hd;
      t3[i] = y[i] + 0.3 * hd;
      t4[i] = y[i] - (11.0 / 54.0) * hd;
      t5[i] = y[i] + (1631.0 / 55296.0) * hd;
      yout[i] = y[i] + (37.0 / 378.0) * hd;
      yerr[i] = ((37.0 / 378.0) - (2825.0 / 27648.0)) * hd;
    }
    geodesic(t1, ak);
    for (int i = 0; i < 6; i++) {
      const Dual yt = h * ak[i];
      t2[i] += (9.0 / 40.0) * yt;
      t3[i] -= 0.9 * yt;
      t4[i] += 2.5 * yt;
      t5[i] += (175.0 / 512.0) * yt;
    }
    geodesic(t2, ak);
    for (int i = 0; i < 6; i++) {
      const Dual yt = h * ak[i];
      t3[i] += 1.2 * yt;
      t4[i] -= (70.0 / 27.0) * yt;
      t5[i] += (575.0 / 13824.0) * yt;
      yout[i] += (250.0 / 621.0) * yt;
      yerr[i] += ((250.0 / 621.0) - (18575.0 / 48384.0)) * yt;
    }
    geodesic(t3, ak);
    for (int i = 0; i < 6; i++) {
      const Dual yt = h * ak[i];
      t4[i] += (35.0 / 27.0) * yt;
      t5[i] += (44275.0 / 110592.0) * yt;
      yout[i] += (125.0 / 594.0) * yt;
      yerr[i] += ((125.0 / 594.0) - (13525.0 / 55296.0)) * yt;
    }
    geodesic(t4, ak);
    for (int i = 0; i < 6; i++) {
      const Dual yt = h * ak[i];
      t5[i] += (253.0 / 4096.0) * yt;
      yerr[i] -= (277.0 / 14336.0) * yt;
    }
    geodesic(t5, ak);
    for (int i = 0; i < 6; i++) {
      const Dual yt = h * ak[i];
      yout[i] += (512.0 / 1771.0) * yt;
      yerr[i] += ((512.0 / 1771.0) - 0.25) * yt;
    }
  }

  // rkqs on the primal values; the tangents ride along the accepted attempt
  __device__ double next_position(Dual* y, const Dual* dydx, double htry, uint32_t& attempts) const {
    double yscal[6];
    for (int i = 0; i < 6; i++) yscal[i] = fabs(y[i].v) + fabs(dydx[i].v * htry) + 1.0e-3;
    double errmax = 0.0, h = htry;
    Dual yerr[6], ytemp[6];
    for (int loop = 0; loop < 40; loop++) {
      rkstep(y, dydx, h, ytemp, yerr);
      attempts++;
      errmax = 0.0;
      for (int i = 0; i < 6; i++) errmax = fmax(errmax, fabs(yerr[i].v / yscal[i]));
      errmax *= 1e11;
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
    for (int i = 0; i < 6; i++) y[i] = ytemp[i];
    return hnext;
  }

  __device__ void initial(DV3 dir, Dual* y, Dual* dydx, double r0, double theta0) {
    // Cartesian::ToSpherical of the direction (vector3d.h:900-918)
    const Dual rr = dsqrt(dir.x * dir.x + dir.y * dir.y + dir.z * dir.z);
    const Dual xx = dir.x / rr, yy = dir.y / rr, zz = dir.z / rr;
    const Dual theta_obs = dacos(zz.v > 1.0 ? mkd(1.0) : (zz.v < -1.0 ? mkd(-1.0) : zz));
    Dual phi_obs = (fabs(xx.v) < 1.0e-6 && fabs(yy.v) < 1.0e-6) ? mkd(0.0) : datan2(yy, xx);
    if (phi_obs.v < 0.0) phi_obs = phi_obs + 2.0 * 3.14159265358979323846;
    const double r = y[0].v, theta = y[1].v;
    const Dual Phi = y[2] - phi_obs;
    const double cost = cos(theta), sint = sin(theta);
    const double sigma = r * r + (a * cost) * (a * cost);
    const double R = sqrt(a2 + r * r);
    const Dual sintobs = dsin(theta_obs), costobs = dcos(theta_obs);
    const Dual v = -sintobs * dcos(Phi);
    const double inv_sigma = 1.0 / sigma;
    const Dual rdot0 = (r * R * v * sint - R * R * costobs * cost) * inv_sigma;
    const Dual thetadot0 = (r * sint * costobs + R * v * cost) * inv_sigma;
    const Dual phidot0 = fabs(sint) < 1e-8 ? mkd(0.0) : sintobs * dsin(Phi) / (R * sint);
    // initial2 (KerrBlackHole.h:310-440)
    const double sintheta = sin(theta0), costheta = cos(theta0);
    double sin2 = sintheta * sintheta;
    const double cos2 = costheta * costheta;
    {
      if (sin2 < 1e-8 * 1e-8) {
        // polar start: the reference's near-pole branch (L = 0)
        const double sg = r0 * r0 + a2, dl = r0 * r0 - 2.0 * M * r0 + a2;
        const Dual e2 = (sg - 2.0 * r0) * (rdot0 * rdot0 / dl + thetadot0 * thetadot0) + dl * (phidot0 * sintheta) * (phidot0 * sintheta);
        const Dual energy = dsqrt(dfabs(e2)) + 1e-10;
        y[4] = rdot0 * sg / dl / energy;
        y[5] = thetadot0 * sg / energy;
        L = mkd(0.0);
        kappa = y[5] * y[5] + a2 * sin2;
        geodesic(y, dydx);
        return;
      }
    }
    const double r2 = r0 * r0;
    const double sg = r2 + a2 * cos2, dl = r2 - 2.0 * M * r0 + a2, s1 = sg - 2.0 * r0;
    const Dual e2 = s1 * (rdot0 * rdot0 / dl + thetadot0 * thetadot0) + dl * sin2 * phidot0 * phidot0;
    const Dual energy = dsqrt(dfabs(e2)) + 1.0e-10;
    y[4] = rdot0 * sg / dl / energy;
    y[5] = thetadot0 * sg / energy;
    L = ((sg * dl * phidot0 - 2.0 * a * r0 * energy) * sin2 / s1) / energy;
    kappa = y[5] * y[5] + a2 * sin2 + L * L / sin2;
    geodesic(y, dydx);
  }
};

__device__ __forceinline__ DV3 bl_to_cart_d(Dual r, Dual th, Dual ph, double a) {
  const Dual rr = dsqrt(r * r + a * a);
  const Dual st = dsin(th);
  return {rr * dcos(ph) * st, rr * dsin(ph) * st, r * dcos(th)};
}

}  // namespace

// one thread per ray; jac_dir: 6 per ray (row-major 3 x 2), jac_bl: 4 per ray
// (d theta / d(s,t), d phi / d(s,t)), grad (adjoint, 2 per ray) = w^T J_dir
__global__ void __launch_bounds__(128) kerr_sens_kernel(DevScene S, GKerr K, const double* __restrict__ rays,
                                                        const double* __restrict__ basis, int64_t n,
                                                        const double* __restrict__ cot, int32_t* __restrict__ status,
                                                        double* __restrict__ jac_dir, double* __restrict__ jac_bl,
                                                        double* __restrict__ grad, uint32_t* __restrict__ err) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double* r = rays + 6 * q;
  const dv3 org = {r[0], r[1], r[2]};
  // unit direction and the two perturbation axes projected off it
  double dl = sqrt(r[3] * r[3] + r[4] * r[4] + r[5] * r[5]);
  const dv3 d = {r[3] / dl, r[4] / dl, r[5] / dl};
  dv3 e1, e2;
  if (basis) {
    const double* b = basis + 6 * q;
    e1 = {b[0], b[1], b[2]};
    e2 = {b[3], b[4], b[5]};
  } else {
    const dv3 up = fabs(d.z) < 0.9 ? dv3{0.0, 0.0, 1.0} : dv3{1.0, 0.0, 0.0};
    e1 = dcross(d, up);
    const double l1 = sqrt(ddot(e1, e1));
    e1 = {e1.x / l1, e1.y / l1, e1.z / l1};
    e2 = dcross(e1, d);
  }
  const double p1 = ddot(d, e1), p2 = ddot(d, e2);
  const DV3 dir = {{d.x, e1.x - d.x * p1, e2.x - d.x * p2},
                   {d.y, e1.y - d.y * p1, e2.y - d.y * p2},
                   {d.z, e1.z - d.z * p1, e2.z - d.z * p2}};
  KerrRayD k{K.a, K.a2, K.M, mkd(0.0), mkd(0.0)};
  Dual y[6], dydx[6];
  double r0, th0, ph0;
  cart_to_bl(org.x - K.pos[0], org.y - K.pos[1], org.z - K.pos[2], K.a, r0, th0, ph0);
  y[0] = mkd(r0);
  y[1] = mkd(th0);
  y[2] = mkd(ph0);
  y[3] = y[4] = y[5] = mkd(0.0);
  int st = -1;
  uint32_t attempts = 0;
  uint64_t nodes = 0, tris = 0;
  DV3 o1 = {mkd(org.x), mkd(org.y), mkd(org.z)}, o2 = o1, dir2 = dir;
  if (r0 < K.Rhor) st = 2;
  if (st < 0) {
    k.initial(dir, y, dydx, r0, th0);
    double h_step = 2.0;
    int c = 0;
    while (c < K.max_steps) {
      double t;
      int ent, prim;
      if (exact_closest(S, {o1.x.v, o1.y.v, o1.z.v}, {dir2.x.v, dir2.y.v, dir2.z.v}, t, ent, prim, err, nodes, tris) &&
          t < 2.0) {
        st = 1;  // a hit (or the horizon): no exit direction
        break;
      }
      k.geodesic(y, dydx);
      if (fabs(h_step) < 1.0e-10) {
        st = 4;
        break;
      }
      h_step = k.next_position(y, dydx, h_step, attempts);
      if (h_step > 2.0) h_step = 2.0;
      if (y[0].v < K.Rhor) {
        st = 2;
        break;
      }
      o1 = o2;
      const DV3 qc = bl_to_cart_d(y[0], y[1], y[2], K.a);
      o2 = {qc.x + K.pos[0], qc.y + K.pos[1], qc.z + K.pos[2]};
      const DV3 dv = {o2.x - o1.x, o2.y - o1.y, o2.z - o1.z};
      const Dual len = dsqrt((dv.x * dv.x + dv.z * dv.z) + dv.y * dv.y);
      dir2 = {dv.x / len, dv.y / len, dv.z / len};
      c++;
      if (K.escape_radius > 0.0 && y[0].v > K.escape_radius) break;
    }
    if (st < 0) {
      double t;
      int ent, prim;
      st = exact_closest(S, {o2.x.v, o2.y.v, o2.z.v}, {dir2.x.v, dir2.y.v, dir2.z.v}, t, ent, prim, err, nodes, tris)
               ? 5
               : 0;
    }
  }
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const bool ok = st == 0;
  if (status) status[q] = st;
  if (jac_dir) {
    const double v[6] = {dir2.x.a, dir2.x.b, dir2.y.a, dir2.y.b, dir2.z.a, dir2.z.b};
    for (int i = 0; i < 6; i++) jac_dir[6 * q + i] = ok ? v[i] : nan;
  }
  if (jac_bl) {
    const double v[4] = {y[1].a, y[1].b, y[2].a, y[2].b};
    for (int i = 0; i < 4; i++) jac_bl[4 * q + i] = ok ? v[i] : nan;
  }
  if (grad && cot) {
    const double* w = cot + 3 * q;
    grad[2 * q] = ok ? w[0] * dir2.x.a + w[1] * dir2.y.a + w[2] * dir2.z.a : nan;
    grad[2 * q + 1] = ok ? w[0] * dir2.x.b + w[1] * dir2.y.b + w[2] * dir2.z.b : nan;
  }
}

cudaError_t launch_kerr_sensitivity(const DevScene& S, const GKerr& K, const double* rays, const double* basis,
                                    int64_t n, const double* cot, int32_t* status, double* jac_dir, double* jac_bl,
                                    double* grad, uint32_t* err, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  kerr_sens_kernel<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(S, K, rays, basis, n, cot, status, jac_dir, jac_bl,
                                                                    grad, err);
  return cudaGetLastError();
}

}  // namespace pr
