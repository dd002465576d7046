// CPU restatement of prender's radiance estimator — TEST INFRASTRUCTURE ONLY.
//
// The oracle the GPU path is checked against.  Every function cites the
// reference file:line it restates (paths inside Sanaxen/prender, proj/).  It
// is loaded only by tests/, the smoke check and bench.py's CPU-baseline leg;
// the product never links or calls it.
//
// Arithmetic is FP64 in the reference's own operation order (see
// oracle_math.h), so that with one thread and the same MT19937-64 seeds the
// images equal the reference's bit for bit.
#include <omp.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../include/prender_gpu.h"
#include "oracle_math.h"

using namespace orc;

namespace {

// ---------------------------------------------------------------- materials
struct Medium {  // ParticipatingMediaPrm.h:85-131 (fields used on the path)
  double scattering = 0, absorbing = 0, transmittance = 0;
  V3 scatteringColor, absorbingColor, transmittanceColor, albedoColor;
  double phase[3] = {0, 0, 0};
  double eta = 0, r_max = 1;
  int level = -1, use_bssrdf = 1;
  // setup_Scattering (ParticipatingMediaPrm.h:133-160)
  void setup(double material_scale) {
    scatteringColor = scatteringColor * material_scale;
    absorbingColor = absorbingColor * material_scale;
    scattering = (scatteringColor.x + scatteringColor.y + scatteringColor.z) / 3;
    absorbing = (absorbingColor.x + absorbingColor.y + absorbingColor.z) / 3;
    transmittance = scattering + absorbing;
    transmittanceColor = scatteringColor + absorbingColor;
    if (transmittance < 1.0e-12) {
      scattering = 0;
      absorbing = 0;
      transmittance = 0.0;
      scatteringColor = V3(1.0, 1.0, 1.0);
      absorbingColor = V3(1.0, 1.0, 1.0);
      albedoColor = V3(1.0, 1.0, 1.0);
    } else {
      albedoColor = V3(scatteringColor.x / transmittanceColor.x, scatteringColor.y / transmittanceColor.y,
                       scatteringColor.z / transmittanceColor.z);
    }
    // channel-sampling table of the absorbing coefficients (k = 1,
    // SAMPLE_ABSORBING, the one the subsurface walk samples): the largest
    // channel, the smallest absorbing channel, one in between (the
    // reference takes the minimum over absorbingColor for every k)
    const V3 sa = absorbingColor;
    double max_s = -9999999.0, min_s = 9999999.0;
    max_i = -1;
    min_i = -1;
    for (int i = 0; i < 3; i++) {
      if (max_s < sa[i]) { max_s = sa[i]; max_i = i; }
      if (min_s > absorbingColor[i]) { min_s = absorbingColor[i]; min_i = i; }
    }
    mid_i = -1;
    for (int i = 0; i < 3; i++)
      if (max_s > sa[i] && min_s < sa[i]) { mid_i = i; break; }
    if (mid_i == -1) {
      const double av = (absorbingColor.x + absorbingColor.y + absorbingColor.z) / 3;
      const double mx = std::max(std::max(sa.x, sa.y), sa.z), mn = std::min(std::min(sa.x, sa.y), sa.z);
      mid_i = (std::fabs(mx - av) < std::fabs(mn - av)) ? max_i : min_i;
    }
    t_sum = sa[0] + sa[1] + sa[2];
    if (t_sum > 1.0e-14) {
      t_[0] = sa[min_i] / t_sum;
      t_[1] = sa[mid_i] / t_sum;
      t_[2] = sa[max_i] / t_sum;
    } else {
      t_[0] = t_[1] = t_[2] = 1.0 / 3.0;
    }
  }
  int max_i = 0, min_i = 0, mid_i = 0;
  double t_sum = 0, t_[3] = {1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0};
  // ParticipatingMedia::sample(u, SAMPLE_ABSORBING, inv) (ParticipatingMediaPrm.h:251-279)
  int sample(double u, int inv) const {
    if (t_sum < 1.0e-14) return std::min(2, (int)(3.0 * u));
    int ii = 0;
    if (inv) ii = min_i;
    if (u < t_[0]) ii = min_i;
    else if (u < t_[0] + t_[1]) ii = mid_i;
    else if (u < t_[0] + t_[1] + t_[2]) ii = max_i;
    if (inv) {
      if (-u < -t_[0]) ii = min_i;
      else if (-u < -t_[0] - t_[1]) ii = mid_i;
      else if (-u < -t_[0] - t_[1] - t_[2]) ii = max_i;
    }
    return ii;
  }
  // transmittanceRatio (ParticipatingMediaPrm.h:336-340)
  V3 tr(double d) const { return vexp(-1.0 * transmittanceColor * d); }
};

struct Material {  // material.h:54-240
  int type = PR_MAT_DIFFUSE;
  V3 color, emission, specular;
  double roughness = 0.0;
  double refractive_index = 1.5;
  double r_refractive_index = 1.0;  // relative index of the subsurface medium (material.h:81)
  int disk_map = 0;                 // 'disk_map' (scene_env.h:1163-1169)
  double ward_ax = 0, ward_ay = 0;  // brdfParameter.ward_brdf (material.h:42-47)
  double phong_n = 0;               // brdfParameter.phong_brdf.specular_exponent
  Medium medium;
  // texture (BitMap cell(i, j) RGB) and IBL image (IBL_Color(i, j) as doubles)
  // (shared: hit_mat copies the material per hit)
  std::shared_ptr<const std::vector<unsigned char>> tex;
  int tex_w = 0, tex_h = 0;
  std::shared_ptr<const std::vector<double>> ibl;
  int ibl_w = 0, ibl_h = 0;
  double ibl_coef = 1.0;
  int repeat = 1;
  int map_flags = 0;
  std::shared_ptr<const std::vector<unsigned char>> bump;  // bump_texture (cell(i, j) RGB), square
  int bump_w = 0, bump_h = 0;
  // Material::isLight (material.h): diffuse, dark, emissive
  bool isLight() const {
    return type == PR_MAT_DIFFUSE && length(color) < 0.001 && length(emission) > 0.001;
  }
};

// ------------------------------------------------------------------ entities
struct Hit {  // IntersectionPos (intersection.h:11-30) + object_id
  double distance = INF;
  V3 normal, position;
  int material = -1;
  int object_id = -1;
  int prim = -1;
  // the hit point's own copy of the material when the entity rewrote it
  // (the accretion disk's texture and Doppler shift, circle.h:264-311)
  bool ov = false;
  V3 ov_color, ov_emission;
  bool ov_spec = false;  // a texture also rewrote the specular colour
  V3 ov_specular;
  bool bump = false;     // IntersectionPos::bump / bump_new_normal
  V3 bump_n;
  bool ov_full = false;  // the hit's whole material copy (a face's OBJ material)
  Material ovm;
};

struct Mesh {
  std::vector<float> vert;   // ObjLoader vert (float)
  std::vector<int> face;     // 0-based
  std::vector<float> fnorm;  // face normals (float, ObjLoader.cpp:577-700)
  std::vector<float> norm;   // vertex normals (float): the vn lines, or the loader's rule
  std::vector<int> norm_id;  // 3 per face
  std::vector<float> uv;     // vt lines (2 per entry)
  std::vector<int> uv_id;    // 3 per face (empty: no vt lines)
  struct ObjMat {            // ObjMaterial (ObjLoader.h:94-150)
    V3 diffuse, specular, emission;
    double alpha = -1.0, ni = 0.0, ns = 5.0, rough = 0.0, ward[2] = {0, 0};
    int refl = -1, smooth = 0, repeat = 1;
    std::vector<unsigned char> tex;  // map_Kd (RGB, cell(i, j))
    int tw = 0, th = 0;
  };
  std::vector<ObjMat> omats;
  std::vector<int> face_omat;  // per face, -1: none (empty: no usemtl)
};

struct Tri {  // Triangle (polygon.h:22-708)
  int mesh, face;
  V3 bmin, bmax, center;  // padded bounding box and its centre
};

struct BVHNode {  // BVH_structure (BVH.h:18-28)
  double box[2][3];
  int children[2] = {-1, -1};
  int axis = 0;
  std::vector<int> objects;  // triangle indices (leaf only)
};

struct QNode {  // QBVH_structure (QBVH.h:53-61)
  float bboxes[2][3][4];
  int64_t children[4];
  int axis_top, axis_left, axis_right;
};

constexpr int64_t QTOP = (int64_t)1 << 63;  // QBVH_TOP_BIT with 64-bit long (QBVH.h:11)

struct QBVH {
  std::vector<QNode> nodes;
  std::vector<int> leaf;  // triangle index, -1 = terminator
};

struct Entity {
  int type = 0, material = -1, normal_inverse = 1;
  // sphere
  V3 position;
  double radius = 0;
  int hemisphere = 0;  // 'hemisphere': the half with y >= 0 about the centre
  // uvplane (plane.h:129-167)
  V3 org, u_axis, v_axis, normal;
  double u_length = 0, v_length = 0;
  // circle (disk): its base UVPlane keeps normal_vector_inverse 1 (circle.h:117-130)
  double radius_inner = 0;
  V3 base_normal;
  V3 du_axis, dv_axis;          // the base UVPlane's unit axes and lengths (plane.h:146-167)
  double du_len = 0, dv_len = 0;
  int blackhole_disk = 0;       // accretion-disk texture index (0 by default, scene_env.h:271)
  // mesh
  int mesh = -1;
  int smooth = 0;  // Mesh::smooth ('smooth' of the OBJECT block)
  std::vector<Tri> tris;
  QBVH qbvh;
  double area = INF;
  bool light = false;
  int light_id = -1;
  V3 bb_min, bb_max;  // Entity::boundingBox (CreateBoundingBox of the entity type)
};

struct Light {  // light.h:13-74
  double power = 0;
  int entity = -1;   // Light::light; an infinity light has none
  int parallel = 0, spot = 0, infinity = 0;
  V3 dir;            // parallel / spot direction; infinity light: as given
  // spot light (light.h:36-46 defaults): cosTotalWidth, cosFalloffStart
  double cos_total = 0, cos_start = 0;
  double falloff = 2.0;
  double att[3] = {1.0, 0.0, 0.0};
  V3 inf_emission;   // infinity_light_emitssin
  V3 center;         // spot: the sphere's centre
  // SpotLightFalloff (light.h:52-63)
  double spot_falloff(V3 w) const {
    const double costheta = dot(dir, w);
    if (costheta < cos_total) return 0.0;
    if (costheta > cos_start) return 1.0;
    const double delta = (costheta - cos_total) / (cos_start - cos_total);
    return std::pow(delta, falloff);
  }
  // SpotLightEmission (light.h:64-73)
  V3 spot_emission(V3 intensity, V3 light_pos, V3 p) const {
    const V3 wi = normalize(light_pos - p);
    const double dist = length(light_pos - p);
    double inv_a = att[0] + dist * (att[1] + att[2] * dist);
    if (inv_a < 1.0e-3) inv_a = 1.0;
    return intensity * spot_falloff(wi * -1.0) / inv_a;
  }
};

struct KerrBH {  // KerrBlackHole (KerrBlackHole.h:86-151) with M = 1, initial_condition 0
  bool on = false;
  V3 position;
  double a = 0, a2 = 0, M = 1.0, Rhor = 0;
  int max_steps = 10000;
  double map_coef[4] = {1, 0, 1, 0};
  double escape_radius = 0;  // 0: the reference's exit by step count only
  std::vector<unsigned char> texture;  // background map, RGB8, cell(y, x) = texture[3 (y W + x)]
  int tex_w = 0, tex_h = 0;
  double texture_coef = 1.0;
  // accretion disk (circle.h:240-335)
  double Rmstable = 0;                  // inner_orbit() (KerrBlackHole.h:215-240)
  int use_temperature = 0;
  double doppler_effect = 0;            // color_doppler_factor_effect
  V3 observer;                          // camera_pos
  std::vector<unsigned char> disk_tex;  // RGBA8, cell(y, x) = disk_tex[4 (y W + x)]
  int disk_w = 0, disk_h = 0;
  uint64_t disk_seed = 0;
};

struct Wormhole {  // WormHole (WormHole.h:126-540) as SceneEnv builds it (scene_env.h:2100-2145)
  bool on = false;
  V3 pos0, pos1;       // position0 ('in'), position1 ('out')
  double Rho = 0, a = 0, M = 1, W = 0;
  int max_steps = 10000;
  int usr_sign = 0;
  V3 camera;
  std::vector<unsigned char> tex[2];
  int tex_w[2] = {0, 0}, tex_h[2] = {0, 0};
  double map_coef[2][4] = {{1, 0, 1, 0}, {1, 0, 1, 0}};
  double tex_coef[2] = {1, 1};
};

struct Scene {
  Wormhole worm;
  KerrBH kerr;
  std::vector<Material> mats;
  std::vector<Entity> ents;
  std::vector<Mesh> meshes;
  std::vector<Light> lights;
  V3 background, env_light;
  Medium medium;
  int media_on = 0;
};

thread_local uint64_t tl_nodes = 0, tl_tris = 0, tl_segments = 0;

// -------------------------------------------------------------- primitives
// Sphere::intersect core (sphere.h:68-96)
// (int) of a double as x86-64's cvttsd2si gives it: NaN and values out of
// range become INT_MIN (the reference's texel indices take NaN at the poles)
inline int trunc_int(double x) {
  if (!(x > -2147483649.0 && x < 2147483648.0)) return INT32_MIN;
  return (int)x;
}

// the repeat wrap of a texture coordinate (sphere.h:189-196, plane.h:241-248)
inline double wrap01(double x) {
  double dmy;
  if (x < 0 || x > 1) x = std::modf(x, &dmy);
  if (x < 0) x = 1.0 - std::fabs(x);
  return x;
}

inline void texel_rgb(const Material& m, int i, int j, V3& c) {
  const unsigned char* t = &(*m.tex)[3 * ((size_t)i * m.tex_w + j)];
  c = V3((double)t[0] / 255.0, (double)t[1] / 255.0, (double)t[2] / 255.0);
}

inline V3 ibl_rgb(const Material& m, int i, int j) {
  const double* t = &(*m.ibl)[3 * ((size_t)i * m.ibl_w + j)];
  return V3(t[0], t[1], t[2]);
}

// the bump normal from the central luminance differences around texel
// (i, j) of a square bump map (sphere.h:411-492, plane.h:290-360; the
// reference wraps the row above the first to W - 1, which a square map keeps
// in range): n + (n x tdir) gx - (n x sdir) gy with n the entity's own
// normal (before its inversion) and g the differences times 0.5 * scale
void bump_normal(const Material& m, int i, int j, V3 n, V3 sdir, V3 tdir, double scale, Hit& h) {
  int u0 = j - 1, u1 = j + 1, v0 = i - 1, v1 = i + 1;
  if (u0 < 0) u0 = m.bump_w - 1;
  if (v0 < 0) v0 = m.bump_w - 1;
  if (u1 < 0) u1 = m.bump_h - 1;
  if (v1 < 0) v1 = m.bump_h - 1;
  if (u0 >= m.bump_w) u0 = 0;
  if (u1 >= m.bump_w) u1 = 0;
  if (v0 >= m.bump_h) v0 = 0;
  if (v1 >= m.bump_h) v1 = 0;
  auto px = [&](int a, int b) {
    const unsigned char* t = &(*m.bump)[3 * ((size_t)a * m.bump_w + b)];
    return V3((double)t[0], (double)t[1], (double)t[2]);
  };
  const V3 Y(0.299, 0.587, 0.114);
  const double gx = scale * dot((px(i, u1) - px(i, u0)), Y) * 0.5;
  const double gy = scale * dot((px(v1, j) - px(v0, j)), Y) * 0.5;
  h.bump_n = n + cross(n, tdir) * gx - cross(n, sdir) * gy;
  h.bump = true;
}

// the sphere's (u, v) of one mapping (sphere.h:117-180, :245-300): the
// spherical angles, then equirectangular, angular and panoramic, each
// replacing the last where set; swap_uv: the IBL block's (theta, phi) order
void sphere_uv(const Material& m, V3 vv, bool swap_uv, bool clamp_angular, double& u, double& v) {
  const double th = std::acos(std::max(-1.0, std::min(1.0, vv.z)));  // SphericalTheta (vector3d.h:259-261)
  double ph = std::atan2(vv.y, vv.x);                                 // SphericalPhi (:262-267)
  if (ph < 0.0) ph += TWOPI;
  if (ph >= TWOPI) ph = 0.0;
  u = swap_uv ? th / PI : ph / TWOPI;
  v = swap_uv ? ph / TWOPI : th / PI;
  if (m.map_flags & PR_MAP_EQUIRECTANGULAR) {
    const double len = std::sqrt(vv.x * vv.x + vv.y * vv.y + vv.z * vv.z);
    if (len == 0.0) {
      u = 0.0;
      v = 0.5;
    } else {
      const double x = vv.x / len, y = vv.y / len, z = vv.z / len;
      const double lambda = std::atan2(z, x);
      const double phi = std::asin(std::fmax(-1.0, std::fmin(1.0, y)));
      double uu = (lambda + PI) / (2.0 * PI);
      double vv2 = (0.5 * PI - phi) / PI;
      uu = uu - std::floor(uu);
      if (vv2 < 0.0) vv2 = 0.0;
      else if (vv2 > 1.0) vv2 = 1.0;
      u = uu;
      v = vv2;
    }
  }
  if (m.map_flags & PR_MAP_ANGULAR) {
    double s = vv.z;
    if (clamp_angular) {
      if (vv.z < -1.0) s = -1.0;
      if (vv.z > 1.0) s = 1.0;
    }
    double r = (1.0 / PI) * std::acos(s);
    r /= std::sqrt(vv.x * vv.x + vv.y * vv.y);
    u = vv.x * r;
    v = vv.y * r;
    u = 0.5 * u + 0.5;
    v = 0.5 * v + 0.5;
  }
  if (m.map_flags & PR_MAP_PANORAMIC) {
    double s = vv.y;
    if (vv.y < -1.0) s = -1.0;
    if (vv.y > 1.0) s = 1.0;
    u = 1.0 + std::atan2(vv.x, -vv.z) / PI;
    v = std::acos(s) / PI;
    const double a = u, b = v;
    u = 0.5 * a;
    v = 1.0 - b;
  }
}

// Sphere::intersect (sphere.h:68-103) with its texture and IBL parts
// (sphere.h:104-240): the hit point's colour and specular from the texture,
// its colour and emission from the IBL image
bool sphere_hit(const Scene& s, const Entity& e, V3 org, V3 dir, Hit& h) {
  const V3 p_o = e.position - org;
  const double b = dot(p_o, dir);
  const double D4 = b * b - dot(p_o, p_o) + e.radius * e.radius;
  if (D4 < 0.0) return false;
  const double sqrt_D4 = std::sqrt(D4);
  const double t1 = b - sqrt_D4, t2 = b + sqrt_D4;
  if (t1 < EPS && t2 < EPS) return false;
  h.distance = (t1 > EPS) ? t1 : t2;
  h.position = org + h.distance * dir;
  h.normal = normalize(h.position - e.position);
  if (e.normal_inverse < 0) h.normal = h.normal * -1.0;
  h.material = e.material;
  const V3 p = h.position - e.position;
  if (e.hemisphere && p.y < 0.0) return false;
  const Material& m = s.mats[e.material];
  if (!m.tex && !m.ibl && !m.bump) return true;
  const double pp[3] = {p.x, p.y, p.z};
  int X = 0, Y = 1, Z = 2;
  if (m.map_flags & PR_MAP_HEMISPHERE) {
    X = 2;
    Y = 0;
    Z = 1;
  }
  const V3 vv(pp[X] / e.radius, pp[Y] / e.radius, pp[Z] / e.radius);
  const bool pole = !(std::fabs(pp[Z] - e.radius) > EPS16);
  V3 color = m.color, emission = m.emission, specular = m.specular;
  bool rewrote = false;
  if (m.tex && !pole) {
    double u, v;
    sphere_uv(m, vv, false, false, u, v);
    if (e.hemisphere) u *= 2.0;
    const double uu = wrap01(u * (double)m.repeat), vw = wrap01(v * (double)m.repeat);
    int j = trunc_int((m.tex_w - 1) * uu);
    int i = trunc_int((m.tex_h - 1) * vw);
    if (m.map_flags & PR_MAP_HEMISPHERE) {
      j = trunc_int((m.tex_w - 1) / 2 + (m.tex_w - 1) * 0.5 * pp[X] / e.radius);
      i = trunc_int((m.tex_h - 1) / 2 + (m.tex_h - 1) * 0.5 * pp[Y] / e.radius);
    }
    if (i < 0) i = 0;
    if (i >= m.tex_h - 1) i = m.tex_h - 1;
    if (j < 0) j = 0;
    if (j >= m.tex_w - 1) j = m.tex_w - 1;
    texel_rgb(m, i, j, color);
    specular = color;
    h.ov_spec = true;
    rewrote = true;
  }
  if (m.ibl && !pole) {
    double u, v;
    sphere_uv(m, vv, true, true, u, v);
    if (e.hemisphere) u *= 2.0;
    int j = trunc_int((m.ibl_w - 1) * u);
    int i = trunc_int((m.ibl_h - 1) * v);
    if (m.map_flags & PR_MAP_HEMISPHERE) {
      j = trunc_int((m.ibl_w - 1) / 2 + (m.ibl_w - 1) * 0.5 * pp[X] / e.radius);
      i = trunc_int((m.ibl_h - 1) / 2 + (m.ibl_h - 1) * 0.5 * pp[Y] / e.radius);
    }
    if (i < 0) i = 0;
    if (i >= m.ibl_h - 1) i = m.ibl_h - 1;
    if (j < 0) j = 0;
    if (j >= m.ibl_w - 1) j = m.ibl_w - 1;
    color = ibl_rgb(m, i, j);
    emission = m.ibl_coef * color;
    rewrote = true;
  }
  if (m.bump && std::fabs(p.z - e.radius) > EPS16) {  // the bump block tests the unmapped p.z
    double u, v;
    sphere_uv(m, vv, true, false, u, v);
    if (e.hemisphere) u *= 2.0;
    int j = trunc_int((m.bump_w - 1) * wrap01(u * (double)m.repeat));
    int i = trunc_int((m.bump_h - 1) * wrap01(v * (double)m.repeat));
    const double th = std::acos(std::max(-1.0, std::min(1.0, vv.z)));
    double phi = std::atan2(vv.y, vv.x);
    if (phi < 0.0) phi += TWOPI;
    if (phi >= TWOPI) phi = 0.0;
    const V3 sdir(std::cos(th) * std::cos(phi), std::cos(th) * std::sin(phi), -std::sin(th));
    const V3 tdir(-std::sin(th) * std::sin(phi), std::sin(th) * std::cos(phi), 0.0);
    const V3 n = e.normal_inverse < 0 ? h.normal * -1.0 : h.normal;
    bump_normal(m, i, j, n, sdir, tdir, 0.1, h);
  }
  if (rewrote) {
    h.ov = true;
    h.ov_color = color;
    h.ov_emission = emission;
    h.ov_specular = specular;
  }
  return true;
}

// UVPlane::intersect (plane.h:220-239) over Plane::intersect (plane.h:86-110)
bool uvplane_hit(const Scene& s, const Entity& e, V3 org, V3 dir, Hit& h) {
  V3 normal2 = e.normal;
  if (e.normal_inverse < 0) normal2 = e.normal * -1.0;
  const double d = dot(dir, normal2);
  if (std::fabs(d) < EPS14) return false;
  h.distance = dot((e.org - org), normal2) / d;
  h.normal = normal2;
  h.position = dir * h.distance + org;
  h.material = e.material;
  if (h.distance < EPS) return false;
  const double u = dot(V3(h.position - e.org), e.u_axis) / e.u_length;
  const double v = dot(V3(h.position - e.org), e.v_axis) / e.v_length;
  if (u < 0 || u > e.u_length) return false;
  if (v < 0 || v > e.v_length) return false;
  // the texture and IBL parts (plane.h:241-273)
  const Material& m = s.mats[e.material];
  if (!m.tex && !m.ibl && !m.bump) return true;
  const double uu = wrap01(u * (double)m.repeat), vw = wrap01(v * (double)m.repeat);
  if (m.bump)
    bump_normal(m, trunc_int((m.bump_h - 1) * vw), trunc_int((m.bump_w - 1) * uu), e.normal, e.u_axis, e.v_axis, 1.0, h);
  if (!m.tex && !m.ibl) return true;
  V3 color = m.color, emission = m.emission, specular = m.specular;
  if (m.tex) {
    texel_rgb(m, trunc_int((m.tex_h - 1) * vw), trunc_int((m.tex_w - 1) * uu), color);
    specular = color;
    h.ov_spec = true;
  }
  if (m.ibl) {
    color = ibl_rgb(m, trunc_int((m.ibl_h - 1) * vw), trunc_int((m.ibl_w - 1) * uu));
    emission = m.ibl_coef * color;
  }
  h.ov = true;
  h.ov_color = color;
  h.ov_emission = emission;
  h.ov_specular = specular;
  return true;
}

inline V3 vtx(const Mesh& m, int id) {
  return V3(m.vert[3 * id], m.vert[3 * id + 1], m.vert[3 * id + 2]);
}

// the scene-global generator the entities' alpha tests draw from
// (SceneEnv::rand_, scene_env.h:213, :306); one per thread here
thread_local MT64* tl_disk_rnd = nullptr;

// the accretion-disk branch of Circle::intersect under a black hole
// (circle.h:240-335); defined with the Kerr restatement
bool kerr_disk_texel(const Scene& s, const Entity& e, Hit& h);

// Circle::intersect (circle.h:177-337): the base UVPlane's plane test with no
// u/v extent (circle = true), the annulus, then, under a black hole, the
// accretion-disk texture (a disk without a material texture takes no other
// branch)
bool circle_hit(const Scene& s, const Entity& e, V3 org, V3 dir, Hit& h) {
  const V3 normal2 = e.base_normal;
  const double d = dot(dir, normal2);
  if (std::fabs(d) < EPS14) return false;
  h.distance = dot((e.org - org), normal2) / d;
  h.normal = normal2;
  h.position = dir * h.distance + org;
  h.material = e.material;
  if (h.distance < EPS) return false;
  if (dot(h.position - e.org, h.position - e.org) > e.radius * e.radius) return false;
  if (dot(h.position - e.org, h.position - e.org) < e.radius_inner * e.radius_inner) return false;
  if (s.kerr.on && e.blackhole_disk >= 0 && s.mats[e.material].disk_map && !s.kerr.disk_tex.empty())
    return kerr_disk_texel(s, e, h);
  return true;
}

// Triangle::CheckIntersection2 (polygon.h:78-129) + Triangle::intersect (:131-173)
bool tri_hit(const Scene& s, const Entity& e, const Tri& tr, V3 org, V3 dir, Hit& h) {
  tl_tris++;
  const Mesh& m = s.meshes[tr.mesh];
  const int* f = &m.face[3 * tr.face];
  const V3 v0 = vtx(m, f[0]);
  const V3 edge1 = vtx(m, f[1]) - v0;
  const V3 edge2 = vtx(m, f[2]) - v0;
  const V3 p = cross(dir, edge2);
  const double det = dot(edge1, p);
  const V3 tv = org - v0;
  const V3 q = cross(tv, edge1);
  const double eps = EPS * 0.1;
  double inv_det, u, v;
  if (det > eps) {
    inv_det = 1.0 / det;
    u = dot(tv, p);
    if (u < 0.0 || u > det) return false;
    v = dot(dir, q);
    if (v < 0.0 || u + v > det) return false;
  } else if (det < -eps) {
    inv_det = 1.0 / det;
    u = dot(tv, p);
    if (u > 0.0 || u < det) return false;
    v = dot(dir, q);
    if (v > 0.0 || u + v < det) return false;
  } else {
    return false;
  }
  const double t = dot(edge2, q) * inv_det;
  u *= inv_det;
  v *= inv_det;
  const double w = 1.0 - u - v;
  if (!(t > EPS)) return false;
  h.distance = t;
  h.position = org + dir * t;
  h.normal = V3(m.fnorm[3 * tr.face], m.fnorm[3 * tr.face + 1], m.fnorm[3 * tr.face + 2]);
  const Mesh::ObjMat* om = nullptr;  // the face's OBJ material (usemtl)
  if (!m.face_omat.empty() && m.face_omat[(size_t)tr.face] >= 0) om = &m.omats[(size_t)m.face_omat[(size_t)tr.face]];
  int smooth = e.smooth;
  if (om && om->smooth) smooth = om->smooth == 1 ? 1 : 0;  // polygon.h:178-188
  if (smooth) {  // polygon.h:186-199
    const int* ni = &m.norm_id[3 * tr.face];
    const V3 n0(m.norm[3 * (size_t)ni[0]], m.norm[3 * (size_t)ni[0] + 1], m.norm[3 * (size_t)ni[0] + 2]);
    const V3 n1(m.norm[3 * (size_t)ni[1]], m.norm[3 * (size_t)ni[1] + 1], m.norm[3 * (size_t)ni[1] + 2]);
    const V3 n2(m.norm[3 * (size_t)ni[2]], m.norm[3 * (size_t)ni[2] + 1], m.norm[3 * (size_t)ni[2] + 2]);
    h.normal = normalize(n0 * w + n1 * u + n2 * v);
  }
  if (e.normal_inverse < 0) h.normal = h.normal * -1.0;
  h.material = e.material;
  h.prim = tr.face;
  // the material's texture / IBL image at the interpolated texture
  // coordinates (polygon.h:206-212, :507-528; no wrap: the coordinates of a
  // textured mesh lie in [0, 1]); bump maps on meshes write the caller's
  // record, which the returned hit overwrites (polygon.h:529-618)
  const Material& mt = s.mats[e.material];
  if (om) {
    // the OBJ material's block of Triangle::intersect (polygon.h:228-400),
    // then the entity's own texture and IBL image (:505-528)
    Material q = mt;
    double hu = 0, hv = 0;
    if (!m.uv_id.empty()) {
      const int* ti = &m.uv_id[3 * tr.face];
      hu = m.uv[2 * (size_t)ti[0]] * w + m.uv[2 * (size_t)ti[1]] * u + m.uv[2 * (size_t)ti[2]] * v;
      hv = m.uv[2 * (size_t)ti[0] + 1] * w + m.uv[2 * (size_t)ti[1] + 1] * u + m.uv[2 * (size_t)ti[2] + 1] * v;
    }
    if (!om->tex.empty()) {
      const double uu = wrap01(hu * om->repeat), vv = wrap01(hv * om->repeat);
      const int j = trunc_int((om->tw - 1) * uu), i = trunc_int((om->th - 1) * vv);
      const unsigned char* t = &om->tex[3 * ((size_t)i * om->tw + j)];
      // base.x * (double)cell.r / 255.0, left to right (polygon.h:257-304)
      auto scaled = [t](V3 b) {
        return V3(b.x * (double)t[0] / 255.0, b.y * (double)t[1] / 255.0, b.z * (double)t[2] / 255.0);
      };
      q.color = scaled(mt.color);
      q.emission = mt.emission;
      if (om->refl >= 0) {
        q.emission = scaled(om->emission);
        q.type = om->refl;
        q.specular = scaled(om->specular);
        q.refractive_index = om->ni;
        q.roughness = om->rough;
        if (q.type == PR_MAT_SPECULAR || q.type == PR_MAT_REFRACTION) q.color = om->specular;
        if (q.type == PR_MAT_WARD) {
          q.ward_ax = om->ward[0];
          q.ward_ay = om->ward[1];
          q.color = scaled(om->diffuse);
        }
        if (q.type == PR_MAT_PHONG) {
          q.phong_n = om->ns;
          q.color = scaled(om->diffuse);
        }
      }
    } else {
      q.color = om->diffuse;
      q.specular = om->specular;
      if (q.type == PR_MAT_DIFFUSE) q.specular = V3();
      q.emission = mt.emission;
      if (om->refl >= 0) {
        q.emission = om->emission;
        q.type = om->refl;
        q.specular = om->specular;
        q.refractive_index = om->ni;
        q.roughness = om->rough;
        if (q.type == PR_MAT_SPECULAR || q.type == PR_MAT_REFRACTION) q.color = om->specular;
        if (q.type == PR_MAT_WARD) {
          q.ward_ax = om->ward[0];
          q.ward_ay = om->ward[1];
          q.color = om->diffuse;
        }
        if (q.type == PR_MAT_PHONG) {
          q.phong_n = om->ns;
          q.color = om->diffuse;
        }
      }
    }
    if (mt.tex) {
      int j = trunc_int((mt.tex_w - 1) * hu), i = trunc_int((mt.tex_h - 1) * hv);
      i = std::min(std::max(i, 0), mt.tex_h - 1);
      j = std::min(std::max(j, 0), mt.tex_w - 1);
      texel_rgb(mt, i, j, q.color);
    }
    if (mt.ibl) {
      int j = trunc_int((mt.ibl_w - 1) * hu), i = trunc_int((mt.ibl_h - 1) * hv);
      i = std::min(std::max(i, 0), mt.ibl_h - 1);
      j = std::min(std::max(j, 0), mt.ibl_w - 1);
      q.color = ibl_rgb(mt, i, j);
      q.emission = mt.ibl_coef * q.color;
    }
    h.ov_full = true;
    h.ovm = q;
    return true;
  }
  if ((mt.tex || mt.ibl) && !m.uv_id.empty()) {
    const int* ti = &m.uv_id[3 * tr.face];
    const double hu = m.uv[2 * (size_t)ti[0]] * w + m.uv[2 * (size_t)ti[1]] * u + m.uv[2 * (size_t)ti[2]] * v;
    const double hv = m.uv[2 * (size_t)ti[0] + 1] * w + m.uv[2 * (size_t)ti[1] + 1] * u + m.uv[2 * (size_t)ti[2] + 1] * v;
    V3 color = mt.color, emission = mt.emission;
    if (mt.tex) {
      int j = trunc_int((mt.tex_w - 1) * hu), i = trunc_int((mt.tex_h - 1) * hv);
      i = std::min(std::max(i, 0), mt.tex_h - 1);
      j = std::min(std::max(j, 0), mt.tex_w - 1);
      texel_rgb(mt, i, j, color);
    }
    if (mt.ibl) {
      int j = trunc_int((mt.ibl_w - 1) * hu), i = trunc_int((mt.ibl_h - 1) * hv);
      i = std::min(std::max(i, 0), mt.ibl_h - 1);
      j = std::min(std::max(j, 0), mt.ibl_w - 1);
      color = ibl_rgb(mt, i, j);
      emission = mt.ibl_coef * color;
    }
    h.ov = true;
    h.ov_color = color;
    h.ov_emission = emission;
  }
  return true;
}

// --------------------------------------------------------------- SAH build
// BoundingBox::CalcSurfaceArea member form (BoundingBox.h:29-33)
inline double area_member(V3 mn, V3 mx) {
  double dx = mx.x - mn.x, dy = mx.y - mn.y, dz = mx.z - mn.z;
  return dx * dy + dx * dz + dy * dz;
}
// BoundingBox::CalcSurfaceArea template form (BoundingBox.h:35-39)
inline double area_template(const double mn[3], const double mx[3]) {
  double d[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
  return d[0] * d[1] + d[1] * d[2] + d[0] * d[2];
}

struct Builder {
  const std::vector<Tri>& tris;
  std::vector<BVHNode> nodes;
  explicit Builder(const std::vector<Tri>& t) : tris(t) {}

  // CalcBoundingBoxOfObjects, Vector3d form (BVH.cpp:137-154)
  void bbox(const std::vector<int>& objs, V3& mn, V3& mx) const {
    mn = tris[objs[0]].bmin;
    mx = tris[objs[0]].bmax;
    for (size_t i = 1; i < objs.size(); i++) {
      const Tri& a = tris[objs[i]];
      if (a.bmin.x < mn.x) mn.x = a.bmin.x;
      if (a.bmin.y < mn.y) mn.y = a.bmin.y;
      if (a.bmin.z < mn.z) mn.z = a.bmin.z;
      if (a.bmax.x > mx.x) mx.x = a.bmax.x;
      if (a.bmax.y > mx.y) mx.y = a.bmax.y;
      if (a.bmax.z > mx.z) mx.z = a.bmax.z;
    }
  }
  // BoundingBox::MergeAnotherBox (BoundingBox.h:229-238)
  static void merge(V3& mn, V3& mx, const Tri& b) {
    mn.x = std::min(mn.x, b.bmin.x);
    mn.y = std::min(mn.y, b.bmin.y);
    mn.z = std::min(mn.z, b.bmin.z);
    mx.x = std::max(mx.x, b.bmax.x);
    mx.y = std::max(mx.y, b.bmax.y);
    mx.z = std::max(mx.z, b.bmax.z);
  }
  void sort_axis(std::vector<int>& v, int axis) const {
    const std::vector<Tri>& t = tris;
    std::sort(v.begin(), v.end(), [&t, axis](int a, int b) -> bool {
      return t[a].center[axis] < t[b].center[axis];
    });
  }
  // BVH::Construct_internal, CONSTRUCTION_OBJECT_SAH (BVH.cpp:194-348)
  void build(const std::vector<int>& targets, int index) {
    {
      V3 mn, mx;
      bbox(targets, mn, mx);
      nodes[index].box[0][0] = mn.x; nodes[index].box[0][1] = mn.y; nodes[index].box[0][2] = mn.z;
      nodes[index].box[1][0] = mx.x; nodes[index].box[1][1] = mx.y; nodes[index].box[1][2] = mx.z;
    }
    const double surf = area_template(nodes[index].box[0], nodes[index].box[1]);
    const double surf_inv = 1.0 / surf;
    int bestAxis = -1, bestIndex = -1;
    double bestCost = -1;
    const size_t n = targets.size();
    std::vector<double> leftAreas(n), rightAreas(n);
    for (int axis = 0; axis < 3; axis++) {
      std::vector<int> L = targets, R;
      sort_axis(L, axis);
      rightAreas[n - 1] = INF;
      R.push_back(L.back());
      L.pop_back();
      V3 mn, mx;
      bbox(R, mn, mx);
      const int sz = (int)L.size();
      for (int i = sz - 1; i >= 0; i--) {
        rightAreas[i] = area_member(mn, mx);
        merge(mn, mx, tris[L[i]]);
        R.push_back(L.back());
        L.pop_back();
      }
      L.push_back(R.back());
      R.pop_back();
      bbox(L, mn, mx);
      const double leafCost = 1.0 * (double)n;
      const int sz2 = (int)R.size();
      for (int i = sz2 - 1, cut = 0; i >= 0; i--, cut++) {
        leftAreas[cut] = area_member(mn, mx);
        merge(mn, mx, tris[R.back()]);
        L.push_back(R.back());
        R.pop_back();
        const double cost = 2 * 1.0 + (leftAreas[cut] * (double)L.size() + rightAreas[cut] * (double)R.size()) * surf_inv * 1.0;
        if ((cost < bestCost || bestCost == -1) && cost < leafCost) {
          bestCost = cost;
          bestIndex = cut;
          bestAxis = axis;
        }
      }
    }
    if (bestAxis == -1) {  // MakeLeaf_internal (BVH.cpp:181-191)
      nodes[index].children[0] = nodes[index].children[1] = -1;
      nodes[index].objects = targets;
      return;
    }
    std::vector<int> lefts = targets;
    sort_axis(lefts, bestAxis);
    std::vector<int> rights(lefts.begin() + bestIndex + 1, lefts.end());
    lefts.resize(bestIndex + 1);
    nodes[index].axis = bestAxis;
    const int c0 = (int)nodes.size();
    nodes[index].children[0] = c0;
    nodes[index].children[1] = c0 + 1;
    nodes.emplace_back();
    nodes.emplace_back();
    build(lefts, c0);
    build(rights, c0 + 1);
  }
};

bool is_leaf(const BVHNode& n) { return n.children[0] == -1; }

struct Flattener {  // QBVH::Construct_internal / MakeLeaf_internal (QBVH.cpp:202-302)
  const std::vector<BVHNode>& bvh;
  QBVH& q;
  Flattener(const std::vector<BVHNode>& b, QBVH& qq) : bvh(b), q(qq) {}
  void make_leaf(size_t index, const BVHNode& leaf, int childindex) {
    const int64_t start = (int64_t)q.leaf.size();
    for (int o : leaf.objects) q.leaf.push_back(o);
    q.leaf.push_back(-1);
    q.nodes[index].children[childindex] = QTOP | start;
  }
  void flatten(size_t nextindex, int target) {
    const BVHNode& nt = bvh[target];
    QNode& cur0 = q.nodes[nextindex];
    memset(&cur0, 0, sizeof(QNode));
    cur0.axis_top = nt.axis;
    const BVHNode* ch[2] = {&bvh[nt.children[0]], &bvh[nt.children[1]]};
    cur0.axis_left = is_leaf(*ch[0]) ? 0 : ch[0]->axis;
    cur0.axis_right = is_leaf(*ch[1]) ? 0 : ch[1]->axis;
    float four[2][3][4];
    memset(four, 0, sizeof(four));
    auto insert = [&four](const BVHNode& b, int slot) {
      for (int xyz = 0; xyz < 3; xyz++) {
        four[0][xyz][slot] = (float)b.box[0][xyz];
        four[1][xyz][slot] = (float)b.box[1][xyz];
      }
    };
    for (int i = 0; i < 2; i++) {
      const BVHNode& child = *ch[i];
      if (is_leaf(child)) {
        const int slot = i * 2;
        make_leaf(nextindex, child, slot);
        q.nodes[nextindex].children[1 + slot] = -1;
        insert(child, slot);
      } else {
        const BVHNode* gc[2] = {&bvh[child.children[0]], &bvh[child.children[1]]};
        const int gci[2] = {child.children[0], child.children[1]};
        for (int j = 0; j < 2; j++) {
          const int slot = i * 2 + j;
          insert(*gc[j], slot);
          if (is_leaf(*gc[j])) {
            make_leaf(nextindex, *gc[j], slot);
          } else {
            const size_t nn = q.nodes.size();
            q.nodes.emplace_back();
            q.nodes[nextindex].children[slot] = (int64_t)nn;
            flatten(nn, gci[j]);
          }
        }
      }
    }
    memcpy(q.nodes[nextindex].bboxes, four, sizeof(four));
  }
};

// ------------------------------------------------------------ traversal
// CheckIntersection4floatAABB (BoundingBox.h:137-178): SSE max/min return
// the second operand when the comparison fails (NaN included).
inline float mx_ps(float a, float b) { return a > b ? a : b; }
inline float mn_ps(float a, float b) { return a < b ? a : b; }

// QBVH::CheckIntersection + CheckIntersection_Leaf (QBVH.cpp:17-159)
bool qbvh_hit(const Scene& s, const Entity& e, V3 org, V3 dir, Hit& out) {
  const int sign[3] = {dir.x >= 0 ? 0 : 1, dir.y >= 0 ? 0 : 1, dir.z >= 0 ? 0 : 1};
  const float ro[3] = {(float)org.x, (float)org.y, (float)org.z};
  const float inf_f = (float)INF;
  const float rid[3] = {dir.x == 0 ? inf_f : (float)(1.0f / dir.x), dir.y == 0 ? inf_f : (float)(1.0f / dir.y),
                        dir.z == 0 ? inf_f : (float)(1.0f / dir.z)};
  const float fmaxv = 3.402823466e+38F;
  std::vector<int64_t> stack;
  stack.push_back(0);
  double dist = -1.0;
  const QBVH& q = e.qbvh;
  while (!stack.empty()) {
    const int64_t ni = stack.back();
    stack.pop_back();
    const QNode& nd = q.nodes[(size_t)ni];
    tl_nodes++;
    bool res[4];
    int any = 0;
    for (int c = 0; c < 4; c++) {
      float tmin = 0.0f, tmax = fmaxv;
      for (int a = 0; a < 3; a++) {
        tmin = mx_ps(tmin, (nd.bboxes[sign[a]][a][c] - ro[a]) * rid[a]);
        tmax = mn_ps(tmax, (nd.bboxes[1 - sign[a]][a][c] - ro[a]) * rid[a]);
      }
      res[c] = tmax >= tmin;
      any |= res[c];
    }
    if (!any) continue;
    int order[4];
    const bool isLeft = sign[nd.axis_top] == 0;
    const int lf = isLeft ? 0 : 2;
    const int rf = (lf + 2) % 4;
    if (sign[nd.axis_left] == 0) { order[lf] = 0; order[lf + 1] = 1; }
    else { order[lf] = 1; order[lf + 1] = 0; }
    if (sign[nd.axis_right] == 0) { order[rf] = 2; order[rf + 1] = 3; }
    else { order[rf] = 3; order[rf + 1] = 2; }
    for (int i = 0; i < 4; i++) {
      const int c = order[i];
      const int64_t ch = nd.children[c];
      if (!res[c] || ch == -1) continue;
      if (ch & QTOP) {
        const int64_t start = ch ^ QTOP;
        double nearest = -1;
        Hit tmp;
        bool got = false;
        for (int64_t k = start; q.leaf[(size_t)k] >= 0; k++) {
          Hit h;
          if (tri_hit(s, e, e.tris[q.leaf[(size_t)k]], org, dir, h) && h.distance > 0 &&
              (nearest < 0 || h.distance < nearest)) {
            tmp = h;
            nearest = h.distance;
            got = true;
          }
        }
        if (got && tmp.distance > EPS) {
          if (dist < 0 || dist > tmp.distance) {
            out = tmp;
            dist = out.distance;
          }
        }
      } else {
        stack.push_back(ch);
      }
    }
  }
  return dist > 0;
}

// intersect_scene_ without a black hole (scene.cpp:83-214)
bool intersect(const Scene& s, V3 org, V3 dir, Hit& isect) {
  tl_segments++;
  isect = Hit();
  isect.distance = INF;
  isect.object_id = -1;
  const V3 o2 = org + dir * 0.000001;
  for (int i = 0; i < (int)s.ents.size(); i++) {
    const Entity& e = s.ents[i];
    Hit h;
    bool got = false;
    switch (e.type) {
      case PR_ENT_SPHERE: got = sphere_hit(s, e, o2, dir, h); break;
      case PR_ENT_UVPLANE: got = uvplane_hit(s, e, o2, dir, h); break;
      case PR_ENT_CIRCLE: got = circle_hit(s, e, o2, dir, h); break;
      case PR_ENT_POLYGON: got = qbvh_hit(s, e, o2, dir, h); break;
      default: break;
    }
    if (got && h.distance < isect.distance) {
      isect = h;
      isect.object_id = i;
    }
  }
  return isect.object_id >= 0;
}

// ------------------------------------------------------------------ setup
int build_scene(const pr_scene_desc* d, Scene& s, std::string& err) {
  if (!d || d->n_entities < 0 || d->n_materials < 0 || d->n_meshes < 0) { err = "bad scene"; return PR_E_ARG; }
  for (int i = 0; i < d->n_materials; i++) {
    const pr_material& pm = d->materials[i];
    Material m;
    m.type = pm.type;
    m.color = V3(pm.color[0], pm.color[1], pm.color[2]);
    m.emission = V3(pm.emission[0], pm.emission[1], pm.emission[2]);
    m.specular = V3(pm.specular[0], pm.specular[1], pm.specular[2]);
    m.roughness = pm.roughness;
    m.refractive_index = pm.refractive_index;
    m.r_refractive_index = pm.r_refractive_index;
    m.disk_map = pm.disk_map;
    m.ward_ax = pm.ward_alpha[0];
    m.ward_ay = pm.ward_alpha[1];
    m.phong_n = pm.phong_exponent;
    if (pm.texture && pm.texture_width > 0 && pm.texture_height > 0) {
      m.tex_w = pm.texture_width;
      m.tex_h = pm.texture_height;
      m.tex = std::make_shared<const std::vector<unsigned char>>(pm.texture, pm.texture + 3 * (size_t)m.tex_w * m.tex_h);
    }
    if ((pm.ibl_rgb8 || pm.ibl_rgbf) && pm.ibl_width > 0 && pm.ibl_height > 0) {
      // IBL_Color (material.h:230-236): a bitmap's bytes / 255, an HDR image's values
      m.ibl_w = pm.ibl_width;
      m.ibl_h = pm.ibl_height;
      const size_t n = 3 * (size_t)m.ibl_w * m.ibl_h;
      auto v = std::make_shared<std::vector<double>>(n);
      for (size_t k = 0; k < n; k++) (*v)[k] = pm.ibl_rgb8 ? (double)pm.ibl_rgb8[k] / 255.0 : (double)pm.ibl_rgbf[k];
      m.ibl = v;
    }
    if (pm.bump && pm.bump_width > 0 && pm.bump_height > 0) {
      m.bump_w = pm.bump_width;
      m.bump_h = pm.bump_height;
      m.bump = std::make_shared<const std::vector<unsigned char>>(pm.bump, pm.bump + 3 * (size_t)m.bump_w * m.bump_h);
    }
    m.ibl_coef = pm.ibl_coef;
    m.repeat = pm.repeat;
    m.map_flags = pm.map_flags;
    if (m.type == PR_MAT_SSS_REFRACTION || m.type == PR_MAT_SSS_DIFFUSE || m.type == PR_MAT_SSS_WARD) {
      // the material's own participatingMediaParam (scene_env.h:1305-1362); the
      // entity set-up calls setup_Scattering when the SCATTERING line is > PS_EPS
      Medium& md = m.medium;
      md.scatteringColor = V3(pm.medium.sigma_s_rgb[0], pm.medium.sigma_s_rgb[1], pm.medium.sigma_s_rgb[2]);
      md.absorbingColor = V3(pm.medium.sigma_a_rgb[0], pm.medium.sigma_a_rgb[1], pm.medium.sigma_a_rgb[2]);
      for (int k = 0; k < 3; k++) md.phase[k] = pm.medium.phase_g[k];
      md.r_max = pm.medium.r_max;
      md.level = pm.medium.level;
      md.use_bssrdf = pm.medium.use_bssrdf;
      const double sc = (md.scatteringColor.x + md.scatteringColor.y + md.scatteringColor.z) / 3;
      if (sc > EPS) md.setup(pm.medium.scale > 0.0 ? pm.medium.scale : 1.0);
      if (m.type != PR_MAT_SSS_REFRACTION || (md.level != -2 && md.level != -1) || !md.use_bssrdf) {
        err = "subsurface scattering: only the directional-dipole forms (reflection reflection + "
              "Subsurface_Scattering, level -2 or -1) are on this path";
        return PR_E_UNSUPPORTED;
      }
    }
    s.mats.push_back(m);
  }
  for (int i = 0; i < d->n_meshes; i++) {
    const pr_mesh& pm = d->meshes[i];
    Mesh m;
    m.vert.assign(pm.vertices, pm.vertices + 3 * (size_t)pm.n_vertices);
    m.face.assign(pm.faces, pm.faces + 3 * (size_t)pm.n_faces);
    m.fnorm.resize(3 * (size_t)pm.n_faces);
    if (pm.vertex_normals && pm.face_vn) {
      m.norm.assign(pm.vertex_normals, pm.vertex_normals + 3 * (size_t)pm.n_vertex_normals);
      m.norm_id.assign(pm.face_vn, pm.face_vn + 3 * (size_t)pm.n_faces);
    } else {
      // Obj::CalcNormalVector without vn lines (ObjLoader.cpp:645-685): the
      // unnormalised face normals summed at each vertex in face order, the
      // mean normalised in float; norm_id = the face's vertex ids
      const int nv = pm.n_vertices;
      m.norm.assign(3 * (size_t)nv, 0.0f);
      m.norm_id = m.face;
      std::vector<int> count((size_t)nv, 0);
      const float* V = m.vert.data();
      for (int f = 0; f < pm.n_faces; f++) {
        const int* fc = &m.face[3 * f];
        float dx1 = V[3 * fc[1]] - V[3 * fc[0]], dy1 = V[3 * fc[1] + 1] - V[3 * fc[0] + 1],
              dz1 = V[3 * fc[1] + 2] - V[3 * fc[0] + 2];
        float dx2 = V[3 * fc[2]] - V[3 * fc[0]], dy2 = V[3 * fc[2] + 1] - V[3 * fc[0] + 1],
              dz2 = V[3 * fc[2] + 2] - V[3 * fc[0] + 2];
        const float fnv[3] = {dy1 * dz2 - dz1 * dy2, dz1 * dx2 - dx1 * dz2, dx1 * dy2 - dy1 * dx2};
        for (int k = 0; k < 3; k++) {
          for (int a = 0; a < 3; a++) m.norm[3 * (size_t)fc[k] + a] += fnv[a];
          count[(size_t)fc[k]]++;
        }
      }
      for (int i2 = 0; i2 < nv; i2++) {
        if (count[(size_t)i2] == 0) continue;
        float* n = &m.norm[3 * (size_t)i2];
        for (int a = 0; a < 3; a++) n[a] /= (double)count[(size_t)i2];
        float a = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (a != 0.0) { n[0] /= a; n[1] /= a; n[2] /= a; }
      }
    }
    if (pm.uv && pm.face_uv) {
      m.uv.assign(pm.uv, pm.uv + 2 * (size_t)pm.n_uv);
      m.uv_id.assign(pm.face_uv, pm.face_uv + 3 * (size_t)pm.n_faces);
    }
    if (pm.obj_materials && pm.face_obj_material && pm.n_obj_materials > 0) {
      for (int k = 0; k < pm.n_obj_materials; k++) {
        const pr_obj_material& q = pm.obj_materials[k];
        Mesh::ObjMat om;
        om.diffuse = V3(q.diffuse[0], q.diffuse[1], q.diffuse[2]);
        om.specular = V3(q.specular[0], q.specular[1], q.specular[2]);
        om.emission = V3(q.emission[0], q.emission[1], q.emission[2]);
        om.alpha = q.alpha;
        om.ni = q.refraction_index;
        om.ns = q.shininess;
        om.rough = q.roughness;
        om.ward[0] = q.ward[0];
        om.ward[1] = q.ward[1];
        om.refl = q.reflection;
        om.smooth = q.smooth;
        om.repeat = q.repeat;
        if (q.texture && q.texture_width > 0 && q.texture_height > 0) {
          om.tw = q.texture_width;
          om.th = q.texture_height;
          om.tex.assign(q.texture, q.texture + 3 * (size_t)om.tw * om.th);
        }
        m.omats.push_back(std::move(om));
      }
      m.face_omat.assign(pm.face_obj_material, pm.face_obj_material + pm.n_faces);
    }
    if (pm.face_normals) {
      memcpy(m.fnorm.data(), pm.face_normals, sizeof(float) * 3 * (size_t)pm.n_faces);
    } else if (pm.vertex_normals && pm.face_vn) {
      // with vn lines: the normalised mean of the face's three (ObjLoader.cpp:617-641)
      for (int f = 0; f < pm.n_faces; f++) {
        float c[3];
        for (int a = 0; a < 3; a++)
          c[a] = (m.norm[3 * (size_t)m.norm_id[3 * f] + a] + m.norm[3 * (size_t)m.norm_id[3 * f + 1] + a] +
                  m.norm[3 * (size_t)m.norm_id[3 * f + 2] + a]) / 3.0;
        double ln = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
        if (ln > 1.0e-16) {
          ln = std::sqrt(ln);
          c[0] /= ln;
          c[1] /= ln;
          c[2] /= ln;
        }
        for (int a = 0; a < 3; a++) m.fnorm[3 * (size_t)f + a] = c[a];
      }
    } else {
      // Obj::CalcNormalVector, no 'vn' lines (ObjLoader.cpp:582-598, :686-697)
      for (int f = 0; f < pm.n_faces; f++) {
        const int* fc = &m.face[3 * f];
        const float* V = m.vert.data();
        float dx1 = V[3 * fc[1]] - V[3 * fc[0]], dy1 = V[3 * fc[1] + 1] - V[3 * fc[0] + 1],
              dz1 = V[3 * fc[1] + 2] - V[3 * fc[0] + 2];
        float dx2 = V[3 * fc[2]] - V[3 * fc[0]], dy2 = V[3 * fc[2] + 1] - V[3 * fc[0] + 1],
              dz2 = V[3 * fc[2] + 2] - V[3 * fc[0] + 2];
        float nx = dy1 * dz2 - dz1 * dy2, ny = dz1 * dx2 - dx1 * dz2, nz = dx1 * dy2 - dy1 * dx2;
        float a = std::sqrt(nx * nx + ny * ny + nz * nz);
        if (a != 0.0) { nx /= a; ny /= a; nz /= a; }
        m.fnorm[3 * f] = nx; m.fnorm[3 * f + 1] = ny; m.fnorm[3 * f + 2] = nz;
      }
    }
    s.meshes.push_back(std::move(m));
  }
  s.background = V3(d->background[0], d->background[1], d->background[2]);
  s.env_light = V3(d->environment_light[0], d->environment_light[1], d->environment_light[2]);
  s.medium.scatteringColor = V3(d->medium.sigma_s_rgb[0], d->medium.sigma_s_rgb[1], d->medium.sigma_s_rgb[2]);
  s.medium.absorbingColor = V3(d->medium.sigma_a_rgb[0], d->medium.sigma_a_rgb[1], d->medium.sigma_a_rgb[2]);
  for (int k = 0; k < 3; k++) s.medium.phase[k] = d->medium.phase_g[k];
  s.medium.setup(1.0);  // scene_env.h:1892
  s.media_on = d->participating_media && !(s.medium.transmittance < EPS12);  // scene_env.h:1893-1896

  for (int i = 0; i < d->n_entities; i++) {
    const pr_entity& pe = d->entities[i];
    if (pe.material < 0 || pe.material >= (int)s.mats.size()) { err = "entity material out of range"; return PR_E_SCENE; }
    Entity e;
    e.type = pe.type;
    e.material = pe.material;
    e.normal_inverse = pe.normal_inverse < 0 ? -1 : 1;
    const Material& m = s.mats[pe.material];
    if (pe.type == PR_ENT_SPHERE) {
      e.position = V3(pe.p[0], pe.p[1], pe.p[2]);
      e.radius = pe.radius;
      e.hemisphere = pe.hemisphere ? 1 : 0;
      e.area = FORPI * e.radius * e.radius;  // Sphere::CalcArea (sphere.h:23-27)
      if (e.hemisphere) {
        e.area = 0.5 * e.area;
        if (m.isLight()) { err = "hemisphere lights are not sampled here"; return PR_E_UNSUPPORTED; }
      }
      const V3 ext(e.radius, e.radius, e.radius), eps(0.01, 0.01, 0.01);  // sphere.h:58-63
      e.bb_min = e.position - ext - eps;
      e.bb_max = e.position + ext + eps;
    } else if (pe.type == PR_ENT_UVPLANE) {  // UVPlane ctor (plane.h:146-167)
      e.org = V3(pe.p[0], pe.p[1], pe.p[2]);
      V3 U(pe.u[0], pe.u[1], pe.u[2]), V(pe.v[0], pe.v[1], pe.v[2]);
      e.u_length = length(U);
      e.v_length = length(V);
      e.u_axis = normalize(U);
      e.v_axis = normalize(V);
      e.normal = normalize(cross(e.u_axis, e.v_axis));
      // UVPlane::CalcArea (plane.h:174-177)
      e.area = length(e.u_axis * e.u_length) * length(e.v_axis * e.v_length) *
               (1.0 - std::pow(dot(e.u_axis, e.v_axis), 2.0));
      {  // UVPlane::CreateBoundingBox (plane.h:191-215)
        const V3 q[4] = {e.org, e.org + e.v_length * 1.0 * e.v_axis, e.org + e.u_length * 1.0 * e.u_axis,
                         e.org + e.u_length * 1.0 * e.u_axis + e.v_length * 1.0 * e.v_axis};
        V3 mn = q[0], mx = q[0];
        for (int k = 1; k < 4; k++) {
          if (mn.x > q[k].x) mn.x = q[k].x;
          if (mn.y > q[k].y) mn.y = q[k].y;
          if (mn.z > q[k].z) mn.z = q[k].z;
          if (mx.x < q[k].x) mx.x = q[k].x;
          if (mx.y < q[k].y) mx.y = q[k].y;
          if (mx.z < q[k].z) mx.z = q[k].z;
        }
        e.bb_min = mn;
        e.bb_max = mx;
      }
    } else if (pe.type == PR_ENT_CIRCLE) {  // Circle ctor (circle.h:117-130)
      e.org = V3(pe.p[0], pe.p[1], pe.p[2]);
      e.radius = pe.radius;
      e.radius_inner = pe.radius_inner;
      V3 w, u, v;
      onb(V3(pe.normal[0], pe.normal[1], pe.normal[2]), w, u, v);
      const V3 U = u * pe.radius, V = v * pe.radius;  // base = UVPlane(o, r*u, r*v)
      e.base_normal = normalize(cross(normalize(U), normalize(V)));
      e.du_len = length(U);  // UVPlane ctor (plane.h:146-157)
      e.dv_len = length(V);
      e.du_axis = normalize(U);
      e.dv_axis = normalize(V);
      e.blackhole_disk = pe.blackhole_disk;
      e.area = e.radius * e.radius * PI;  // Circle::CalcArea
    } else if (pe.type == PR_ENT_POLYGON) {
      if (pe.mesh < 0 || pe.mesh >= (int)s.meshes.size()) { err = "entity mesh out of range"; return PR_E_SCENE; }
      e.mesh = pe.mesh;
      e.smooth = pe.smooth;
      const Mesh& mesh = s.meshes[pe.mesh];
      const int nf = (int)mesh.face.size() / 3;
      // Polygon::MakeTrianglesEntity + Triangle::CreateBoundingBox (polygon.h:686-703, :912-969)
      for (int f = 0; f < nf; f++) {
        Tri t;
        t.mesh = pe.mesh;
        t.face = f;
        V3 mn(INF, INF, INF), mx(-INF, -INF, -INF);
        for (int k = 0; k < 3; k++) {
          V3 v = vtx(mesh, mesh.face[3 * f + k]);
          if (mn.x > v.x) mn.x = v.x;
          if (mn.y > v.y) mn.y = v.y;
          if (mn.z > v.z) mn.z = v.z;
          if (mx.x < v.x) mx.x = v.x;
          if (mx.y < v.y) mx.y = v.y;
          if (mx.z < v.z) mx.z = v.z;
        }
        const V3 eps(0.01, 0.01, 0.01);
        t.bmin = mn - eps;
        t.bmax = mx + eps;
        t.center = (t.bmin + t.bmax) / 2.0;
        e.tris.push_back(t);
      }
      if (nf == 0) { err = "empty mesh"; return PR_E_SCENE; }
      {  // Polygon::CreateBoundingBox over the mesh vertices (polygon.h:875-889)
        V3 mn(INF, INF, INF), mx(-INF, -INF, -INF);
        for (size_t k = 0; k + 2 < mesh.vert.size(); k += 3) {
          const V3 v(mesh.vert[k], mesh.vert[k + 1], mesh.vert[k + 2]);
          if (mn.x > v.x) mn.x = v.x;
          if (mn.y > v.y) mn.y = v.y;
          if (mn.z > v.z) mn.z = v.z;
          if (mx.x < v.x) mx.x = v.x;
          if (mx.y < v.y) mx.y = v.y;
          if (mx.z < v.z) mx.z = v.z;
        }
        const V3 eps(0.01, 0.01, 0.01);
        e.bb_min = mn - eps;
        e.bb_max = mx + eps;
      }
      // QBVH::Construct (QBVH.cpp:161-186)
      Builder b(e.tris);
      b.nodes.emplace_back();
      std::vector<int> all(nf);
      for (int f = 0; f < nf; f++) all[f] = f;
      b.build(all, 0);
      if (is_leaf(b.nodes[0])) { err = "mesh too small for a QBVH root (reference falls back to BVH)"; return PR_E_BUILD; }
      e.qbvh.nodes.emplace_back();
      Flattener fl(b.nodes, e.qbvh);
      fl.flatten(0, 0);
      if (m.isLight()) { err = "mesh lights are not sampled by the reference's NEE"; return PR_E_UNSUPPORTED; }
    } else if (pe.type == PR_ENT_INF_LIGHT) {
      // 'infinity_light': no geometry (scene_env.h:1525-1541)
    } else {
      err = "entity type not supported by the oracle";
      return PR_E_UNSUPPORTED;
    }
    s.ents.push_back(std::move(e));
  }
  if (d->wormhole.enabled) {
    const pr_wormhole& w = d->wormhole;
    if (d->kerr.enabled) { err = "a scene has a black hole or a wormhole"; return PR_E_UNSUPPORTED; }
    Wormhole& wh = s.worm;
    wh.on = true;
    wh.pos0 = V3(w.in[0], w.in[1], w.in[2]);
    wh.pos1 = V3(w.out[0], w.out[1], w.out[2]);
    wh.Rho = w.rho;
    wh.W = w.w;
    wh.a = std::fabs(w.a);
    wh.M = wh.W / 1.42953;
    wh.max_steps = w.max_steps;
    wh.usr_sign = w.sign;
    wh.camera = V3(w.camera[0], w.camera[1], w.camera[2]);
    for (int k = 0; k < 2; k++) {
      for (int q = 0; q < 4; q++) wh.map_coef[k][q] = w.map_coef[k][q];
      wh.tex_coef[k] = w.texture_coef[k];
      if (w.texture[k] && w.texture_width[k] > 0 && w.texture_height[k] > 0) {
        wh.tex_w[k] = w.texture_width[k];
        wh.tex_h[k] = w.texture_height[k];
        wh.tex[k].assign(w.texture[k], w.texture[k] + 3 * (size_t)wh.tex_w[k] * wh.tex_h[k]);
      }
    }
  }
  if (d->kerr.enabled) {
    s.kerr.on = true;
    s.kerr.position = V3(d->kerr.position[0], d->kerr.position[1], d->kerr.position[2]);
    s.kerr.a = d->kerr.a;
    s.kerr.a2 = s.kerr.a * s.kerr.a;
    s.kerr.M = 1.0;
    s.kerr.Rhor = s.kerr.M + std::sqrt(s.kerr.M * s.kerr.M - s.kerr.a2) + 1e-10;  // KerrBlackHole.h:116
    s.kerr.max_steps = d->kerr.max_steps;
    for (int k = 0; k < 4; k++) s.kerr.map_coef[k] = d->kerr.map_coef[k];
    s.kerr.escape_radius = d->kerr.escape_radius;
    s.kerr.texture_coef = d->kerr.texture_coef;
    if (d->kerr.texture && d->kerr.texture_width > 0 && d->kerr.texture_height > 0) {
      s.kerr.tex_w = d->kerr.texture_width;
      s.kerr.tex_h = d->kerr.texture_height;
      s.kerr.texture.assign(d->kerr.texture, d->kerr.texture + 3 * (size_t)s.kerr.tex_w * s.kerr.tex_h);
    }
    // inner_orbit (KerrBlackHole.h:215-240) with M = 1 and the class's own
    // cbrt(x) = pow(x, 1/3)
    {
      const double M = s.kerr.M, a = s.kerr.a, a2 = s.kerr.a2, m2 = M * M;
      auto cbrt_r = [](double x) { return std::pow(x, 1.0 / 3.0); };
      const double z1 = 1 + cbrt_r(1 - a2 / m2) * (cbrt_r(1 + a / M) + cbrt_r(1 - a / M));
      const double z2 = std::sqrt(3 * a2 / m2 + z1 * z1);
      s.kerr.Rmstable = M * (3 + z2 - std::sqrt((3 - z1) * (3 + z1 + 2 * z2)));
    }
    s.kerr.use_temperature = d->kerr.use_accretion_disk_temperature;
    s.kerr.doppler_effect = d->kerr.color_doppler_factor_effect;
    s.kerr.observer = V3(d->kerr.observer[0], d->kerr.observer[1], d->kerr.observer[2]);
    s.kerr.disk_seed = d->kerr.disk_seed;
    if (d->kerr.disk_texture && d->kerr.disk_texture_width > 0 && d->kerr.disk_texture_height > 0) {
      s.kerr.disk_w = d->kerr.disk_texture_width;
      s.kerr.disk_h = d->kerr.disk_texture_height;
      s.kerr.disk_tex.assign(d->kerr.disk_texture, d->kerr.disk_texture + 4 * (size_t)s.kerr.disk_w * s.kerr.disk_h);
    }
    for (const Entity& e : s.ents) {
      if (e.type != PR_ENT_CIRCLE || e.blackhole_disk < 0 || !s.mats[e.material].disk_map) continue;
      // the reference indexes its texture list with blackhole_disk (circle.h:240-242)
      if (s.kerr.disk_tex.empty() || e.blackhole_disk != 0) {
        err = "a disk_map disk under the black hole needs accretion-disk texture 0";
        return PR_E_SCENE;
      }
    }
  }
  // light registration in entity order (scene_env.h:1525-1541, :1567-1586,
  // :1645-1663, :1692-1719) + random_light_setup's sort (light.h:97).
  // Entity::light_id stays the registration index, which the reference
  // later uses to index the sorted list (directLight_radiance.h:541).
  for (int i = 0; i < (int)s.ents.size(); i++) {
    Entity& e = s.ents[i];
    const pr_entity& pe = d->entities[i];
    const Material& m = s.mats[e.material];
    if (!m.isLight()) continue;
    Light l;
    const V3 dir(pe.light_dir[0], pe.light_dir[1], pe.light_dir[2]);
    if (e.type == PR_ENT_INF_LIGHT) {
      l.infinity = 1;
      l.dir = dir;
      l.inf_emission = m.emission;
      l.power = length(m.emission);
      s.lights.push_back(l);
      continue;
    }
    e.light = true;
    l.entity = i;
    l.parallel = pe.parallel_light;
    l.spot = pe.spot_light;
    l.dir = dir;
    if (e.type == PR_ENT_UVPLANE && l.parallel && length(dir) < 1.0e-16) l.dir = e.normal * (double)e.normal_inverse;
    e.light_id = (int)s.lights.size();
    l.power = e.area * length(m.emission);
    if (l.spot) {
      // SpotLightPower of the default cone, before the entity's own angles are set
      l.cos_total = std::cos(30.0 * RAD);
      l.cos_start = std::cos(25.0 * RAD);
      l.power = length(m.emission) * 2.0 * PI * (1.0 - .5 * (l.cos_start + l.cos_total));
      l.cos_total = std::cos(pe.spot_angle[0] * RAD);
      l.cos_start = std::cos((pe.spot_angle[0] - pe.spot_angle[1]) * RAD);
      l.falloff = pe.spot_falloff;
      for (int k = 0; k < 3; k++) l.att[k] = pe.spot_attenuation[k];
      l.center = e.position;
    }
    s.lights.push_back(l);
  }
  std::sort(s.lights.begin(), s.lights.end(), [](const Light& a, const Light& b) { return a.power > b.power; });
  return PR_OK;
}

// --------------------------------------------------------------- radiance
struct Ctx {
  const Scene& s;
  Sampler& rnd;
  int nee, media;
  int depth_cfg, depth_limit;
  int hg_correct;
};

V3 radiance(Ctx& c, V3 org, V3 dir, int depth);

// LightList::randomLight (light.h:132-155): probability reported as 1
const Light& random_light(Ctx& c) {
  const double next = c.rnd.Next01();
  const int n = (int)c.s.lights.size();
  int index = (int)((next) * (double)(n - 1) + 0.5);
  if (index >= n) index = n - 1;
  if (index < 0) index = 0;
  return c.s.lights[index];
}

// eval_direct_radiance for area lights and a diffuse receiver (directLight_radiance.h:19-313)
Material hit_mat(const Scene& s, const Hit& h);

// the BRDF direct_radiance_sample evaluates towards the light: the vertex's
// own reflection type (directLight_radiance.h:211-290)
enum { NEE_DIFFUSE = 0, NEE_WARD = 1, NEE_PHONG = 2 };

V3 eval_direct(Ctx& c, const Light& light, const Hit& v0, V3 orienting_normal, V3 light_pos, int depth,
               int brdf = NEE_DIFFUSE, V3 ray_dir = V3()) {
  V3 light_normal;
  double pdf = 1.0;
  V3 emission;
  if (!light.infinity) {
    const Entity& le = c.s.ents[light.entity];
    if (le.type == PR_ENT_SPHERE) {
      light_normal = normalize(light_pos - le.position);
      if (le.normal_inverse < 0) light_normal = light_normal * -1.0;
      pdf = 1.0 / le.area;
    } else if (le.type == PR_ENT_UVPLANE) {
      light_normal = le.normal;
      if (le.normal_inverse < 0) light_normal = light_normal * -1.0;
      pdf = 1.0 / le.area;
    }
    emission = c.s.mats[le.material].emission;
  } else {
    light_normal = light.dir;
    pdf = 1.0;
    emission = light.inf_emission;
  }
  V3 light_dir = normalize(light_pos - v0.position);
  double dist2 = sqr(light_pos - v0.position);
  double dot0 = dot(orienting_normal, light_dir);
  double dot1 = dot(light_normal, -1.0 * light_dir);
  // directional kinds: fixed direction, no distance or light-side cosine
  // (directLight_radiance.h:84-122); a spot light keeps the cosine of the
  // sampled point at the receiver
  if (light.infinity || light.parallel) {
    light_dir = light.dir * -1.0;
    pdf = 1.0;
    dot1 = 1.0;
    dist2 = 1.0;
    dot0 = dot(orienting_normal, light_dir);
  }
  if (light.spot) {
    light_dir = normalize(light.center - v0.position);
    pdf = 1.0;
    dot1 = 1.0;
    dist2 = 1.0;
  }
  const bool point = light.infinity || light.parallel || light.spot;
  V3 rad;
  if (dot0 >= 0 && dot1 >= 0) {
    const double G = dot0 * dot1 / dist2;
    Hit is;
    const bool isect = intersect(c.s, v0.position, light_dir, is);
    if (isect || light.infinity) {
      const bool cond = point || std::fabs(std::sqrt(dist2) - is.distance) < 1e-3;
      if (cond) {
        if (is.object_id >= 0 && is.object_id != light.entity) return V3();
        if (light.spot) emission = light.spot_emission(emission, light.center, v0.position);
        if (light.infinity) emission = light.inf_emission;
        if (c.media && !light.infinity) {  // env->participatingMedia (directLight_radiance.h:188-204)
          const double t = light.spot ? length(v0.position - light.center) : length(v0.position - light_pos);
          emission = emission * c.s.medium.tr(t);
        }
        const Material vm = hit_mat(c.s, v0);
        if (brdf == NEE_WARD) {
          V3 w, u, v;
          onb(orienting_normal, w, u, v);
          const V3 in = -1.0 * ray_dir;
          const V3 halfv = normalize(in + light_dir);
          const V3 dir = light_dir;
          const double ww0 = std::pow(dot(halfv, orienting_normal), 2.0);
          if (std::fabs(ww0) < 1.0e-16) return V3();
          const double ww1 = (std::pow(dot(halfv, u) / vm.ward_ax, 2.0) + std::pow(dot(halfv, v) / vm.ward_ay, 2.0)) / ww0;
          const double ww2 = 4.0 * PI * vm.ward_ax * vm.ward_ay * std::sqrt(dot(dir, orienting_normal) * dot(in, orienting_normal));
          if (std::fabs(ww2) < 1.0e-16) return V3();
          const double ww = std::exp(-ww1) / ww2;
          if (ww < 0.0) return V3();
          rad = (emission * (vm.specular * ww)) * G / pdf;
        } else if (brdf == NEE_PHONG) {
          const V3 ref = normalize(ray_dir - orienting_normal * 2.0 * dot(orienting_normal, ray_dir));
          if (dot(ref, light_dir) < 0.0) return V3();
          const double ww1 = std::pow(dot(ref, light_dir), vm.phong_n);
          const double ww = ((vm.phong_n + 2) / TWOPI) * ww1;
          if (ww < 0.0) return V3();
          rad = (emission * (vm.specular * ww)) * G / pdf;
        } else if (point) {  // not a diffuse surface light: BRDF = colour (directLight_radiance.h:260-283)
          rad = (emission * vm.color) * G / pdf;
        } else {
          rad = (emission * (vm.color * INV_PI)) * G / pdf;
        }
      }
    }
  }
  // a bump map scales the term by the tilted normal's cosine (directLight_radiance.h:303-310)
  if (v0.bump) rad = (std::max(0.0, dot(light_dir, v0.bump_n)) / dot(light_dir, v0.normal)) * rad;
  return rad;
}

// direct_radiance_sample (directLight_radiance.h:318-387), area lights
V3 direct_sample(Ctx& c, const Light& light, const Hit& v0, V3 orienting_normal, int depth, int brdf = NEE_DIFFUSE,
                 V3 ray_dir = V3()) {
  V3 light_pos;  // an infinity light draws no point (light_pos stays zero)
  if (light.infinity) return eval_direct(c, light, v0, orienting_normal, light_pos, depth, brdf, ray_dir);
  const Entity& le = c.s.ents[light.entity];
  if (le.type == PR_ENT_SPHERE) {  // rnd->Next01() (directLight_radiance.h:343-360)
    const double r1 = TWOPI * c.rnd.Next01();
    const double r2 = 1.0 - 2.0 * c.rnd.Next01();
    const double sq = std::sqrt(1.0 - r2 * r2);
    light_pos = le.position + ((le.radius + EPS) * V3(sq * std::cos(r1), sq * std::sin(r1), r2));
  } else if (le.type == PR_ENT_UVPLANE) {
    const double t = le.v_length * c.rnd.Next01();
    const double s = le.u_length * c.rnd.Next01();
    light_pos = le.org + le.u_axis * s + le.v_axis * t + le.normal * EPS;
  }
  return eval_direct(c, light, v0, orienting_normal, light_pos, depth, brdf, ray_dir);
}

// direct_light_perfect_refrection (directLight_radiance.h:516-556): the
// infinity light met by a miss (infinity_light_direct + InfinityLight,
// light.h:157-173), else a light entity's emission, for a parallel or spot
// light (the kind of the light the entity's registration index points to in
// the sorted list) times the cosine to its direction and the spot's
// emission (parallel_light_direct / spot_light_direct, :406-477); org is the
// specular vertex
V3 direct_perfect(Ctx& c, V3 org, V3 dir, int depth) {
  Hit lid;
  const bool isect = intersect(c.s, org, dir, lid);
  V3 d;
  int exist_infinity_light = 0;
  if (!isect) {
    for (const Light& l : c.s.lights)
      if (l.infinity && std::fabs(dot(l.dir, dir * -1.0) - 1.0) < 1.0e-3) {
        exist_infinity_light++;
        d = l.inf_emission;
        break;
      }
  }
  if (isect && c.s.ents[lid.object_id].light && !exist_infinity_light) {
    const V3 em = c.s.mats[lid.material].emission;
    d = em;
    const Light& light = c.s.lights[c.s.ents[lid.object_id].light_id];
    if (light.parallel) {
      const double dot0 = dot(dir, light.dir * -1.0);
      d = dot0 >= 0.0 ? em * dot0 : V3();
    }
    if (light.spot) {
      const V3 intensity = light.spot_emission(em, light.center, org);
      const double dot0 = dot(dir, normalize(light.center - org));
      d = dot0 >= 0.0 ? intensity * dot0 : V3();
    }
    if (c.media) d = c.s.medium.tr(lid.distance) * d;
  }
  return d;
}

// Entity::isInsideDir (entity.h:98-114); media_ignore_front_back is 0
bool inside_dir(V3 normal, V3 raydir) {
  const V3 on = dot(normal, raydir) < 0.0 ? normal : (-1.0 * normal);
  return dot(on, normal) > 0;
}

// the material of a hit point: the scene's, or the copy the entity rewrote
Material hit_mat(const Scene& s, const Hit& h) {
  if (h.ov_full) return h.ovm;
  Material m = s.mats[h.material];
  if (h.ov) {
    m.color = h.ov_color;
    m.emission = h.ov_emission;
  }
  if (h.ov_spec) m.specular = h.ov_specular;
  return m;
}

// BRDF_Diffuse (brdf.h:408-700), no bump / shadow planes / IBL
V3 brdf_diffuse(Ctx& c, V3 raydir, const Hit& hp, int ent, V3 on, double p_rr, double p_scat, int depth) {
  const Scene& s = c.s;
  const Entity& obj = s.ents[ent];
  const Material mat = hit_mat(s, hp);
  const bool ins = inside_dir(hp.normal, raydir);
  V3 emission = mat.emission;
  V3 trr(1, 1, 1);
  if (c.media) trr = s.medium.tr(hp.distance);
  if (obj.light && obj.type == PR_ENT_UVPLANE) {
    if (dot(hp.normal, raydir) >= 0.0) return V3();
  }
  if (c.nee) {
    if (obj.light) {
      if (depth == 0) return (trr * mat.emission) / p_rr / (1.0 - p_scat);
      return V3();
    }
  } else if (obj.light) {
    return (trr * mat.emission) / p_rr / (1.0 - p_scat);
  }
  V3 w, u, v;
  onb(on, w, u, v);
  const double r1 = TWOPI * c.rnd.next01();
  const double r2 = c.rnd.next01(), r2s = std::sqrt(r2);
  const V3 dir = normalize((u * std::cos(r1) * r2s + v * std::sin(r1) * r2s + w * std::sqrt(1.0 - r2)));
  V3 incoming = radiance(c, hp.position, dir, depth + 1);
  V3 weight = mat.color / p_rr / (1.0 - p_scat);
  if (hp.bump) weight = weight * (std::max(0.1, dot(dir, hp.bump_n)) / dot(dir, hp.normal));  // brdf.h:552-557
  V3 direct;
  if (c.nee && !s.lights.empty()) {
    for (int i = 0; i < 3; i++) {  // SHADOW_RAY_SAMPLING (def.h:10)
      const Light& l = random_light(c);
      direct = direct + direct_sample(c, l, hp, on, depth) / 1.0;
    }
    direct = direct / 3;
    direct = direct / p_rr / (1.0 - p_scat);
  }
  if (!c.nee && !s.lights.empty()) {  // parallel, spot and infinity lights only (brdf.h:590-605)
    for (int i = 0; i < 3; i++) {
      const Light& l = random_light(c);
      if (l.parallel || l.spot || l.infinity) direct = direct + direct_sample(c, l, hp, on, depth) / 1.0;
    }
    direct = direct / 3;
    direct = direct / p_rr / (1.0 - p_scat);
  }
  if (c.media && ins) {
    direct = trr * direct;
    emission = trr * emission;
    incoming = trr * incoming;
  }
  return s.env_light + emission + direct + weight * incoming;
}

// BRDF_Phong (brdf.h:16-190) and BRDF_Ward (brdf.h:192-319): one direction
// from the lobe (cos^n about the mirror direction; Ward's anisotropic
// half-vector sampling about the orienting normal, Walter's "Notes on the
// Ward BRDF"), its radiance first, then three next-event samples evaluated
// with the same lobe; a direction below the surface returns zero for the
// whole vertex
V3 brdf_glossy(Ctx& c, V3 raydir, const Hit& hp, V3 on, double p_rr, double p_scat, int depth, int brdf) {
  const Scene& s = c.s;
  const Material mat = hit_mat(s, hp);
  const bool ins = inside_dir(hp.normal, raydir);
  V3 emission = mat.emission;
  V3 trr(1, 1, 1);
  if (c.media) trr = s.medium.tr(hp.distance);
  V3 dir;
  double ww;
  if (brdf == NEE_PHONG) {
    V3 w, u, v;
    onb(normalize(raydir - on * 2.0 * dot(on, raydir)), w, u, v);
    const double ph = TWOPI * c.rnd.next01();
    double cost = std::pow(c.rnd.next01(), 1.0 / (mat.phong_n + 1.0));
    if (cost > 1.0) cost = 1.0;
    if (cost < -1.0) cost = -1.0;
    const double sint = std::sqrt(1.0 - cost * cost);
    dir = normalize((u * std::cos(ph) * sint + v * std::sin(ph) * sint + w * cost));
    if (dot(on, dir) < 0.0) return V3();
    ww = (mat.phong_n + 2) / (mat.phong_n + 1);
  } else {
    const double ax = mat.ward_ax, ay = mat.ward_ay;
    const V3 in = -1.0 * raydir;
    V3 w, u, v;
    onb(on, w, u, v);
    const double u1 = c.rnd.next01();
    const double u2 = c.rnd.next01();
    double phi = std::atan(ay / ax * std::tan(TWOPI * u2));
    if (0.25 <= u2 && u2 <= 0.75) phi += PI;
    else if (0.75 < u2) phi += TWOPI;
    const double theta = std::atan(std::sqrt(-std::log(u1) / (std::pow(std::cos(phi), 2) / std::pow(ax, 2) +
                                                                 std::pow(std::sin(phi), 2) / std::pow(ay, 2))));
    const V3 halfv = normalize((u * std::cos(phi) * std::sin(theta) + v * std::sin(phi) * std::sin(theta) +
                                w * std::cos(theta)));
    dir = normalize(2.0 * dot(in, halfv) * halfv - in);
    if (dot(on, dir) < 0.0) return V3();
    ww = dot(halfv, in) * std::pow(dot(halfv, on), 3) * std::sqrt(dot(dir, on) / dot(in, on));
  }
  V3 incoming = radiance(c, hp.position, dir, depth + 1);
  V3 weight = mat.specular * ww / p_rr / (1.0 - p_scat);
  if (hp.bump) weight = weight * (std::max(0.1, dot(dir, hp.bump_n)) / dot(dir, hp.normal));  // brdf.h:102-108, :310-316
  V3 direct;
  if (c.nee && !s.lights.empty()) {
    for (int i = 0; i < 3; i++) {
      const Light& l = random_light(c);
      direct = direct + direct_sample(c, l, hp, on, depth, brdf, raydir) / 1.0;
    }
    direct = direct / 3;
    direct = direct / p_rr / (1.0 - p_scat);
  }
  if (!c.nee && !s.lights.empty()) {  // parallel, spot and infinity lights only (brdf.h:128-146)
    for (int i = 0; i < 3; i++) {
      const Light& l = random_light(c);
      if (l.parallel || l.spot || l.infinity) direct = direct + direct_sample(c, l, hp, on, depth, brdf, raydir) / 1.0;
    }
    direct = direct / 3;
    direct = direct / p_rr / (1.0 - p_scat);
  }
  if (c.media && ins) {
    direct = trr * direct;
    emission = trr * emission;
    incoming = trr * incoming;
  }
  return s.env_light + emission + direct + weight * incoming;
}

// BRDF_Specular (brdf.h:702-761)
V3 brdf_specular(Ctx& c, V3 raydir, const Hit& hp, double p_rr, double p_scat, int depth) {
  const Scene& s = c.s;
  const Material mat = hit_mat(s, hp);
  const bool ins = inside_dir(hp.normal, raydir);
  V3 emission = mat.emission;
  V3 trr(1, 1, 1);
  if (c.media) trr = s.medium.tr(hp.distance);
  const V3 dir = normalize(raydir - hp.normal * 2.0 * dot(hp.normal, raydir));
  V3 incoming = radiance(c, hp.position, dir, depth + 1);
  V3 weight = mat.color / p_rr / (1.0 - p_scat);
  if (c.nee) incoming = incoming + direct_perfect(c, hp.position, dir, depth);
  if (hp.bump) weight = weight * (std::max(0.1, dot(dir, hp.bump_n)) / dot(dir, hp.normal));  // brdf.h:740-745
  if (c.media && ins) {
    emission = trr * emission;
    incoming = trr * incoming;
  }
  return s.env_light + emission + weight * incoming;
}

// BRDF_Refraction (brdf.h:763-953), no bump
V3 brdf_refraction(Ctx& c, V3 raydir, const Hit& hp, int mat_type, V3 on, double p_rr, double p_scat, int depth) {
  const Scene& s = c.s;
  const Material mat = hit_mat(s, hp);
  const bool ins = inside_dir(hp.normal, raydir);
  V3 emission = mat.emission;
  V3 trr(1, 1, 1);
  if (c.media) trr = s.medium.tr(hp.distance);
  V3 incoming, weight(1, 1, 1), direct, direct_r;
  const V3 refl = normalize(raydir - hp.normal * 2.0 * dot(hp.normal, raydir));
  const bool into = dot(hp.normal, on) > 0.0;
  if (c.nee) direct = direct_perfect(c, hp.position, refl, depth);
  const double nc = 1.0;
  const double nt = mat.refractive_index;  // FORMULA0 (material.h)
  const double nnt = into ? nc / nt : nt / nc;
  const double ddn = dot(raydir, on);
  const double cos2t = 1.0 - nnt * nnt * (1.0 - ddn * ddn);
  if (cos2t < 0.0) {
    incoming = radiance(c, hp.position, refl, depth + 1);
    weight = mat.color / p_rr / (1.0 - p_scat);
    incoming = incoming + direct;
  } else {
    const V3 tdir = normalize(raydir * nnt - hp.normal * (into ? 1.0 : -1.0) * (ddn * nnt + std::sqrt(std::fabs(cos2t))));
    const double a = nt - nc, b = nt + nc;
    const double R0 = (a * a) / (b * b);
    const double cc = 1.0 - (into ? -ddn : dot(tdir, -1.0 * on));
    double Re = R0 + (1.0 - R0) * std::pow(cc, 5.0);
    const double nnt2 = std::pow(into ? nc / nt : nt / nc, 2.0);
    double Tr = (1.0 - Re) * nnt2;
    double probability = 0.25 + 0.5 * Re;
    if (mat_type == PR_MAT_REFRACTION_FRESNEL) {
      if (into) { probability = 1.0; Re = 1.0; Tr = 0.0; }
      else { probability = 0.0; Re = 0.0; Tr = 1.0; }
    }
    if (c.nee) direct_r = direct_perfect(c, hp.position, tdir, depth);
    if (depth > 2) {
      if (c.rnd.next01() < probability) {
        incoming = (radiance(c, hp.position, refl, depth + 1)) * Re;
        weight = mat.color / (probability * p_rr) / (1.0 - p_scat);
        incoming = incoming + direct;
      } else {
        incoming = (radiance(c, hp.position, tdir, depth + 1)) * Tr;
        weight = mat.color / ((1.0 - probability) * p_rr) / (1.0 - p_scat);
        incoming = incoming + direct_r;
      }
    } else {
      // g++ evaluates the right operand of the reference's
      // 'radiance(refl)*Re + radiance(tdir)*Tr' first (brdf.h:928-930)
      const V3 l2 = radiance(c, hp.position, tdir, depth + 1);
      const V3 l1 = radiance(c, hp.position, refl, depth + 1);
      incoming = l1 * Re + l2 * Tr;
      weight = mat.color / (p_rr) / (1.0 - p_scat);
      incoming = incoming + direct + direct_r;
    }
  }
  if (c.media && ins) {
    emission = trr * emission;
    incoming = trr * incoming;
  }
  return s.env_light + emission + weight * incoming;
}

// sampleSphere / sampleHG (sampler.h:24-93)
V3 sample_sphere(Ctx& c) {
  const double r1 = TWOPI * c.rnd.next01();
  const double r2 = 1.0 - 2.0 * c.rnd.next01();
  const double r22 = (r2 < 1.0) ? 1.0 - r2 * r2 : 0.0;
  const double sq = std::sqrt(r22);
  return normalize(V3(sq * std::cos(r1), sq * std::sin(r1), r2));
}
V3 sample_hg(Ctx& c, V3 raydir, double g) {
  if (g == 0.0) return sample_sphere(c);
  V3 w, u, v;
  onb(raydir, w, u, v);
  const double r1 = TWOPI * c.rnd.next01();
  const double r2 = c.rnd.next01();
  const double s = (1.0 - g * g) / (1.0 - g + 2.0 * g * r2);
  // the reference parses (1.0 / 2.0*g) as (1/2)*g (sampler.h:55-56)
  const double cost = c.hg_correct ? (1.0 / (2.0 * g)) * (1.0 + g * g - s * s) : (1.0 / 2.0 * g) * (1.0 + g * g - s * s);
  const double sint = std::sqrt(std::max(0.0, 1.0 - cost * cost));
  return normalize(sint * std::cos(r1) * u + sint * std::sin(r1) * v + cost * w);
}
// PhaseFunction_HenyeyGreenstein (phase.h:14-20)
double phase_hg(double g, double costheta) {
  const double w = 1.0 + g * g - 2.0 * g * costheta;
  if (std::fabs(w) < EPS12) return 0.0;
  return (INV_FORPI) * (1.0 - g * g) / std::pow(w, 3.0 / 2.0);
}

// eval_direct_radiance_media / direct_radiance_sample_media (ParticipatingMedia.h:27-268)
V3 direct_media(Ctx& c, const Light& light, V3 pos, int depth) {
  V3 light_pos, light_normal;
  double pdf = 1.0;
  V3 emission;
  if (!light.infinity) {
    const Entity& le = c.s.ents[light.entity];
    if (le.type == PR_ENT_SPHERE) {
      const double r1 = 2 * PI * c.rnd.next01();
      const double r2 = 1.0 - 2.0 * c.rnd.next01();
      light_pos = le.position + ((le.radius + EPS) * V3(std::sqrt(1.0 - r2 * r2) * std::cos(r1), std::sqrt(1.0 - r2 * r2) * std::sin(r1), r2));
    } else if (le.type == PR_ENT_UVPLANE) {
      const double t = le.v_length * c.rnd.next01();
      const double s = le.u_length * c.rnd.next01();
      light_pos = le.org + le.u_axis * s + le.v_axis * t;
    }
  }
  // transmittance over the distance to the point (spot: the centre; infinity: none)
  double tt = length(pos - light_pos);
  if (light.spot) tt = length(pos - light.center);
  if (light.infinity) tt = 0.0;
  const V3 trr = c.s.medium.tr(tt);
  // eval_direct_radiance_media
  if (!light.infinity) {
    const Entity& le = c.s.ents[light.entity];
    if (le.type == PR_ENT_SPHERE) {
      light_normal = normalize(light_pos - le.position);
      pdf = 1.0 / le.area;
    } else {
      light_normal = le.normal;
      pdf = 1.0 / le.area;
    }
    emission = c.s.mats[le.material].emission;
  } else {
    light_normal = light.dir;
    pdf = 1.0;
    emission = light.inf_emission;
  }
  V3 light_dir = normalize(light_pos - pos);
  double dist2 = sqr(light_pos - pos);
  double dot1 = dot(light_normal, -1.0 * light_dir);
  if (light.infinity || light.parallel) {
    light_dir = light.dir * -1.0;
    pdf = 1.0;
    dot1 = 1.0;
    dist2 = 1.0;
  }
  if (light.spot) {
    light_dir = normalize(light.center - pos);
    pdf = 1.0;
    dot1 = 1.0;
    dist2 = 1.0;
  }
  const bool point = light.infinity || light.parallel || light.spot;
  V3 rad;
  if (dot1 >= 0) {
    const double G = dot1 / dist2;
    Hit is;
    const bool isect = intersect(c.s, pos, light_dir, is);
    if (isect || light.infinity) {
      if (point || std::fabs(std::sqrt(dist2) - is.distance) < 1e-3) {
        if (!(is.object_id >= 0 && is.object_id != light.entity)) {
          if (light.spot) emission = light.spot_emission(emission, light.center, pos);
          rad = point ? emission * G / pdf : emission * (1.0 / PI) * G / pdf;
        }
      }
    }
  }
  return rad * trr;
}

// participatingMedia_radiance (ParticipatingMedia.h:300-461)
V3 media_radiance(Ctx& c, V3 org, V3 raydir, const Hit& hp, int ent, double p_rr, double p_scat, int depth) {
  const Scene& s = c.s;
  const Medium& md = s.medium;
  const Entity& obj = s.ents[ent];
  const int select = std::min(2, (int)(3.0 * c.rnd.next01()));
  const double u = c.rnd.next01();
  const double d = -std::log(1.0 + u * (std::exp(-md.transmittance * hp.distance) - 1.0)) / md.transmittance;
  const double pdf = std::exp(-md.transmittance * d) * (-md.transmittance / (std::exp(-md.transmittance * hp.distance) - 1.0));
  V3 next_dir;
  double phase;
  const double g = md.phase[select];
  if (g == 0.0 || std::fabs(g) > 1.0) {
    next_dir = sample_sphere(c);
    phase = INV_FORPI;
  } else {
    next_dir = sample_hg(c, raydir, g);
    phase = phase_hg(g, dot(next_dir, raydir));
  }
  const double dirPdf = phase;
  const V3 npos = org + d * raydir;
  const V3 trr = md.tr(d);
  V3 direct;
  if (!obj.light) {
    if (!s.lights.empty()) {
      for (int i = 0; i < 3; i++) {
        const Light& l = random_light(c);
        direct = direct + direct_media(c, l, npos, depth) / 1.0;
      }
      direct = direct / 3;
    }
  }
  if (pdf == 0.0) return V3();
  if (obj.light) {
    if (depth == 0) return trr * hit_mat(s, hp).emission;
    return V3();
  }
  V3 L = direct + radiance(c, npos, next_dir, depth + 1);
  L = trr * md.scatteringColor * L * phase / pdf / dirPdf / p_scat / p_rr;
  return L;
}

// ---------------------------------------------------------------- BSSRDF
// Directional dipole of Frisvad, Hachisuka and Kjeldsen, "Directional
// Dipole Model for Subsurface Scattering" (ACM TOG 2014), as the reference
// evaluates it (bssrdf.h:48-248), and the dipole branch of BRDF_SSS2_
// (Subsurface_Scattering.h:630-1181) for level -2 materials.
double dd_C1(double n) {  // 2 C1 / 2 of the paper's moment polynomials (bssrdf.h:48-61)
  double r;
  if (n > 1.0) r = -9.23372 + n * (22.2272 + n * (-20.9292 + n * (10.2291 + n * (-2.54396 + 0.254913 * n))));
  else r = 0.919317 + n * (-3.4793 + n * (6.75335 + n * (-7.80989 + n * (4.98554 - 1.36881 * n))));
  return r / 2.0;
}
double dd_C2(double n) {  // bssrdf.h:63-67
  double r = -1641.1 + n * (1213.67 + n * (-568.556 + n * (164.798 + n * (-27.0181 + 1.91826 * n))));
  r += (((135.926 / n) - 656.175) / n + 1376.53) / n;
  return r / 3.0;
}
inline V3 vsqrt(V3 a) { return V3(std::sqrt(a.x), std::sqrt(a.y), std::sqrt(a.z)); }
inline V3 vdiv(V3 a, V3 b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline double vmin(V3 a) {  // Vector3d::Min
  double m = a.x;
  if (m > a.y) m = a.y;
  if (m > a.z) m = a.z;
  return m;
}
inline double comp(V3 a, int j) { return j == 0 ? a.x : (j == 1 ? a.y : a.z); }

struct Dipole {  // DirectionalDipole (bssrdf.h:75-128)
  V3 sigma_s, sigma_a, sigma_t, sigma_sp, sigma_tp, albedo_p, D, sigma_tr, de;
  double Cp, Ce, A, eta;
  Dipole(const Material& m, double eta_) {
    eta = eta_;
    sigma_a = m.medium.absorbingColor;
    sigma_s = m.medium.scatteringColor;
    sigma_t = sigma_s + sigma_a;
    sigma_sp = sigma_s * (V3(1.0, 1.0, 1.0) - V3(m.medium.phase[0], m.medium.phase[1], m.medium.phase[2]));
    sigma_tp = sigma_sp + sigma_a;
    albedo_p = vdiv(sigma_sp, sigma_tp);
    D = vdiv(V3(1.0, 1.0, 1.0), 3.0 * sigma_tp);
    sigma_tr = vsqrt(vdiv(sigma_a, D));
    de = vdiv(2.131 * D, vsqrt(albedo_p));
    Cp = (1.0 - 2.0 * dd_C1(eta)) / 4.0;
    Ce = (1.0 - 3.0 * dd_C2(eta)) / 2.0;
    A = (1.0 - Ce) / (2.0 * Cp);
  }
};

// Sp_d (bssrdf.h:131-172)
double dd_sp(const Dipole& dd, V3 x, V3 w, double r, V3 n0, int j) {
  const double s_tr_r = comp(dd.sigma_tr, j) * r;
  const double s_tr_r_one = 1.0 + s_tr_r;
  const double x_dot_w = dot(x, w);
  const double r_sqr = r * r;
  const double exp_tr = std::exp(-s_tr_r);
  const double t0 = 1.0 / (4.0 * dd.Cp) * (0.02533029591058444286096986580243191) * exp_tr / (r * r_sqr);
  const double t1 = r_sqr / comp(dd.D, j) + 3.0 * s_tr_r_one * x_dot_w;
  const double t2 = 3.0 * comp(dd.D, j) * s_tr_r_one * dot(w, n0);
  const double t3 = (s_tr_r_one + 3.0 * comp(dd.D, j) * (3.0 * s_tr_r_one + s_tr_r * s_tr_r) / r_sqr * x_dot_w) * dot(x, n0);
  return t0 * (dd.Cp * t1 - dd.Ce * (t2 - t3));
}

// bssrdf (bssrdf.h:188-236)
double dd_bssrdf(const Dipole& dd, V3 xi, V3 ni, V3 wi, V3 xo, V3 no, V3 wo, int j) {
  (void)wo;
  const V3 xoxi = xo - xi;
  const double r = length(xoxi);
  V3 ni_s = cross(normalize(xoxi), normalize(cross(ni, xoxi)));
  if (r < 1.0e-8) ni_s = ni;
  const double nnt = 1.0 / dd.eta, ddn = -dot(wi, ni);
  const V3 w12 = normalize(wi * -nnt - ni * (ddn * nnt + std::sqrt(1.0 - nnt * nnt * (1.0 - ddn * ddn))));
  const V3 wv = w12 - ni_s * (2.0 * dot(w12, ni_s));
  const double dej = comp(dd.de, j), Dj = comp(dd.D, j);
  const double cos_beta = -std::sqrt((r * r - dot(xoxi, w12) * dot(xoxi, w12)) / (r * r + dej * dej));
  double dr;
  const double mu0 = -dot(no, w12);
  if (mu0 > 0.0) {
    double tmp = (Dj * mu0) * ((Dj * mu0) - dej * cos_beta * 2.0) + r * r;
    if (tmp < 0) tmp = 0.0;
    dr = std::sqrt(tmp);
  } else {
    const double st = comp(dd.sigma_t, j);
    double tmp = 1.0 / (3.0 * st * 3.0 * st) + r * r;
    if (tmp < 0) tmp = 0.0;
    dr = std::sqrt(tmp);
  }
  const V3 xoxv = xo - (xi + ni_s * (2.0 * dd.A * dej));
  const double dv = length(xoxv);
  const double result = dd_sp(dd, xoxi, w12, dr, no, j) - dd_sp(dd, xoxv, wv, dv, no, j);
  return (result < 0.0) ? 0.0 : result;
}

// fresnel (bssrdf.h:239-247)
double dd_fresnel(double cos_theta, double eta) {
  const double sin_theta_t_sqr = 1.0 / (eta * eta) * (1.0 - cos_theta * cos_theta);
  if (sin_theta_t_sqr >= 1.0) return 1.0;
  const double cos_theta_t = std::sqrt(1.0 - sin_theta_t_sqr);
  const double r_s = (cos_theta - eta * cos_theta_t) / (cos_theta + eta * cos_theta_t);
  const double r_p = (eta * cos_theta - cos_theta_t) / (eta * cos_theta + cos_theta_t);
  return (r_s * r_s + r_p * r_p) * 0.5;
}

// gaussianSample2D / gaussianSample2DPdf (Subsurface_Scattering.h:612-628)
V3 gauss_sample_2d(double u1, double u2, double falloff, double rmax) {
  const double r = std::sqrt(std::log(1.0 - u1 * (1.0 - std::exp(-falloff * rmax * rmax))) / -falloff);
  const double theta = TWOPI * u2;
  return V3(r * std::cos(theta), r * std::sin(theta), 0);
}
double gauss_pdf_2d(V3 pc, V3 ps, V3 N, double falloff, double rmax) {
  const V3 d = ps - pc;
  const V3 projected = d - N * dot(d, N);
  const double pdf = falloff * std::exp(-falloff * sqr(projected)) / PI;
  return pdf / (1.0f - std::exp(-falloff * rmax * rmax));
}

V3 radiance(Ctx& c, V3 org, V3 dir, int depth);
V3 direct_sample(Ctx& c, const Light& light, const Hit& v0, V3 orienting_normal, int depth, int brdf, V3 ray_dir);
V3 brdf_refraction(Ctx& c, V3 raydir, const Hit& hp, int mat_type, V3 on, double p_rr, double p_scat, int depth);
const Light& random_light(Ctx& c);
bool inside_dir(V3 normal, V3 raydir);

// BRDF_SSS2_ (Subsurface_Scattering.h:630-1181) for level -2: Gaussian-disk
// probe rays for the exit point, the directional dipole, NEE at the exit,
// or (accept 0.5) the Fresnel-surface refraction; raydir is the refracted
// direction radiance() passes in
V3 radiance(Ctx& c, V3 org, V3 dir, int depth);

// radiance_through_media (Subsurface_Scattering.h:31-543): a walk inside the
// subsurface object in_ent with at most sc_max scattering events.  At
// sc_depth 0 it always scatters: a distance sampled towards the far side,
// a phase-function direction retried (up to 145 times) until it leaves the
// object or enters another; at sc_max it leaves: across the object's
// surface (refracted, or mirrored under total internal reflection) with
// the surface colour and three next-event samples there, or into another
// object.  The Fresnel factors it computes are not applied.
V3 through_media(Ctx& c, V3 org, V3 dir, int depth, int in_ent, int sc_depth, int sc_max) {
  const Scene& s = c.s;
  const Material& im = s.mats[s.ents[in_ent].material];
  const Medium& pm = im.medium;
  double dirPdf = 1.0, phase = 1.0;
  double rr2 = 1.0;
  if (depth > c.depth_limit * 30) {
    rr2 *= std::min(std::pow(0.5, depth - c.depth_limit), std::pow(0.5, sc_depth));
    if (c.rnd.next01() >= rr2) return im.emission;
  } else {
    rr2 = 1.0;
  }
  Hit out;
  if (!intersect(s, org, dir, out)) return V3();
  const double sig0 = pm.transmittanceColor[pm.sample(c.rnd.next01(), 0)];
  double probability = 1.0 - std::exp(-sig0 * out.distance);
  if (probability < 0) probability = 0;
  else if (probability > 1.0) probability = 1.0;
  if (sc_depth == 0) probability = 1.0;
  if (sc_depth == sc_max || out.distance < 1.0e-4) probability = 0;
  bool sss = (c.rnd.next01() < probability);
  if (sss) {
    double d = 0.0, pdf = 1.0;
    const double p_pdf = 1;
    V3 new_org = org, nd = dir;
    sss = false;
    for (int kk = 0; kk < 145; kk++) {
      (void)pm.sample(c.rnd.next01(), 1);  // an unused channel draw
      const int ii = pm.sample(c.rnd.next01(), 1);
      const double st = pm.transmittanceColor[ii];
      const double b = out.distance;
      const double t = -std::log(1.0 + c.rnd.next01() * (std::exp(-st * b) - 1.0)) / st;
      pdf = std::exp(-st * t) * (-st / (std::exp(-st * b) - 1.0));
      d = t;
      new_org = org + d * dir;
      nd = dir;
      if (sc_depth < 1) {
        Hit w;
        if (intersect(s, org, dir, w) && w.distance < length(new_org - org) && w.object_id == in_ent) continue;
      }
      const int select = pm.sample(c.rnd.next01(), 0);
      const double g = pm.phase[select];
      if (g == 0.0 || std::fabs(g) > 1.0) {
        nd = sample_sphere(c);
        phase = INV_FORPI;
      } else {
        nd = sample_hg(c, dir, g);
        phase = phase_hg(g, dot(dir, nd));
      }
      dirPdf = phase;
      Hit w;
      if (!intersect(s, new_org, nd, w)) continue;
      const bool insidedir = inside_dir(w.normal, nd);
      if (w.object_id == in_ent) {
        if (insidedir) continue;
        sss = true;
        break;
      }
      if (insidedir) {
        sss = true;
        break;
      }
    }
    if (!sss) return V3();
    const V3 Tr = pm.tr(d);
    const V3 Ld = through_media(c, new_org, nd, depth + 1, in_ent, sc_depth + 1, sc_max);
    const V3 Li = Tr * pm.scatteringColor * Ld * phase / pdf / dirPdf / probability / rr2 / p_pdf;
    if (length(Li) > 100) return V3();  // OVER_RADIANCE_CUT0
    return Li;
  }
  const V3 Tr = pm.tr(out.distance);
  if (out.object_id != in_ent) return Tr * radiance(c, out.position, dir, depth + 1) / (1.0 - probability) / rr2;
  // leaving across the object's own surface
  const V3 out_on = dot(out.normal, dir) < 0.0 ? out.normal : (-1.0 * out.normal);
  const V3 refl = normalize(dir - out.normal * 2.0 * dot(out.normal, dir));
  V3 nd = dir;
  {
    const double nc = 1.0, nt = s.mats[out.material].refractive_index;
    const bool into = dot(out.normal, dir) < 0.0;
    const double nnt = into ? nc / nt : nt / nc;
    const double ddn = dot(dir, out_on);
    const double cos2t = 1.0 - nnt * nnt * (1.0 - ddn * ddn);
    if (cos2t > 0) nd = normalize(dir * nnt - out.normal * (into ? 1.0 : -1.0) * (ddn * nnt + std::sqrt(std::fabs(cos2t))));
    if (cos2t < 0) nd = refl;
  }
  const V3 weight = Tr * s.mats[out.material].color / (1.0 - probability) / rr2;
  const V3 Li = radiance(c, out.position, nd, depth + 1);
  V3 direct;
  if (c.nee && !s.lights.empty()) {
    for (int i = 0; i < 3; i++) {
      const Light& l = random_light(c);
      direct = direct + direct_sample(c, l, out, out.normal, depth, NEE_DIFFUSE, V3()) / 1.0;
    }
    direct = direct / 3;
  }
  if (!c.nee && !s.lights.empty()) {  // parallel, spot and infinity lights only (Subsurface_Scattering.h:519-535)
    for (int i = 0; i < 3; i++) {
      const Light& l = random_light(c);
      if (l.parallel || l.spot || l.infinity)
        direct = direct + direct_sample(c, l, out, out.normal, depth, NEE_DIFFUSE, V3()) / 1.0;
    }
    direct = direct / 3;
  }
  return (direct + Li) * weight;
}

V3 brdf_sss2(Ctx& c, V3 raydir, const Hit& hp, int ent, V3 on, double p_rr, double p_scat, int depth) {
  const Scene& s = c.s;
  const Material& hm = s.mats[hp.material];
  const bool ins = inside_dir(hp.normal, raydir);
  V3 emission = hm.emission;
  V3 trr(1, 1, 1);
  if (c.media) trr = s.medium.tr(hp.distance);
  const double eta = hm.r_refractive_index;
  const Dipole dd(hm, eta);
  const Entity& obj = s.ents[ent];
  const Medium& pm = s.mats[obj.material].medium;
  V3 incoming, weight(1, 1, 1), direct;
  Hit out = hp;
  out.object_id = ent;
  double samplePDF = 1.0, sampleDir = 1.0;
  const int sampleN = 40;
  int err = 1;
  // samplingType 2 (Gaussian disk), rmax heuristic (:701-714)
  double sigmaTr = vmin(dd.sigma_tp);
  const double sigmaTrCoef = 0.001;
  double rmax;
  {
    const double skipRatio = 1.0e-4;
    const double x = vmin(pm.scatteringColor);
    double y = 2.0 - 1.0 / (1.0 + std::exp(-4.0 * (x - 1.6)));
    if (pm.absorbing < 0.001) y *= 1.3 - std::exp(vmin(pm.absorbingColor) * 1000.0);
    rmax = 1.25 * std::sqrt(std::log(skipRatio) / -sigmaTr) * y * pm.r_max;
  }
  const double ln = length(obj.bb_max - obj.bb_min);
  if (rmax > ln) rmax = ln * 0.3;
  const double step = 0.5 * rmax / sampleN;
  V3 on2, dir;
  for (int i = sampleN; i >= 1; i--) {
    err = 1;
    V3 ww, u, v;
    onb(on, ww, u, v);
    // g++ evaluates 'gaussianSample2D(rnd->next01(), rnd->next01(), ...)'
    // right to left: the second argument draws first
    const double u2 = c.rnd.next01();
    const double u1 = c.rnd.next01();
    const V3 pSample = gauss_sample_2d(u1, u2, sigmaTr * sigmaTrCoef, rmax);
    const V3 p = hp.position + pSample.x * u + pSample.y * v;
    const double halfProbeLength = i * step;
    // intersect_scene ignores its target id: the probe takes the closest hit
    if (!intersect(s, p - on * halfProbeLength, on, out)) continue;
    on2 = out.normal;
    samplePDF = gauss_pdf_2d(V3(0, 0, 0), pSample, V3(0, 0, 1), sigmaTr * sigmaTrCoef, rmax);
    if (dot(hp.normal, on) < 0) on2 = -1.0 * on2;
    onb(on2, ww, u, v);
    const double r1 = TWOPI * c.rnd.next01();
    const double r2 = c.rnd.next01(), r2s = std::sqrt(r2);
    dir = normalize((u * std::cos(r1) * r2s + v * std::sin(r1) * r2s + ww * std::sqrt(1.0 - r2)));
    sampleDir = dot(on2, dir) * INV_PI;
    if (sampleDir > 0) {
      err = 0;
      break;
    }
  }
  if (err) return V3();
  const V3 w = -1.0 * raydir, x = hp.position, n = on;
  const V3 sw = dir, sp = out.position, sn = on2;
  const double cos_wi_n = dot(sn, sw);
  if (cos_wi_n < 0.0) return V3();
  const double T21 = std::max(1.0 - dd_fresnel(dot(w, n), eta), 0.0);
  const double T12 = std::max(1.0 - dd_fresnel(cos_wi_n, eta), 0.0);
  double accept_prob = 0.5;
  const bool into = dot(hp.normal, on) > 0.0;
  if (!into) accept_prob = 0;
  if (c.rnd.next01() < accept_prob) {
    double pms = 0.5;
    if (pm.level == -2) pms = 1;
    if (c.rnd.next01() < pms) {
      V3 result;
      result.x = dd_bssrdf(dd, sp, sn, sw, x, n, w, 0);
      result.y = dd_bssrdf(dd, sp, sn, sw, x, n, w, 1);
      result.z = dd_bssrdf(dd, sp, sn, sw, x, n, w, 2);
      weight = hm.color * T12 * result * cos_wi_n * T21 / samplePDF / sampleDir / accept_prob / p_rr /
               (1.0 - p_scat) / pms;
      incoming = radiance(c, sp, sw, depth + 1);
      if (c.nee && !s.lights.empty()) {
        for (int k = 0; k < 3; k++) {
          const Light& l = random_light(c);
          direct = direct + direct_sample(c, l, out, on2, depth, NEE_DIFFUSE, V3()) / 1.0;
        }
        direct = direct / 3;
        direct = direct * T12 * result * cos_wi_n * T21 / samplePDF / sampleDir / accept_prob / p_rr /
                 (1.0 - p_scat);
      }
      if (!c.nee && !s.lights.empty()) {
        // parallel, spot and infinity lights only, sampled at the ENTRY point
        // with its orienting normal (Subsurface_Scattering.h:989-1010; the
        // NEE branch above takes the exit point)
        for (int k = 0; k < 3; k++) {
          const Light& l = random_light(c);
          if (l.parallel || l.spot || l.infinity)
            direct = direct + direct_sample(c, l, hp, on, depth, NEE_DIFFUSE, V3()) / 1.0;
        }
        direct = direct / 3;
        direct = direct * T12 * result * cos_wi_n * T21 / samplePDF / sampleDir / accept_prob / p_rr /
                 (1.0 - p_scat);
      }
      if (length(incoming * weight) > 100) return V3();  // OVER_RADIANCE_CUT2
    } else {
      // single scattering (level -1): the walk radiance_through_media takes
      // from just inside the entry point along the refracted direction
      weight = hm.color / accept_prob / p_rr / (1.0 - p_scat) / (1.0 - pms);
      incoming = through_media(c, hp.position - hp.normal * 0.0001, raydir, depth + 1, ent, 0, 1);
      if (length(incoming * weight) > 100) return V3();  // OVER_RADIANCE_CUT2
    }
  } else {
    V3 Tr(1, 1, 1);
    if (!into) Tr = pm.tr(hp.distance);
    weight = Tr / (1.0 - accept_prob);
    incoming = brdf_refraction(c, raydir, hp, PR_MAT_REFRACTION, on, p_rr, p_scat, depth);
    if (length(incoming * weight) > 200) return V3();  // OVER_RADIANCE_CUT3
    direct = V3();
  }
  if (c.media && ins) {
    direct = trr * direct;
    emission = trr * emission;
    incoming = trr * incoming;
  }
  return s.env_light + emission + direct + weight * incoming;
}

// Kerr branch of intersect_scene (defined with the Kerr restatement below);
// on a miss, miss_color is what radiance() returns for it (radiance.h:30-43)
bool kerr_query(const Scene& s, V3 org, V3 dir, Hit& hit, V3& miss_color);
bool worm_query(const Scene& s, V3 org, V3 dir, Hit& hit, V3& miss_color);

// radiance() (radiance.h:25-556): diffuse / specular / refraction / media
V3 radiance(Ctx& c, V3 org, V3 dir, int depth) {
  const Scene& s = c.s;
  Hit hp;
  if (s.kerr.on) {
    V3 miss;
    if (!kerr_query(s, org, dir, hp, miss)) return miss;
  } else if (s.worm.on) {
    V3 miss;
    if (!worm_query(s, org, dir, hp, miss)) return miss;
  } else if (!intersect(s, org, dir, hp)) {
    return s.background;
  }
  const Material mat = hit_mat(s, hp);
  // an object with an IBL image gives its hit point's emission and nothing
  // else (radiance.h:45-50, IBL_LIGHT 0)
  if (mat.ibl) return mat.emission;
  const V3 on = dot(hp.normal, dir) < 0.0 ? hp.normal : (-1.0 * hp.normal);
  V3 rw = mat.emission;
  switch (mat.type) {
    case PR_MAT_WARD: rw = rw + mat.color + mat.specular; break;
    case PR_MAT_PHONG: rw = rw + mat.specular; break;
    default: rw = rw + mat.color; break;
  }
  // RGB_MAX (def.h): std::max(x, std::max(y, z))
  const double myz = (rw.y < rw.z) ? rw.z : rw.y;
  double p_rr = (rw.x < myz) ? myz : rw.x;
  if (depth > c.depth_limit) p_rr *= std::pow(0.5, depth - c.depth_limit);
  if (depth > c.depth_cfg) {
    if (c.rnd.next01() >= p_rr) {
      V3 trr(1, 1, 1);
      if (c.media) trr = s.medium.tr(hp.distance);
      return trr * mat.emission;
    }
  } else {
    p_rr = 1.0;
  }
  const bool from_outside = inside_dir(hp.normal, dir);
  double p_scat = 0.0;
  if (c.media && from_outside) {
    p_scat = 1.0 - std::exp(-s.medium.scattering * hp.distance);
    if (p_scat < 0.01) p_scat = 0.01;
    else if (p_scat > 0.99) p_scat = 0.99;
    if (c.rnd.next01() < p_scat) return media_radiance(c, org, dir, hp, hp.object_id, p_rr, p_scat, depth);
  }
  switch (mat.type) {
    case PR_MAT_DIFFUSE:
      if (c.rnd.next01() < mat.roughness) return brdf_diffuse(c, dir, hp, hp.object_id, on, p_rr, p_scat, depth);
      return brdf_specular(c, dir, hp, p_rr, p_scat, depth);
    case PR_MAT_SPECULAR:
      if (c.rnd.next01() < 1.0 - mat.roughness) return brdf_specular(c, dir, hp, p_rr, p_scat, depth);
      return brdf_diffuse(c, dir, hp, hp.object_id, on, p_rr, p_scat, depth);
    case PR_MAT_PHONG:  // radiance.h:470-484: diffuse with probability roughness
      if (c.rnd.next01() < mat.roughness) return brdf_diffuse(c, dir, hp, hp.object_id, on, p_rr, p_scat, depth);
      return brdf_glossy(c, dir, hp, on, p_rr, p_scat, depth, NEE_PHONG);
    case PR_MAT_WARD: {  // radiance.h:493-509: diffuse with probability rd / (rd + rs)
      const double rd = (mat.color.x + mat.color.y + mat.color.z) / 3.0;
      const double rs = (mat.specular.x + mat.specular.y + mat.specular.z) / 3.0;
      const double diffuse_probability = rd / (rs + rd);
      const double u = c.rnd.next01();
      if (u < diffuse_probability) return brdf_diffuse(c, dir, hp, hp.object_id, on, p_rr, p_scat, depth);
      return brdf_glossy(c, dir, hp, on, p_rr, p_scat, depth, NEE_WARD);
    }
    case PR_MAT_REFRACTION:
    case PR_MAT_REFRACTION_FRESNEL:
      return brdf_refraction(c, dir, hp, mat.type, on, p_rr, p_scat, depth);
    case PR_MAT_SSS_REFRACTION: {
      // radiance.h:154-224 (use_brssdf, level -2): refract into the object,
      // then the dipole (BRDF_SSS2) with the refracted direction
      const bool into = dot(hp.normal, on) > 0.0;
      const double nc = 1.0;
      const double nt = mat.refractive_index;
      const double nnt = into ? nc / nt : nt / nc;
      const double ddn = dot(dir, on);
      const double cos2t = 1.0 - nnt * nnt * (1.0 - ddn * ddn);
      V3 tdir = normalize(dir * nnt - hp.normal * (into ? 1.0 : -1.0) * (ddn * nnt + std::sqrt(std::fabs(cos2t))));
      if (cos2t < 0) tdir = normalize(dir - on * 2.0 * dot(on, dir));
      V3 tr(1, 1, 1);
      if (!into) tr = mat.medium.tr(hp.distance);
      const double probability = 1;
      (void)c.rnd.next01();  // 'if (rnd->next01() < probability)' with probability 1
      return tr * brdf_sss2(c, tdir, hp, hp.object_id, on, p_rr, p_scat, depth) / probability;
    }
    default:
      return V3();
  }
}

struct OracleScene {
  Scene s;
  std::string err;
  uint64_t nodes = 0, tris = 0, segments = 0;
};

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" {

void* oracle_scene_create(const pr_scene_desc* d, int* status, char* err, int errlen) {
  auto* o = new OracleScene();
  int st = build_scene(d, o->s, o->err);
  if (status) *status = st;
  if (st != PR_OK) {
    if (err && errlen > 0) snprintf(err, errlen, "%s", o->err.c_str());
    delete o;
    return nullptr;
  }
  return o;
}

void oracle_scene_destroy(void* h) { delete static_cast<OracleScene*>(h); }

int oracle_qbvh_info(void* h, int ent, int64_t* nn, int64_t* nl) {
  auto* o = static_cast<OracleScene*>(h);
  if (!o || ent < 0 || ent >= (int)o->s.ents.size() || o->s.ents[ent].type != PR_ENT_POLYGON) return PR_E_ARG;
  *nn = (int64_t)o->s.ents[ent].qbvh.nodes.size();
  *nl = (int64_t)o->s.ents[ent].qbvh.leaf.size();
  return PR_OK;
}

int oracle_qbvh_export(void* h, int ent, float* boxes, int64_t* children, int32_t* axes, int32_t* leaf) {
  auto* o = static_cast<OracleScene*>(h);
  if (!o || ent < 0 || ent >= (int)o->s.ents.size() || o->s.ents[ent].type != PR_ENT_POLYGON) return PR_E_ARG;
  const QBVH& q = o->s.ents[ent].qbvh;
  for (size_t i = 0; i < q.nodes.size(); i++) {
    memcpy(boxes + 24 * i, q.nodes[i].bboxes, 24 * sizeof(float));
    for (int c = 0; c < 4; c++) children[4 * i + c] = q.nodes[i].children[c];
    axes[3 * i] = q.nodes[i].axis_top;
    axes[3 * i + 1] = q.nodes[i].axis_left;
    axes[3 * i + 2] = q.nodes[i].axis_right;
  }
  for (size_t i = 0; i < q.leaf.size(); i++) {
    const int t = q.leaf[i];
    leaf[i] = t < 0 ? -1 : o->s.ents[ent].tris[t].face;
  }
  return PR_OK;
}

// intersect_scene_ per ray; also reports the QBVH face id, hit position and normal
int oracle_first_hit(void* h, const double* rays, int64_t n, int32_t* ent, int32_t* prim, double* t,
                     double* pos, double* nrm, uint64_t* nodes_visited, uint64_t* tri_tests) {
  auto* o = static_cast<OracleScene*>(h);
  if (!o || !rays || n < 0) return PR_E_ARG;
  tl_nodes = tl_tris = 0;
  for (int64_t k = 0; k < n; k++) {
    const double* r = rays + 6 * k;
    Hit hit;
    const bool got = intersect(o->s, V3(r[0], r[1], r[2]), V3(r[3], r[4], r[5]), hit);
    ent[k] = got ? hit.object_id : -1;
    prim[k] = got ? hit.prim : -1;
    t[k] = got ? hit.distance : -1.0;
    if (pos) { pos[3 * k] = hit.position.x; pos[3 * k + 1] = hit.position.y; pos[3 * k + 2] = hit.position.z; }
    if (nrm) { nrm[3 * k] = hit.normal.x; nrm[3 * k + 1] = hit.normal.y; nrm[3 * k + 2] = hit.normal.z; }
  }
  if (nodes_visited) *nodes_visited = tl_nodes;
  if (tri_tests) *tri_tests = tl_tris;
  return PR_OK;
}

// radiance() roots from one MT19937-64 stream (the reference harness' 'radiance' command)
int oracle_radiance(void* h, const double* rays, int64_t n, uint64_t seed, const pr_render_params* prm, double* out) {
  auto* o = static_cast<OracleScene*>(h);
  if (!o || !rays || !prm || n < 0) return PR_E_ARG;
  MT64 rnd(seed);
  MT64 drnd((uint64_t)(unsigned)o->s.kerr.disk_seed);
  tl_disk_rnd = &drnd;
  Ctx c{o->s, rnd, prm->nee, prm->media && o->s.media_on, prm->depth, prm->depth_limit, (prm->flags & PR_FLAG_HG_CORRECT) != 0};
  for (int64_t k = 0; k < n; k++) {
    const double* r = rays + 6 * k;
    const V3 v = radiance(c, V3(r[0], r[1], r[2]), V3(r[3], r[4], r[5]), 0);
    out[3 * k] = v.x; out[3 * k + 1] = v.y; out[3 * k + 2] = v.z;
  }
  return PR_OK;
}

// sampleHG (sampler.h:24-93) about one incoming direction, n draws from one
// MT19937-64 stream: the reference's (g/2) form, or with correct != 0 the
// Henyey-Greenstein inverse CDF.  out: n x 3 unit directions.
int oracle_sample_hg(double g, int correct, uint64_t seed, const double* raydir, int64_t n, double* out) {
  if (!raydir || !out || n < 0) return PR_E_ARG;
  static const Scene empty{};
  MT64 rnd(seed);
  Ctx c{empty, rnd, 0, 0, 0, 0, correct};
  const V3 d = normalize(V3(raydir[0], raydir[1], raydir[2]));
  for (int64_t k = 0; k < n; k++) {
    const V3 v = sample_hg(c, d, g);
    out[3 * k] = v.x; out[3 * k + 1] = v.y; out[3 * k + 2] = v.z;
  }
  return PR_OK;
}

// Render::Run (render.h:1125-1455) over rows [row0, row1): per-thread MT
// streams seeded thread_id+1, OpenMP dynamic rows, tent filter, luminance
// cutoff and sensor response.  image: W*H*3 doubles (reference row order).
// With threads == 1 the result equals the reference bit for bit.
static int render_rows(OracleScene* o, const pr_camera* cam, const pr_render_params* prm, int threads,
                       const std::vector<int>& rows, double* image, double* seconds, uint64_t* segments);

int oracle_render(void* h, const pr_camera* cam, const pr_render_params* prm, int threads, int row0, int row1,
                  double* image, double* seconds, uint64_t* segments) {
  auto* o = static_cast<OracleScene*>(h);
  if (!o || !cam || !prm || !image || threads < 1) return PR_E_ARG;
  const int H = cam->height;
  if (row0 < 0) row0 = 0;
  if (row1 <= 0 || row1 > H) row1 = H;
  std::vector<int> rows;
  for (int y = row0; y < row1; y++) rows.push_back(y);
  return render_rows(o, cam, prm, threads, rows, image, seconds, segments);
}

// The same over an explicit list of rows (each in [0, H)), e.g. every k-th
// row of the frame for a CPU sample spread over the whole image.
int oracle_render_rows(void* h, const pr_camera* cam, const pr_render_params* prm, int threads, const int32_t* rows,
                       int n_rows, double* image, double* seconds, uint64_t* segments) {
  auto* o = static_cast<OracleScene*>(h);
  if (!o || !cam || !prm || !image || threads < 1 || n_rows < 0 || (n_rows > 0 && !rows)) return PR_E_ARG;
  std::vector<int> r(rows, rows + n_rows);
  for (int y : r)
    if (y < 0 || y >= cam->height) return PR_E_ARG;
  return render_rows(o, cam, prm, threads, r, image, seconds, segments);
}

constexpr int32_t kOracleTentSubpixels = 1 << 16;

static int render_rows(OracleScene* o, const pr_camera* cam, const pr_render_params* prm, int threads,
                       const std::vector<int>& rows, double* image, double* seconds, uint64_t* segments) {
  const Scene& s = o->s;
  const int W = cam->width, H = cam->height;
  const int n_rows = (int)rows.size();
  // CameraScreenPram (render.h:105-150)
  V3 cpos(cam->position[0], cam->position[1], cam->position[2]);
  V3 cdir(cam->dir[0], cam->dir[1], cam->dir[2]);
  const V3 cup(cam->up[0], cam->up[1], cam->up[2]);
  double cam_phi = std::atan2(cdir.y, cdir.x);
  if (cam_phi < 0.0) cam_phi += 2.0 * PI;
  if (std::fabs(cam_phi - PI) < 1.0e-6 || cam_phi < 1.0e-6 || std::fabs(cam_phi - 2.0 * PI) < 1.0e-6) {
    cdir.y += 1.0e-6;
    const double len = std::sqrt(cdir.x * cdir.x + cdir.y * cdir.y + cdir.z * cdir.z);
    cdir.x /= len; cdir.y /= len; cdir.z /= len;
  }
  const double sw = cam->screen_width * W / H;
  const double sh = cam->screen_height;
  const V3 sx = normalize(cross(cdir, cup)) * sw;
  const V3 sy = normalize(cross(sx, cdir)) * sh;
  const V3 center = cpos + cdir * cam->screen_dist;
  const double iw = 1.0 / W, ih = 1.0 / H;
  int samples = prm->samples, ss = prm->supersamples;
  double rate = (1.0 / ss);
  // Render::Run folds the sub-pixels into the samples under the tent filter
  // (render.h:1180-1186), which leaves every sample in sub-pixel (0, 0);
  // kOracleTentSubpixels keeps the 2 x 2 sub-pixels instead, the footprint
  // of generate_new_path (render.h:273-293): the expectation of the
  // Metropolis image (a test-only switch of this oracle)
  if (prm->tent_filter && !(prm->flags & kOracleTentSubpixels)) { samples = samples * (ss * ss); ss = 1; rate = 0.5; }
  else if (prm->tent_filter) rate = 0.5;
  const double smp = 1.0 / samples / (ss * ss);
  const float cutoff = (float)prm->luminance_cutoff;
  std::vector<V3> img((size_t)W * H);
  std::vector<std::unique_ptr<MT64>> rnd;
  for (int i = 0; i < threads; i++) rnd.emplace_back(new MT64((uint64_t)(unsigned)(i + 1)));
  // the entities' alpha-test stream (SceneEnv::rand_): one generator seeded
  // with the disk seed on one thread, as the reference's shared one is
  std::vector<std::unique_ptr<MT64>> drnd;
  for (int i = 0; i < threads; i++) drnd.emplace_back(new MT64((uint64_t)(unsigned)(s.kerr.disk_seed + i)));
  std::atomic<uint64_t> seg_total(0);
  const auto t0 = std::chrono::steady_clock::now();
  for (int sidx = 0; sidx < samples; sidx++) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int ri = 0; ri < n_rows; ri++) {
      const int y = rows[ri];
      const int tid = omp_get_thread_num();
      tl_segments = 0;
      tl_disk_rnd = drnd[tid].get();
      Ctx c{s, *rnd[tid], prm->nee, prm->media && s.media_on, prm->depth, prm->depth_limit,
            (prm->flags & PR_FLAG_HG_CORRECT) != 0};
      for (int x = 0; x < W; x++) {
        const int idx = (H - y - 1) * W + x;
        for (int syy = 0; syy < ss; syy++) {
          for (int sxx = 0; sxx < ss; sxx++) {
            V3 acc;
            double dx = 0, dy = 0;
            if (prm->tent_filter) {
              const double rr1 = 2.0 * c.rnd.next01();
              const double rr2 = 2.0 * c.rnd.next01();
              dx = rr1 < 1.0 ? std::sqrt(rr1) - 1.0 : 1.0 - std::sqrt(2.0 - rr1);
              dy = rr2 < 1.0 ? std::sqrt(rr2) - 1.0 : 1.0 - std::sqrt(2.0 - rr2);
            }
            const double r1 = (sxx + 0.5 + dx) * rate;
            const double r2 = (syy + 0.5 + dy) * rate;
            const V3 sp = center + sx * ((r1 + x) * iw - 0.5) + sy * ((r2 + y) * ih - 0.5);
            const V3 dir = normalize(sp - cpos);
            const V3 v = radiance(c, cpos, dir, 0) * smp;
            acc = acc + v * 1.0;
            if (cutoff > 0.0) {  // render.h:1375-1384
              const float lum = (float)dot(V3(0.2126, 0.7152, 0.0722), acc);
              if (lum > cutoff) {
                const float xs = cutoff / lum;
                acc = acc * (double)xs;
              }
            }
            img[idx] = img[idx] + acc;
          }
        }
      }
      seg_total += tl_segments;
    }
  }
  for (size_t i = 0; i < img.size(); i++) img[i] = img[i] * prm->sensor_response;
  const auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  if (segments) *segments = seg_total.load();
  for (size_t i = 0; i < img.size(); i++) {
    image[3 * i] = img[i].x; image[3 * i + 1] = img[i].y; image[3 * i + 2] = img[i].z;
  }
  return PR_OK;
}

// ---------------------------------------------------------------- PSSMLT
}  // extern "C"

namespace {

// Mutate0 (mlt.h:40-53): the step from LuxRender, |2r - 1| through fabsf
double mlt_mutate0(MT64& rnd, double x) {
  const double r = rnd.next01();
  const double s1 = 1.0 / 512.0, s2 = 1.0 / 16.0;
  const double dx = s1 / (s1 / s2 + (double)std::fabs((float)(2.0 * r - 1.0))) - s1 / (s1 / s2 + 1.0);
  if (r < 0.5) {
    const double x1 = x + dx;
    return (x1 < 1.0) ? x1 : x1 - 1.0;
  }
  const double x1 = x - dx;
  return (x1 < 0.0) ? x1 + 1.0 : x1;
}

// KelemenMLT (mlt.h:86-168): primary samples with lazy mutation, a stack
// of the values a rejected proposal restores; every draw of the
// primary-sample generator (construction, growth, mutations) comes from the
// thread's MTRandom, as random() returns it
struct KelemenSampler : Sampler {
  struct PS {
    int modify_time = 0;
    double value = 0.0;
  };
  MT64& rnd;
  int global_time = 0, large_step = 0, large_step_time = 0, used = 0;
  std::vector<PS> ps;
  std::vector<PS> stack;
  explicit KelemenSampler(MT64& r) : rnd(r) { grow(128); }
  double Next01() override { return rnd.next01(); }
  void grow(size_t n) {  // vector::resize: each new PrimarySample draws its value
    const size_t old = ps.size();
    ps.resize(n);
    for (size_t i = old; i < n; i++) {
      ps[i].modify_time = 0;
      ps[i].value = rnd.next01();
    }
  }
  double next01() override {
    if (ps.size() <= (size_t)used) grow((size_t)(ps.size() * 1.5));
    PS& p = ps[(size_t)used];
    if (p.modify_time < global_time) {
      if (large_step > 0) {
        stack.push_back(p);
        p.modify_time = global_time;
        p.value = rnd.next01();
      } else {
        if (p.modify_time < large_step_time) {
          p.modify_time = large_step_time;
          p.value = rnd.next01();
        }
        while (p.modify_time < global_time - 1) {
          p.value = mlt_mutate0(rnd, p.value);
          p.modify_time++;
        }
        stack.push_back(p);
        p.value = mlt_mutate0(rnd, p.value);
        p.modify_time = global_time;
      }
    }
    used++;
    return ps[(size_t)used - 1].value;
  }
  void restore() {
    int idx = used - 1;
    while (!stack.empty()) {
      ps[(size_t)idx--] = stack.back();
      stack.pop_back();
    }
  }
};

struct MltPath {  // PathSample (mlt.h:177-190)
  int x = 0, y = 0;
  double weight = 0.0;
  V3 F;
  bool cancel = true;
};

struct MltCamera {
  V3 cpos, center, sx, sy;
  double iw, ih;
  int W, H;
};

// generate_new_path (render.h:195-357) with its image-plane branch off (the
// `if (0 && ...)`): pixel and sub-pixel from primary samples, the tent
// filter the MLT set-up forces, radiance() drawing from the sampler
MltPath mlt_new_path(Ctx& c, KelemenSampler& k, const MltCamera& cam) {
  double pdf = 1.0;
  pdf *= cam.W;
  pdf *= cam.H;
  float x, y;
  do {
    x = (float)(k.next01() * cam.W);
    y = (float)(k.next01() * cam.H);
  } while (x < 0 || cam.W <= x || y < 0 || cam.H <= y);
  const int xx = (int)x, yy = (int)y;
  const int sxx = k.next01() < 0.5 ? 0 : 1;
  const int syy = k.next01() < 0.5 ? 0 : 1;
  const double rr1 = 2.0 * k.next01();
  const double rr2 = 2.0 * k.next01();
  const double dx = rr1 < 1.0 ? std::sqrt(rr1) - 1.0 : 1.0 - std::sqrt(2.0 - rr1);
  const double dy = rr2 < 1.0 ? std::sqrt(rr2) - 1.0 : 1.0 - std::sqrt(2.0 - rr2);
  pdf *= 4.0;
  const double r1 = (sxx + 0.5 + dx) * 0.5;
  const double r2 = (syy + 0.5 + dy) * 0.5;
  const V3 sp = cam.center + cam.sx * ((r1 + xx) * cam.iw - 0.5) + cam.sy * ((r2 + yy) * cam.ih - 0.5);
  const V3 dir = normalize(sp - cam.cpos);
  MltPath p;
  p.x = xx;
  p.y = yy;
  p.F = radiance(c, cam.cpos, dir, 0) * 1.0;
  p.weight = pdf;
  p.cancel = p.F.x == 0.0 && p.F.y == 0.0 && p.F.z == 0.0;
  return p;
}

inline double mlt_luminance(V3 c) { return dot(V3(0.2126, 0.7152, 0.0722), c); }  // mlt.h:171-174

}  // namespace

extern "C" {

// Render::RunMLT (render.h:363-785) on one thread: `samples` chains, each
// with W H pre_sample seed paths (large steps), a start path drawn by
// luminance (SPPMLTSamplingPath, mlt.h:201-219), b = their mean luminance,
// and (int)(W H mutation) mutations with p_large 0.5 and Kelemen's weights
// of the proposal and the current path; every chain's image is added up and
// scaled by sensor_response / 4 (scene_env.h:1956) / samples.  The primary
// samples' generator is MTRandom seeded prime_numbers[32] = 137.
int oracle_render_mlt(void* h, const pr_camera* cam, const pr_render_params* prm, double mutation, double pre_sample,
                      double* image) {
  auto* o = static_cast<OracleScene*>(h);
  if (!o || !cam || !prm || !image) return PR_E_ARG;
  const Scene& s = o->s;
  MltCamera mc;
  mc.W = cam->width;
  mc.H = cam->height;
  mc.cpos = V3(cam->position[0], cam->position[1], cam->position[2]);
  V3 cdir(cam->dir[0], cam->dir[1], cam->dir[2]);
  const V3 cup(cam->up[0], cam->up[1], cam->up[2]);
  double cam_phi = std::atan2(cdir.y, cdir.x);
  if (cam_phi < 0.0) cam_phi += 2.0 * PI;
  if (std::fabs(cam_phi - PI) < 1.0e-6 || cam_phi < 1.0e-6 || std::fabs(cam_phi - 2.0 * PI) < 1.0e-6) {
    cdir.y += 1.0e-6;
    const double len = std::sqrt(cdir.x * cdir.x + cdir.y * cdir.y + cdir.z * cdir.z);
    cdir.x /= len; cdir.y /= len; cdir.z /= len;
  }
  const double sw = cam->screen_width * mc.W / mc.H;
  mc.sx = normalize(cross(cdir, cup)) * sw;
  mc.sy = normalize(cross(mc.sx, cdir)) * cam->screen_height;
  mc.center = mc.cpos + cdir * cam->screen_dist;
  mc.iw = 1.0 / mc.W;
  mc.ih = 1.0 / mc.H;
  const int size = mc.W * mc.H;
  const int seeds = (int)(size * pre_sample);
  const int M = (int)(size * mutation);
  // the reference prints progress every seeds / 10 and M / 10 steps (a
  // division by zero below ten)
  if (seeds < 10 || M < 10 || prm->samples < 1) return PR_E_ARG;
  MT64 rnd((uint64_t)(unsigned)137);
  tl_disk_rnd = &rnd;
  std::vector<V3> img((size_t)size);
  for (int chain = 0; chain < prm->samples; chain++) {
    std::vector<V3> tmp((size_t)size);
    KelemenSampler k(rnd);
    k.large_step = 1;
    Ctx c{s, k, prm->nee, prm->media && s.media_on, prm->depth, prm->depth_limit,
          (prm->flags & PR_FLAG_HG_CORRECT) != 0};
    std::vector<MltPath> seed((size_t)seeds);
    double sumI = 0.0;
    for (int i = 0; i < seeds; i++) {
      k.used = 0;
      seed[(size_t)i] = mlt_new_path(c, k, mc);
      k.global_time++;
      k.stack.clear();
      sumI += mlt_luminance(seed[(size_t)i].F);
    }
    if (sumI < 1.0e-14) continue;
    auto pick = [&]() {
      const double r = rnd.next01() * sumI;
      int sel = (int)(rnd.next01() * seeds);
      if (sel >= seeds) sel = seeds - 1;
      double acc = 0.0;
      for (int i = 0; i < seeds; i++) {
        acc += mlt_luminance(seed[(size_t)i].F);
        if (r <= acc) {
          sel = i;
          break;
        }
      }
      return sel;
    };
    int sel = pick();
    for (int q = 0; q < seeds && seed[(size_t)sel].cancel; q++) sel = pick();
    const double b = sumI / seeds;
    const double p_large = 0.5;
    const double iM = 1.0 / M;
    MltPath old = seed[(size_t)sel];
    for (int i = 0; i < M; i++) {
      k.used = 0;
      k.large_step = (rnd.next01() < p_large) ? 1 : 0;
      const MltPath np = mlt_new_path(c, k, mc);
      const double Lnew = mlt_luminance(np.F), Lold = mlt_luminance(old.F);
      double a = 1.0;
      if (Lold > 1.0e-16) a = std::min(1.0, Lnew / Lold);
      const double wn = (a + k.large_step) / (Lnew / b + p_large) * iM;
      const double wo = (1.0 - a) / (Lold / b + p_large) * iM;
      const size_t ni = (size_t)((mc.H - np.y - 1) * mc.W + np.x), oi = (size_t)((mc.H - old.y - 1) * mc.W + old.x);
      tmp[oi] = tmp[oi] + wo * old.weight * old.F;
      tmp[ni] = tmp[ni] + wn * np.weight * np.F;
      if (rnd.next01() < a) {
        old = np;
        if (k.large_step) k.large_step_time = k.global_time;
        k.global_time++;
        k.stack.clear();
      } else {
        k.restore();
      }
    }
    for (int i = 0; i < size; i++) img[(size_t)i] = img[(size_t)i] + tmp[(size_t)i];
  }
  const double w = 0.25 * prm->sensor_response / (double)prm->samples;
  for (int i = 0; i < size; i++) {
    const V3 v = img[(size_t)i] * w;
    image[3 * i] = v.x;
    image[3 * i + 1] = v.y;
    image[3 * i + 2] = v.z;
  }
  return PR_OK;
}

int oracle_light_count(void* h) {
  auto* o = static_cast<OracleScene*>(h);
  return o ? (int)o->s.lights.size() : -1;
}

}  // extern "C"

// ======================================================================
// Kerr geodesics: the Kerr branch of intersect_scene (scene.cpp:448-732)
// with KerrBlackHole's set-up, initial conditions and Cash-Karp RK45
// (KerrBlackHole.h:86-151, :310-440, :660-852, :1239-1431), FP64 in the
// reference's operation order.
// ======================================================================
namespace {

inline double clampd(double v, double lo, double hi) {  // Clamp (vector3d.h:236)
  if (v < lo) return lo;
  else if (v > hi) return hi;
  else return v;
}

// Cartesian::ToBoyerLindquist (vector3d.h:941-951)
inline void cart_to_bl(double x, double y, double z, double a, double& r, double& th, double& ph) {
  double r0 = x * x + y * y + z * z;
  const double u = r0 - a * a;
  const double zz = 2. * a * z;
  r0 = std::sqrt((u + std::sqrt(u * u + zz * zz)) / 2.);
  th = std::acos(clampd(z / r0, -1.0, 1.0));
  double phi = std::atan2(y / r0, x / r0);
  if (phi < 0.0) phi += TWOPI;
  if (phi >= TWOPI) phi = 0.0;
  r = r0;
  ph = phi;
}

// Spherical::ToBoyerLindquist (vector3d.h:888-898): BL (r, th, ph) -> Cartesian
inline V3 bl_to_cart(double r, double th, double ph, double a) {
  const double rr = std::sqrt(r * r + a * a);
  const double sint = std::sin(th);
  return V3(rr * std::cos(ph) * sint, rr * std::sin(ph) * sint, r * std::cos(th));
}

// Cartesian::ToSpherical (vector3d.h:900-918)
inline void cart_to_sph(double x, double y, double z, double& r, double& th, double& ph) {
  r = std::sqrt(x * x + y * y + z * z);
  double xx = 0, yy = 0, zz = 0;
  if (r > 1.0e-16) {
    xx = x / r;
    yy = y / r;
    zz = z / r;
  } else {
    th = 0;
    ph = 0;
    return;
  }
  th = std::acos(clampd(zz, -1.0, 1.0));
  double phi;
  if (std::fabs(xx) < 1.0e-6 && std::fabs(yy) < 1.0e-6) phi = 0.0;
  else phi = std::atan2(yy, xx);
  if (phi < 0.0) phi += 2.0 * PI;
  if (phi >= 2.0 * PI) phi = 0.0;
  ph = phi;
}

struct KerrRay {
  const KerrBH& k;
  double L = 0, kappa = 0;
  double traceDir = 1.0;
  explicit KerrRay(const KerrBH& kk) : k(kk) {}

  // KerrBlackHole::geodesic (KerrBlackHole.h:1239-1281)
  void geodesic(const double* y, double* dydx) const {
    const double r = y[0];
    const double theta = y[1];
    const double pr = y[4];
    const double ptheta = y[5];
    const double r2 = r * r;
    const double twor = 2.0 * k.M * r;
    const double sintheta = std::sin(theta);
    double sin2 = sintheta * sintheta;
    const double costheta = std::cos(theta);
    const double cos2 = costheta * costheta;
    const double sigma = r2 + k.a2 * cos2;
    const double delta = r2 - twor + k.a2;
    const double sd = sigma * delta;
    const double siginv = 1.0 / sigma;
    const double bot = 1.0 / sd;
    if (std::fabs(sin2) < 1.0e-16) {
      if (sin2 < 0.0) sin2 = -1.0e-16;
      else sin2 = 1.0e-16;
    }
    dydx[0] = -pr * delta * siginv;
    dydx[1] = -ptheta * siginv;
    dydx[2] = -(twor * k.a + (sigma - twor) * L / sin2) * bot;
    dydx[3] = -(1.0 + (twor * (r2 + k.a2) - twor * k.a * L) * bot);
    dydx[4] = -(((r - 1.0) * (-kappa) + twor * (r2 + k.a2) - 2.0 * k.a * L) * bot - 2.0 * pr * pr * (r - 1.0) * siginv);
    dydx[5] = -sintheta * costheta * (L * L / (sin2 * sin2) - k.a2) * siginv;
  }

  // rkstep (KerrBlackHole.h:1288-1361)
  void rkstep(const double* y, const double* dydx, double h, double* yout, double* yerr) const {
    double ak[6], t1[6], t2[6], t3[6], t4[6], t5[6];
    h *= traceDir;
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
    for (int i = 0; i < 6; i++) {
      const double yt = h * ak[i];
      t2[i] += (9.0 / 40.0) * yt;
      t3[i] -= 0.9 * yt;
      t4[i] += 2.5 * yt;
      t5[i] += (175.0 / 512.0) * yt;
    }
    geodesic(t2, ak);
    for (int i = 0; i < 6; i++) {
      const double yt = h * ak[i];
      t3[i] += 1.2 * yt;
      t4[i] -= (70.0 / 27.0) * yt;
      t5[i] += (575.0 / 13824.0) * yt;
      yout[i] += (250.0 / 621.0) * yt;
      yerr[i] += ((250.0 / 621.0) - (18575.0 / 48384.0)) * yt;
    }
    geodesic(t3, ak);
    for (int i = 0; i < 6; i++) {
      const double yt = h * ak[i];
      t4[i] += (35.0 / 27.0) * yt;
      t5[i] += (44275.0 / 110592.0) * yt;
      yout[i] += (125.0 / 594.0) * yt;
      yerr[i] += ((125.0 / 594.0) - (13525.0 / 55296.0)) * yt;
    }
    geodesic(t4, ak);
    for (int i = 0; i < 6; i++) {
      const double yt = h * ak[i];
      t5[i] += (253.0 / 4096.0) * yt;
      yerr[i] -= (277.0 / 14336.0) * yt;
    }
    geodesic(t5, ak);
    for (int i = 0; i < 6; i++) {
      const double yt = h * ak[i];
      yout[i] += (512.0 / 1771.0) * yt;
      yerr[i] += ((512.0 / 1771.0) - 0.25) * yt;
    }
  }

  // rkqs (KerrBlackHole.h:1366-1431); returns hnext, updates y
  double rkqs(double* y, const double* dydx, double htry, double escal, const double* yscal, int& attempts) const {
    double errmax = 0.0, h = htry, htemp;
    double yerr[6], ytemp[6];
    const int loopMax = 40;
    int loopCnt = 0;
    while (loopCnt < loopMax) {
      rkstep(y, dydx, h, ytemp, yerr);
      attempts++;
      errmax = 0.0;
      for (int i = 0; i < 6; i++) {
        const double temp = std::fabs(yerr[i] / yscal[i]);
        if (temp > errmax) errmax = temp;
      }
      errmax *= escal;
      if (errmax <= 1.0) break;
      htemp = 0.9 * h / std::sqrt(std::sqrt(errmax));
      h *= 0.1;
      if (h >= 0.0) {
        if (htemp > h) h = htemp;
      } else {
        if (htemp < h) h = htemp;
      }
      loopCnt++;
    }
    double hnext;
    if (errmax > 1.89e-4) hnext = 0.9 * h * std::pow(errmax, -0.2);
    else hnext = 5.0 * h;
    for (int i = 0; i < 6; i++) y[i] = ytemp[i];
    return hnext;
  }

  // NextPosition (KerrBlackHole.h:471-522)
  double next_position(double* y, const double* dydx, double htry, int& attempts) const {
    const double escal = 1e11;
    double yscal[6];
    for (int i = 0; i < 6; i++) yscal[i] = std::fabs(y[i]) + std::fabs(dydx[i] * htry) + 1.0e-3;
    return rkqs(y, dydx, htry, escal, yscal, attempts);
  }

  // initial2 (KerrBlackHole.h:310-440) for theta0 = y[1]
  void initial2(double* y0, double* ydot0, double r0, double theta0) {
    y0[3] = 0;
    y0[4] = 0;
    y0[5] = 0;
    double sintheta = std::sin(theta0), costheta = std::cos(theta0);
    const double cos2 = costheta * costheta;
    double sin2 = sintheta * sintheta;
    const double POLE_THRESHOLD = 1e-8;
    const bool near_pole = (sin2 < POLE_THRESHOLD * POLE_THRESHOLD);
    if (near_pole) {
      const double sigma = r0 * r0 + k.a2;
      const double delta = r0 * r0 - 2.0 * k.M * r0 + k.a2;
      const double vphi_sin = ydot0[2] * sintheta;
      const double rdot0 = ydot0[0];
      const double thetadot0 = ydot0[1];
      const double energy2 = (sigma - 2.0 * r0) * (rdot0 * rdot0 / delta + thetadot0 * thetadot0) + delta * vphi_sin * vphi_sin;
      const double energy = std::sqrt(std::fabs(energy2)) + 1e-10;
      y0[4] = rdot0 * sigma / delta / energy;
      y0[5] = thetadot0 * sigma / energy;
      L = 0.0;
      kappa = y0[5] * y0[5] + k.a2 * sin2;
    } else {
      if (sin2 < 1e-16) {
        sintheta = 1e-16;
        sin2 = 1e-32;
      }
      const double rdot0 = ydot0[0];
      const double thetadot0 = ydot0[1];
      const double r2 = r0 * r0;
      const double sigma = r2 + k.a2 * cos2;
      const double delta = r2 - 2.0 * k.M * r0 + k.a2;
      const double s1 = sigma - 2.0 * r0;
      y0[4] = rdot0 * sigma / delta;
      y0[5] = thetadot0 * sigma;
      const double phidot0 = ydot0[2];
      const double energy2 = s1 * (rdot0 * rdot0 / delta + thetadot0 * thetadot0) + delta * sin2 * phidot0 * phidot0;
      const double energy = std::sqrt(std::fabs(energy2)) + 1.0e-10;
      y0[4] = y0[4] / energy;
      y0[5] = y0[5] / energy;
      L = ((sigma * delta * phidot0 - 2.0 * k.a * r0 * energy) * sin2 / s1) / energy;
      kappa = y0[5] * y0[5] + k.a2 * sin2 + L * L / sin2;
    }
    geodesic(y0, ydot0);
  }

  // RayToOrdinaryDifferentialEquationInitial, initial_condition 0 (KerrBlackHole.h:660-852)
  void initial(const V3& dir, double* y, double* dydx, double r0, double theta0) {
    y[3] = 0;
    y[4] = 0;
    y[5] = 0;
    const double r = y[0], theta = y[1], phi = y[2];
    double rs, theta_obs, phi_obs;
    cart_to_sph(dir.x, dir.y, dir.z, rs, theta_obs, phi_obs);
    const double Phi = phi - phi_obs;
    const double cost = std::cos(theta);
    const double sintobs = std::sin(theta_obs);
    const double rr = r * r;
    const double sigma = rr + (k.a * cost) * (k.a * cost);
    const double R = std::sqrt(k.a2 + rr);
    const double v = -sintobs * std::cos(Phi);
    const double zdot = 1.;
    const double inv_sigma = 1.0 / sigma;
    const double sint = std::sin(theta);
    const double rdot0 = zdot * (r * R * v * sint - R * R * std::cos(theta_obs) * cost) * inv_sigma;
    const double thetadot0 = zdot * (r * sint * std::cos(theta_obs) + R * v * cost) * inv_sigma;
    double phidot0;
    const double POLE_THRESHOLD = 1e-8;
    if (std::fabs(sint) < POLE_THRESHOLD) phidot0 = 0.0;
    else phidot0 = zdot * sintobs * std::sin(Phi) / (R * sint);
    dydx[0] = rdot0;
    dydx[1] = thetadot0;
    dydx[2] = phidot0;
    initial2(y, dydx, r0, theta0);
  }
};

}  // namespace

namespace {

// The Kerr branch of intersect_scene for one ray (scene.cpp:448-732).
// Returns the status (0 background, 1 entity hit, 2 event horizon, 4 step
// underflow, 5 entity ahead of the last step); y is the final state, dir2
// the last polyline direction, cnt the steps taken, hit the accepted hit.
// ---- accretion disk under the black hole (circle.h:240-335) -------------
// calculateLuminance (color.h:47-49), BT.709 weights in source order
inline double luminance(V3 c) { return 0.2126 * c.x + 0.7152 * c.y + 0.0722 * c.z; }

// adjustLuminance / adjustToSourceLuminance (color.h:51-74): the target is
// rescaled to the source's luminance and rounded to 0..255 integer levels
V3 adjust_to_source_luminance(V3 source, V3 target) {
  const double want = luminance(source);
  const double cur = luminance(target);
  if (cur == 0.0) {
    const int value = (int)clampd((double)(int)std::round(want / 0.2126), 0, 255);
    return V3(value, value, value);
  }
  const double scale = want / cur;
  return V3(clampd((double)(int)std::round(target.x * scale), 0, 255),
            clampd((double)(int)std::round(target.y * scale), 0, 255),
            clampd((double)(int)std::round(target.z * scale), 0, 255));
}

// accretionDiskTemperatureGeom (KerrBlackHole.h:1565-1593): thin-disk
// T^4 ~ (Mdot / r^3)(1 - sqrt(r_in / r)) with Mdot a tenth of Eddington
double disk_temperature(double r, double M, double r_in) {
  const double mdot_edd = (4.0 * PI * 1.67262192369e-27) / (0.1 * 6.6524587158e-29);
  const double mdot = 0.1 * mdot_edd;
  (void)M;
  if (r <= r_in) return 0.0;
  const double factor = mdot / (r * r * r);
  double inner = 1.0 - std::sqrt(r_in / r);
  if (inner < 0) inner = 0;
  return std::pow(factor * inner, 0.25);
}

// temperatureToRGB (KerrBlackHole.h:1595-1646): the piecewise blackbody fit
// the reference uses (temperature clamped to 1000..40000 K)
V3 temperature_rgb(double temp) {
  temp = clampd(temp, 1000.0, 40000.0);
  temp /= 100.0;
  double r, g, b;
  if (temp <= 66) {
    r = 255;
  } else {
    r = clampd(329.698727446 * std::pow(temp - 60, -0.1332047592), 0.0, 255.0);
  }
  if (temp <= 66) {
    g = clampd(99.4708025861 * std::log(temp) - 161.1195681661, 0.0, 255.0);
  } else {
    g = clampd(288.1221695283 * std::pow(temp - 60, -0.0755148492), 0.0, 255.0);
  }
  if (temp >= 66) b = 255;
  else if (temp <= 19) b = 0;
  else b = clampd(138.5177312231 * std::log(temp - 10) - 305.0447927307, 0.0, 255.0);
  return V3(r / 255.0, g / 255.0, b / 255.0);
}

// wavelengthToIntensity (relativistic.h:64-81): a Gaussian of width 100 nm
// around the channel's wavelength, faded outside 380..750 nm
double wl_intensity(double wl, double center) {
  const double width = 100.0;
  const double diff = wl - center;
  double it = std::exp(-(diff * diff) / (2.0 * width * width));
  if (wl < 380.0 || wl > 750.0) {
    double fade = 1.0;
    if (wl < 380.0) fade = std::exp(-(380.0 - wl) / 50.0);
    else fade = std::exp(-(wl - 750.0) / 50.0);
    it *= fade;
  }
  return it;
}

// applyDopplerShiftWavelength (relativistic.h:84-108): each channel's
// wavelength (700 / 546.1 / 435.8 nm) divided by the factor, redistributed
V3 doppler_wavelength(V3 c, double f) {
  const double R = 700.0, G = 546.1, B = 435.8;
  const double rw = R / f, gw = G / f, bw = B / f;
  V3 o;
  o.x += c.x * wl_intensity(rw, R);
  o.y += c.x * wl_intensity(rw, G);
  o.z += c.x * wl_intensity(rw, B);
  o.x += c.y * wl_intensity(gw, R);
  o.y += c.y * wl_intensity(gw, G);
  o.z += c.y * wl_intensity(gw, B);
  o.x += c.z * wl_intensity(bw, R);
  o.y += c.z * wl_intensity(bw, G);
  o.z += c.z * wl_intensity(bw, B);
  return V3(clampd(o.x, 0, 1), clampd(o.y, 0, 1), clampd(o.z, 0, 1));
}

// applyDopplerShiftFull (relativistic.h:141-170): beaming D^4 blended with
// the wavelength shift by the effect strength, clamped to [0, 1]
V3 doppler_full(V3 c, double d, double effect) {
  const double it = d * d * d * d;
  const V3 wl = doppler_wavelength(c, 1.0 + (d - 1.0) * effect);
  const V3 si = c * it;
  const V3 sh = wl * effect + si * (1.0 - effect);
  return V3(clampd(sh.x, 0, 1), clampd(sh.y, 0, 1), clampd(sh.z, 0, 1));
}

// the deterministic part of the disk branch at hit point pos: false where
// the disk is not there (inside the ISCO, beyond the radius, off the
// texture); else its colour, emission and alpha
bool disk_shade(const Scene& s, const Entity& e, V3 pos, V3& color_out, V3& emission_out, double& alp_out) {
  const KerrBH& kb = s.kerr;
  Hit hh;
  hh.position = pos;
  Hit& h = hh;
  const V3 p = h.position - kb.position;  // Coordinate_transformation (KerrBlackHole.h:461-468)
  double sr, sth, sph;
  cart_to_bl(p.x, p.y, p.z, kb.a, sr, sth, sph);
  if (sr < kb.Rhor) return false;
  if (sr > e.radius) return false;
  if (!(sr >= kb.Rmstable)) return false;
  // the base UVPlane's (u, v) of the hit (plane.h:228-229)
  const double u = dot(h.position - e.org, e.du_axis) / e.du_len;
  const double v = dot(h.position - e.org, e.dv_axis) / e.dv_len;
  // DiscMapping::MapUV (circle.h:53-77) with rMin = Rmstable, disk_r = radius
  const double theta = std::atan2(u / sr, v / sr);
  const double rn = (sr - kb.Rmstable) / (e.radius - kb.Rmstable);
  const double fx = kb.disk_w * 0.5 + kb.disk_w * rn * std::cos(theta);
  const double fy = kb.disk_h * 0.5 + kb.disk_h * rn * std::sin(theta);
  // int conversion truncates toward zero: in range iff -1 < f < size
  if (!(fx > -1.0 && fx < kb.disk_w) || !(fy > -1.0 && fy < kb.disk_h)) return false;
  const int xi = (int)fx, yi = (int)fy;
  const unsigned char* t = &kb.disk_tex[4 * ((size_t)yi * kb.disk_w + xi)];
  const double tmp_r = length(h.position - kb.position);
  V3 color(t[0] / 255.0, t[1] / 255.0, t[2] / 255.0);
  if (kb.use_temperature) {
    const double temp = disk_temperature(tmp_r, 1.0, kb.Rmstable);
    color = adjust_to_source_luminance(color, temperature_rgb(temp));
  }
  V3 emission = s.mats[e.material].emission * color;
  double alp = t[3] / 255.0;
  const double cl = length(color) / 3.0;
  alp = (cl < alp) ? cl : alp;  // std::min(alp, |colour| / 3)
  // getDiskVelocity (KerrBlackHole.h:1507-1531) about +z with sign -1, then
  // the circular-orbit speed seen by a locally non-rotating observer
  V3 vel;
  {
    const V3 rv = h.position - kb.position;
    const double r = length(rv);
    if (r < 1e-6) {
      vel = V3();
    } else {
      const double vm = std::sqrt(1.0 / r);
      V3 vd(0.0 * rv.z - 1.0 * rv.y, 1.0 * rv.x - 0.0 * rv.z, 0.0 * rv.y - 0.0 * rv.x);
      vd = normalize(vd);
      vel = vd * (vm * -1.0);
    }
  }
  const double a = kb.a;
  const double omg = 1.0 / (std::pow(tmp_r, 3.0 / 2.0) + a);
  const double delt = tmp_r * tmp_r - 2.0 * tmp_r + a * a;
  const double A = std::pow(tmp_r, 4.0) + a * a * tmp_r * tmp_r + 2.0 * a * a * tmp_r;
  const double o = 2.0 * a * tmp_r / A;
  vel = normalize(vel) * (omg - o) * A / (tmp_r * tmp_r * std::sqrt(delt));
  // calculateDopplerFactorFromObserver (KerrBlackHole.h:1534-1562)
  double doppler = 1.0;
  {
    const V3 view = normalize(h.position - kb.observer);
    const double beta = length(vel);
    if (!(beta < 1e-6)) {
      const V3 vdir = normalize(vel);
      const double cos_t = dot(view, vdir);
      const double gamma = 1.0 / std::sqrt(1.0 - beta * beta);
      doppler = 1.0 / (gamma * (1.0 - beta * cos_t));
    }
  }
  color_out = doppler_full(color, doppler, kb.doppler_effect);
  emission_out = doppler_full(emission, doppler, kb.doppler_effect);
  alp_out = alp;
  return true;
}

bool kerr_disk_texel(const Scene& s, const Entity& e, Hit& h) {
  const KerrBH& kb = s.kerr;
  V3 color, emission;
  double alp;
  if (!disk_shade(s, e, h.position, color, emission, alp)) return false;
  if (alp == 0.0) return false;
  if (alp < 0.99) {
    if (!tl_disk_rnd) {  // an entry point that set no stream (first-hit queries)
      thread_local MT64 fallback((uint64_t)(unsigned)kb.disk_seed);
      tl_disk_rnd = &fallback;
    }
    if (alp <= tl_disk_rnd->next01()) return false;
  }
  h.ov = true;
  h.ov_color = color;
  h.ov_emission = emission;
  return true;
}

int kerr_trace_one(const Scene& s, V3 org, V3 dir, Hit& hit, double* y, V3& dir2, int& cnt) {
  const KerrBH& kb = s.kerr;
  KerrRay K(kb);
  double dydx[6];
  const V3 rel = org - kb.position;  // Setup (KerrBlackHole.h:153-166)
  double r0, th0, ph0;
  cart_to_bl(rel.x, rel.y, rel.z, kb.a, r0, th0, ph0);
  cnt = 0;
  V3 org2 = org, org1 = org;
  dir2 = dir;
  y[0] = r0; y[1] = th0; y[2] = ph0; y[3] = 0; y[4] = 0; y[5] = 0;
  if (r0 < kb.Rhor) return 2;
  K.traceDir = 1.0;
  K.initial(1.0 * dir, y, dydx, r0, th0);
  const double h_dist = 2.0;
  double h_step = h_dist;
  int attempts = 0;
  while ((kb.max_steps < 0) ? 1 : (cnt < kb.max_steps)) {
    if (intersect(s, org1, dir2, hit)) {
      if (hit.distance < h_dist) {
        const V3 c = hit.position - kb.position;
        double sr, sth, sph;
        cart_to_bl(c.x, c.y, c.z, kb.a, sr, sth, sph);
        return (sr < kb.Rhor) ? 2 : 1;
      }
    }
    K.geodesic(y, dydx);
    if (std::fabs(h_step) < 1.0e-10) return 4;
    const double r_before = y[0];
    h_step = K.next_position(y, dydx, h_step, attempts);
    if (h_step > h_dist) h_step = h_dist;
    if (y[0] < kb.Rhor) return 2;
    org1 = org2;
    const V3 c = bl_to_cart(y[0], y[1], y[2], kb.a);
    org2 = c + kb.position;
    dir2 = normalize(org2 - org1);
    cnt++;
    // optional early exit (not in the reference): far out and receding
    if (kb.escape_radius > 0.0 && y[0] > kb.escape_radius && y[0] > r_before) break;
  }
  if (intersect(s, org2, dir2, hit)) return 5;
  return 0;
}

// background colour of an escaped ray (scene.cpp:711-727 + SphericalMapping::Map, circle.h:92-105)
V3 kerr_background(const KerrBH& kb, const double* yy, const V3& bg) {
  if (kb.texture.empty()) return bg;
  double y1 = yy[1] * kb.map_coef[0] + kb.map_coef[1];
  double y2 = yy[2] * kb.map_coef[2] + kb.map_coef[3];
  y1 = std::fmod(y1, PI);
  y2 = std::fmod(y2, 2.0 * PI);
  double phi = y2, theta = y1;
  if (phi < 0.0) phi += 2.0 * PI;
  if (theta < 0.0) theta = -theta;
  if (!(phi == phi) || !(theta == theta)) return V3();  // non-finite state: no texel (the reference reads out of range)
  int x = (int)(phi / (2.0 * PI) * kb.tex_w);
  x = x % kb.tex_w;
  const int y1i = (int)(theta / PI * kb.tex_h);
  const int yv = y1i % kb.tex_h;
  const unsigned char* t = &kb.texture[3 * ((size_t)yv * kb.tex_w + x)];
  return V3(kb.texture_coef * t[0] / 255.0, kb.texture_coef * t[1] / 255.0, kb.texture_coef * t[2] / 255.0);
}

// ------------------------------------------------------------ wormhole
// WormHole.h restated: the Dneg wormhole's radius r(l) and dr/dl, the
// inverse r -> l by Newton's method, the ray's frame (a basis whose x axis
// points from the mouth to the camera) and its inverse by cofactors, the
// geodesic equations (A7) with the initial conditions (A9), and Cash-Karp
// RK45 with the class's own step control.

inline V3 sph_to_cart(double r, double th, double ph) {  // Spherical::ToCartesian (vector3d.h:879-887)
  const double sint = std::sin(th);
  return V3(r * std::cos(ph) * sint, r * std::sin(ph) * sint, r * std::cos(th));
}

// Matrix4D * Vector3d (vector3d.h:760-768): the upper 3x3 block, row major
inline V3 mat_mul3(const double* m, V3 v) {
  return V3(v.x * m[0] + v.y * m[1] + v.z * m[2], v.x * m[4] + v.y * m[5] + v.z * m[6],
            v.x * m[8] + v.y * m[9] + v.z * m[10]);
}

// InvertMatrix_ (vector3d.h:577-755): cofactors in the published (Mesa GLU)
// order; a determinant below 1e-16 leaves B as it was
bool invert4(const double* A, double* B) {
  double inv[16];
  inv[0] = A[5] * A[10] * A[15] - A[5] * A[11] * A[14] - A[9] * A[6] * A[15] + A[9] * A[7] * A[14] +
           A[13] * A[6] * A[11] - A[13] * A[7] * A[10];
  inv[4] = -A[4] * A[10] * A[15] + A[4] * A[11] * A[14] + A[8] * A[6] * A[15] - A[8] * A[7] * A[14] -
           A[12] * A[6] * A[11] + A[12] * A[7] * A[10];
  inv[8] = A[4] * A[9] * A[15] - A[4] * A[11] * A[13] - A[8] * A[5] * A[15] + A[8] * A[7] * A[13] +
           A[12] * A[5] * A[11] - A[12] * A[7] * A[9];
  inv[12] = -A[4] * A[9] * A[14] + A[4] * A[10] * A[13] + A[8] * A[5] * A[14] - A[8] * A[6] * A[13] -
            A[12] * A[5] * A[10] + A[12] * A[6] * A[9];
  inv[1] = -A[1] * A[10] * A[15] + A[1] * A[11] * A[14] + A[9] * A[2] * A[15] - A[9] * A[3] * A[14] -
           A[13] * A[2] * A[11] + A[13] * A[3] * A[10];
  inv[5] = A[0] * A[10] * A[15] - A[0] * A[11] * A[14] - A[8] * A[2] * A[15] + A[8] * A[3] * A[14] +
           A[12] * A[2] * A[11] - A[12] * A[3] * A[10];
  inv[9] = -A[0] * A[9] * A[15] + A[0] * A[11] * A[13] + A[8] * A[1] * A[15] - A[8] * A[3] * A[13] -
           A[12] * A[1] * A[11] + A[12] * A[3] * A[9];
  inv[13] = A[0] * A[9] * A[14] - A[0] * A[10] * A[13] - A[8] * A[1] * A[14] + A[8] * A[2] * A[13] +
            A[12] * A[1] * A[10] - A[12] * A[2] * A[9];
  inv[2] = A[1] * A[6] * A[15] - A[1] * A[7] * A[14] - A[5] * A[2] * A[15] + A[5] * A[3] * A[14] +
           A[13] * A[2] * A[7] - A[13] * A[3] * A[6];
  inv[6] = -A[0] * A[6] * A[15] + A[0] * A[7] * A[14] + A[4] * A[2] * A[15] - A[4] * A[3] * A[14] -
           A[12] * A[2] * A[7] + A[12] * A[3] * A[6];
  inv[10] = A[0] * A[5] * A[15] - A[0] * A[7] * A[13] - A[4] * A[1] * A[15] + A[4] * A[3] * A[13] +
            A[12] * A[1] * A[7] - A[12] * A[3] * A[5];
  inv[14] = -A[0] * A[5] * A[14] + A[0] * A[6] * A[13] + A[4] * A[1] * A[14] - A[4] * A[2] * A[13] -
            A[12] * A[1] * A[6] + A[12] * A[2] * A[5];
  inv[3] = -A[1] * A[6] * A[11] + A[1] * A[7] * A[10] + A[5] * A[2] * A[11] - A[5] * A[3] * A[10] -
           A[9] * A[2] * A[7] + A[9] * A[3] * A[6];
  inv[7] = A[0] * A[6] * A[11] - A[0] * A[7] * A[10] - A[4] * A[2] * A[11] + A[4] * A[3] * A[10] +
           A[8] * A[2] * A[7] - A[8] * A[3] * A[6];
  inv[11] = -A[0] * A[5] * A[11] + A[0] * A[7] * A[9] + A[4] * A[1] * A[11] - A[4] * A[3] * A[9] -
            A[8] * A[1] * A[7] + A[8] * A[3] * A[5];
  inv[15] = A[0] * A[5] * A[10] - A[0] * A[6] * A[9] - A[4] * A[1] * A[10] + A[4] * A[2] * A[9] +
            A[8] * A[1] * A[6] - A[8] * A[2] * A[5];
  double det = A[0] * inv[0] + A[1] * inv[4] + A[2] * inv[8] + A[3] * inv[12];
  if (det < 1.0e-16) return false;
  det = 1.0 / det;
  for (int i = 0; i < 16; i++) B[i] = inv[i] * det;
  return true;
}

struct WormRay {  // the per-ray copy of the class (scene.cpp:738)
  const Wormhole& w;
  double l0 = 0, theta0 = 0, phi0 = 0;
  double n_l = 0, n_ph = 0, n_th = 0;
  double Mat[16], invMat[16];
  explicit WormRay(const Wormhole& w_) : w(w_) {}

  double r_wh(double l) const {  // WormHole.h:172-180
    const double x = 2.0 * (std::fabs(l) - w.a) / (PI * w.M);
    if (std::fabs(l) > w.a) return w.Rho + w.M * (x * std::atan(x) - 0.5 * std::log(1.0 + x * x));
    return w.Rho;
  }
  double drdl(double l) const {  // :182-193
    double sg = 1;
    if (l < 0) sg = -1;
    if (l == 0.0) sg = 0.0;
    if (std::fabs(l) > w.a) return (2.0 * std::atan((2.0 * (-w.a + std::fabs(l))) / (w.M * PI)) * sg) / PI;
    return 0;
  }
  double rtol(double r, double linit) const {  // :195-238, Newton from the start, then from a
    const double M = w.M, Rho = w.Rho;
    double x = 2.0 * (std::fabs(linit) - w.a) / (PI * M);
    int stat = -1;
    for (int i = 0; i < 30; i++) {
      const double xi = x;
      x = x - (Rho + M * (x * std::atan(x) - 0.5 * std::log(1.0 + x * x)) - r) / (M * std::atan(x));
      if (std::fabs(x - xi) < 1.0e-6) {
        stat = 0;
        break;
      }
      if (!std::isfinite(x)) break;
    }
    double l = x * PI * M * 0.5 + w.a;
    if (stat != 0) {
      x = w.a;
      for (int i = 0; i < 30; i++) {
        const double xi = x;
        x = x - (Rho + M * (x * std::atan(x) - 0.5 * std::log(1.0 + x * x)) - r) / (M * std::atan(x));
        if (std::fabs(x - xi) < 1.0e-6) {
          l = x * PI * M * 0.5 + w.a;
          break;
        }
        if (!std::isfinite(x)) break;
      }
    }
    return (linit < 0) ? -std::fabs(l) : std::fabs(l);
  }
  // Setup (WormHole.h:321-395) with sgn: the ray's mouth
  void setup(V3 org, double sgn) {
    const V3 mouth = sgn >= 0 ? w.pos0 : w.pos1;
    const V3 pos = org - mouth;
    double pr, pth, pph;
    cart_to_sph(pos.x, pos.y, pos.z, pr, pth, pph);
    for (int i = 0; i < 16; i++) Mat[i] = invMat[i] = (i % 5 == 0) ? 1.0 : 0.0;
    const V3 X = normalize(w.camera - mouth);
    V3 Y = normalize(cross(V3(0, 0, 1), X));
    if (length(Y) < 1.0e-16) Y = normalize(cross(V3(0, 1, 0), X));
    const V3 Z = normalize(cross(X, Y));
    // Matrix4D(X.x, Y.x, Z.x, 0, X.y, Y.y, Z.y, 0, X.z, Y.z, Z.z, 0, 0, 0, 0, 1) transposed
    const double m0[16] = {X.x, Y.x, Z.x, 0, X.y, Y.y, Z.y, 0, X.z, Y.z, Z.z, 0, 0, 0, 0, 1.0};
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) Mat[4 * i + j] = m0[4 * j + i];
    (void)invert4(Mat, invMat);
    const V3 pv = sph_to_cart(pr, pth, pph);
    const V3 q = mat_mul3(Mat, pv);
    double qr, qth, qph;
    cart_to_sph(q.x, q.y, q.z, qr, qth, qph);
    theta0 = qth;
    phi0 = qph;
    l0 = rtol(qr, sgn * w.a / 2);
  }
  // initial (WormHole.h:399-428): the direction in the frame, (A9)
  void initial(double* y, double rr, double rth, double rph) {
    const V3 rc = mat_mul3(Mat, sph_to_cart(rr, rth, rph));
    double r_, th, ph;
    cart_to_sph(rc.x, rc.y, rc.z, r_, th, ph);
    const double sint = std::sin(th);
    const double Nx = sint * std::cos(ph), Ny = sint * std::sin(ph), Nz = std::cos(th);
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
  void geodesic(const double* y, double* dydx) const {
    const double r = r_wh(y[0]);
    const double r2 = r * r;
    double sint = std::sin(y[1]);
    if (std::fabs(sint) < 1.0e-8) sint = sint > 0.0 ? 1.0e-8 : -1.0e-8;
    const double sint2 = sint * sint;
    const double r_l0 = r_wh(l0);
    const double b = r_l0 * std::sin(theta0) * n_ph;
    const double B2 = r_l0 * r_l0 * (n_th * n_th + n_ph * n_ph);
    const double invr2 = 1.0 / r2;
    dydx[0] = y[3];
    dydx[1] = y[4] * invr2;
    dydx[2] = b * invr2 / sint2;
    dydx[3] = B2 * drdl(y[0]) * invr2 / r;
    dydx[4] = (b * b * invr2) * (std::cos(y[1]) / (sint * sint2));
  }
  // rkstep (WormHole.h:541-612): Cash-Karp with h negated (traceDir 1)
  void rkstep(const double* y, const double* dydx, double h, double* yout, double* yerr) const {
    double ak[5], t1[5], t2[5], t3[5], t4[5], t5[5];
    h *= -1.0 * 1.0;
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
  double next_position(double* y, const double* dydx, double htry) const {
    const double escal = 1e11;
    double yscal[5], ytemp[5], yerr[5];
    for (int i = 0; i < 5; i++) yscal[i] = std::fabs(y[i]) + std::fabs(dydx[i] * htry) + 1.0e-3;
    double h = htry, errmax = 0.0, htemp;
    int loops = 0;
    while (loops < 2000) {
      rkstep(y, dydx, h, ytemp, yerr);
      errmax = 0.0;
      for (int i = 0; i < 5; i++) {
        const double temp = std::fabs(yerr[i] / yscal[i]);
        if (temp > errmax) errmax = temp;
      }
      errmax *= escal;
      if (errmax <= 1.0) break;
      htemp = 0.9 * h / std::sqrt(std::sqrt(errmax));
      h *= 0.1;
      if (h >= 0.0) {
        if (htemp > h) h = htemp;
      } else {
        if (htemp < h) h = htemp;
      }
      loops++;
    }
    const double hnext = errmax > 1.89e-4 ? 0.9 * h * std::pow(errmax, -0.2) : 5.0 * h;
    for (int i = 0; i < 5; i++) y[i] = ytemp[i];
    return hnext;
  }
  V3 world(V3 q, double sgn) const {  // WorldAxisSystem (WormHole.h:430-447)
    return mat_mul3(invMat, q) + (sgn >= 0 ? w.pos0 : w.pos1);
  }
};

// intersect_scene__ (scene.cpp:735-925): 1 entity hit; 0 background 1
// (l >= 0); 3 background 2 (l < 0); y: the final state with (theta, phi)
// of the last polyline direction
int worm_trace_one(const Scene& s, V3 org, V3 dir, Hit& hit, double* y, V3& dir2, int& cnt) {
  const Wormhole& wh = s.worm;
  WormRay kb(wh);
  double rr, rth, rph;
  cart_to_sph(dir.x, dir.y, dir.z, rr, rth, rph);
  const double sign = length(org) > 1000000 ? -1.0 : 1.0;
  kb.setup(org, sign);
  double dydx[5];
  kb.initial(y, rr, rth, rph);
  cnt = 0;
  const int cntMax = wh.max_steps;
  V3 org2 = org, org1 = org;
  dir2 = dir;
  double h_dist = 0.5;
  if (std::fabs(y[0]) < wh.a || kb.r_wh(y[0]) <= wh.Rho) h_dist = h_dist * 0.15;
  double h_step = h_dist;
  while (cntMax < 0 ? true : cnt < cntMax) {
    if (std::fabs(y[0]) > 1.0e10 || std::fabs(kb.r_wh(y[0])) > 1.0e10 || !std::isfinite(y[0])) break;
    if (intersect(s, org1, dir2, hit) && hit.distance < h_dist) return 1;
    kb.geodesic(y, dydx);
    if (std::fabs(h_step) < 1.0e-14) h_step = 1.0e-14;
    h_step = kb.next_position(y, dydx, h_step);
    if (h_step > h_dist) h_step = h_dist;
    org1 = org2;
    org2 = kb.world(sph_to_cart(kb.r_wh(y[0]), y[1], y[2]), y[0]);
    dir2 = normalize(org2 - org1);
    cnt++;
  }
  if (wh.usr_sign) y[0] = wh.usr_sign * y[0];
  double dr, dth, dph;
  cart_to_sph(dir2.x, dir2.y, dir2.z, dr, dth, dph);
  y[1] = dth;
  y[2] = dph;
  return y[0] >= 0 ? 0 : 3;
}

// the colour of a ray that ended on a background (scene.cpp:860-920 +
// SphericalMapping::Map, circle.h:92-105); no texture: BACKGROUND
V3 worm_background(const Wormhole& wh, int side, const double* yy, const V3& bg) {
  if (wh.tex[side].empty()) return bg;
  double y1 = yy[1] * wh.map_coef[side][0] + wh.map_coef[side][1];
  double y2 = yy[2] * wh.map_coef[side][2] + wh.map_coef[side][3];
  y1 = std::fmod(y1, PI);
  y2 = std::fmod(y2, 2.0 * PI);
  double phi = y2, theta = y1;
  if (phi < 0.0) phi += 2.0 * PI;
  if (theta < 0.0) theta = -theta;
  if (!(phi == phi) || !(theta == theta)) return V3();
  int x = (int)(phi / (2.0 * PI) * wh.tex_w[side]);
  x = x % wh.tex_w[side];
  const int yv = ((int)(theta / PI * wh.tex_h[side])) % wh.tex_h[side];
  const unsigned char* t = &wh.tex[side][3 * ((size_t)yv * wh.tex_w[side] + x)];
  const double c = wh.tex_coef[side];
  return V3(c * t[0] / 255.0, c * t[1] / 255.0, c * t[2] / 255.0);
}

bool worm_query(const Scene& s, V3 org, V3 dir, Hit& hit, V3& miss_color) {
  double y[5];
  V3 dir2;
  int cnt;
  const int st = worm_trace_one(s, org, dir, hit, y, dir2, cnt);
  if (st == 1) return true;
  miss_color = worm_background(s.worm, st == 0 ? 0 : 1, y, s.background);
  return false;
}

bool kerr_query(const Scene& s, V3 org, V3 dir, Hit& hit, V3& miss_color) {
  double y[6];
  V3 dir2;
  int cnt;
  const int st = kerr_trace_one(s, org, dir, hit, y, dir2, cnt);
  if (st == 1) return true;
  if (st == 2) miss_color = V3();
  else if (st == 0) miss_color = kerr_background(s.kerr, y, s.background);
  else miss_color = s.background;
  return false;
}

}  // namespace

extern "C" {

// One Kerr trace per ray (intersect_scene's Kerr branch, scene.cpp:448-732).
static void kerr_trace_ray(OracleScene* o, const double* rays, int64_t q, int32_t* status, double* final_bl,
                           double* exit_dir, int32_t* steps, int32_t* hit_entity, double* hit_t, double* hit_color,
                           double* hit_emission) {
  const double* rr = rays + 6 * q;
  Hit hit;
  double y[6];
  V3 dir2;
  int cnt = 0;
  const int st = kerr_trace_one(o->s, V3(rr[0], rr[1], rr[2]), V3(rr[3], rr[4], rr[5]), hit, y, dir2, cnt);
  status[q] = st;
  steps[q] = cnt;
  for (int k = 0; k < 3; k++) final_bl[3 * q + k] = y[k];
  exit_dir[3 * q] = dir2.x;
  exit_dir[3 * q + 1] = dir2.y;
  exit_dir[3 * q + 2] = dir2.z;
  hit_entity[q] = (st == 1 || st == 5) ? hit.object_id : -1;
  hit_t[q] = (st == 1 || st == 5) ? hit.distance : -1.0;
  // the hit point's material colour and emission (the disk's rewritten copy)
  if (hit_color && hit_emission) {
    V3 c, em;
    if (st == 1 || st == 5) {
      const Material m = hit_mat(o->s, hit);
      c = m.color;
      em = m.emission;
    }
    for (int k = 0; k < 3; k++) {
      hit_color[3 * q + k] = c[k];
      hit_emission[3 * q + k] = em[k];
    }
  }
}

// One wormhole trace per ray (intersect_scene__, scene.cpp:735-925):
// status 1 entity hit, 0 background 1, 3 background 2; the final state
// (l, theta, phi of the last polyline direction), that direction, the steps
// and the hit entity (-1: none).  Rays are independent: threads split them.
int oracle_wormhole_trace(void* h, int threads, const double* rays, int64_t n, int32_t* status, double* final_y,
                          double* exit_dir, int32_t* steps, int32_t* hit_entity) {
  auto* o = static_cast<OracleScene*>(h);
  if (!o || !rays || n < 0 || !o->s.worm.on) return PR_E_ARG;
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads > 0 ? threads : 1)
  for (int64_t q = 0; q < n; q++) {
    const double* rr = rays + 6 * q;
    Hit hit;
    double y[5];
    V3 dir2;
    int cnt = 0;
    const int st = worm_trace_one(o->s, V3(rr[0], rr[1], rr[2]), V3(rr[3], rr[4], rr[5]), hit, y, dir2, cnt);
    status[q] = st;
    steps[q] = cnt;
    for (int k = 0; k < 3; k++) final_y[3 * q + k] = y[k];
    exit_dir[3 * q] = dir2.x;
    exit_dir[3 * q + 1] = dir2.y;
    exit_dir[3 * q + 2] = dir2.z;
    hit_entity[q] = st == 1 ? hit.object_id : -1;
  }
  return PR_OK;
}

int oracle_kerr_trace(void* h, const double* rays, int64_t n, int32_t* status, double* final_bl, double* exit_dir,
                      int32_t* steps, int32_t* hit_entity, double* hit_t, double* hit_color, double* hit_emission) {
  auto* o = static_cast<OracleScene*>(h);
  if (!o || !rays || n < 0 || !o->s.kerr.on) return PR_E_ARG;
  MT64 drnd((uint64_t)(unsigned)o->s.kerr.disk_seed);
  tl_disk_rnd = &drnd;
  for (int64_t q = 0; q < n; q++)
    kerr_trace_ray(o, rays, q, status, final_bl, exit_dir, steps, hit_entity, hit_t, hit_color, hit_emission);
  return PR_OK;
}

// The same on several threads, for scenes without a textured accretion disk
// (whose alpha test draws from one stream over the rays in their order: those
// run on one thread).  Rays are independent otherwise, so the results equal
// the one-thread call's.
int oracle_kerr_trace_threads(void* h, int threads, const double* rays, int64_t n, int32_t* status, double* final_bl,
                              double* exit_dir, int32_t* steps, int32_t* hit_entity, double* hit_t, double* hit_color,
                              double* hit_emission) {
  auto* o = static_cast<OracleScene*>(h);
  if (!o || !rays || n < 0 || !o->s.kerr.on) return PR_E_ARG;
  if (threads <= 1 || !o->s.kerr.disk_tex.empty())
    return oracle_kerr_trace(h, rays, n, status, final_bl, exit_dir, steps, hit_entity, hit_t, hit_color,
                             hit_emission);
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
  for (int64_t q = 0; q < n; q++)
    kerr_trace_ray(o, rays, q, status, final_bl, exit_dir, steps, hit_entity, hit_t, hit_color, hit_emission);
  return PR_OK;
}

// The accretion disk's shading at given points of disk entity ent
// (circle.h:240-322 without the alpha test): valid, colour, emission, alpha.
int oracle_kerr_disk_shade(void* h, int ent, const double* points, int64_t n, int32_t* valid, double* color,
                           double* emission, double* alpha) {
  auto* o = static_cast<OracleScene*>(h);
  if (!o || !points || n < 0 || !o->s.kerr.on || ent < 0 || ent >= (int)o->s.ents.size()) return PR_E_ARG;
  const Entity& e = o->s.ents[ent];
  if (e.type != PR_ENT_CIRCLE || o->s.kerr.disk_tex.empty()) return PR_E_ARG;
  for (int64_t q = 0; q < n; q++) {
    V3 c, em;
    double a = 0.0;
    const bool ok = disk_shade(o->s, e, V3(points[3 * q], points[3 * q + 1], points[3 * q + 2]), c, em, a);
    valid[q] = ok ? 1 : 0;
    for (int k = 0; k < 3; k++) {
      color[3 * q + k] = ok ? c[k] : 0.0;
      emission[3 * q + k] = ok ? em[k] : 0.0;
    }
    alpha[q] = ok ? a : 0.0;
  }
  return PR_OK;
}

}  // extern "C"
