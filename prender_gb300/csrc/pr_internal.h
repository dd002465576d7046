// Host/device shared layout of the uploaded scene.
//
// The GPU scene is a flat set of arrays in HBM:
//   * entities and materials (a few dozen records, read through the
//     read-only cache);
//   * one QBVH per mesh, all meshes' nodes concatenated, 128-byte nodes
//     (six float4 of child boxes in SoA form, one int4 of children, one int4
//     of axes and leaf sizes) so that a node is eight 128-bit loads;
//   * triangles stored in QBVH leaf order, three float4 each (vertex 0, 1, 2
//     as the mesh keeps them in float, face id in v0.w), so a leaf is a
//     contiguous run and the FP64 re-test reads the exact float vertices;
//   * face normals per mesh face (float3, ObjLoader's rule).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/prender_gpu.h"

namespace pr {

constexpr int kMaxEntities = 48;
constexpr int kMaxLights = 16;
constexpr int kStackSize = 64;          // QBVH traversal stack (entries)
constexpr int kWStack = 32;             // wide-tree traversal stack (node groups); a tree may be this deep
constexpr int kSplitStack = 4;          // pending glass branches (depth <= 2 splits)
constexpr int32_t kChildInvalid = -1;   // QBVH child slot without a child
// leaf child = kLeafBit | first leaf slot; inner child = node index (>= 0)
constexpr uint32_t kLeafBit = 0x80000000u;

struct alignas(16) GNode {   // 128 bytes
  float bmin_x[4], bmax_x[4];
  float bmin_y[4], bmax_y[4];
  float bmin_z[4], bmax_z[4];
  int32_t child[4];
  int32_t axes;            // axis_top | axis_left << 2 | axis_right << 4
  uint16_t count[4];       // triangles in each leaf child
  int32_t pad;
};
static_assert(sizeof(GNode) == 128, "GNode must be 128 bytes");

// The render path's node: eight children with boxes quantised to 8 bits per
// plane on a per-node grid (compressed wide BVH node after Ylitie, Karras
// and Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed
// Wide BVHs", HPG 2017), 80 bytes = five 128-bit loads.  Child box of slot s
// on axis a: [p_a + qlo_a[s] * 2^ea, p_a + qhi_a[s] * 2^ea].  Inner children
// are stored contiguously from child_base in slot order (child of slot s =
// child_base + popcount(imask below s)); the triangles of the leaf children
// (at most 3 each) contiguously from tri_base in slot order.  meta byte s of
// a leaf = (1 << count) - 1 << 5 | offset of its first triangle from
// tri_base; 0 for inner and empty slots.  An empty slot has qlo > qhi.
// Slots are assigned so that a ray whose direction has sign bits k (bit a
// set: negative along axis a) meets the children roughly near to far in the
// order slot = i ^ k, i = 0..7.
struct alignas(16) WNode {   // 80 bytes
  float p[3];
  uint32_t e_imask;        // ex | ey << 8 | ez << 16 (biased float exponents) | imask << 24
  int32_t child_base;
  int32_t tri_base;
  uint32_t meta[2];        // byte s of the pair
  uint32_t qlo_x[2], qlo_y[2], qlo_z[2];
  uint32_t qhi_x[2], qhi_y[2], qhi_z[2];
};
static_assert(sizeof(WNode) == 80, "WNode must be 80 bytes");

struct GMaterial {
  int32_t type;
  float roughness;
  float ior;
  float pad;
  float color[3];
  float emission[3];
  double color_d[3];
  double emission_d[3];
  double roughness_d;
  double ior_d;
  // directional dipole of a level -2 subsurface material (bssrdf.h:75-128),
  // from the material's own medium after setup_Scattering
  int32_t sss;             // 1: PR_MAT_SSS_REFRACTION with the dipole
  float sss_eta;           // r_refractive_index
  float sss_Cp, sss_Ce, sss_A;
  float sss_sigma_tr[3], sss_D[3], sss_de[3], sss_sigma_t[3];
  float sss_falloff;       // Gaussian-disk falloff: min(sigma_t') * 0.001
  float sss_rmax0;         // probe-disk radius before the object-size clamp
  float sss_tr[3];         // the medium's transmittanceColor (exit attenuation)
  // level -1 adds the single-scattering walk (radiance_through_media)
  int32_t sss_level;       // -2 or -1
  float sss_ss[3];         // scatteringColor
  float sss_g[3];          // phase parameters (PAHASE)
  float sss_t[3];          // channel-sampling table: absorbing coefficients of the
  float sss_tsum;          //   smallest / middle / largest channel over their sum
  int32_t sss_idx;         // those channels: min | mid << 4 | max << 8
  // glossy lobes (brdf.h:16-319)
  float specular[3];
  float ward_ax, ward_ay;  // Ward roughness along the orienting normal's u / v axes
  float phong_n;           // Phong exponent
  // textures (sphere.h:104-240, plane.h:241-273): offsets of the texel
  // records in DevScene::texels (RGB / 255, -1: none) and of the IBL
  // image's in DevScene::ibl_texels (-1: none)
  int32_t tex_off, tex_w, tex_h;
  int32_t ibl_off, ibl_w, ibl_h;
  float ibl_coef;
  int32_t repeat;
  int32_t map_flags;       // PR_MAP_*
  int32_t bump_off, bump_w, bump_h;  // bump map texels in DevScene::bump_texels (-1: none)
  // a material derived for the faces of an OBJ material (polygon.h:228-400):
  // its map_Kd texture (texels in DevScene::texels, -1: none), '#REPEAT',
  // which of colour / specular / emission (1 / 2 / 4) the texel scales, and
  // '#SMOOTH' (0 the entity's choice, 1 on, 2 off)
  int32_t mtex_off, mtex_w, mtex_h, mtex_repeat, mtex_mask, mesh_smooth;
};

struct GEntity {
  int32_t type;
  int32_t material;
  int32_t normal_inverse;
  int32_t is_light;
  // sphere / disk centre, uvplane origin (FP64: the hit test runs in FP64)
  double p[3];
  double radius;
  double radius_inner;     // disk (annulus) inner radius
  // uvplane: unit axes, lengths and normal (plane.h:146-167)
  double u_axis[3], v_axis[3], normal[3];
  double u_length, v_length;
  double area;
  // mesh
  int32_t node_base;       // root node index in the concatenated node array
  int32_t slot_base;       // first leaf slot of this mesh
  int32_t rnode_base;      // root of the mesh's render-path tree (DevScene::rnodes)
  int32_t mesh_flags;      // mesh: 1 smooth, 2 texture coordinates (DevScene::fuv), 4 OBJ
                           // materials (DevScene::fmat), 8 vertex normals (DevScene::fvn)
  int32_t face_base;       // first face-normal record of this mesh
  int32_t n_faces;
  float bmin[3], bmax[3];  // bounds (for scene extents)
  double bb_min[3], bb_max[3];  // Entity::boundingBox of the reference (sphere / mesh / uvplane)
  double sss_rmax;
  // accretion disk under the black hole (circle.h:240-335): set when the
  // disk's material has disk_map and the hole has a disk texture
  int32_t kerr_disk;
  int32_t hemisphere;      // 'hemisphere': only the half with y >= y_centre is hit (sphere.h:98-103)
  double du_axis[3], dv_axis[3];  // the base UVPlane's unit axes and lengths (plane.h:146-157)
  double du_len, dv_len;
  double disk_em[3];              // the material's emission, FP64
};

// FP32 copy of an entity for the render path (no FP64 conversions in the
// inner loops); lives inside DevScene, i.e. in the kernel parameter space.
struct GEntF {
  int32_t type, material, normal_inverse, is_light;
  float p[3];
  float radius_eps;  // sphere radius + PS_EPS (light sampling, directLight_radiance.h:346)
  float u[3];
  float u_length;
  float v[3];
  float v_length;
  float n[3];
  float area;
  int32_t face_base, node_base;  // node_base: the render-path tree's root (DevScene::rnodes)
  float sss_rmax;  // subsurface probe-disk radius for this object (its bounding-box clamp applied)
  int32_t light_id;  // lights: registration index (Entity::light_id), which the reference
                     // uses as an index into the sorted list (directLight_radiance.h:541)
  // disk: u_length = radius, v_length = inner radius, n = the plane normal
};

// One entry of the light list in LightList::random_light_setup's order
// (sorted by power, light.h:97): what next-event estimation needs of each
// light kind (light.h:13-74, directLight_radiance.h:19-133).
enum { PR_LIGHT_AREA = 0, PR_LIGHT_PARALLEL = 1, PR_LIGHT_SPOT = 2, PR_LIGHT_INFINITY = 3 };
struct GLight {
  int32_t ent;        // the emitting entity (an infinity light's own type-0 entity)
  int32_t kind;       // PR_LIGHT_*
  int32_t mat;        // material whose emission the light gives off
  float falloff;      // spot: SpotLightFalloff exponent
  float dir[3];       // parallel: unit direction the light travels; spot: cone axis;
                      // infinity: the direction as given (not normalised)
  float cos_total;    // spot: cos(cone width), spot_light_cos_angle[0]
  float center[3];    // spot: sphere centre
  float cos_start;    // spot: cos(cone - falloff width), spot_light_cos_angle[1]
  float att[3];       // spot: attenuation a0 + d (a1 + a2 d)
  float dir_len;      // |dir| (infinity lights: the shadow ray runs along -dir / |dir|)
};

struct GMedium {
  float sigma_s_mean;      // ParticipatingMedia::scattering
  float sigma_t_mean;      // ParticipatingMedia::transmittance
  float sigma_s[3];        // scatteringColor
  float sigma_t[3];        // transmittanceColor
  float g[3];              // phase_prm
  int32_t on;
};

// WormHole state shared by every ray of a scene (WormHole.h:126-540 as
// SceneEnv builds it, scene_env.h:2100-2145); mat / inv: the frame Setup
// builds from the camera position for rays at mouth 0 ([0]) and mouth 1
// ([1]) and its cofactor inverse, row major 4 x 4 (computed on the host)
struct GWorm {
  int32_t enabled;
  int32_t max_steps;       // geodesics_max_length
  double pos[2][3];        // position0 ('in'), position1 ('out')
  double Rho, a, M;        // throat radius, half length, lensing (M = W / 1.42953)
  int32_t usr_sign;        // 'sign'
  int32_t pad;
  double mat[2][16];
  double inv[2][16];
  const unsigned char* tex[2];  // backgrounds, RGB8 rows as cell(y, x) reads them; null = none
  int32_t tex_w[2], tex_h[2];
  double map_coef[2][4];
  double tex_coef[2];
};

// KerrBlackHole state shared by every ray of a scene (KerrBlackHole.h:86-151;
// M = 1 as SceneEnv constructs it, scene_env.h:2067)
struct GKerr {
  int32_t enabled;
  int32_t max_steps;       // geodesics_max_length
  double pos[3];           // black hole centre (world)
  double a, a2, M, Rhor;   // spin, spin^2, mass, horizon radius + 1e-10
  double map_coef[4];      // background (theta, phi) affine map
  double escape_radius;    // 0: integrate to max_steps as the reference does
  double texture_coef;     // background texture scale (background_texture_coef)
  const unsigned char* texture;  // background texture, RGB8 rows as cell(y, x) reads them
  int32_t tex_w, tex_h;
  int32_t precision;             // PR_KERR_FP64 / PR_KERR_FP32
  double scene_radius;           // farthest scene geometry from the hole (BL-safe bound)
  double scene_inner;            // nearest scene geometry to the hole (0: something at the hole)
  // accretion disk (circle.h:240-335)
  double Rmstable;               // inner_orbit() (KerrBlackHole.h:215-240)
  double doppler_effect;         // color_doppler_factor_effect
  double observer[3];            // camera_pos of the black hole
  const uchar4* disk_tex;        // RGBA8 rows as cell(y, x) reads them; null = none
  int32_t disk_w, disk_h;
  int32_t use_temp;              // use_accretion_disk_temperature
  int32_t pad0;
  uint64_t disk_seed;            // key of the alpha-test stream
};

// Everything a kernel needs, passed by value (fits the 4 KB param space).
struct DevScene {
  const GEntity* ents;
  const GMaterial* mats;
  const GNode* nodes;      // the reference's trees (exact first-hit path)
  const float4* tris;      // 3 per leaf slot
  const WNode* rnodes;     // the render path's trees (render_bvh.h)
  const float4* rtris;     // 3 per triangle slot of those
  const float* fnorm;      // 3 per face
  const float4* texels;    // every material's texture, RGB / 255 (cell(i, j) order)
  const float4* ibl_texels;  // every IBL image, IBL_Color(i, j) order
  const float* bump_texels;  // every bump map: the texel's luminance 0.299 r + 0.587 g + 0.114 b (0..255)
  const float* fvn;        // 9 per face: the vertex normals of smooth meshes (null: none)
  const float* fuv;        // 6 per face: the texture coordinates of textured meshes (null: none)
  const int32_t* fmat;     // per face: the derived material of its OBJ material (-1: the entity's; null: none)
  int32_t n_ents;
  int32_t n_lights;
  int32_t n_point_lights;  // parallel, spot and infinity lights (sampled even without NEE)
  GLight lights[kMaxLights];
  double background[3];
  double env_light[3];
  float bg[3];
  float env[3];
  GMedium medium;
  float scene_scale;       // max |coordinate| of the scene bounds
  int32_t has_sss;         // a subsurface (dipole) material is present
  int32_t has_glossy;      // a Ward or Phong material is present
  int32_t has_tex;         // 1: a material has a texture, an IBL image or a bump map; 2: a mesh is smooth
  GEntF entf[kMaxEntities];
};

}  // namespace pr
