/*
 * prender_gpu.h — C ABI of the GB300 (sm_103a) radiance estimator and Kerr
 * geodesic tracer that drops in for prender's render loop.
 *
 * Every entry point is plain C: pointers, sizes and status codes.  All calls
 * return an int status: PR_OK (0) or a negative PR_E* code; pr_last_error()
 * gives a human-readable reason.  Nothing aborts or traps.  A context owns one
 * CUDA device and is not thread-safe (one context per host thread).
 *
 * Output buffers are caller-allocated.  Functions whose name ends in _dev
 * take device pointers; the others take host pointers and copy.
 *
 * Each declaration cites the reference interface it replaces
 * (paths are inside Sanaxen/prender).
 */
#ifndef PRENDER_GPU_H
#define PRENDER_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PR_ABI_VERSION 8

/* ---- status codes --------------------------------------------------- */
enum {
  PR_OK = 0,
  PR_E_ARG = -1,        /* bad argument (null pointer, size out of range)   */
  PR_E_CUDA = -2,       /* a CUDA runtime call failed                        */
  PR_E_SCENE = -3,      /* scene description is invalid or not uploaded      */
  PR_E_BUILD = -4,      /* acceleration structure could not be built         */
  PR_E_DEVICE = -5,     /* a device-side check fired (see pr_last_error)     */
  PR_E_NOMEM = -6,      /* allocation failed                                 */
  PR_E_UNSUPPORTED = -7 /* feature outside this build                        */
};

/* device-side error bits, reported through PR_E_DEVICE */
enum {
  PR_DEV_STACK_OVERFLOW = 1,  /* QBVH traversal stack exceeded its capacity  */
  PR_DEV_LOOP_CAP = 2,        /* a bounded device loop hit its iteration cap */
  PR_DEV_BAD_INDEX = 4,       /* a node/primitive index was out of range     */
  PR_DEV_QUEUE_OVERFLOW = 8,  /* a wavefront queue exceeded its capacity     */
  PR_DEV_NONFINITE = 16       /* a non-finite value was produced             */
};

/* ---- scene description (semantics of SceneEnv, scene_env.h:155-261) ---- */

/* material.h:19-29 ReflectionType, same numbering */
enum {
  PR_MAT_DIFFUSE = 0,
  PR_MAT_SPECULAR = 1,
  PR_MAT_REFRACTION = 2,
  PR_MAT_WARD = 3,
  PR_MAT_PHONG = 4,
  PR_MAT_SSS_REFRACTION = 5,
  PR_MAT_SSS_DIFFUSE = 6,
  PR_MAT_SSS_WARD = 7,
  PR_MAT_REFRACTION_FRESNEL = 8
};

/* entity.h:18-25 EntityType, same numbering.  PR_ENT_INF_LIGHT is an
 * 'infinity_light x y z' OBJECT (scene_env.h:891-894, :1525-1541): no
 * geometry, a directional light at infinity whose emission is its
 * material's; it counts as an entity here (the reference keeps it out of
 * its entity list, so later entity indices are one higher than its). */
enum {
  PR_ENT_INF_LIGHT = 0,
  PR_ENT_SPHERE = 1,
  PR_ENT_UVPLANE = 3,
  PR_ENT_CIRCLE = 4,
  PR_ENT_POLYGON = 5
};

/* Per-object homogeneous medium (ParticipatingMediaPrm.h:85-131): the
 * *_rgb colours are the raw keyword values; the host derives the scalar
 * means and transmittance exactly as setup_Scattering does. */
typedef struct pr_medium {
  double sigma_s_rgb[3];   /* SCATTERING colour line                         */
  double sigma_a_rgb[3];   /* ABSORBING colour line                          */
  double phase_g[3];       /* PAHASE (HG g per RGB channel)                  */
  double eta;              /* refractive index of the medium (BSSRDF)        */
  double scale;            /* MATERIAL_SCALE                                 */
  double r_max;            /* MATERIAL_R_MAX                                 */
  int32_t level;           /* -2 dipole, -1 single+multi, >=0 volumetric walk */
  int32_t use_bssrdf;
} pr_medium;

/* material.h:54-240 Material (texture fields out of scope) */
typedef struct pr_material {
  int32_t type;            /* PR_MAT_*                                       */
  int32_t disk_map;        /* 'disk_map' (scene_env.h:1163-1169): a disk with
                              this material under a black hole is shaded from
                              the accretion-disk texture (circle.h:240-335)  */
  double color[3];
  double emission[3];
  double specular[3];
  double roughness;        /* 'reflection diffuse' sets 1, 'specular' sets 0  */
  double refractive_index; /* default 1.5 (REFRACTIVE_INDEX_OF_GLASS)         */
  pr_medium medium;        /* used by the SSS material types                 */
  double r_refractive_index; /* 'r_refractive_index' (relative index of the
                                subsurface medium, default 1.0)               */
  double ward_alpha[2];    /* 'ward_brdf lo_d lo_s alp_x alp_y' roughness along
                              the orienting normal's u and v axes (material.h:42-47) */
  double phong_exponent;   /* 'phong_brdf lo_d lo_s n' specular exponent     */
  /* Textures on spheres, hemispheres and uvplanes (sphere.h:117-240,
   * plane.h:241-273).  texture: 'texture file.bmp', RGB8 rows as
   * BitMap::cell(y, x) reads them; a hit takes its colour and specular from
   * the texel.  ibl_*: 'ibl_texture file.bmp|.hdr': a hit takes its colour
   * from the texel and its emission from ibl_coef times the texel
   * (ibl_texture_coef); give the image as RGB8 (ibl_rgb8, a BMP) or as float
   * RGB (ibl_rgbf, a Radiance HDR as HDRImage holds it), not both.  NULL
   * pointers: no texture.  map_flags: PR_MAP_* (several may be set, applied
   * in the reference's order). */
  const uint8_t* texture;
  int32_t texture_width, texture_height;
  const uint8_t* ibl_rgb8;
  const float* ibl_rgbf;
  int32_t ibl_width, ibl_height;
  double ibl_coef;         /* ibl_texture_coef (default 1)                   */
  int32_t repeat;          /* 'repeat' (default 1)                           */
  int32_t map_flags;
  /* 'bump_texture file.bmp' (sphere.h:320-492, plane.h:274-360): RGB8 rows
   * as BitMap::cell(y, x) reads them, square; the luminance gradient tilts
   * a normal that scales the hit's scattered and next-event weights */
  const uint8_t* bump;
  int32_t bump_width, bump_height;
} pr_material;

/* texture mappings of spheres (material.h:188-192) */
enum {
  PR_MAP_HEMISPHERE = 1,     /* hemisphere_map    */
  PR_MAP_ANGULAR = 2,        /* angular_map       */
  PR_MAP_PANORAMIC = 4,      /* panoramic_map     */
  PR_MAP_EQUIRECTANGULAR = 8 /* equirectangular_map */
};

/* One OBJECT block (scene_env.h:854-1851) after its transforms. */
typedef struct pr_entity {
  int32_t type;            /* PR_ENT_*                                       */
  int32_t material;        /* index into pr_scene_desc.materials             */
  int32_t normal_inverse;  /* 'normal' keyword: 1 or -1                      */
  int32_t mesh;            /* PR_ENT_POLYGON: index into meshes              */
  double p[3];             /* sphere centre / uvplane origin / disk centre   */
  double radius;           /* sphere or disk radius                          */
  double u[3], v[3];       /* uvplane U and V edge vectors (unnormalised)    */
  double normal[3];        /* disk normal                                    */
  double radius_inner;     /* disk2 inner radius                             */
  int32_t blackhole_disk;  /* 'blackhole_disk' (scene_env.h:1177-1181, :1627):
                              index of the accretion-disk texture; 0 is the
                              reference's default, -1 = none                 */
  /* light kinds of an emitting entity (light.h:13-74, scene_env.h:1210-1252).
   * Only meaningful when the material is a light (diffuse, |colour| < 1e-3,
   * |emission| > 1e-3).  parallel_light: a uvplane or sphere whose light
   * arrives along -light_dir from wherever the entity is seen (a uvplane
   * with light_dir zero takes its own normal * normal_inverse).
   * spot_light: a sphere whose intensity |emission| falls off outside the
   * cone around light_dir (SpotLightFalloff) and with distance
   * (spot_attenuation).  Next-event estimation samples both kinds even when
   * it is off for area lights (brdf.h:590-605). */
  int32_t parallel_light;  /* 'parallel_light 1'                              */
  int32_t spot_light;      /* 'spot_light 1' (spheres only)                  */
  int32_t hemisphere;      /* PR_ENT_SPHERE: 'hemisphere x y z r', the half
                              with y >= 0 about the centre (sphere.h:98-103) */
  double light_dir[3];     /* parallel_light_dir / spot_light_dir, unit length
                              as the parser leaves them; PR_ENT_INF_LIGHT: the
                              'infinity_light' direction as given (its length
                              scales the light, as in the reference)         */
  double spot_angle[2];    /* spot_light_angle: cone and falloff widths in
                              degrees (cos(a0), cos(a0 - a1) bound the falloff) */
  double spot_falloff;     /* spot_light_falloff exponent (parser default 0) */
  double spot_attenuation[3]; /* spot_attenuation a0 a1 a2: intensity divided by
                              a0 + d (a1 + a2 d) (parser default 0 0 1)      */
  int32_t smooth;          /* PR_ENT_POLYGON: 'smooth 1' shades with the
                              normal interpolated from the vertex normals
                              (polygon.h:186-199)                            */
  int32_t pad_smooth;
} pr_entity;

/* Triangle mesh as ObjLoader keeps it (ObjLoader.h:153-233): float vertices,
 * 0-based faces.  face_normals may be NULL, in which case they are derived
 * with the loader's rule (ObjLoader.cpp:577-700).  A smooth entity's
 * vertex normals: vertex_normals[face_vn[3 f + k]] (the OBJ's vn lines and
 * face ids); both NULL derives them with the loader's rule (the mean of the
 * unnormalised face normals around each vertex, normalised; face_vn = the
 * face's vertex ids).  Texture coordinates (vt lines, 2 floats each) with
 * face_uv (3 ids per face) place textures and IBL images on the mesh
 * (polygon.h:206-212, :507-528); NULL for none. */
/* An OBJ material (newmtl in an mtllib file, ObjLoader.cpp:704-900;
 * ObjMaterial, ObjLoader.h:94-150) that faces select with usemtl.  A face's
 * hit takes the entity's material and then, as Triangle::intersect does
 * (polygon.h:228-400): the colour Kd and specular Ks (0 for a diffuse
 * entity material), or with a map_Kd texture the entity colour times the
 * texel; with '#REFLECTION t' also the type t, '#EMISSION', Ni, '#ROUGHNESS',
 * '#WARD' / Ns and the type's colours (texel-scaled with a texture). */
typedef struct pr_obj_material {
  double diffuse[3];          /* Kd (or '#COLOR')                            */
  double alpha;               /* d (or 1 - Tr); -1: none                     */
  double specular[3];         /* Ks (or '#SPECULAR')                         */
  double emission[3];         /* '#EMISSION'                                 */
  double refraction_index;    /* Ni (0 default; 1.5 for '#REFLECTION 2')     */
  double shininess;           /* Ns (default 5)                              */
  double roughness;           /* '#ROUGHNESS' (0; '#REFLECTION 0/1' set 0)    */
  double ward[2];             /* '#WARD ax ay'                               */
  int32_t reflection;         /* '#REFLECTION' type (-1: none)               */
  int32_t smooth;             /* '#SMOOTH': 0 unset, 1 on, 2 off             */
  int32_t repeat;             /* '#REPEAT' (default 1)                       */
  int32_t texture_width, texture_height;
  int32_t pad0;
  const uint8_t* texture;     /* map_Kd, RGB8 as BitMap::cell(y, x) reads it */
} pr_obj_material;

typedef struct pr_mesh {
  int32_t n_vertices;
  int32_t n_faces;
  const float* vertices;      /* 3 * n_vertices                              */
  const int32_t* faces;       /* 3 * n_faces                                 */
  const float* face_normals;  /* 3 * n_faces or NULL                         */
  int32_t n_vertex_normals;
  int32_t n_uv;
  const float* vertex_normals;  /* 3 * n_vertex_normals or NULL              */
  const int32_t* face_vn;       /* 3 * n_faces or NULL                       */
  const float* uv;              /* 2 * n_uv or NULL                          */
  const int32_t* face_uv;       /* 3 * n_faces or NULL                       */
  int32_t n_obj_materials;
  int32_t pad_obj;
  const pr_obj_material* obj_materials;  /* usemtl targets or NULL           */
  const int32_t* face_obj_material;      /* per face, -1: none; NULL: none   */
} pr_mesh;

/* Kerr integrator precision: PR_KERR_FP64 runs the reference's FP64
 * arithmetic in its order (exit directions within 1e-6 rad of it).
 * PR_KERR_FP32 is the mixed form: the reference's FP64 steps near the hole
 * and among the scene, FP32 fixed h = 2 steps for outbound rays beyond
 * max(200, scene radius + 2) while the FP64 error estimate stays small, and
 * an inbound ray inside all scene geometry with no radial turning point
 * left reported as captured (status 4) at once.  Renders take that
 * shortcut only on a black BACKGROUND, where a captured ray's colour does
 * not depend on whether the reference would end it in the horizon (2) or
 * by step underflow (4).  Its error against the FP64 form is stated by the
 * tests. */
enum { PR_KERR_FP64 = 0, PR_KERR_FP32 = 1 };

/* KerrBlackHole constructor inputs (KerrBlackHole.h:86-151, scene_env.h:701-766,2056-2098) */
typedef struct pr_kerr {
  int32_t enabled;
  int32_t max_steps;          /* geodesics_max_length                        */
  double position[3];         /* black hole centre (world)                   */
  double a;                   /* angular_momentum (spin, M = 1)              */
  double map_coef[4];         /* background (theta, phi) affine coefficients */
  double escape_radius;       /* 0 = reference behaviour (no escape test)    */
  double texture_coef;        /* background texture scale ('coef', default 1) */
  const uint8_t* texture;     /* background texture, RGB8, row y of W pixels as
                                 Bitmap::cell(y, x) returns it; NULL = none   */
  int32_t texture_width;
  int32_t texture_height;
  int32_t precision;          /* PR_KERR_FP64 (default) or PR_KERR_FP32      */
  int32_t use_accretion_disk_temperature;  /* scene_env.h:496-500           */
  double color_doppler_factor_effect;      /* scene_env.h:502-507           */
  double observer[3];         /* camera_position the black hole was built with
                                 (KerrBlackHole::camera_pos, scene_env.h:2067):
                                 the disk's Doppler factor is taken from it   */
  const uint8_t* disk_texture;  /* accretion_disk_texture 0, RGBA8 rows as
                                   Bitmap::cell(y, x) returns them; NULL = none */
  int32_t disk_texture_width;
  int32_t disk_texture_height;
  uint64_t disk_seed;         /* stream of the disk's alpha test (the reference
                                 draws it from the scene's generator, seeded
                                 from the clock, scene_env.h:306)             */
} pr_kerr;

/* A traversable wormhole (WormHole.h:126-540, scene_env.h:767-856,
 * :2100-2145): the Dneg metric of James, von Tunzelmann, Franklin and
 * Thorne ("Visualizing Interstellar's wormhole", 2015) with throat radius
 * rho, length 2a and lensing width w (M = w / 1.42953).  Every scene query
 * of radiance() follows a geodesic from the ray's origin (its mouth chosen
 * by |origin| > 1e6), stepped by Cash-Karp RK45 and tested against the
 * scene segment by segment; a ray that leaves ends on background 1 (l >= 0)
 * or 2 (l < 0).  Renders without next-event estimation and media. */
typedef struct pr_wormhole {
  int32_t enabled;
  int32_t max_steps;          /* geodesics_max_length                        */
  double in[3];               /* 'in' mouth (position0); the reference's
                                 default is CAMERA_POS + CAMERA_DIR * dist   */
  double out[3];              /* 'out' mouth (position1; default 0 0 0)      */
  double rho, a, w;           /* Rho, a, W                                   */
  int32_t sign;               /* 'sign': a nonzero value multiplies the final
                                 l before the side is read (usr_set_sign_)   */
  int32_t pad0;
  double camera[3];           /* camera_position the wormhole was built with
                                 (its frame's x axis points from the mouth to it) */
  const uint8_t* texture[2];  /* background_texture1 / 2, RGB8 rows as
                                 BitMap::cell(y, x) reads them; NULL = none   */
  int32_t texture_width[2];
  int32_t texture_height[2];
  double map_coef[2][4];      /* map_coef1 / map_coef2 (theta, phi) affine  */
  double texture_coef[2];     /* coef1 / coef2                               */
} pr_wormhole;

typedef struct pr_scene_desc {
  int32_t n_materials;
  int32_t n_entities;
  int32_t n_meshes;
  int32_t participating_media;  /* 'participatingMedia' keyword            */
  const pr_material* materials;
  const pr_entity* entities;
  const pr_mesh* meshes;
  double background[3];         /* BACKGROUND                               */
  double environment_light[3];  /* ENVLIGHT                                 */
  pr_medium medium;             /* global SCATTERING / ABSORBING / PAHASE   */
  pr_kerr kerr;
  pr_wormhole wormhole;
} pr_scene_desc;

/* CameraScreenPram (render.h:70-158) inputs, after SceneEnv::Load. */
typedef struct pr_camera {
  double position[3];
  double dir[3];              /* normalised by SceneEnv::Load (scene_env.h:1920) */
  double up[3];
  double screen_width;        /* world_screen_width  (CAMERA_ANGLE rule applied) */
  double screen_height;       /* world_screen_height                             */
  double screen_dist;         /* world_screen_dist                               */
  int32_t width, height;      /* IMAGE                                           */
} pr_camera;

/* render modes */
/* PR_MODE_MLT: primary-sample-space Metropolis light transport
 * (Render::RunMLT, render.h:363-785; Kelemen et al. 2002) over the same
 * radiance estimator: many independent chains on the GPU sharing one
 * bootstrap (W H pre_sample x samples seed paths; b their mean luminance),
 * each started from a seed drawn by luminance and running its share of the
 * samples x W x H x mutation mutations (p_large 0.5, Kelemen's weights); the
 * tent filter and the x 1/4 sensor scale of the reference's MLT set-up
 * apply; no luminance clamp. */
enum { PR_MODE_MEGAKERNEL = 0, PR_MODE_WAVEFRONT = 1, PR_MODE_MLT = 2 };

/* Render::Run (render.h:1125-1455) parameters. */
typedef struct pr_render_params {
  int32_t samples;            /* SAMPLING                                    */
  int32_t supersamples;       /* SUPERSAMPLING                               */
  int32_t tent_filter;        /* tentfilter                                  */
  int32_t depth;              /* DEPTH (RR starts after it)                  */
  int32_t depth_limit;        /* DEPTH_LIMIT                                 */
  int32_t nee;                /* nextEventEstimation                         */
  int32_t media;              /* participatingMedia (global medium on/off)   */
  int32_t mode;               /* PR_MODE_*                                   */
  uint64_t seed;              /* counter-based stream key                    */
  double luminance_cutoff;    /* per-sample clamp (default 0.025)            */
  double sensor_response;     /* final image scale (default 1)               */
  int32_t max_path_vertices;  /* device cap on path length (0 = 512)         */
  int32_t flags;              /* PR_FLAG_*                                   */
  int32_t total_spp;          /* samples of the whole frame when this call
                                 renders one shard of it; 0 = this call's
                                 samples*supersamples^2.  Sets the per-sample
                                 weight 1/total_spp and so the luminance
                                 clamp (render.h:1139, :1375-1384)          */
  int32_t pad1;
  double mlt_mutation;        /* PR_MODE_MLT: mutations per pixel and chain
                                 ('mutation', default 2)                     */
  double mlt_pre_sample;      /* seed paths per pixel and chain ('pre_sample',
                                 default 0.4)                                */
  int32_t mlt_chains;         /* GPU chains (0: enough to fill the device)   */
  int32_t pad2;
} pr_render_params;

enum {
  PR_FLAG_HG_CORRECT = 1,     /* sample HG with cos = 1/(2g)(...) instead of
                                 the reference's (g/2)(...) (sampler.h:55)   */
  PR_FLAG_EXACT_HITS = 2      /* FP64-confirmed closest hits while rendering */
};

typedef struct pr_ctx pr_ctx;

/* ---- context ---------------------------------------------------------- */
/* Replaces process start-up in main.cpp:21-60. */
pr_ctx* pr_create(int device, int* status);
void pr_destroy(pr_ctx* ctx);
const char* pr_last_error(const pr_ctx* ctx);
int pr_abi_version(void);
/* sizeof of the ABI structs, in the order pr_medium, pr_material,
 * pr_entity, pr_mesh, pr_kerr, pr_scene_desc, pr_camera,
 * pr_render_params, pr_render_stats (0..8); 0 for other values.  Lets a
 * binding check its struct mirrors. */
size_t pr_abi_sizeof(int which);

/* ---- scene -------------------------------------------------------------- */
/* Replaces SceneEnv::Load + CreateEntList (scene_env.h:357, scene.cpp:38):
 * uploads entities, materials, lights (light list built as in
 * LightList::random_light_setup, light.h:95) and builds one QBVH per mesh
 * with the reference's SAH rules (BVH.cpp:194-348, QBVH.cpp:161-302). */
int pr_scene_upload(pr_ctx* ctx, const pr_scene_desc* scene);

/* The checks pr_scene_upload makes of a scene description (sizes, indices,
 * materials, light kinds, the black hole), on the host, with no device and
 * no tree build.  Returns the status pr_scene_upload would; on an error
 * the reason goes to msg (msg_len bytes, NUL-terminated) when msg is not
 * null. */
int pr_scene_check(const pr_scene_desc* scene, char* msg, int msg_len);

/* QBVH statistics of a mesh entity: node count and leaf-array length.
 * Replaces QBVH::Construct bookkeeping (QBVH.cpp:161-186). */
int pr_qbvh_info(pr_ctx* ctx, int entity, int64_t* n_nodes, int64_t* n_leaf_slots);

/* Copies a mesh QBVH in the reference's layout (QBVH.h:53-61): per node
 * 24 floats of boxes [min/max][xyz][4], 4 int64 children (leaf = top bit |
 * leaf start, invalid = -1) and 3 int32 axes; leaf slots hold face ids with
 * -1 terminators.  Used to check the build against the reference. */
int pr_qbvh_export(pr_ctx* ctx, int entity, float* boxes, int64_t* children,
                   int32_t* axes, int32_t* leaf_faces);

/* Host-only build of one mesh's QBVH with the reference's rules (SAH
 * binary tree, BVH.cpp:194-348, flattened by QBVH.cpp:161-302), in the same
 * export layout as pr_qbvh_export.  Needs no GPU.  Call with null output
 * arrays to obtain n_nodes / n_leaf_slots, then again to fill them. */
int pr_qbvh_build_host(const float* vertices, int32_t n_vertices, const int32_t* faces, int32_t n_faces,
                       int64_t* n_nodes, int64_t* n_leaf_slots, float* boxes, int64_t* children,
                       int32_t* axes, int32_t* leaf_faces);

/* The render path's own tree of one mesh (no reference counterpart; the
 * reference builds only the QBVH above): a binned-SAH binary tree collapsed
 * to compressed 8-wide nodes, built on the host (on_gpu = 0) or on the GPU
 * (on_gpu = 1; pr_scene_upload uses it for meshes of 4096 faces and more).
 * Both builders make the same split decisions, so the nodes are equal and
 * only the order of triangles within a leaf may differ.  nodes: 80 bytes per
 * node (grid origin as 3 floats, x/y/z grid exponents and the inner-child
 * mask as 4 bytes, first inner child, first triangle slot, 8 leaf bytes,
 * then the children's lower and upper planes as 6 x 8 bytes), node 0 the
 * root; tri_faces: the face id of each triangle slot.  Outputs may be NULL
 * (counts only); PR_E_ARG if a capacity is too small (counts still set). */
int pr_render_bvh_export(pr_ctx* ctx, const pr_mesh* mesh, int on_gpu, void* nodes, int64_t nodes_cap,
                         int32_t* tri_faces, int64_t tris_cap, int64_t* n_nodes, int64_t* n_tris);

/* ---- closest hit ---------------------------------------------------------- */
/* intersect_scene_ (scene.cpp:83-214) for n rays, including the 1e-6 origin
 * push, the linear entity loop and QBVH::CheckIntersection (QBVH.cpp:17-137).
 * Rays are FP64 (org xyz, dir xyz interleaved, 6 per ray).  Outputs: entity
 * index (-1 = miss), face id for meshes (-1 otherwise), distance from the
 * pushed origin (FP64, bit-exact with the reference).  Host buffers. */
int pr_first_hit(pr_ctx* ctx, const double* rays, int64_t n, int32_t* entity,
                 int32_t* prim, double* t);
/* same, device buffers */
int pr_first_hit_dev(pr_ctx* ctx, const double* rays, int64_t n, int32_t* entity,
                     int32_t* prim, double* t);

/* The renderer's own FP32 closest-hit query (near-first QBVH traversal with
 * culling) on the same ray batch, for checking it against pr_first_hit:
 * rays are converted to FP32 and the origin is used as given (no 1e-6
 * push).  Outputs as pr_first_hit, t in FP64 holding the FP32 distance. */
int pr_trace_fast(pr_ctx* ctx, const double* rays, int64_t n, int32_t* entity, int32_t* prim, double* t);

/* ---- rendering -------------------------------------------------------- */
/* Render::Run (render.h:1125-1455): accumulates samples [sample_offset,
 * sample_offset + samples*supersamples^2) of every pixel into rgb_accum
 * (W*H*3 floats, row order of the reference image: index (H-y-1)*W+x),
 * already multiplied by 1/(total samples) and by sensor_response.  With
 * sample_offset = 0 and accumulate = 0 the buffer is overwritten. */
int pr_render(pr_ctx* ctx, const pr_camera* cam, const pr_render_params* prm,
              float* rgb_accum, uint64_t sample_offset, int accumulate);
int pr_render_dev(pr_ctx* ctx, const pr_camera* cam, const pr_render_params* prm,
                  float* rgb_accum_dev, uint64_t sample_offset, int accumulate);

/* Allocation-free variant of pr_render_dev for the megakernel form (no
 * counterpart in the reference, which renders on the CPU).  For callers that
 * must not allocate device memory while rendering: a frame loop with a hard
 * time budget, which cannot absorb the device-wide synchronisation that
 * cudaMalloc / cudaFree may cause, or a host application whose device memory
 * is all handed out by its own pool allocator, so that an allocation behind
 * its back can fail or break its accounting.  It calls no cudaMalloc /
 * cudaFree; its scratch is a 16 MiB
 * static device array that every GPU loading this library keeps until exit,
 * so images of at most 1,398,080 pixels are accepted (larger ones return
 * PR_E_ARG).  The first call on a device looks up that array's address in
 * the device's primary context and keeps it; make that first call before
 * any stream capture starts.  The kept address is not valid in a context
 * made with the driver API, nor after cudaDeviceReset.  Calls that overlap
 * on the GPU share the array and race.  The scene must already be uploaded
 * with pr_scene_upload (which allocates, at set-up).  Result as
 * pr_render_dev, except where pr_render_dev's per-chunk partial images
 * (min(ceil(1.2e6 / pixels), spp) chunks of W*H*3 floats) would not fit in
 * the array: there the samples are summed in fewer chunks, so the image
 * agrees with pr_render_dev's to float rounding rather than bit for bit. */
int pr_render_dev_noalloc(pr_ctx* ctx, const pr_camera* cam, const pr_render_params* prm, float* rgb_accum_dev,
                          uint64_t sample_offset, int accumulate);

/* Per-launch statistics of the last render: paths, path segments (extension
 * plus shadow rays), QBVH nodes visited, triangle tests, device milliseconds.
 * Kerr renders and pr_kerr_trace report straight-segment scene tests as
 * segments, accepted RK45 steps as nodes_visited and RK45 attempts as
 * tri_tests. */
typedef struct pr_render_stats {
  uint64_t paths;
  uint64_t segments;
  uint64_t nodes_visited;
  uint64_t tri_tests;
  double device_ms;
  uint64_t kernel_launches;  /* kernels of this library launched by the call */
} pr_render_stats;
int pr_last_render_stats(pr_ctx* ctx, pr_render_stats* stats);
/* Autotuner (no reference counterpart): times one short wavefront frame
 * (the caller's camera and parameters with enough camera samples per pixel
 * to fill the largest pool twice over) for each candidate path-pool size
 * {2^19 .. 2^22} and traversal grid {4, 8, 16} blocks per SM, and keeps the
 * fastest for later pr_render calls on this context.  Images do not depend
 * on either choice.  Outputs may be NULL. */
int pr_autotune_wavefront(pr_ctx* ctx, const pr_camera* camera, const pr_render_params* params,
                          int32_t* slots, int32_t* trace_blocks_per_sm, double* frame_ms);

/* Per-kernel device time of the last wavefront render when it ran with the
 * host-driven loop (environment PR_WF_HOST_LOOP=1; zeros otherwise): ms[0..3]
 * = shade, extend, shadow, control (n entries written, at most 4); and
 * shadow_counts[0..2] = the frame's shadow rays, node visits and triangle
 * tests (may be NULL).  No reference counterpart (diagnostics). */
int pr_last_kernel_times(pr_ctx* ctx, double* ms, unsigned long long* shadow_counts, int n);

/* ---- Batches ---------------------------------------------------------- */
/* A scene object: an uploaded scene owned by the context, independent of the
 * one pr_scene_upload sets (SceneEnv::Load + CreateEntList per object). */
typedef struct pr_scene_obj pr_scene_obj;
pr_scene_obj* pr_scene_create(pr_ctx* ctx, const pr_scene_desc* desc, int* status);
void pr_scene_release(pr_ctx* ctx, pr_scene_obj* scene);

typedef struct pr_job {
  const pr_scene_obj* scene;
  pr_camera camera;
  pr_render_params params;    /* params.mode: plain (megakernel) or wavefront form */
  float* rgb_dev;             /* W*H*3 floats on the device, image row order  */
  uint64_t sample_offset;
  int32_t accumulate;
  int32_t pad;
} pr_job;

/* Renders n jobs (no reference counterpart: the reference renders one scene
 * per process).  Plain-form jobs (and Kerr scenes) run as one captured CUDA
 * graph, on parallel branches; each such image equals pr_render_dev of the
 * same inputs up to float summation order (a batch uses fewer sample chunks
 * per pixel).  Wavefront-form jobs share the context's path pool and run one
 * after another after that graph, each as pr_render_dev would run it (one
 * graph launch per pass), with the same image.  Scene objects must stay
 * alive until the call returns. */
int pr_render_batch(pr_ctx* ctx, int n, const pr_job* jobs);

/* ---- Differentiation ------------------------------------------------- */
/* Adjoint of pr_render by path replay (no reference counterpart: the
 * reference renders only).  Given dL_drgb = dLoss/d(image) for the image that
 * pr_render produced with the same camera, parameters and sample_offset
 * (3 floats per pixel, same row order), ADDS dLoss/d(material colour) to
 * d_color and dLoss/d(material emission) to d_emission (3 doubles per
 * material each, in pr_scene_desc material order; either may be NULL), and
 * writes dLoss/d(s) for a common scale s of every emission at s = 1 to
 * *d_emission_scale (may be NULL).  Sampling decisions are held fixed;
 * scenes with participating media or more than 16 materials are rejected
 * (PR_E_UNSUPPORTED).  pr_render_adjoint takes host buffers. */
int pr_render_adjoint(pr_ctx* ctx, const pr_camera* camera, const pr_render_params* params,
                      const float* dl_drgb, uint64_t sample_offset, double* d_color,
                      double* d_emission, double* d_emission_scale);
int pr_render_adjoint_dev(pr_ctx* ctx, const pr_camera* camera, const pr_render_params* params,
                          const float* dl_drgb_dev, uint64_t sample_offset, double* d_color_dev,
                          double* d_emission_dev);

/* ---- Kerr geodesics --------------------------------------------------- */
/* The Kerr branch of intersect_scene (scene.cpp:448-732) for n camera rays
 * (FP64, 6 per ray).  Per ray: status (0 reached background, 1 hit an
 * entity, 2 event horizon, 3 initial-condition failure, 4 step underflow),
 * final Boyer-Lindquist (r, theta, phi), final polyline direction, steps
 * taken, hit entity and hit distance.  Host buffers. */
int pr_kerr_trace(pr_ctx* ctx, const double* rays, int64_t n, int32_t* status,
                  double* final_bl, double* exit_dir, int32_t* steps,
                  int32_t* hit_entity, double* hit_t);
int pr_kerr_trace_dev(pr_ctx* ctx, const double* rays, int64_t n, int32_t* status,
                      double* final_bl, double* exit_dir, int32_t* steps,
                      int32_t* hit_entity, double* hit_t);

/* ---- Wormhole geodesics ---------------------------------------------- */
/* The wormhole branch of intersect_scene__ (scene.cpp:735-925) for n rays
 * (FP64, 6 per ray).  Per ray: status (1 hit an entity, 0 ended on
 * background 1 (final l >= 0), 3 on background 2 (l < 0)), final state
 * (l, then theta and phi of the last polyline direction), that direction,
 * steps taken and the hit entity (-1: none).  Host buffers; the _dev form
 * takes device pointers.  Any output may be NULL. */
int pr_wormhole_trace(pr_ctx* ctx, const double* rays, int64_t n, int32_t* status,
                      double* final_y, double* exit_dir, int32_t* steps,
                      int32_t* hit_entity);
int pr_wormhole_trace_dev(pr_ctx* ctx, const double* rays, int64_t n, int32_t* status,
                          double* final_y, double* exit_dir, int32_t* steps,
                          int32_t* hit_entity);

/* Ray-bundle Jacobian of the Kerr map (no reference counterpart).  The
 * initial direction d of each ray is perturbed as normalize(d + s e1 + t e2);
 * basis holds e1, e2 (6 doubles per ray) or is NULL (then e1 = unit(d x z),
 * or d x x near the z axis, and e2 = e1 x d).  For rays that leave the scene
 * (status 0) jac_dir gets d(exit direction)/d(s, t), 3 x 2 row-major, and
 * jac_bl gets d(final theta, phi)/d(s, t), 2 x 2 row-major; other statuses
 * give NaN.  Forward mode on dual numbers through the FP64 tracer, along the
 * primal trace's steps.  Host buffers; any output may be NULL. */
int pr_kerr_sensitivity(pr_ctx* ctx, const double* rays, int64_t n, const double* basis,
                        int32_t* status, double* jac_dir, double* jac_bl);
/* Adjoint form: grad (2 per ray) = cotangent^T d(exit direction)/d(s, t)
 * for a cotangent of 3 doubles per ray (evaluated from the same forward
 * tangents: two inputs per ray make forward mode the cheaper one). */
int pr_kerr_sensitivity_adjoint(pr_ctx* ctx, const double* rays, int64_t n, const double* basis,
                                const double* cotangent, double* grad);

/* ---- output --------------------------------------------------------- */
/* 8-bit output of an image (Render::OutputBmp, render.h:1563-1589, with
 * ppm.h:22-27): per channel int(pow(clamp(x, 0, 1), g) * 255 + 0.5), g =
 * 1/2.2, or g = gamma_offset when |gamma_offset| > 0.01 (the reference uses
 * the offset itself as the exponent; negative offsets are refused).  in:
 * W*H*3 floats in pr_render's row order; out: W*H*3 bytes in the bitmap's
 * cell(i, j) order (row i = image row H-1-i), R, G, B.  _dev: device
 * buffers; the plain form takes host buffers. */
int pr_image_to_rgb8(pr_ctx* ctx, const float* rgb, int32_t width, int32_t height, double gamma_offset,
                     uint8_t* out);
int pr_image_to_rgb8_dev(pr_ctx* ctx, const float* rgb_dev, int32_t width, int32_t height, double gamma_offset,
                         uint8_t* out_dev);

/* HDR output of an image (Render::OutputHdr, render.h:1649-1667, with
 * HDRImage::HDRPixel, hdr.h:30-44): Radiance RGBE bytes, 4 per pixel (R, G, B
 * mantissas and the exponent + 128; zero where max(R, G, B) <= 1e-32), the
 * file's scanline order (scanline r = row r of pr_render's order).  in: W*H*3
 * floats; out: W*H*4 bytes (4-byte aligned for _dev).  The header and the
 * scanline framing are the writer's (prender_gb300.scene.write_hdr). */
int pr_image_to_rgbe(pr_ctx* ctx, const float* rgb, int32_t width, int32_t height, uint8_t* out);
int pr_image_to_rgbe_dev(pr_ctx* ctx, const float* rgb_dev, int32_t width, int32_t height, uint8_t* out_dev);

/* Accretion-disk shading test hook: the texture, temperature and Doppler
 * branch of Circle::intersect under the black hole (circle.h:240-322, no
 * alpha test) at n world points of disk entity `entity`.  Host buffers:
 * points 3n in; valid n (0 where the disk is not there: inside the ISCO,
 * beyond the radius, off the texture), colour 3n, emission 3n, alpha n out.
 * PR_E_SCENE without a disk texture; the scene's disk_map flag is not
 * required. */
int pr_kerr_disk_shade(pr_ctx* ctx, int entity, const double* points, int64_t n, int32_t* valid,
                       double* color, double* emission, double* alpha);

/* ---- scene files ---------------------------------------------------- */
/* The reference's scene text format read on the host (SceneEnv::Load,
 * scene_env.h:357-2160, with its expression evaluator Expr.h for every
 * value it evaluates: VAR variables, arithmetic, functions, %NAME%
 * environment references; OBJ meshes as Obj::Load reads them, quads and
 * vertex normals included; rotation / translate / scale of spheres and
 * meshes; TARGET_POS and CAMERA_MATRIX; BMP textures), replacing the
 * `prender scene.txt` front end (main.cpp) for callers that render through
 * this library.  No GPU is touched.  pr_scene_file_load returns NULL on
 * failure with "file:line: message" in err (errlen bytes): a missing file,
 * a value the evaluator rejects, or a keyword of a feature this library
 * does not render (other lights, object textures, transformed uvplanes and
 * disks, lens, MLT, wormholes, OBJ materials), which is refused rather than
 * skipped.  Lines that do not change the image are skipped and listed by
 * pr_scene_file_warnings.  The reference's overrides of settings by
 * environment variables (SAMPLING, IMAGE_X, ...) are not applied. */
typedef struct pr_scene_file pr_scene_file;
pr_scene_file* pr_scene_file_load(const char* path, char* err, int errlen);
/* The scene, for pr_scene_upload / pr_scene_create; its buffers live until
 * pr_scene_file_free. */
const pr_scene_desc* pr_scene_file_desc(const pr_scene_file* file);
/* Camera (CAMERA_ANGLE rule applied, direction normalised), render
 * parameters (mode PR_MODE_MEGAKERNEL, seed 0: set them before pr_render)
 * and gamma_offset (for pr_image_to_rgb8); any pointer may be NULL. */
int pr_scene_file_camera(const pr_scene_file* file, pr_camera* cam, pr_render_params* prm, double* gamma_offset);
const char* pr_scene_file_warnings(const pr_scene_file* file);
void pr_scene_file_free(pr_scene_file* file);

#ifdef __cplusplus
}
#endif
#endif /* PRENDER_GPU_H */
