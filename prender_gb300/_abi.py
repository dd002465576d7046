"""ctypes mirror of include/prender_gpu.h (the C ABI).

Field order and types must match the header exactly; tests check the sizes
against the shared library's own sizeof report.
"""
import ctypes as C

PR_OK = 0
PR_E_ARG = -1
PR_E_CUDA = -2
PR_E_SCENE = -3
PR_E_BUILD = -4
PR_E_DEVICE = -5
PR_E_NOMEM = -6
PR_E_UNSUPPORTED = -7

# material.h:19-29 ReflectionType
PR_MAT_DIFFUSE = 0
PR_MAT_SPECULAR = 1
PR_MAT_REFRACTION = 2
PR_MAT_WARD = 3
PR_MAT_PHONG = 4
PR_MAT_SSS_REFRACTION = 5
PR_MAT_SSS_DIFFUSE = 6
PR_MAT_SSS_WARD = 7
PR_MAT_REFRACTION_FRESNEL = 8

# entity.h:18-25 EntityType
PR_ENT_INF_LIGHT = 0
PR_ENT_SPHERE = 1
PR_ENT_UVPLANE = 3
PR_ENT_CIRCLE = 4
PR_KERR_FP64 = 0
PR_KERR_FP32 = 1
PR_ENT_POLYGON = 5
PR_MAP_HEMISPHERE = 1
PR_MAP_ANGULAR = 2
PR_MAP_PANORAMIC = 4
PR_MAP_EQUIRECTANGULAR = 8

PR_MODE_MEGAKERNEL = 0
PR_MODE_WAVEFRONT = 1
PR_MODE_MLT = 2

PR_FLAG_HG_CORRECT = 1
PR_FLAG_EXACT_HITS = 2

D3 = C.c_double * 3


class pr_medium(C.Structure):
    _fields_ = [
        ("sigma_s_rgb", D3),
        ("sigma_a_rgb", D3),
        ("phase_g", D3),
        ("eta", C.c_double),
        ("scale", C.c_double),
        ("r_max", C.c_double),
        ("level", C.c_int32),
        ("use_bssrdf", C.c_int32),
    ]


class pr_material(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("disk_map", C.c_int32),
        ("color", D3),
        ("emission", D3),
        ("specular", D3),
        ("roughness", C.c_double),
        ("refractive_index", C.c_double),
        ("medium", pr_medium),
        ("r_refractive_index", C.c_double),
        ("ward_alpha", C.c_double * 2),
        ("phong_exponent", C.c_double),
        ("texture", C.POINTER(C.c_uint8)),
        ("texture_width", C.c_int32),
        ("texture_height", C.c_int32),
        ("ibl_rgb8", C.POINTER(C.c_uint8)),
        ("ibl_rgbf", C.POINTER(C.c_float)),
        ("ibl_width", C.c_int32),
        ("ibl_height", C.c_int32),
        ("ibl_coef", C.c_double),
        ("repeat", C.c_int32),
        ("map_flags", C.c_int32),
        ("bump", C.POINTER(C.c_uint8)),
        ("bump_width", C.c_int32),
        ("bump_height", C.c_int32),
    ]


class pr_entity(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("material", C.c_int32),
        ("normal_inverse", C.c_int32),
        ("mesh", C.c_int32),
        ("p", D3),
        ("radius", C.c_double),
        ("u", D3),
        ("v", D3),
        ("normal", D3),
        ("radius_inner", C.c_double),
        ("blackhole_disk", C.c_int32),
        ("parallel_light", C.c_int32),
        ("spot_light", C.c_int32),
        ("hemisphere", C.c_int32),
        ("light_dir", D3),
        ("spot_angle", C.c_double * 2),
        ("spot_falloff", C.c_double),
        ("spot_attenuation", D3),
        ("smooth", C.c_int32),
        ("pad_smooth", C.c_int32),
    ]


class pr_obj_material(C.Structure):
    _fields_ = [
        ("diffuse", D3),
        ("alpha", C.c_double),
        ("specular", D3),
        ("emission", D3),
        ("refraction_index", C.c_double),
        ("shininess", C.c_double),
        ("roughness", C.c_double),
        ("ward", C.c_double * 2),
        ("reflection", C.c_int32),
        ("smooth", C.c_int32),
        ("repeat", C.c_int32),
        ("texture_width", C.c_int32),
        ("texture_height", C.c_int32),
        ("pad0", C.c_int32),
        ("texture", C.c_void_p),
    ]


class pr_mesh(C.Structure):
    _fields_ = [
        ("n_vertices", C.c_int32),
        ("n_faces", C.c_int32),
        ("vertices", C.POINTER(C.c_float)),
        ("faces", C.POINTER(C.c_int32)),
        ("face_normals", C.POINTER(C.c_float)),
        ("n_vertex_normals", C.c_int32),
        ("n_uv", C.c_int32),
        ("vertex_normals", C.POINTER(C.c_float)),
        ("face_vn", C.POINTER(C.c_int32)),
        ("uv", C.POINTER(C.c_float)),
        ("face_uv", C.POINTER(C.c_int32)),
        ("n_obj_materials", C.c_int32),
        ("pad_obj", C.c_int32),
        ("obj_materials", C.POINTER(pr_obj_material)),
        ("face_obj_material", C.POINTER(C.c_int32)),
    ]


class pr_kerr(C.Structure):
    _fields_ = [
        ("enabled", C.c_int32),
        ("max_steps", C.c_int32),
        ("position", D3),
        ("a", C.c_double),
        ("map_coef", C.c_double * 4),
        ("escape_radius", C.c_double),
        ("texture_coef", C.c_double),
        ("texture", C.c_void_p),
        ("texture_width", C.c_int32),
        ("texture_height", C.c_int32),
        ("precision", C.c_int32),
        ("use_accretion_disk_temperature", C.c_int32),
        ("color_doppler_factor_effect", C.c_double),
        ("observer", D3),
        ("disk_texture", C.c_void_p),
        ("disk_texture_width", C.c_int32),
        ("disk_texture_height", C.c_int32),
        ("disk_seed", C.c_uint64),
    ]


class pr_wormhole(C.Structure):
    _fields_ = [
        ("enabled", C.c_int32),
        ("max_steps", C.c_int32),
        ("in_", D3),
        ("out", D3),
        ("rho", C.c_double),
        ("a", C.c_double),
        ("w", C.c_double),
        ("sign", C.c_int32),
        ("pad0", C.c_int32),
        ("camera", D3),
        ("texture", C.c_void_p * 2),
        ("texture_width", C.c_int32 * 2),
        ("texture_height", C.c_int32 * 2),
        ("map_coef", (C.c_double * 4) * 2),
        ("texture_coef", C.c_double * 2),
    ]


class pr_scene_desc(C.Structure):
    _fields_ = [
        ("n_materials", C.c_int32),
        ("n_entities", C.c_int32),
        ("n_meshes", C.c_int32),
        ("participating_media", C.c_int32),
        ("materials", C.POINTER(pr_material)),
        ("entities", C.POINTER(pr_entity)),
        ("meshes", C.POINTER(pr_mesh)),
        ("background", D3),
        ("environment_light", D3),
        ("medium", pr_medium),
        ("kerr", pr_kerr),
        ("wormhole", pr_wormhole),
    ]


class pr_camera(C.Structure):
    _fields_ = [
        ("position", D3),
        ("dir", D3),
        ("up", D3),
        ("screen_width", C.c_double),
        ("screen_height", C.c_double),
        ("screen_dist", C.c_double),
        ("width", C.c_int32),
        ("height", C.c_int32),
    ]


class pr_render_params(C.Structure):
    _fields_ = [
        ("samples", C.c_int32),
        ("supersamples", C.c_int32),
        ("tent_filter", C.c_int32),
        ("depth", C.c_int32),
        ("depth_limit", C.c_int32),
        ("nee", C.c_int32),
        ("media", C.c_int32),
        ("mode", C.c_int32),
        ("seed", C.c_uint64),
        ("luminance_cutoff", C.c_double),
        ("sensor_response", C.c_double),
        ("max_path_vertices", C.c_int32),
        ("flags", C.c_int32),
        ("total_spp", C.c_int32),
        ("pad1", C.c_int32),
        ("mlt_mutation", C.c_double),
        ("mlt_pre_sample", C.c_double),
        ("mlt_chains", C.c_int32),
        ("pad2", C.c_int32),
    ]


class pr_render_stats(C.Structure):
    _fields_ = [
        ("paths", C.c_uint64),
        ("segments", C.c_uint64),
        ("nodes_visited", C.c_uint64),
        ("tri_tests", C.c_uint64),
        ("device_ms", C.c_double),
        ("kernel_launches", C.c_uint64),
    ]


class pr_job(C.Structure):
    _fields_ = [
        ("scene", C.c_void_p),
        ("camera", pr_camera),
        ("params", pr_render_params),
        ("rgb_dev", C.c_void_p),
        ("sample_offset", C.c_uint64),
        ("accumulate", C.c_int32),
        ("pad", C.c_int32),
    ]
