"""Scene description with the semantics of prender's SceneEnv.

Mirrors the OBJECT / global keywords of the reference's scene format
(scene_env.h:357-2160): materials follow the reference's defaults (diffuse
type with roughness 0 unless 'reflection diffuse' sets 1, glass IOR 1.5),
lights are entities whose material passes Material::isLight (material.h),
and the camera follows CameraScreenPram (render.h:105-150) with the
CAMERA_ANGLE rule (scene_env.h:1881-1886).

A Scene can be handed to the GPU library (``to_desc``) and written out in
the reference's own text format (``write_reference``), so that the same
bytes drive both.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _abi as A


@dataclass
class Medium:
    """Homogeneous medium (ParticipatingMediaPrm.h:85-131)."""
    sigma_s_rgb: Sequence[float] = (0.0, 0.0, 0.0)
    sigma_a_rgb: Sequence[float] = (0.0, 0.0, 0.0)
    phase_g: Sequence[float] = (0.0, 0.0, 0.0)
    eta: float = 0.0
    scale: float = 1.0
    r_max: float = 1.0
    level: int = -1
    use_bssrdf: int = 1

    def to_c(self) -> A.pr_medium:
        m = A.pr_medium()
        m.sigma_s_rgb[:] = [float(x) for x in self.sigma_s_rgb]
        m.sigma_a_rgb[:] = [float(x) for x in self.sigma_a_rgb]
        m.phase_g[:] = [float(x) for x in self.phase_g]
        m.eta, m.scale, m.r_max = float(self.eta), float(self.scale), float(self.r_max)
        m.level, m.use_bssrdf = int(self.level), int(self.use_bssrdf)
        return m


@dataclass
class Material:
    """Material (material.h:54-240); defaults are the reference's."""
    type: int = A.PR_MAT_DIFFUSE
    color: Sequence[float] = (0.0, 0.0, 0.0)
    emission: Sequence[float] = (0.0, 0.0, 0.0)
    specular: Sequence[float] = (0.0, 0.0, 0.0)
    roughness: float = 0.0
    refractive_index: float = 1.5
    medium: Medium = field(default_factory=Medium)
    r_refractive_index: float = 1.0
    disk_map: int = 0
    ward_alpha: Sequence[float] = (0.1, 0.1)
    phong_exponent: float = 1.0
    # textures (sphere.h:104-240, plane.h:241-273): texture (H, W, 3) uint8
    # rows as BitMap::cell(y, x) reads them; ibl (H, W, 3) uint8 (a bitmap)
    # or float32 (a Radiance HDR image, IBL_Color(i, j) order); map_flags
    # PR_MAP_*; compared by identity, not value
    texture: Optional[np.ndarray] = field(default=None, compare=False, repr=False)
    ibl: Optional[np.ndarray] = field(default=None, compare=False, repr=False)
    ibl_coef: float = 1.0
    repeat: int = 1
    map_flags: int = 0
    bump: Optional[np.ndarray] = field(default=None, compare=False, repr=False)  # (N, N, 3) uint8

    @staticmethod
    def diffuse(color, emission=(0.0, 0.0, 0.0)) -> "Material":
        """'reflection diffuse' (scene_env.h:1444-1448): roughness 1."""
        return Material(A.PR_MAT_DIFFUSE, tuple(color), tuple(emission), roughness=1.0)

    @staticmethod
    def mirror(color) -> "Material":
        """'reflection specular' (scene_env.h:1486-1490): roughness 0."""
        return Material(A.PR_MAT_SPECULAR, tuple(color), roughness=0.0)

    @staticmethod
    def ward(color, specular, alpha_x: float, alpha_y: float, emission=(0.0, 0.0, 0.0)) -> "Material":
        """'reflection ward_brdf' with 'ward_brdf 1 1 alpha_x alpha_y'
        (scene_env.h:1417-1425, :1492-1495): diffuse colour with probability
        rd / (rd + rs) of the mean reflectances, else Ward's anisotropic
        glossy lobe weighted by specular (brdf.h:192-319)."""
        return Material(A.PR_MAT_WARD, tuple(color), tuple(emission), tuple(specular),
                        ward_alpha=(float(alpha_x), float(alpha_y)))

    @staticmethod
    def phong(color, specular, exponent: float, roughness: float = 0.0, emission=(0.0, 0.0, 0.0)) -> "Material":
        """'reflection phong_brdf' with 'phong_brdf 1 1 exponent' (scene_env.h
        :1427-1435, :1497-1500): diffuse with probability roughness, else the
        cos^n lobe about the mirror direction weighted by specular
        (brdf.h:16-190, radiance.h:470-484)."""
        return Material(A.PR_MAT_PHONG, tuple(color), tuple(emission), tuple(specular), roughness=float(roughness),
                        phong_exponent=float(exponent))

    @staticmethod
    def glass(color, ior: float = 1.5) -> "Material":
        """'reflection reflection' (scene_env.h:1450-1458)."""
        return Material(A.PR_MAT_REFRACTION, tuple(color), refractive_index=ior)

    @staticmethod
    def subsurface(color, sigma_s, sigma_a, g=0.0, eta: float = 1.3, ior: float = 1.5, r_max: float = 1.0,
                   scale: float = 1.0, level: int = -2) -> "Material":
        """'reflection reflection' + 'reflection Subsurface_Scattering' with the
        material's SCATTERING / ABSORBING / PAHASE, 'level' (-2: directional
        dipole; -1: dipole or a single-scattering walk, half each;
        scene_env.h:1305-1362) and r_refractive_index eta."""
        g3 = tuple(g) if hasattr(g, "__len__") else (float(g),) * 3
        return Material(A.PR_MAT_SSS_REFRACTION, tuple(color), refractive_index=ior, r_refractive_index=eta,
                        medium=Medium(sigma_s_rgb=tuple(sigma_s), sigma_a_rgb=tuple(sigma_a), phase_g=g3, scale=scale,
                                      r_max=r_max, level=int(level), use_bssrdf=1))

    def is_light(self) -> bool:
        """Material::isLight (material.h)."""
        return (self.type == A.PR_MAT_DIFFUSE and math.sqrt(sum(c * c for c in self.color)) < 0.001
                and math.sqrt(sum(e * e for e in self.emission)) > 0.001)

    def to_c(self, keep=None) -> A.pr_material:
        """keep: a list that takes the texture arrays the struct points to
        (without it the struct carries no textures)"""
        m = A.pr_material()
        m.type = int(self.type)
        m.color[:] = [float(x) for x in self.color]
        m.emission[:] = [float(x) for x in self.emission]
        m.specular[:] = [float(x) for x in self.specular]
        m.roughness = float(self.roughness)
        m.refractive_index = float(self.refractive_index)
        m.medium = self.medium.to_c()
        m.r_refractive_index = float(self.r_refractive_index)
        m.disk_map = int(self.disk_map)
        m.ward_alpha[:] = [float(x) for x in self.ward_alpha]
        m.phong_exponent = float(self.phong_exponent)
        m.ibl_coef = float(self.ibl_coef)
        m.repeat = int(self.repeat)
        m.map_flags = int(self.map_flags)
        if keep is not None:
            if self.texture is not None:
                t = np.ascontiguousarray(self.texture, dtype=np.uint8)
                if t.ndim != 3 or t.shape[2] != 3:
                    raise ValueError("texture must be (H, W, 3) uint8")
                keep.append(t)
                m.texture = t.ctypes.data_as(C.POINTER(C.c_uint8))
                m.texture_height, m.texture_width = t.shape[0], t.shape[1]
            if self.ibl is not None:
                if self.ibl.dtype == np.uint8:
                    t = np.ascontiguousarray(self.ibl)
                    m.ibl_rgb8 = t.ctypes.data_as(C.POINTER(C.c_uint8))
                else:
                    t = np.ascontiguousarray(self.ibl, dtype=np.float32)
                    m.ibl_rgbf = t.ctypes.data_as(C.POINTER(C.c_float))
                if t.ndim != 3 or t.shape[2] != 3:
                    raise ValueError("ibl image must be (H, W, 3)")
                keep.append(t)
                m.ibl_height, m.ibl_width = t.shape[0], t.shape[1]
            if self.bump is not None:
                t = np.ascontiguousarray(self.bump, dtype=np.uint8)
                if t.ndim != 3 or t.shape[2] != 3:
                    raise ValueError("bump texture must be (H, W, 3) uint8")
                keep.append(t)
                m.bump = t.ctypes.data_as(C.POINTER(C.c_uint8))
                m.bump_height, m.bump_width = t.shape[0], t.shape[1]
        return m


@dataclass
class Entity:
    type: int
    material: int
    normal_inverse: int = 1
    mesh: int = -1
    p: Sequence[float] = (0.0, 0.0, 0.0)
    radius: float = 0.0
    u: Sequence[float] = (0.0, 0.0, 0.0)
    v: Sequence[float] = (0.0, 0.0, 0.0)
    normal: Sequence[float] = (0.0, 0.0, 1.0)
    radius_inner: float = 0.0
    blackhole_disk: int = 0
    # light kinds (light.h:13-74): parallel / spot flags, the direction as
    # the C ABI takes it (parallel_light_dir / spot_light_dir normalised the
    # way the reference's parser does; an infinity light's as given), the
    # spot cone in degrees, falloff exponent and distance attenuation (the
    # parser's defaults).  light_dir_text keeps the unnormalised direction a
    # scene file gives, for the file writer.
    parallel_light: int = 0
    spot_light: int = 0
    light_dir: Sequence[float] = (0.0, 0.0, 0.0)
    spot_angle: Sequence[float] = (0.0, 0.0)
    spot_falloff: float = 0.0
    spot_attenuation: Sequence[float] = (0.0, 0.0, 1.0)
    light_dir_text: Optional[Sequence[float]] = field(default=None, compare=False, repr=False)
    hemisphere: int = 0
    smooth: int = 0  # meshes: 'smooth 1', normals interpolated from the vertex normals

    def to_c(self) -> A.pr_entity:
        e = A.pr_entity()
        e.type, e.material, e.normal_inverse, e.mesh = self.type, self.material, self.normal_inverse, self.mesh
        e.p[:] = [float(x) for x in self.p]
        e.radius = float(self.radius)
        e.u[:] = [float(x) for x in self.u]
        e.v[:] = [float(x) for x in self.v]
        e.normal[:] = [float(x) for x in self.normal]
        e.radius_inner = float(self.radius_inner)
        e.blackhole_disk = int(self.blackhole_disk)
        e.parallel_light = int(self.parallel_light)
        e.spot_light = int(self.spot_light)
        e.hemisphere = int(self.hemisphere)
        e.light_dir[:] = [float(x) for x in self.light_dir]
        e.spot_angle[:] = [float(x) for x in self.spot_angle]
        e.spot_falloff = float(self.spot_falloff)
        e.spot_attenuation[:] = [float(x) for x in self.spot_attenuation]
        e.smooth = int(self.smooth)
        return e


def _normalize_ref(v):
    """normalize (vector3d.h:162-165): v * (1 / length), the squared length
    summed as (x x + z z) + y y (Vector3d::sqr's SSE2 pairing,
    vector3d.h:99-117), so that the result is the reference parser's double"""
    inv = 1.0 / math.sqrt((v[0] * v[0] + v[2] * v[2]) + v[1] * v[1])
    return [v[0] * inv, v[1] * inv, v[2] * inv]


@dataclass
class ObjMaterial:
    """An OBJ material (newmtl, ObjLoader.cpp:704-900) with the loader's
    defaults; texture is the map_Kd image ((H, W, 3) uint8, cell(y, x) rows)."""
    diffuse: Sequence[float] = (0.0, 0.0, 0.0)
    alpha: float = -1.0
    specular: Sequence[float] = (0.0, 0.0, 0.0)
    emission: Sequence[float] = (0.0, 0.0, 0.0)
    refraction_index: float = 0.0
    shininess: float = 5.0
    roughness: float = 0.0
    ward: Sequence[float] = (0.0, 0.0)
    reflection: int = -1
    smooth: int = 0
    repeat: int = 1
    texture: Optional[np.ndarray] = field(default=None, compare=False, repr=False)
    name: str = ""

    def to_c(self, keep: list) -> A.pr_obj_material:
        # ObjMaterial keeps floats (the MTL reader's sscanf %f)
        def f32(x):
            return float(np.float32(x))
        o = A.pr_obj_material()
        o.diffuse[:] = [f32(x) for x in self.diffuse]
        o.alpha = f32(self.alpha)
        o.specular[:] = [f32(x) for x in self.specular]
        o.emission[:] = [f32(x) for x in self.emission]
        o.refraction_index, o.shininess, o.roughness = f32(self.refraction_index), f32(self.shininess), f32(self.roughness)
        o.ward[:] = [f32(x) for x in self.ward]
        o.reflection, o.smooth, o.repeat = int(self.reflection), int(self.smooth), int(self.repeat)
        if self.texture is not None:
            t = np.ascontiguousarray(self.texture, dtype=np.uint8)
            keep.append(t)
            o.texture = t.ctypes.data
            o.texture_height, o.texture_width = t.shape[0], t.shape[1]
        return o


@dataclass
class Mesh:
    vertices: np.ndarray  # (n, 3) float32
    faces: np.ndarray     # (m, 3) int32, 0-based
    # (m, 3) float32 shading normals per face, or None for the OBJ loader's
    # rule from the vertices (an OBJ file with vertex normals, or a mesh
    # moved by rotation / scale, carries its own)
    face_normals: Optional[np.ndarray] = None
    # vn lines (k, 3) float32 with their ids per face (m, 3); None: a smooth
    # entity derives them with the loader's rule from the vertices.  Given
    # vertex normals also decide the face normals (the normalised mean of a
    # face's three, ObjLoader.cpp:617-641) unless face_normals is given.
    vertex_normals: Optional[np.ndarray] = None
    face_vn: Optional[np.ndarray] = None
    # vt lines (k, 2) float32 with their ids per face (m, 3): where textures
    # and IBL images land on the mesh
    uv: Optional[np.ndarray] = None
    face_uv: Optional[np.ndarray] = None
    # OBJ materials (mtllib) and each face's (usemtl; -1 none)
    obj_materials: Optional[list] = None
    face_material: Optional[np.ndarray] = None

    def __post_init__(self):
        self.vertices = np.ascontiguousarray(self.vertices, dtype=np.float32)
        self.faces = np.ascontiguousarray(self.faces, dtype=np.int32)
        if self.face_normals is not None:
            self.face_normals = np.ascontiguousarray(self.face_normals, dtype=np.float32).reshape(-1, 3)
            if self.face_normals.shape[0] != self.faces.shape[0]:
                raise ValueError("face_normals needs one normal per face")
        for arr, ids, k, what in (("vertex_normals", "face_vn", 3, "vertex normals"), ("uv", "face_uv", 2, "uv")):
            a, i = getattr(self, arr), getattr(self, ids)
            if (a is None) != (i is None):
                raise ValueError(f"{what} need both the values and their face ids")
            if a is not None:
                setattr(self, arr, np.ascontiguousarray(a, dtype=np.float32).reshape(-1, k))
                setattr(self, ids, np.ascontiguousarray(i, dtype=np.int32).reshape(-1, 3))
                if getattr(self, ids).shape[0] != self.faces.shape[0]:
                    raise ValueError(f"{what}: one id triple per face")
        if (self.obj_materials is None) != (self.face_material is None):
            raise ValueError("OBJ materials need both the materials and each face's index")
        if self.face_material is not None:
            self.face_material = np.ascontiguousarray(self.face_material, dtype=np.int32).reshape(-1)
            if self.face_material.shape[0] != self.faces.shape[0]:
                raise ValueError("face_material: one index per face")


@dataclass
class Camera:
    """SceneEnv camera fields (scene_env.h:170-178) with the reference defaults."""
    position: Sequence[float] = (50.0, 52.0, 220.0)
    dir: Sequence[float] = (0.0, -0.04, -1.0)
    up: Sequence[float] = (0.0, 1.0, 0.0)
    screen: Sequence[float] = (30.0, 30.0, 40.0)  # SCREEN w h dist
    angle: Optional[float] = None                 # CAMERA_ANGLE (degrees)
    width: int = 320
    height: int = 240

    def to_c(self) -> A.pr_camera:
        c = A.pr_camera()
        c.position[:] = [float(x) for x in self.position]
        d = np.asarray(self.dir, dtype=np.float64)
        # SceneEnv::Load normalises camera_dir at the end (scene_env.h:1920)
        ln = math.sqrt((d[0] * d[0] + d[2] * d[2]) + d[1] * d[1])
        c.dir[:] = [float(x * (1.0 / ln)) for x in d]
        c.up[:] = [float(x) for x in self.up]
        w, h, dist = (float(x) for x in self.screen)
        if self.angle is not None:  # scene_env.h:1881-1886
            w = 2.0 * dist * math.tan(self.angle * (math.pi / 180.0) / 2.0)
            h = w
        c.screen_width, c.screen_height, c.screen_dist = w, h, dist
        c.width, c.height = int(self.width), int(self.height)
        return c


@dataclass
class RenderSettings:
    """Render::Run inputs (render.h:1125-1200) with the reference defaults
    (scene_env.h:262-350; luminance_cutoff 0.025, scene_env.h:221)."""
    samples: int = 8
    supersamples: int = 2
    tent_filter: int = 0
    depth: int = 8
    depth_limit: int = 64
    nee: int = 0
    media: int = 0
    mode: int = A.PR_MODE_MEGAKERNEL
    seed: int = 0
    luminance_cutoff: float = 0.025
    sensor_response: float = 1.0
    max_path_vertices: int = 0
    flags: int = 0
    total_spp: int = 0
    # PR_MODE_MLT (metropolisTransport): mutations and seed paths per pixel
    # and chain (the reference's 'mutation' and 'pre_sample'), GPU chains
    mutation: float = 2.0
    pre_sample: float = 0.4
    mlt_chains: int = 0

    def to_c(self) -> A.pr_render_params:
        p = A.pr_render_params()
        for k in ("samples", "supersamples", "tent_filter", "depth", "depth_limit", "nee", "media", "mode",
                  "max_path_vertices", "flags", "total_spp"):
            setattr(p, k, int(getattr(self, k)))
        p.seed = int(self.seed)
        p.luminance_cutoff = float(self.luminance_cutoff)
        p.sensor_response = float(self.sensor_response)
        p.mlt_mutation = float(self.mutation)
        p.mlt_pre_sample = float(self.pre_sample)
        p.mlt_chains = int(self.mlt_chains)
        return p

    @property
    def spp(self) -> int:
        return self.samples * self.supersamples * self.supersamples


class SceneDesc:
    """Holds a pr_scene_desc and every buffer it points to."""

    def __init__(self, scene: "Scene"):
        self._tex = []
        self._mats = (A.pr_material * max(1, len(scene.materials)))(*[m.to_c(self._tex) for m in scene.materials])
        self._ents = (A.pr_entity * max(1, len(scene.entities)))(*[e.to_c() for e in scene.entities])
        self._mesh_arrays = []
        meshes = []
        for m in scene.meshes:
            v = np.ascontiguousarray(m.vertices, dtype=np.float32)
            f = np.ascontiguousarray(m.faces, dtype=np.int32)
            self._mesh_arrays += [v, f]
            pm = A.pr_mesh()
            pm.n_vertices, pm.n_faces = v.shape[0], f.shape[0]
            pm.vertices = v.ctypes.data_as(C.POINTER(C.c_float))
            pm.faces = f.ctypes.data_as(C.POINTER(C.c_int32))
            pm.face_normals = None
            if m.face_normals is not None:
                fn = np.ascontiguousarray(m.face_normals, dtype=np.float32)
                self._mesh_arrays.append(fn)
                pm.face_normals = fn.ctypes.data_as(C.POINTER(C.c_float))
            if m.vertex_normals is not None:
                vn, fv = m.vertex_normals, m.face_vn
                self._mesh_arrays += [vn, fv]
                pm.n_vertex_normals = vn.shape[0]
                pm.vertex_normals = vn.ctypes.data_as(C.POINTER(C.c_float))
                pm.face_vn = fv.ctypes.data_as(C.POINTER(C.c_int32))
            if m.uv is not None:
                uv, fu = m.uv, m.face_uv
                self._mesh_arrays += [uv, fu]
                pm.n_uv = uv.shape[0]
                pm.uv = uv.ctypes.data_as(C.POINTER(C.c_float))
                pm.face_uv = fu.ctypes.data_as(C.POINTER(C.c_int32))
            if m.obj_materials is not None:
                om = (A.pr_obj_material * max(1, len(m.obj_materials)))(*[o.to_c(self._tex) for o in m.obj_materials])
                fm = m.face_material
                self._mesh_arrays += [om, fm]
                pm.n_obj_materials = len(m.obj_materials)
                pm.obj_materials = C.cast(om, C.POINTER(A.pr_obj_material))
                pm.face_obj_material = fm.ctypes.data_as(C.POINTER(C.c_int32))
            meshes.append(pm)
        self._meshes = (A.pr_mesh * max(1, len(meshes)))(*meshes)
        d = A.pr_scene_desc()
        d.n_materials, d.n_entities, d.n_meshes = len(scene.materials), len(scene.entities), len(scene.meshes)
        d.participating_media = int(scene.participating_media)
        d.materials = C.cast(self._mats, C.POINTER(A.pr_material))
        d.entities = C.cast(self._ents, C.POINTER(A.pr_entity))
        d.meshes = C.cast(self._meshes, C.POINTER(A.pr_mesh))
        d.background[:] = [float(x) for x in scene.background]
        d.environment_light[:] = [float(x) for x in scene.environment_light]
        d.medium = scene.medium.to_c()
        k = A.pr_kerr()
        k.texture_coef = 1.0
        self._keep = []
        if scene.kerr is not None:
            k.enabled = 1
            k.max_steps = int(scene.kerr["max_steps"])
            k.position[:] = [float(x) for x in scene.kerr["position"]]
            k.a = float(scene.kerr["a"])
            k.map_coef[:] = [float(x) for x in scene.kerr.get("map_coef", (1.0, 0.0, 1.0, 0.0))]
            k.escape_radius = float(scene.kerr.get("escape_radius", 0.0))
            k.texture_coef = float(scene.kerr.get("texture_coef", 1.0))
            k.precision = int(scene.kerr.get("precision", A.PR_KERR_FP64))
            tex = scene.kerr.get("texture")
            if tex is not None:
                tex = np.ascontiguousarray(tex, dtype=np.uint8)
                if tex.ndim != 3 or tex.shape[2] != 3:
                    raise ValueError("background texture must be (H, W, 3) uint8")
                self._keep.append(tex)
                k.texture = tex.ctypes.data
                k.texture_height, k.texture_width = tex.shape[0], tex.shape[1]
            k.use_accretion_disk_temperature = int(bool(scene.kerr.get("disk_temperature", False)))
            k.color_doppler_factor_effect = float(scene.kerr.get("doppler_effect", 0.0))
            obs = scene.kerr.get("observer")
            k.observer[:] = [float(x) for x in (scene.camera.position if obs is None else obs)]
            k.disk_seed = int(scene.kerr.get("disk_seed", 1)) & 0xFFFFFFFF
            dt = scene.kerr.get("disk_texture")
            if dt is not None:
                dt = _rgba(dt)
                self._keep.append(dt)
                k.disk_texture = dt.ctypes.data
                k.disk_texture_height, k.disk_texture_width = dt.shape[0], dt.shape[1]
        d.kerr = k
        wm = A.pr_wormhole()
        if scene.wormhole is not None:
            w = scene.wormhole
            wm.enabled = 1
            wm.max_steps = int(w["max_steps"])
            wm.in_[:] = list(w["in"])
            wm.out[:] = list(w["out"])
            wm.rho, wm.a, wm.w = w["rho"], w["a"], w["w"]
            wm.sign = int(w["sign"])
            cam_pos = w.get("camera") or scene.camera.position
            wm.camera[:] = [float(x) for x in cam_pos]
            for k2 in range(2):
                tex = w["textures"][k2]
                if tex is not None:
                    tex = np.ascontiguousarray(tex, dtype=np.uint8)
                    if tex.ndim != 3 or tex.shape[2] != 3:
                        raise ValueError("wormhole background must be (H, W, 3) uint8")
                    self._keep.append(tex)
                    wm.texture[k2] = tex.ctypes.data
                    wm.texture_height[k2], wm.texture_width[k2] = tex.shape[0], tex.shape[1]
                for q in range(4):
                    wm.map_coef[k2][q] = w["map_coef"][k2][q]
                wm.texture_coef[k2] = w["texture_coef"][k2]
        d.wormhole = wm
        self.desc = d

    def ptr(self):
        return C.byref(self.desc)


@dataclass
class Scene:
    materials: List[Material] = field(default_factory=list)
    entities: List[Entity] = field(default_factory=list)
    meshes: List[Mesh] = field(default_factory=list)
    background: Sequence[float] = (0.0, 0.0, 0.0)
    environment_light: Sequence[float] = (0.0, 0.0, 0.0)
    participating_media: int = 0
    medium: Medium = field(default_factory=Medium)
    kerr: Optional[dict] = None
    wormhole: Optional[dict] = None
    camera: Camera = field(default_factory=Camera)
    settings: RenderSettings = field(default_factory=RenderSettings)

    # ---- building (one OBJECT block each) ----
    def _mat(self, m: Material) -> int:
        self.materials.append(m)
        return len(self.materials) - 1

    def add_sphere(self, center, radius, material: Material, normal_inverse: int = 1) -> int:
        self.entities.append(Entity(A.PR_ENT_SPHERE, self._mat(material), normal_inverse, p=tuple(center),
                                    radius=float(radius)))
        return len(self.entities) - 1

    def add_hemisphere(self, center, radius, material: Material, normal_inverse: int = 1) -> int:
        """'hemisphere x y z r': the half of the sphere with y >= y_centre
        (sphere.h:98-103), e.g. a sky dome with an IBL image"""
        i = self.add_sphere(center, radius, material, normal_inverse)
        self.entities[i].hemisphere = 1
        return i

    def add_uvplane(self, org, U, V, material: Material, normal_inverse: int = 1) -> int:
        self.entities.append(Entity(A.PR_ENT_UVPLANE, self._mat(material), normal_inverse, p=tuple(org),
                                    u=tuple(U), v=tuple(V)))
        return len(self.entities) - 1

    def add_disk(self, center, normal, radius, material: Material, radius_inner: float = 0.0,
                 normal_inverse: int = 1) -> int:
        """An annulus ('disk2 x y z r r_inner' + 'normal nx ny nz'; circle.h)."""
        self.entities.append(Entity(A.PR_ENT_CIRCLE, self._mat(material), normal_inverse, p=tuple(center),
                                    radius=float(radius), normal=tuple(normal), radius_inner=float(radius_inner)))
        return len(self.entities) - 1

    def set_black_hole(self, position, a: float, max_steps: int = 10000,
                       map_coef=(1.0, 0.0, 1.0, 0.0), escape_radius: float = 0.0,
                       texture=None, texture_coef: float = 1.0, precision: int = A.PR_KERR_FP64,
                       disk_texture=None, disk_temperature: bool = False, doppler_effect: float = 0.0,
                       observer=None, disk_seed: int = 1) -> None:
        """A Kerr black hole of mass 1 ('BLACKHOLE x y z' block, scene_env.h:701-766);
        texture is the background map as an (H, W, 3) uint8 array indexed
        [y, x] the way the reference's Bitmap::cell(y, x) reads its image.

        disk_texture ((H, W, 3) or (H, W, 4) uint8, same indexing) is
        accretion_disk_texture 0: disks whose material has disk_map set are
        shaded from it with the ISCO cut, the Doppler shift of the disk's
        orbital motion seen from observer (default: the camera position) and
        the texture's alpha test (circle.h:240-335).  disk_temperature and
        doppler_effect are use_accretion_disk_temperature and
        color_doppler_factor_effect; disk_seed seeds the alpha-test stream."""
        self.kerr = {"position": tuple(float(x) for x in position), "a": float(a), "max_steps": int(max_steps),
                     "map_coef": tuple(float(x) for x in map_coef), "escape_radius": float(escape_radius),
                     "texture": texture, "texture_coef": float(texture_coef), "precision": int(precision),
                     "disk_texture": disk_texture, "disk_temperature": bool(disk_temperature),
                     "doppler_effect": float(doppler_effect),
                     "observer": None if observer is None else tuple(float(x) for x in observer),
                     "disk_seed": int(disk_seed)}

    def add_infinity_light(self, direction, emission) -> int:
        """'infinity_light x y z' (scene_env.h:891-894, :1525-1541): light from
        infinitely far along direction (as given; its length scales the
        light the way the reference's unnormalised vector does)"""
        self.entities.append(Entity(A.PR_ENT_INF_LIGHT, self._mat(Material.diffuse((0.0, 0.0, 0.0), emission)),
                                    light_dir=tuple(float(x) for x in direction)))
        return len(self.entities) - 1

    def add_spot_light(self, center, radius, emission, direction, angle, falloff: float = 0.0,
                       attenuation=(0.0, 0.0, 1.0)) -> int:
        """A spot light: an emitting sphere with 'spot_light 1',
        spot_light_dir, spot_light_angle (cone, falloff widths in degrees),
        spot_light_falloff and spot_attenuation (scene_env.h:1223-1252)"""
        i = self.add_sphere(center, radius, Material.diffuse((0.0, 0.0, 0.0), emission))
        e = self.entities[i]
        e.spot_light = 1
        e.light_dir_text = tuple(float(x) for x in direction)
        e.light_dir = tuple(_normalize_ref(e.light_dir_text))
        e.spot_angle = tuple(float(x) for x in angle)
        e.spot_falloff = float(falloff)
        e.spot_attenuation = tuple(float(x) for x in attenuation)
        return i

    def make_parallel_light(self, index: int, direction=None) -> None:
        """'parallel_light 1' (+ parallel_light_dir) on emitting entity index:
        its light arrives along -direction (a uvplane without one takes its
        own normal, scene_env.h:1572-1578)"""
        e = self.entities[index]
        e.parallel_light = 1
        if direction is not None:
            e.light_dir_text = tuple(float(x) for x in direction)
            e.light_dir = tuple(_normalize_ref(e.light_dir_text))

    def set_wormhole(self, in_pos, out_pos=(0.0, 0.0, 0.0), rho: float = 1.3, a: float = 0.5, w: float = 0.05,
                     max_steps: int = 10000, sign: int = 0, textures=(None, None),
                     map_coef=((1.0, 0.0, 1.0, 0.0), (1.0, 0.0, 1.0, 0.0)), texture_coef=(1.0, 1.0),
                     camera=None) -> None:
        """A wormhole ('WORMHOLE' block, scene_env.h:767-856): mouths in / out,
        throat radius rho, length 2a, lensing width w; textures are the two
        backgrounds as (H, W, 3) uint8 arrays indexed [y, x] as
        BitMap::cell(y, x) reads them; camera: the camera position its frame
        is built from (default: the scene camera's)"""
        self.wormhole = {"in": tuple(float(x) for x in in_pos), "out": tuple(float(x) for x in out_pos),
                         "rho": float(rho), "a": float(a), "w": float(w), "max_steps": int(max_steps),
                         "sign": int(sign), "textures": tuple(textures),
                         "map_coef": tuple(tuple(float(x) for x in m) for m in map_coef),
                         "texture_coef": tuple(float(x) for x in texture_coef),
                         "camera": None if camera is None else tuple(float(x) for x in camera)}

    def add_mesh(self, vertices, faces, material: Material, normal_inverse: int = 1, smooth: int = 0,
                 vertex_normals=None, face_vn=None, uv=None, face_uv=None) -> int:
        self.meshes.append(Mesh(vertices, faces, vertex_normals=vertex_normals, face_vn=face_vn, uv=uv,
                                face_uv=face_uv))
        self.entities.append(Entity(A.PR_ENT_POLYGON, self._mat(material), normal_inverse,
                                    mesh=len(self.meshes) - 1, smooth=int(smooth)))
        return len(self.entities) - 1

    def to_desc(self) -> SceneDesc:
        return SceneDesc(self)

    # ---- reference text format ----
    def write_reference(self, directory: str, name: str = "scene.txt", threads: int = 1) -> str:
        """Writes the scene in the reference's text format (scene_env.h
        keywords) plus one OBJ per mesh; returns the scene file path."""
        os.makedirs(directory, exist_ok=True)
        cam, st = self.camera, self.settings

        def f3(v):
            return " ".join(_fmt(x) for x in v)

        out = [
            "IMAGE", f"{cam.width} {cam.height}", "",
            "THREAD", str(threads), "",
            "OUTPUT", "out.bmp", "",
            "SCREEN", f3(cam.screen), "",
            "SAMPLING", str(st.samples), "",
            "SUPERSAMPLING", str(st.supersamples), "",
            "tentfilter", str(st.tent_filter), "",
            "DEPTH", str(st.depth), "",
            "DEPTH_LIMIT", str(st.depth_limit), "",
            "luminance_cutoff", _fmt(st.luminance_cutoff), "",
            "sensor_response", _fmt(st.sensor_response), "",
            "nextEventEstimation", str(st.nee), "",
            "metropolisTransport", str(1 if st.mode == A.PR_MODE_MLT else 0), "",
            "mutation", _fmt(st.mutation), "",
            "pre_sample", _fmt(st.pre_sample), "",
            "IMAGEDUMP", "1000000", "",
            "participatingMedia", str(int(self.participating_media and st.media)), "",
            "CAMERA_POS", f3(cam.position), "",
            "CAMERA_DIR", f3(cam.dir), "",
            "CAMERA_UPVEC", f3(cam.up), "",
            "BACKGROUND", f3(self.background), "",
            "ENVLIGHT", f3(self.environment_light), "",
        ]
        if cam.angle is not None:
            out += ["CAMERA_ANGLE", _fmt(cam.angle), ""]
        if self.kerr is not None:
            k = self.kerr
            if k.get("escape_radius", 0.0) or k.get("precision", A.PR_KERR_FP64) != A.PR_KERR_FP64:
                raise ValueError("escape_radius and the FP32 integrator have no reference counterpart")
            out += [f"BLACKHOLE {f3(k['position'])}",
                    f"geodesics_max_length {int(k['max_steps'])}",
                    f"angular_momentum {_fmt(k['a'])}",
                    "initial_condition 0",
                    f"map_coef {f3(k.get('map_coef', (1.0, 0.0, 1.0, 0.0)))}"]
            if k.get("texture") is not None:
                tex_path = os.path.join(directory, "background.bmp")
                _write_bmp24(tex_path, np.asarray(k["texture"], dtype=np.uint8))
                out += [f"background_texture {tex_path}", f"coef {_fmt(k.get('texture_coef', 1.0))}"]
            if k.get("disk_texture") is not None:
                dt = _rgba(k["disk_texture"])
                if (dt[:, :, 3] != 255).any():
                    raise ValueError("the 24-bit BMP writer carries no alpha; give an opaque disk texture")
                disk_path = os.path.join(directory, "disk.bmp")
                _write_bmp24(disk_path, np.ascontiguousarray(dt[:, :, :3]))
                out.append(f"accretion_disk_texture {disk_path}")
            out.append("")
            obs = k.get("observer")
            if obs is not None and tuple(float(x) for x in obs) != tuple(float(x) for x in cam.position):
                raise ValueError("the reference takes the disk's observer from CAMERA_POS")
            if k.get("disk_temperature"):
                out += ["use_accretion_disk_temperature", "1", ""]
            if k.get("doppler_effect", 0.0):
                out += ["color_doppler_factor_effect", _fmt(k["doppler_effect"]), ""]
        if self.wormhole is not None:
            w = self.wormhole
            if w.get("camera") is not None and tuple(w["camera"]) != tuple(float(x) for x in cam.position):
                raise ValueError("the reference builds the wormhole's frame from CAMERA_POS")
            out += ["WORMHOLE", f"in {f3(w['in'])}", f"out {f3(w['out'])}", f"Rho {_fmt(w['rho'])}",
                    f"a {_fmt(w['a'])}", f"W {_fmt(w['w'])}", f"sign {int(w['sign'])}",
                    f"geodesics_max_length {int(w['max_steps'])}"]
            for k2 in range(2):
                if w["textures"][k2] is not None:
                    tp = os.path.join(directory, f"worm_bg{k2 + 1}.bmp")
                    _write_bmp24(tp, np.asarray(w["textures"][k2], dtype=np.uint8))
                    out.append(f"background_texture{k2 + 1} {tp}")
                out.append(f"map_coef{k2 + 1} {f3(w['map_coef'][k2])}")
                out.append(f"coef{k2 + 1} {_fmt(w['texture_coef'][k2])}")
            out.append("")
        md = self.medium
        out += ["SCATTERING", "0", f3(md.sigma_s_rgb), "",
                "ABSORBING", "0", f3(md.sigma_a_rgb), "",
                f"PAHASE {f3(md.phase_g)}", ""]
        refl = {A.PR_MAT_DIFFUSE: "reflection diffuse", A.PR_MAT_SPECULAR: "reflection specular",
                A.PR_MAT_REFRACTION: "reflection reflection", A.PR_MAT_WARD: "reflection ward_brdf",
                A.PR_MAT_PHONG: "reflection phong_brdf",
                A.PR_MAT_SSS_REFRACTION: "reflection reflection\nreflection Subsurface_Scattering"}
        for ei, e in enumerate(self.entities):
            m = self.materials[e.material]
            out.append("OBJECT")
            if e.type == A.PR_ENT_SPHERE:
                out.append(f"{'hemisphere' if e.hemisphere else 'sphere'} {f3(e.p)} {_fmt(e.radius)}")
            elif e.type == A.PR_ENT_UVPLANE:
                out += [f"uvplane {f3(e.p)}", f"U {f3(e.u)}", f"V {f3(e.v)}"]
            elif e.type == A.PR_ENT_CIRCLE:
                out += [f"disk2 {f3(e.p)} {_fmt(e.radius)} {_fmt(e.radius_inner)}", f"normal {f3(e.normal)}"]
                # the keyword sets a scene-wide value every later disk inherits (scene_env.h:1177-1181)
                out.append(f"blackhole_disk {int(e.blackhole_disk)}")
            elif e.type == A.PR_ENT_INF_LIGHT:
                out.append(f"infinity_light {f3(e.light_dir)}")
            elif e.type == A.PR_ENT_POLYGON:
                if self.meshes[e.mesh].face_normals is not None:
                    raise ValueError("a mesh with its own face normals has no reference writer")
                objname = f"mesh{e.mesh}.obj"
                _write_obj(os.path.join(directory, objname), self.meshes[e.mesh])
                out.append(f"objfile {os.path.join(directory, objname)}")
                if e.smooth:
                    out.append(f"smooth {int(e.smooth)}")
            else:
                raise ValueError("entity type has no reference writer")
            if m.type in (A.PR_MAT_REFRACTION, A.PR_MAT_SSS_REFRACTION) and m.refractive_index != 1.5:
                out.append(f"refractive_index {_fmt(m.refractive_index)}")
            if m.type == A.PR_MAT_SSS_REFRACTION:
                md = m.medium
                if len(set(float(x) for x in md.phase_g)) != 1:
                    raise ValueError("the reference's 'PAHASE x y z' keeps x for y; give one g")
                mean_s = sum(float(x) for x in md.sigma_s_rgb) / 3.0
                mean_a = sum(float(x) for x in md.sigma_a_rgb) / 3.0
                out += ["SCATTERING", _fmt(round(mean_s, 12)), f3(md.sigma_s_rgb),
                        "ABSORBING", _fmt(round(mean_a, 12)), f3(md.sigma_a_rgb),
                        "PAHASE", _fmt(md.phase_g[0]),
                        "level", str(int(md.level)),
                        "MATERIAL_R_MAX", _fmt(md.r_max),
                        f"r_refractive_index {_fmt(m.r_refractive_index)}"]
                if float(md.scale) != 1.0:
                    out += ["MATERIAL_SCALE", _fmt(md.scale)]
            out += [f"emission {f3(m.emission)}", f"color {f3(m.color)}"]
            if m.type in (A.PR_MAT_WARD, A.PR_MAT_PHONG):
                out.append(f"specular {f3(m.specular)}")
                if m.type == A.PR_MAT_WARD:
                    out.append(f"ward_brdf 1 1 {_fmt(m.ward_alpha[0])} {_fmt(m.ward_alpha[1])}")
                else:
                    out.append(f"phong_brdf 1 1 {_fmt(m.phong_exponent)}")
            if m.disk_map:
                out.append(f"disk_map {int(m.disk_map)}")
            if m.texture is not None:
                tp = os.path.join(directory, f"tex{ei}.bmp")
                _write_bmp24(tp, np.asarray(m.texture, dtype=np.uint8))
                out.append(f"texture {tp}")
            if m.ibl is not None:
                if m.ibl.dtype == np.uint8:
                    ip = os.path.join(directory, f"ibl{ei}.bmp")
                    _write_bmp24(ip, np.asarray(m.ibl))
                else:
                    ip = os.path.join(directory, f"ibl{ei}.hdr")
                    write_hdr(ip, hdr_rgbe(np.asarray(m.ibl, dtype=np.float32))[::-1])
                out.append(f"ibl_texture {ip}")
                if float(m.ibl_coef) != 1.0:
                    out.append(f"ibl_texture_coef {_fmt(m.ibl_coef)}")
            if m.bump is not None:
                bp = os.path.join(directory, f"bump{ei}.bmp")
                _write_bmp24(bp, np.asarray(m.bump, dtype=np.uint8))
                out.append(f"bump_texture {bp}")
            if int(m.repeat) != 1:
                out.append(f"repeat {int(m.repeat)}")
            for bit, key in ((A.PR_MAP_HEMISPHERE, "hemisphere_map"), (A.PR_MAP_ANGULAR, "angular_map"),
                             (A.PR_MAP_PANORAMIC, "panoramic_map"), (A.PR_MAP_EQUIRECTANGULAR, "equirectangular_map")):
                if int(m.map_flags) & bit:
                    out.append(f"{key} 1")
            ldir = e.light_dir_text if e.light_dir_text is not None else e.light_dir
            if e.parallel_light:
                out.append("parallel_light 1")
                if any(float(x) for x in ldir):
                    out.append(f"parallel_light_dir {f3(ldir)}")
            if e.spot_light:
                out += ["spot_light 1", f"spot_light_dir {f3(ldir)}",
                        f"spot_light_angle {_fmt(e.spot_angle[0])} {_fmt(e.spot_angle[1])}",
                        f"spot_light_falloff {_fmt(e.spot_falloff)}",
                        f"spot_attenuation {f3(e.spot_attenuation)}"]
            if e.normal_inverse < 0:
                out.append("normal -1")
            if m.type in refl:
                # 'reflection diffuse' forces roughness 1 and 'specular' 0; an
                # explicit roughness line written after keeps other values
                out.append(refl[m.type])
                default_r = {A.PR_MAT_DIFFUSE: 1.0, A.PR_MAT_SPECULAR: 0.0, A.PR_MAT_PHONG: 0.0,
                             A.PR_MAT_WARD: 0.0}.get(m.type)
                if default_r is not None and float(m.roughness) != default_r:
                    out.append(f"roughness {_fmt(m.roughness)}")
            else:
                raise ValueError("material type has no reference writer")
            out.append("")
        path = os.path.join(directory, name)
        with open(path, "w", newline="\n") as fh:
            fh.write("\n".join(out) + "\n")
        return path


def _fmt(x) -> str:
    """Positional decimal that the reference's expression reader (Expr.h:210-280)
    turns into the same double: at most 15 significant digits, so that its
    digit accumulation is exact and the single division correctly rounded."""
    x = float(x)
    s = np.format_float_positional(x, unique=True, trim="-")
    digits = s.lstrip("-").replace(".", "").lstrip("0")
    if len(digits) > 15:
        raise ValueError(f"{x!r} needs more than 15 significant digits in the reference scene format")
    return s


def _rgba(tex) -> np.ndarray:
    """(H, W, 3) or (H, W, 4) uint8 texture as contiguous RGBA (alpha 255
    where none is given, as BitMap::Read sets it for 24-bit images,
    bitmap.cpp:116-123)."""
    t = np.asarray(tex, dtype=np.uint8)
    if t.ndim != 3 or t.shape[2] not in (3, 4):
        raise ValueError("disk texture must be (H, W, 3) or (H, W, 4) uint8")
    if t.shape[2] == 3:
        t = np.concatenate([t, np.full(t.shape[:2] + (1,), 255, np.uint8)], axis=2)
    return np.ascontiguousarray(t)


def hdr_rgbe(img: np.ndarray) -> np.ndarray:
    """RGBE bytes (H, W, 4) that HDRImage::load_unsafe (hdr.h:82-210) reads
    back as exactly these values (byte * 2^(e - 136) per channel); raises
    if a value has no such form (more than 8 significant bits against the
    texel's largest channel)"""
    f = np.asarray(img, dtype=np.float64)
    mx = f.max(axis=2)
    m, e = np.frexp(mx)
    ex = np.where(mx > 0, e + 128, 0).astype(np.int64)
    if (ex < 0).any() or (ex > 255).any():
        raise ValueError("value out of the RGBE exponent range")
    b = np.where(mx[..., None] > 0, f * np.ldexp(1.0, (136 - ex))[..., None], 0.0)
    if (b != np.floor(b)).any() or (b > 255).any():
        raise ValueError("an HDR value that RGBE cannot hold exactly")
    return np.concatenate([b.astype(np.uint8), ex.astype(np.uint8)[..., None]], axis=2)


def rgbe_values(rgbe: np.ndarray) -> np.ndarray:
    """the values HDRImage::load_unsafe gives RGBE bytes: byte *
    pow(2, e - 128) / 256 (hdr.h:203-208; e = 0 included), as float32"""
    q = np.asarray(rgbe, dtype=np.uint8)
    return (q[..., :3].astype(np.float64) * np.ldexp(1.0, q[..., 3:4].astype(np.int64) - 136)).astype(np.float32)


def write_hdr(path: str, rgbe: np.ndarray) -> None:
    """Writes a Radiance .hdr file from (H, W, 4) RGBE bytes in scanline order
    (what Context.to_rgbe returns) as HDRImage::save does (hdr.h:213-246):
    the same header lines, '-Y H +X W', then per scanline the new-style
    marker 2 2 and the width, and each of the four byte planes as literal
    runs of at most 127 bytes."""
    q = np.ascontiguousarray(rgbe, dtype=np.uint8)
    h, w = q.shape[0], q.shape[1]
    out = bytearray()
    out += b"#?RADIANCE\n# Made with 100% pure HDR Shop\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0000000000000\n\n"
    out += f"-Y {h} +X {w}\n".encode()
    for r in range(h):
        out += bytes((2, 2, (w >> 8) & 0xFF, w & 0xFF))
        for c in range(4):
            plane = q[r, :, c].tobytes()
            for k in range(0, w, 127):
                chunk = plane[k:k + 127]
                out.append(len(chunk))
                out += chunk
    with open(path, "wb") as f:
        f.write(bytes(out))


def write_bmp(path: str, rgb8: np.ndarray) -> None:
    """Writes a 24-bit BMP from (H, W, 3) uint8 rows in the bitmap's
    cell(i, j) order (what Context.to_rgb8 returns), as Render::OutputBmp's
    BitMap::Write would."""
    _write_bmp24(path, np.ascontiguousarray(rgb8, dtype=np.uint8))


def _write_bmp24(path: str, tex: np.ndarray) -> None:
    """24-bit BMP whose decoded image, read back through the reference's
    BitMap::cell(y, x) (bitmap.h:187-190: row H-1-y of the top-down decode),
    is tex[y, x]: the file's bottom row is tex[0]."""
    h, w, _ = tex.shape
    row = w * 3
    pad = (4 - row % 4) % 4
    size = 54 + (row + pad) * h
    hdr = bytearray(54)
    hdr[0:2] = b"BM"
    hdr[2:6] = size.to_bytes(4, "little")
    hdr[10:14] = (54).to_bytes(4, "little")
    hdr[14:18] = (40).to_bytes(4, "little")
    hdr[18:22] = w.to_bytes(4, "little")
    hdr[22:26] = h.to_bytes(4, "little")  # positive height: rows stored bottom-up
    hdr[26:28] = (1).to_bytes(2, "little")
    hdr[28:30] = (24).to_bytes(2, "little")
    hdr[34:38] = ((row + pad) * h).to_bytes(4, "little")
    with open(path, "wb") as fh:
        fh.write(bytes(hdr))
        for y in range(h):  # stored bottom row first = tex[0]
            fh.write(tex[y, :, ::-1].tobytes() + b"\0" * pad)


def _write_mtl(path: str, mats, texdir: str) -> None:
    with open(path, "w", newline="\n") as fh:
        for i, o in enumerate(mats):
            fh.write(f"newmtl m{i}\n")
            fh.write("Kd %.9g %.9g %.9g\n" % tuple(float(x) for x in o.diffuse))
            fh.write("Ks %.9g %.9g %.9g\n" % tuple(float(x) for x in o.specular))
            if float(o.alpha) >= 0.0:
                fh.write("d %.9g\n" % float(o.alpha))
            if float(o.shininess) != 5.0:
                fh.write("Ns %.9g\n" % float(o.shininess))
            if o.texture is not None:
                tp = f"mtex{i}.bmp"
                _write_bmp24(os.path.join(texdir, tp), np.asarray(o.texture, dtype=np.uint8))
                fh.write(f"map_Kd {tp}\n")
            if int(o.smooth):
                fh.write(f"#SMOOTH {1 if int(o.smooth) == 1 else 0}\n")
            if int(o.repeat) != 1:
                fh.write(f"#REPEAT {int(o.repeat)}\n")
            if any(float(x) for x in o.emission):
                fh.write("#EMISSION %.9g %.9g %.9g\n" % tuple(float(x) for x in o.emission))
            if any(float(x) for x in o.ward):
                fh.write("#WARD %.9g %.9g\n" % tuple(float(x) for x in o.ward))
            if int(o.reflection) >= 0:
                # Ni before '#REFLECTION 2' keeps an explicit index; the
                # loader then sets 0.0 to 1.5 and '#REFLECTION 0/1' the roughness to 0
                if float(o.refraction_index) != 0.0:
                    fh.write("Ni %.9g\n" % float(o.refraction_index))
                fh.write(f"#REFLECTION {int(o.reflection)}\n")
            elif float(o.refraction_index) != 0.0:
                fh.write("Ni %.9g\n" % float(o.refraction_index))
            if float(o.roughness) != 0.0:
                fh.write("#ROUGHNESS %.9g\n" % float(o.roughness))


def _write_obj(path: str, mesh: Mesh) -> None:
    # %.9g round-trips float32 exactly through sscanf("%f")
    with open(path, "w", newline="\n") as fh:
        if mesh.obj_materials is not None:
            mtl = os.path.splitext(path)[0] + ".mtl"
            _write_mtl(mtl, mesh.obj_materials, os.path.dirname(path))
            fh.write(f"mtllib {os.path.basename(mtl)}\n")
        for v in mesh.vertices:
            fh.write("v %.9g %.9g %.9g\n" % (float(v[0]), float(v[1]), float(v[2])))
        if mesh.vertex_normals is not None:
            for n in mesh.vertex_normals:
                fh.write("vn %.9g %.9g %.9g\n" % (float(n[0]), float(n[1]), float(n[2])))
        if mesh.uv is not None:
            for t in mesh.uv:
                fh.write("vt %.9g %.9g\n" % (float(t[0]), float(t[1])))
        cur_mtl = None
        for q, f in enumerate(mesh.faces):
            if mesh.face_material is not None and int(mesh.face_material[q]) != cur_mtl:
                cur_mtl = int(mesh.face_material[q])
                fh.write(f"usemtl m{cur_mtl}\n" if cur_mtl >= 0 else "usemtl none\n")
            corners = []
            for k in range(3):
                c = "%d" % (int(f[k]) + 1)
                if mesh.uv is not None and mesh.vertex_normals is not None:
                    c += "/%d/%d" % (int(mesh.face_uv[q][k]) + 1, int(mesh.face_vn[q][k]) + 1)
                elif mesh.vertex_normals is not None:
                    c += "//%d" % (int(mesh.face_vn[q][k]) + 1)
                elif mesh.uv is not None:
                    c += "/%d" % (int(mesh.face_uv[q][k]) + 1)
                corners.append(c)
            fh.write("f %s\n" % " ".join(corners))
