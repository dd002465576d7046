"""Scene files in the reference's text format, read by the library's native
reader (pr_scene_file_load; SceneEnv::Load, scene_env.h:357-2160).

    scene = scene_file.load("CornellBox.txt")
    ctx.upload(scene)
    img = ctx.render(scene)

The returned Scene holds copies of everything the file named (materials,
entities, OBJ meshes, BMP textures), the resolved camera and the render
settings, so it renders through the same calls as a Scene built in Python.
Features this library does not render make the load fail with the line that
asked for them; lines that do not change the image are listed in
``scene.file_warnings``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi as A
from ._lib import load as _load_lib
from .scene import Camera, Entity, Material, Medium, Mesh, ObjMaterial, RenderSettings, Scene


class SceneFileError(ValueError):
    """The scene file could not be read, or asks for a feature this library
    does not render."""


@dataclass
class ResolvedCamera(Camera):
    """A camera as SceneEnv::Load leaves it: direction already normalised and
    the screen already sized by CAMERA_ANGLE, so ``to_c`` passes the values
    through unchanged."""

    def to_c(self) -> A.pr_camera:
        c = A.pr_camera()
        c.position[:] = [float(x) for x in self.position]
        c.dir[:] = [float(x) for x in self.dir]
        c.up[:] = [float(x) for x in self.up]
        c.screen_width, c.screen_height, c.screen_dist = (float(x) for x in self.screen)
        c.width, c.height = int(self.width), int(self.height)
        return c


def _v(a, n=3):
    return tuple(float(a[i]) for i in range(n))


def _image(ptr, h, w, dtype):
    """a copy of an (h, w, 3) image the reader holds, or None"""
    if not ptr or h <= 0 or w <= 0:
        return None
    return np.ctypeslib.as_array(ptr, shape=(h * w * 3,)).reshape(h, w, 3).astype(dtype, copy=True)


def _medium(m: A.pr_medium) -> Medium:
    return Medium(sigma_s_rgb=_v(m.sigma_s_rgb), sigma_a_rgb=_v(m.sigma_a_rgb), phase_g=_v(m.phase_g),
                  eta=float(m.eta), scale=float(m.scale), r_max=float(m.r_max), level=int(m.level),
                  use_bssrdf=int(m.use_bssrdf))


def _texture(ptr, w: int, h: int, ch: int):
    if not ptr or w <= 0 or h <= 0:
        return None
    buf = (C.c_uint8 * (w * h * ch)).from_address(ptr)
    return np.frombuffer(buf, np.uint8).reshape(h, w, ch).copy()


def load(path: str) -> Scene:
    """Reads a scene file (and the OBJ and BMP files it names) into a Scene."""
    L = _load_lib()
    err = C.create_string_buffer(1024)
    f = L.pr_scene_file_load(str(path).encode(), err, len(err))
    if not f:
        raise SceneFileError(err.value.decode(errors="replace"))
    try:
        d = C.cast(L.pr_scene_file_desc(f), C.POINTER(A.pr_scene_desc)).contents
        cam, prm, gamma = A.pr_camera(), A.pr_render_params(), C.c_double(0.0)
        if L.pr_scene_file_camera(f, C.byref(cam), C.byref(prm), C.byref(gamma)) != 0:
            raise SceneFileError("pr_scene_file_camera failed")
        warnings = L.pr_scene_file_warnings(f).decode(errors="replace")
        s = Scene()
        for i in range(d.n_materials):
            m = d.materials[i]
            s.materials.append(Material(
                type=int(m.type), color=_v(m.color), emission=_v(m.emission), specular=_v(m.specular),
                roughness=float(m.roughness), refractive_index=float(m.refractive_index), medium=_medium(m.medium),
                r_refractive_index=float(m.r_refractive_index), disk_map=int(m.disk_map),
                ward_alpha=_v(m.ward_alpha, 2), phong_exponent=float(m.phong_exponent),
                texture=_image(m.texture, m.texture_height, m.texture_width, np.uint8),
                ibl=(_image(m.ibl_rgb8, m.ibl_height, m.ibl_width, np.uint8) if m.ibl_rgb8
                     else _image(m.ibl_rgbf, m.ibl_height, m.ibl_width, np.float32)),
                ibl_coef=float(m.ibl_coef), repeat=int(m.repeat), map_flags=int(m.map_flags),
                bump=_image(m.bump, m.bump_height, m.bump_width, np.uint8)))
        for i in range(d.n_entities):
            e = d.entities[i]
            s.entities.append(Entity(
                type=int(e.type), material=int(e.material), normal_inverse=int(e.normal_inverse), mesh=int(e.mesh),
                p=_v(e.p), radius=float(e.radius), u=_v(e.u), v=_v(e.v), normal=_v(e.normal),
                radius_inner=float(e.radius_inner), blackhole_disk=int(e.blackhole_disk),
                parallel_light=int(e.parallel_light), spot_light=int(e.spot_light), light_dir=_v(e.light_dir),
                spot_angle=_v(e.spot_angle, 2), spot_falloff=float(e.spot_falloff),
                spot_attenuation=_v(e.spot_attenuation), hemisphere=int(e.hemisphere), smooth=int(e.smooth)))
        for i in range(d.n_meshes):
            pm = d.meshes[i]
            v = np.ctypeslib.as_array(pm.vertices, shape=(pm.n_vertices * 3,)).reshape(-1, 3).copy()
            fc = np.ctypeslib.as_array(pm.faces, shape=(pm.n_faces * 3,)).reshape(-1, 3).copy()
            fn = None
            if pm.face_normals:
                fn = np.ctypeslib.as_array(pm.face_normals, shape=(pm.n_faces * 3,)).reshape(-1, 3).copy()
            vn = fvn = uv = fuv = None
            if pm.vertex_normals and pm.face_vn:
                vn = np.ctypeslib.as_array(pm.vertex_normals, shape=(pm.n_vertex_normals * 3,)).reshape(-1, 3).copy()
                fvn = np.ctypeslib.as_array(pm.face_vn, shape=(pm.n_faces * 3,)).reshape(-1, 3).copy()
            if pm.uv and pm.face_uv:
                uv = np.ctypeslib.as_array(pm.uv, shape=(pm.n_uv * 2,)).reshape(-1, 2).copy()
                fuv = np.ctypeslib.as_array(pm.face_uv, shape=(pm.n_faces * 3,)).reshape(-1, 3).copy()
            oms = fm = None
            if pm.obj_materials and pm.face_obj_material and pm.n_obj_materials > 0:
                oms = []
                for k in range(pm.n_obj_materials):
                    q = pm.obj_materials[k]
                    oms.append(ObjMaterial(diffuse=_v(q.diffuse), alpha=float(q.alpha), specular=_v(q.specular),
                                           emission=_v(q.emission), refraction_index=float(q.refraction_index),
                                           shininess=float(q.shininess), roughness=float(q.roughness),
                                           ward=_v(q.ward, 2), reflection=int(q.reflection), smooth=int(q.smooth),
                                           repeat=int(q.repeat),
                                           texture=_texture(q.texture, q.texture_width, q.texture_height, 3)))
                fm = np.ctypeslib.as_array(pm.face_obj_material, shape=(pm.n_faces,)).copy()
            s.meshes.append(Mesh(v, fc, fn, vertex_normals=vn, face_vn=fvn, uv=uv, face_uv=fuv, obj_materials=oms,
                                 face_material=fm))
        s.background = _v(d.background)
        s.environment_light = _v(d.environment_light)
        s.participating_media = int(d.participating_media)
        s.medium = _medium(d.medium)
        k = d.kerr
        if k.enabled:
            s.kerr = {"position": _v(k.position), "a": float(k.a), "max_steps": int(k.max_steps),
                      "map_coef": _v(k.map_coef, 4), "escape_radius": float(k.escape_radius),
                      "texture": _texture(k.texture, k.texture_width, k.texture_height, 3),
                      "texture_coef": float(k.texture_coef), "precision": int(k.precision),
                      "disk_texture": _texture(k.disk_texture, k.disk_texture_width, k.disk_texture_height, 4),
                      "disk_temperature": bool(k.use_accretion_disk_temperature),
                      "doppler_effect": float(k.color_doppler_factor_effect), "observer": _v(k.observer),
                      "disk_seed": int(k.disk_seed)}
        w = d.wormhole
        if w.enabled:
            s.set_wormhole(_v(w.in_), _v(w.out), rho=float(w.rho), a=float(w.a), w=float(w.w),
                           max_steps=int(w.max_steps), sign=int(w.sign),
                           textures=tuple(_texture(w.texture[k], w.texture_width[k], w.texture_height[k], 3)
                                          for k in range(2)),
                           map_coef=tuple(tuple(float(x) for x in w.map_coef[k]) for k in range(2)),
                           texture_coef=(float(w.texture_coef[0]), float(w.texture_coef[1])),
                           camera=_v(w.camera))
        s.camera = ResolvedCamera(position=_v(cam.position), dir=_v(cam.dir), up=_v(cam.up),
                                  screen=(float(cam.screen_width), float(cam.screen_height), float(cam.screen_dist)),
                                  angle=None, width=int(cam.width), height=int(cam.height))
        s.settings = RenderSettings(samples=prm.samples, supersamples=prm.supersamples, tent_filter=prm.tent_filter,
                                    depth=prm.depth, depth_limit=prm.depth_limit, nee=prm.nee, media=prm.media,
                                    mode=prm.mode, seed=int(prm.seed), luminance_cutoff=float(prm.luminance_cutoff),
                                    sensor_response=float(prm.sensor_response), mutation=float(prm.mlt_mutation),
                                    pre_sample=float(prm.mlt_pre_sample))
        s.gamma_offset = float(gamma.value)
        s.file_warnings = warnings
        return s
    finally:
        L.pr_scene_file_free(f)
