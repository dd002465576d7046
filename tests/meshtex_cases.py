"""Meshes with smooth shading and textures (polygon.h:178-528), shared by the
golden-vector generator and the tests.

* 'smooth', 'smooth_nonee': the sphere Cornell box with 'smooth 1' meshes:
  a diffuse icosphere and a glass icosphere whose vertex normals come from
  the loader's rule (no vn lines), and a wavy panel whose own vn lines tilt
  its shading normals (drawn with 'normal -1' and its faces reversed), with
  next-event estimation on and off.
* 'mesh_tex', 'mesh_tex_nonee': textured meshes (vt lines): a smooth
  icosphere with a spherical mapping, a Phong panel (the texel is its
  colour, the specular colour stays), a panel with an IBL bitmap (its hits
  return the texel's emission), and a ball with a bump map (which the
  reference's mesh hit does not keep; without vt lines its lookup reads
  outside the map), NEE on and off.
* 'obj_mtl', 'obj_mtl_nonee': OBJ materials chosen per face (usemtl): Kd
  over a diffuse entity (its Ks dropped), a '#REFLECTION 4' Phong, a map_Kd
  texture with '#REPEAT 2' (the entity colour times the texel), a mirror; on
  a panel a textured Ward with '#EMISSION' (colour, specular and emission
  times the texel), a '#SMOOTH 1' material and a glass one.

Textures are seeded synthetic images."""
import numpy as np

from prender_gb300.scene import Camera, Material, ObjMaterial, RenderSettings, Scene
from prender_gb300.scenes import icosphere

from texture_cases import _walls, bump_map, checker

CASES = ["smooth", "smooth_nonee", "mesh_tex", "mesh_tex_nonee", "obj_mtl", "obj_mtl_nonee"]


def _ball(subdiv, center, radius):
    v, f = icosphere(subdiv)
    return (v * radius + np.asarray(center)).astype(np.float32), f, v


def _wavy_panel(center, size, n, seed):
    """an n x n grid in the xz plane with vertex normals tilted by a seeded
    wave (vn lines of their own, one per vertex)"""
    rng = np.random.default_rng(seed)
    xs = np.linspace(-0.5, 0.5, n + 1) * size
    gx, gz = np.meshgrid(xs, xs, indexing="ij")
    v = np.stack([gx.ravel() + center[0], np.full(gx.size, center[1]), gz.ravel() + center[2]], 1).astype(np.float32)
    ph = rng.uniform(0, 6.28, 2)
    nx = 0.35 * np.sin(gx.ravel() / size * 12.0 + ph[0])
    nz = 0.35 * np.cos(gz.ravel() / size * 9.0 + ph[1])
    vn = np.stack([nx, np.ones_like(nx), nz], 1)
    vn /= np.linalg.norm(vn, axis=1, keepdims=True)
    f = []
    for i in range(n):
        for j in range(n):
            a, b, c, d = i * (n + 1) + j, (i + 1) * (n + 1) + j, (i + 1) * (n + 1) + j + 1, i * (n + 1) + j + 1
            f += [(a, c, b), (a, d, c)]  # facing +y
    uv = np.stack([(gx.ravel() / size + 0.5), (gz.ravel() / size + 0.5)], 1)
    return v, np.array(f, np.int32), vn.astype(np.float32), np.clip(uv, 0.0, 1.0).astype(np.float32)


def _sphere_uv(unit):
    u = np.arctan2(unit[:, 2], unit[:, 0]) / (2 * np.pi) + 0.5
    v = np.arccos(np.clip(unit[:, 1], -1, 1)) / np.pi
    return np.clip(np.stack([u, v], 1), 0.0, 1.0).astype(np.float32)


def build(name: str, width: int, height: int, samples: int, supersamples: int = 2) -> Scene:
    s = Scene()
    _walls(s)
    s.add_sphere((50, 76, 81.6), 5, Material.diffuse((0, 0, 0), (36, 36, 36)))
    nee = 0 if name.endswith("_nonee") else 1
    if name in ("smooth", "smooth_nonee"):
        v, f, _ = _ball(2, (27, 14, 60), 14)
        s.add_mesh(v, f, Material.diffuse((0.7, 0.4, 0.3)), smooth=1)
        v, f, _ = _ball(2, (73, 13, 78), 13)
        s.add_mesh(v, f, Material.glass((0.99, 0.99, 0.99)), smooth=1)
        v, f, vn, _ = _wavy_panel((50, 1.0, 110), 40, 6, 7)
        # faces reversed and drawn with normal -1: the same surface from above
        s.add_mesh(v, f[:, ::-1].copy(), Material.diffuse((0.6, 0.7, 0.75)), normal_inverse=-1, smooth=1,
                   vertex_normals=vn, face_vn=f[:, ::-1].copy())
    elif name in ("mesh_tex", "mesh_tex_nonee"):
        v, f, unit = _ball(2, (27, 14, 60), 14)
        m = Material.diffuse((0.5, 0.5, 0.5))
        m.texture = checker(32, 64, 8, (220, 60, 40), (40, 200, 60), 41)
        s.add_mesh(v, f, m, smooth=1, uv=_sphere_uv(unit), face_uv=f)
        pv, pf, _, puv = _wavy_panel((72, 1.0, 70), 36, 3, 9)
        ph = Material.phong((0.3, 0.3, 0.3), (0.5, 0.5, 0.5), exponent=25.0, roughness=0.4)
        ph.texture = checker(24, 24, 4, (250, 250, 60), (40, 40, 220), 42)
        s.add_mesh(pv, pf, ph, uv=puv, face_uv=pf)
        # an upright IBL panel at the back (x = 20..50, y = 20..50, z = 30;
        # a grid: the reference's QBVH needs more than one leaf)
        iv, iff, _, iuv = _wavy_panel((35, 30, 35), 30, 3, 10)
        iv = np.ascontiguousarray(iv[:, [0, 2, 1]])
        ibl = Material.diffuse((0.0, 0.0, 0.0))
        ibl.ibl = checker(16, 16, 4, (250, 200, 120), (60, 90, 160), 43)
        ibl.ibl_coef = 0.5
        s.add_mesh(iv, iff, ibl, uv=iuv, face_uv=iff)
        bv, bf, bunit = _ball(1, (62, 40, 45), 8)
        bm = Material.diffuse((0.3, 0.5, 0.8))
        bm.bump = bump_map(16, 44)
        s.add_mesh(bv, bf, bm, uv=_sphere_uv(bunit), face_uv=bf)
    elif name in ("obj_mtl", "obj_mtl_nonee"):
        # OBJ materials (usemtl) over a diffuse entity material
        base = Material.diffuse((0.5, 0.5, 0.5))
        mats = [
            ObjMaterial(diffuse=(0.8, 0.3, 0.2), specular=(0.4, 0.4, 0.4)),                # Kd; Ks dropped (diffuse B)
            ObjMaterial(diffuse=(0.2, 0.5, 0.2), specular=(0.5, 0.5, 0.5), shininess=20.0,
                        reflection=4, roughness=0.3),                                      # Phong
            ObjMaterial(texture=checker(16, 32, 4, (250, 220, 60), (40, 60, 220), 61), repeat=2),  # B colour x texel
            ObjMaterial(specular=(0.9, 0.9, 0.9), reflection=1),                           # mirror
        ]
        v, f, unit = _ball(2, (27, 14, 60), 14)
        fm = (np.arange(len(f)) % 5 - 1).astype(np.int32)  # -1, 0, 1, 2, 3 in turn
        s.add_mesh(v, f, base, uv=_sphere_uv(unit), face_uv=f)
        s.meshes[-1].obj_materials, s.meshes[-1].face_material = mats, fm
        pv, pf, pvn, puv = _wavy_panel((66, 1.0, 80), 40, 4, 12)
        pmats = [
            ObjMaterial(diffuse=(0.3, 0.6, 0.8), specular=(0.5, 0.4, 0.3), emission=(0.2, 0.1, 0.0),
                        ward=(0.1, 0.25), reflection=3,
                        texture=checker(16, 16, 4, (240, 240, 240), (90, 90, 90), 62)),   # Ward, texel-scaled
            ObjMaterial(diffuse=(0.7, 0.7, 0.3), smooth=1),                                # '#SMOOTH 1'
            ObjMaterial(refraction_index=1.4, specular=(0.95, 0.95, 0.95), reflection=2),  # glass
        ]
        pfm = (np.arange(len(pf)) % 3).astype(np.int32)
        s.add_mesh(pv, pf, Material.diffuse((0.6, 0.6, 0.6)), vertex_normals=pvn, face_vn=pf, uv=puv, face_uv=pf)
        s.meshes[-1].obj_materials, s.meshes[-1].face_material = pmats, pfm
    else:
        raise KeyError(name)
    s.camera = Camera(position=(50, 52, 220), dir=(0, -0.04, -1), angle=30, width=width, height=height)
    s.settings = RenderSettings(samples=samples, supersamples=supersamples, tent_filter=1, depth=5, nee=nee, seed=0)
    return s


def one_thread_cases():
    """name -> scene for one-thread renders (bit-exact against the reference)"""
    return {k: build(k, 32, 24, 1, 2) for k in CASES}


def highspp_case(name: str):
    """64 x 48, 64 x 2^2 tent-filtered samples (256 spp) per batch"""
    return build(name, 64, 48, 64, 2)
