"""Seeded synthetic scenes with the shapes of the benchmark configurations.

No reference meshes or textures ship with prender's test scenes, so every
input here is generated from a seed: the edupt-style sphere Cornell box,
the triangle-mesh Cornell box with a Perlin-displaced icosphere, and the
media / Kerr variants.  Each builder returns a :class:`Scene` that can be
rendered by the GPU library and written in the reference's scene format.
"""
from __future__ import annotations

import math

import numpy as np

from . import _abi as A
from .scene import Camera, Material, Medium, RenderSettings, Scene


def cornell_spheres(width: int = 256, height: int = 192, samples: int = 4, supersamples: int = 2,
                    depth: int = 5, seed: int = 0) -> Scene:
    """Sphere Cornell box: five radius-1e5 walls (proj/test/CornellBox.txt
    minus its black front wall), a diffuse, a mirror and a glass sphere, and
    a radius-5 emissive sphere light inside the box under the ceiling."""
    s = Scene()
    s.add_sphere((100001, 40.8, 81.6), 100000, Material.diffuse((0.75, 0.25, 0.25)))   # left
    s.add_sphere((-99901, 40.8, 81.6), 100000, Material.diffuse((0.25, 0.25, 0.75)))   # right
    s.add_sphere((50, 40.8, 100000), 100000, Material.diffuse((0.75, 0.75, 0.75)))     # back
    s.add_sphere((50, 100000, 81.6), 100000, Material.diffuse((0.75, 0.75, 0.75)))     # floor
    s.add_sphere((50, -99918.4, 81.6), 100000, Material.diffuse((0.75, 0.75, 0.75)))   # ceiling
    s.add_sphere((65, 20, 20), 20, Material.diffuse((0.25, 0.75, 0.25)))
    s.add_sphere((27, 16.5, 47), 16.5, Material.mirror((0.99, 0.99, 0.99)))
    s.add_sphere((77, 16.5, 78), 16.5, Material.glass((0.99, 0.99, 0.99)))
    s.add_sphere((50, 76, 81.6), 5, Material.diffuse((0, 0, 0), (36, 36, 36)))         # light
    s.camera = Camera(position=(50, 52, 220), dir=(0, -0.04, -1), angle=30, width=width, height=height)
    s.settings = RenderSettings(samples=samples, supersamples=supersamples, tent_filter=1, depth=depth,
                                nee=0, seed=seed)
    return s


# ---------------------------------------------------------------- meshes
def box_mesh(lo, hi):
    """Closed axis-aligned box, 12 triangles."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], dtype=np.float32)
    f = np.array([[0, 1, 2], [0, 2, 3],      # z0
                  [4, 6, 5], [4, 7, 6],      # z1
                  [0, 4, 5], [0, 5, 1],      # y0
                  [3, 2, 6], [3, 6, 7],      # y1
                  [0, 3, 7], [0, 7, 4],      # x0
                  [1, 5, 6], [1, 6, 2]],     # x1
                 dtype=np.int32)
    return v, f


def icosphere(subdiv: int):
    """Unit icosphere: 20*4^subdiv faces, 10*4^subdiv+2 vertices."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
             (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.array(verts, dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(faces, dtype=np.int64)
    for _ in range(subdiv):
        nv = v.shape[0]
        edges = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        key = np.minimum(edges[:, 0], edges[:, 1]) * (nv + 1) + np.maximum(edges[:, 0], edges[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        a = uniq // (nv + 1)
        b = uniq % (nv + 1)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid], axis=0)
        m = inv.reshape(3, -1).T + nv  # midpoints of edges (01, 12, 20) per face
        f0, f1, f2 = f[:, 0], f[:, 1], f[:, 2]
        m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([f0, m01, m20], 1), np.stack([f1, m12, m01], 1),
                            np.stack([f2, m20, m12], 1), np.stack([m01, m12, m20], 1)], axis=0)
    return v, f.astype(np.int32)


def _perlin3(p: np.ndarray, seed: int) -> np.ndarray:
    """Improved gradient noise (Perlin 2002) with a seeded permutation."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256)
    perm = np.concatenate([perm, perm])
    grads = np.array([[1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1],
                      [-1, 0, -1], [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1], [1, 1, 0], [-1, 1, 0],
                      [0, -1, 1], [0, -1, -1]], dtype=np.float64)
    pi = np.floor(p).astype(np.int64)
    pf = p - pi
    pi &= 255
    fade = pf * pf * pf * (pf * (pf * 6 - 15) + 10)

    def h(ix, iy, iz):
        return perm[perm[perm[ix] + iy] + iz] & 15

    out = np.zeros(p.shape[0])
    acc = []
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                g = grads[h((pi[:, 0] + dx) & 255, (pi[:, 1] + dy) & 255, (pi[:, 2] + dz) & 255)]
                d = pf - np.array([dx, dy, dz], dtype=np.float64)
                acc.append((g * d).sum(1))
    u, v, w = fade[:, 0], fade[:, 1], fade[:, 2]
    lerp = lambda a, b, t: a + t * (b - a)  # noqa: E731
    x00 = lerp(acc[0], acc[1], u)
    x10 = lerp(acc[2], acc[3], u)
    x01 = lerp(acc[4], acc[5], u)
    x11 = lerp(acc[6], acc[7], u)
    out = lerp(lerp(x00, x10, v), lerp(x01, x11, v), w)
    return out


def displaced_icosphere(subdiv: int, center, radius: float, amp: float = 0.05, freq: float = 4.0,
                        seed: int = 0):
    v, f = icosphere(subdiv)
    n = _perlin3(v * freq + 17.0, seed)
    r = radius * (1.0 + amp * n)
    verts = (v * r[:, None] + np.asarray(center, dtype=np.float64)).astype(np.float32)
    return verts, f


def mesh_cornell(width: int = 1024, height: int = 768, samples: int = 16, supersamples: int = 2,
                 subdiv: int = 7, material: str = "diffuse", depth: int = 5, seed: int = 0) -> Scene:
    """Triangle-mesh Cornell box: a 12-triangle box, a uvplane area light
    under the ceiling (U, V of length 5 as in proj/test/CornellBoxMLT2*.txt)
    and a Perlin-displaced icosphere (subdiv 7 = 327,680 triangles) that is
    diffuse, glass, ward or phong.  NEE on; 16 x 2^2 tent-filtered samples = 64 spp."""
    s = Scene()
    bv, bf = box_mesh((1, 0, 0), (99, 81.6, 250))
    s.add_mesh(bv, bf, Material.diffuse((0.75, 0.75, 0.75)))
    s.add_uvplane((47.5, 81.5, 78.5), (5, 0, 0), (0, 0, 5), Material.diffuse((0, 0, 0), (36, 36, 36)))
    iv, jf = displaced_icosphere(subdiv, (50, 24, 70), 20.0, amp=0.05, seed=seed)
    if material == "glass":
        mat = Material.glass((0.99, 0.99, 0.99))
    elif material == "ward":  # anisotropic brushed-metal lobe over a dark diffuse base
        mat = Material.ward((0.10, 0.25, 0.10), (0.60, 0.55, 0.45), alpha_x=0.08, alpha_y=0.30)
    elif material == "phong":  # glossy lobe (n = 40), diffuse on 30 % of hits
        mat = Material.phong((0.25, 0.60, 0.25), (0.55, 0.55, 0.55), exponent=40.0, roughness=0.3)
    else:
        mat = Material.diffuse((0.25, 0.75, 0.25))
    s.add_mesh(iv, jf, mat)
    s.camera = Camera(position=(50, 52, 220), dir=(0, -0.04, -1), angle=30, width=width, height=height)
    s.settings = RenderSettings(samples=samples, supersamples=supersamples, tent_filter=1, depth=depth,
                                nee=1, seed=seed)
    return s


def diff_cornell(width: int = 512, height: int = 512, samples: int = 16, supersamples: int = 2, subdiv: int = 5,
                 albedo=None, emission_scale: float = 1.0, depth: int = 5, seed: int = 0) -> Scene:
    """Cornell box for differentiable rendering: eight Lambertian materials
    (five walls as uv-planes, a displaced icosphere and two boxes) with RGB
    albedo drawn U(0.1, 0.9) from the seed (or given as an (8, 3) array), and
    the ceiling light whose emission is scaled by emission_scale.  NEE on;
    16 x 2^2 tent-filtered samples = 64 spp."""
    rng = np.random.default_rng(seed)
    alb = rng.uniform(0.1, 0.9, (8, 3)) if albedo is None else np.asarray(albedo, dtype=np.float64)
    s = Scene()
    X0, X1, Y1, Z0, Z1 = 1.0, 99.0, 81.6, 0.0, 250.0
    # walls facing into the box (normal = normalize(U x V))
    s.add_uvplane((X0, 0.0, Z0), (0.0, 0.0, Z1), (X1 - X0, 0.0, 0.0), Material.diffuse(alb[0]))   # floor, +y
    s.add_uvplane((X0, Y1, Z0), (X1 - X0, 0.0, 0.0), (0.0, 0.0, Z1), Material.diffuse(alb[1]))    # ceiling, -y
    s.add_uvplane((X0, 0.0, Z0), (X1 - X0, 0.0, 0.0), (0.0, Y1, 0.0), Material.diffuse(alb[2]))   # back, +z
    s.add_uvplane((X0, 0.0, Z0), (0.0, Y1, 0.0), (0.0, 0.0, Z1), Material.diffuse(alb[3]))        # left, +x
    s.add_uvplane((X1, 0.0, Z0), (0.0, 0.0, Z1), (0.0, Y1, 0.0), Material.diffuse(alb[4]))        # right, -x
    iv, jf = displaced_icosphere(subdiv, (50, 20, 70), 16.0, amp=0.05, seed=seed)
    s.add_mesh(iv, jf, Material.diffuse(alb[5]))
    bv, bf = box_mesh((14, 0, 30), (34, 30, 50))
    s.add_mesh(bv, bf, Material.diffuse(alb[6]))
    bv, bf = box_mesh((66, 0, 95), (86, 18, 115))
    s.add_mesh(bv, bf, Material.diffuse(alb[7]))
    e = 36.0 * float(emission_scale)
    s.add_uvplane((47.5, 81.5, 78.5), (5, 0, 0), (0, 0, 5), Material.diffuse((0, 0, 0), (e, e, e)))
    s.camera = Camera(position=(50, 52, 220), dir=(0, -0.04, -1), angle=30, width=width, height=height)
    s.settings = RenderSettings(samples=samples, supersamples=supersamples, tent_filter=1, depth=depth,
                                nee=1, seed=seed)
    return s


def sss_cornell(width: int = 128, height: int = 96, samples: int = 4, supersamples: int = 2, subdiv: int = 5,
                sigma_s=(1.0, 0.9, 0.8), sigma_a=(0.01, 0.02, 0.03), g: float = 0.0, eta: float = 1.3,
                depth: int = 5, seed: int = 0, level: int = -2) -> Scene:
    """Mesh Cornell box whose displaced icosphere is a subsurface material:
    directional-dipole BSSRDF (level -2; level -1 adds the single-scattering
    walk) with sigma_s' ~ 1, sigma_a ~ 0.01 per unit and relative index eta
    1.3 inside a Fresnel surface (IOR 1.5)."""
    s = mesh_cornell(width, height, samples, supersamples, subdiv=subdiv, depth=depth, seed=seed)
    s.materials[s.entities[2].material] = Material.subsurface((0.9, 0.8, 0.7), sigma_s=sigma_s, sigma_a=sigma_a,
                                                              g=g, eta=eta, level=level)
    return s


def media_cornell(width: int = 128, height: int = 96, samples: int = 4, supersamples: int = 2,
                  sigma_s: float = 0.05, sigma_a: float = 0.01, g: float = 0.3, subdiv: int = 3,
                  depth: int = 5, seed: int = 0) -> Scene:
    """Cornell box filled with a homogeneous medium (global SCATTERING /
    ABSORBING / PAHASE) around a diffuse icosphere, NEE on."""
    s = mesh_cornell(width, height, samples, supersamples, subdiv=subdiv, depth=depth, seed=seed)
    s.participating_media = 1
    s.medium = Medium(sigma_s_rgb=(sigma_s,) * 3, sigma_a_rgb=(sigma_a,) * 3, phase_g=(g,) * 3)
    s.settings.media = 1
    return s


def media_batch(n: int = 32, seed: int = 0, sizes=(128, 256, 384, 512, 768, 1024), samples: int = 16,
                supersamples: int = 2, subdiv: int = 5, bssrdf: bool = True):
    """n Cornell variants for one batched launch: a homogeneous medium with
    sigma_s U(0.05, 0.5), sigma_a 0.01 and HG g U(-0.6, 0.8) around a
    20k-triangle displaced icosphere (subdiv 5) that is a directional-dipole
    BSSRDF material (sigma_s' ~ 1, sigma_a ~ 0.01 per unit, relative index
    1.3; diffuse with bssrdf=False), square images of uneven sizes
    (128^2 .. 1024^2), 16 x 2^2 tent-filtered samples (64 spp)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        side = int(rng.choice(sizes))
        # parameters rounded to 6 decimals, so that the reference's scene format holds them exactly
        s = media_cornell(side, side, samples, supersamples, sigma_s=round(float(rng.uniform(0.05, 0.5)), 6),
                          sigma_a=0.01, g=round(float(rng.uniform(-0.6, 0.8)), 6), subdiv=subdiv, seed=seed)
        if bssrdf:
            s.materials[s.entities[2].material] = Material.subsurface(
                (0.9, 0.8, 0.7), sigma_s=(1.0, 0.95, 0.9), sigma_a=(0.01, 0.012, 0.015), eta=1.3, level=-2)
        s.settings.seed = seed + i
        out.append(s)
    return out


def celestial_texture(width: int = 1024, height: int = 512, stars: int = 10000, seed: int = 0,
                      cells=(24, 12)) -> np.ndarray:
    """Procedural celestial sphere for the Kerr background map: a seeded
    two-tone checker in (phi, theta) plus point stars; (H, W, 3) uint8
    indexed [y, x] as the background lookup's cell(y, x)."""
    rng = np.random.default_rng(seed)
    ys, xs = np.meshgrid(np.arange(height), np.arange(width), indexing="ij")
    cx = (xs * cells[0]) // width
    cy = (ys * cells[1]) // height
    even = ((cx + cy) % 2 == 0)[..., None]
    tex = np.where(even, np.array([38, 44, 70], np.uint8), np.array([16, 14, 30], np.uint8)).astype(np.uint8)
    sx = rng.integers(0, width, stars)
    sy = rng.integers(0, height, stars)
    b = rng.integers(120, 256, stars)
    tint = rng.integers(0, 3, stars)
    col = np.stack([b, b, b], 1)
    col[np.arange(stars), tint] = np.minimum(255, col[np.arange(stars), tint] + 40)
    tex[sy, sx] = col.astype(np.uint8)
    return np.ascontiguousarray(tex)


def kerr_disk(width: int = 256, height: int = 192, a: float = 0.9, max_steps: int = 400,
              samples: int = 1, supersamples: int = 1, escape_radius: float = 0.0, texture=None) -> Scene:
    """A spinning black hole of mass 1 at the origin (spin axis z) with a thin
    emitting annulus in its equatorial plane (r 3..12), a diffuse sphere behind
    it that the hole lenses, and a camera 30 M away, 8 degrees above the disk
    plane; the scene of the reference's BLACKHOLE examples at test scale."""
    s = Scene()
    s.add_disk((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 12.0,
               Material.diffuse((0.75, 0.75, 0.75), emission=(4.0, 2.5, 1.0)), radius_inner=3.0)
    s.add_sphere((6.0, 40.0, 6.0), 6.0, Material.diffuse((0.25, 0.55, 0.85), emission=(0.4, 0.8, 1.2)))
    s.set_black_hole((0.0, 0.0, 0.0), a, max_steps=max_steps, escape_radius=escape_radius, texture=texture)
    el = math.radians(8.0)
    c, sn = round(math.cos(el), 12), round(math.sin(el), 12)  # decimal-exact in the scene text
    s.camera = Camera(position=(0.0, round(-30.0 * c, 10), round(30.0 * sn, 10)), dir=(0.0, c, -sn), up=(0.0, 0.0, 1.0),
                      width=width, height=height, angle=40.0)
    s.settings = RenderSettings(samples=samples, supersamples=supersamples, depth=1, depth_limit=1, nee=0)
    return s


def kerr_lensing(a: float = 0.999, width: int = 2048, height: int = 1024, max_steps: int = 4000,
                 fov: float = 60.0, texture=None, escape_radius: float = 0.0, r_cam: float = 6.03) -> Scene:
    """Kerr lensing view: camera at Boyer-Lindquist r = 6.03 M in the
    equatorial plane (theta = pi/2) looking at the hole, a thin emitting
    accretion disk r 3..15 M in that plane, and a procedural celestial
    sphere as the background map (seeded checker + 10k point stars)."""
    s = Scene()
    s.add_disk((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 15.0,
               Material.diffuse((0.0, 0.0, 0.0), emission=(1.6, 0.9, 0.4)), radius_inner=3.0)
    if texture is None:
        texture = celestial_texture(1024, 512, stars=10000, seed=0)
    s.set_black_hole((0.0, 0.0, 0.0), a, max_steps=max_steps, escape_radius=escape_radius, texture=texture)
    y = round(-math.sqrt(r_cam * r_cam + a * a), 12)  # BL (r, pi/2, 3 pi/2) in Cartesian
    s.camera = Camera(position=(0.0, y, 0.0), dir=(0.0, 1.0, 0.0), up=(0.0, 0.0, 1.0), width=width, height=height,
                      angle=fov)
    s.settings = RenderSettings(samples=1, supersamples=1, depth=1, depth_limit=1, nee=0)
    return s


def accretion_texture(width: int = 512, height: int = 512, seed: int = 0, arms: int = 7) -> np.ndarray:
    """Procedural accretion-disk map for DiscMapping::MapUV (circle.h:53-77):
    the disk's normalised radius rn maps to the distance rn * size from the
    image centre, so the annulus rn in [0, 0.5] fills the image.  Hot white
    inner rim cooling to orange and deep red outward, seeded spiral
    turbulence streaks; (H, W, 3) uint8 indexed [y, x] as cell(y, x)."""
    rng = np.random.default_rng(seed)
    ys, xs = np.meshgrid(np.arange(height), np.arange(width), indexing="ij")
    dx = (xs + 0.5) / width - 0.5
    dy = (ys + 0.5) / height - 0.5
    rn = np.sqrt(dx * dx + dy * dy) * 2.0  # 0 at the ISCO, 1 at the image edge
    th = np.arctan2(dy, dx)
    phase = rng.uniform(0.0, 2.0 * np.pi, arms)
    twist = rng.uniform(4.0, 9.0, arms)
    turb = np.zeros_like(rn)
    for k in range(arms):
        turb += np.sin((k + 2) * th + twist[k] * np.log1p(6.0 * rn) + phase[k])
    turb = 0.5 + 0.5 * turb / arms
    heat = np.clip(1.0 - rn, 0.0, 1.0)
    bright = np.clip((0.35 + 0.65 * turb) * (0.25 + 0.75 * heat ** 0.7), 0.0, 1.0)
    r = np.clip(255.0 * bright * (0.85 + 0.15 * heat), 0, 255)
    g = np.clip(255.0 * bright * (0.25 + 0.7 * heat ** 1.5), 0, 255)
    b = np.clip(255.0 * bright * (0.05 + 0.9 * heat ** 3.0), 0, 255)
    tex = np.stack([r, g, b], axis=-1)
    tex[rn > 1.0] = 0.0
    return np.ascontiguousarray(tex.astype(np.uint8))


def kerr_accretion(a: float = 0.999, width: int = 2048, height: int = 1024, max_steps: int = 4000,
                   fov: float = 60.0, texture=None, disk_texture=None, doppler_effect: float = 0.3,
                   disk_temperature: bool = False, escape_radius: float = 0.0, r_cam: float = 6.03,
                   samples: int = 1, supersamples: int = 1, precision: int = A.PR_KERR_FP64,
                   disk_seed: int = 1, elevation: float = 0.0) -> Scene:
    """The Kerr lensing view with a textured accretion disk: 'disk2 0 0 0 15 3'
    with 'blackhole_disk 0' and a disk_map material, the procedural disk map
    as accretion_disk_texture, color_doppler_factor_effect doppler_effect
    and the celestial sphere behind; camera at Boyer-Lindquist r = r_cam M
    in the disk plane looking at the hole (elevation > 0 degrees lifts it
    above the plane at the same Cartesian distance)."""
    s = Scene()
    m = Material.diffuse((0.0, 0.0, 0.0), emission=(2.0, 2.0, 2.0))
    m.disk_map = 1
    s.add_disk((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 15.0, m, radius_inner=3.0)
    if texture is None:
        texture = celestial_texture(1024, 512, stars=10000, seed=0)
    elif texture is False:  # no background map: escaped rays take BACKGROUND
        texture = None
    if disk_texture is None:
        disk_texture = accretion_texture(512, 512, seed=0)
    s.set_black_hole((0.0, 0.0, 0.0), a, max_steps=max_steps, escape_radius=escape_radius, texture=texture,
                     precision=precision, disk_texture=disk_texture, disk_temperature=disk_temperature,
                     doppler_effect=doppler_effect, disk_seed=disk_seed)
    dist = math.sqrt(r_cam * r_cam + a * a)  # BL (r, pi/2, 3 pi/2) in Cartesian
    if elevation == 0.0:
        s.camera = Camera(position=(0.0, round(-dist, 12), 0.0), dir=(0.0, 1.0, 0.0), up=(0.0, 0.0, 1.0),
                          width=width, height=height, angle=fov)
    else:
        el = math.radians(elevation)
        c, sn = round(math.cos(el), 12), round(math.sin(el), 12)  # decimal-exact in the scene text
        s.camera = Camera(position=(0.0, round(-dist * c, 10), round(dist * sn, 10)), dir=(0.0, c, -sn),
                          up=(0.0, 0.0, 1.0), width=width, height=height, angle=fov)
    s.settings = RenderSettings(samples=samples, supersamples=supersamples, depth=1, depth_limit=1, nee=0)
    return s


def random_rays(scene_bounds_lo, scene_bounds_hi, n: int, seed: int = 0, inside=True) -> np.ndarray:
    """n rays (org xyz, dir xyz) with origins uniform in the box and
    directions uniform on the sphere; FP64, 6 per ray."""
    rng = np.random.default_rng(seed)
    lo = np.asarray(scene_bounds_lo, dtype=np.float64)
    hi = np.asarray(scene_bounds_hi, dtype=np.float64)
    org = lo + (hi - lo) * rng.random((n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.ascontiguousarray(np.concatenate([org, d], axis=1))


def camera_rays(scene: Scene, jitter_seed: int = 0) -> np.ndarray:
    """One primary ray per pixel through the pixel centre of CameraScreenPram
    (render.h:1261-1269); FP64, 6 per ray, row-major in (y, x)."""
    c = scene.camera.to_c()
    W, H = c.width, c.height
    pos = np.array(c.position[:])
    d = np.array(c.dir[:])
    up = np.array(c.up[:])
    sw = c.screen_width * W / H
    sx = np.cross(d, up)
    sx = sx / np.linalg.norm(sx) * sw
    sy = np.cross(sx, d)
    sy = sy / np.linalg.norm(sy) * c.screen_height
    center = pos + d * c.screen_dist
    rng = np.random.default_rng(jitter_seed)
    ys, xs = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    jx = rng.random(ys.shape) if jitter_seed else 0.5
    jy = rng.random(ys.shape) if jitter_seed else 0.5
    px = ((xs + jx) / W - 0.5)[..., None]
    py = ((ys + jy) / H - 0.5)[..., None]
    sp = center + sx * px + sy * py
    dirs = sp - pos
    dirs /= np.linalg.norm(dirs, axis=-1, keepdims=True)
    org = np.broadcast_to(pos, dirs.shape)
    return np.ascontiguousarray(np.concatenate([org, dirs], axis=-1).reshape(-1, 6))


def rays_toward(vertices: np.ndarray, lo, hi, n: int, seed: int = 0) -> np.ndarray:
    """n rays from random points in the box [lo, hi] aimed at random mesh
    vertices (jittered), so that most of them reach the mesh; FP64."""
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    org = lo + (hi - lo) * rng.random((n, 3))
    tgt = vertices[rng.integers(0, vertices.shape[0], n)].astype(np.float64) + rng.normal(scale=0.05, size=(n, 3))
    d = tgt - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.ascontiguousarray(np.concatenate([org, d], axis=1))
