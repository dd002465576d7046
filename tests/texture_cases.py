"""Scenes with textures and image-based lighting on hits (sphere.h:104-240,
plane.h:241-273), shared by the golden-vector generator and the tests.

* 'tex_maps': the sphere Cornell box with textured spheres in each mapping
  (the spherical default with repeat 2, equirectangular, angular,
  panoramic, hemisphere_map), a textured Ward sphere (the texel is also its
  specular colour), a textured uvplane panel (repeat 3) and a textured
  hemisphere, lit by the area light with next-event estimation.
* 'ibl_dome': an open scene under a sky dome (a hemisphere seen from
  inside) whose colour and emission come from a Radiance HDR image
  (ibl_texture_coef 1.5, angular map); a uvplane floor with a bitmap IBL
  image (emission from the bitmap), diffuse, mirror, glass and Phong
  spheres.  The dome is not a light (its material is dark and emits
  nothing of its own), so paths collect it where they hit it.
* 'ibl_nonee': the same without next-event estimation.
* 'ibl_panoramic': a full sphere dome with a bitmap IBL image in the
  panoramic map, and the equirectangular and hemisphere_map variants on
  smaller spheres.
* 'bump', 'bump_nonee': bump maps (square, smooth noise) on a diffuse
  uvplane floor (nothing below it: the reference's weight divides by the
  cosine to the plane's own normal, which a ray from underneath turns
  negative), a diffuse, a Ward, a mirror and a textured sphere, with
  next-event estimation on and off; the tilted normal scales each
  scattered weight and next-event term.

Textures are seeded synthetic images (checkerboards, gradients, noise);
the HDR image holds values that RGBE stores exactly."""
import numpy as np

from prender_gb300 import _abi as A
from prender_gb300.scene import Camera, Material, RenderSettings, Scene, rgbe_values

CASES = ["tex_maps", "ibl_dome", "ibl_nonee", "ibl_panoramic", "bump", "bump_nonee"]


def checker(h, w, n, c0, c1, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    board = ((y * n // h + x * n // w) % 2).astype(bool)
    img = np.where(board[..., None], np.array(c0), np.array(c1)).astype(np.float64)
    img += rng.integers(-20, 21, (h, w, 3))
    img[:, :, 2] += 40.0 * x / w  # a gradient across u
    return np.clip(img, 0, 255).astype(np.uint8)


def sky_hdr(h, w, seed):
    """an HDR sky: RGBE bytes with a bright region (exponent 130) over a
    dimmer one (126-128), decoded as the reference decodes them"""
    rng = np.random.default_rng(seed)
    q = np.zeros((h, w, 4), np.uint8)
    q[..., :3] = rng.integers(60, 256, (h, w, 3))
    e = np.full((h, w), 127)
    e[: h // 3] = 129
    e[h // 3: h // 3 + 2, w // 4: w // 4 + 3] = 132  # a sun
    e += rng.integers(-1, 2, (h, w))
    q[..., 3] = e
    return rgbe_values(q)


def bump_map(n, seed, blur=3, amp=255.0):
    rng = np.random.default_rng(seed)
    a = rng.uniform(0, 255, (n, n))
    for _ in range(blur):  # smooth, wrapping
        a = (a + np.roll(a, 1, 0) + np.roll(a, -1, 0) + np.roll(a, 1, 1) + np.roll(a, -1, 1)) / 5.0
    a = (a - a.min()) / (a.max() - a.min() + 1e-9) * amp
    g = np.clip(a, 0, 255).astype(np.uint8)
    return np.stack([g, np.roll(g, 3, 1), g], axis=2)


def _walls(s):
    s.add_sphere((100001, 40.8, 81.6), 100000, Material.diffuse((0.75, 0.25, 0.25)))
    s.add_sphere((-99901, 40.8, 81.6), 100000, Material.diffuse((0.25, 0.25, 0.75)))
    s.add_sphere((50, 40.8, 100000), 100000, Material.diffuse((0.75, 0.75, 0.75)))
    s.add_sphere((50, 100000, 81.6), 100000, Material.diffuse((0.75, 0.75, 0.75)))
    s.add_sphere((50, -99918.4, 81.6), 100000, Material.diffuse((0.75, 0.75, 0.75)))


def _textured(color_tex, maps=0, repeat=1, base=None):
    m = base if base is not None else Material.diffuse((0.5, 0.5, 0.5))
    m.texture = color_tex
    m.map_flags = maps
    m.repeat = repeat
    return m


def build(name: str, width: int, height: int, samples: int, supersamples: int = 2) -> Scene:
    s = Scene()
    if name == "tex_maps":
        _walls(s)
        s.add_sphere((25, 14, 60), 14, _textured(checker(32, 64, 8, (220, 60, 40), (40, 200, 60), 1), repeat=2))
        s.add_sphere((75, 14, 60), 14, _textured(checker(48, 48, 6, (240, 240, 60), (40, 40, 200), 2),
                                                 A.PR_MAP_EQUIRECTANGULAR))
        s.add_sphere((50, 10, 95), 10, _textured(checker(40, 40, 5, (250, 250, 250), (30, 30, 30), 3),
                                                 A.PR_MAP_ANGULAR))
        s.add_sphere((20, 42, 40), 8, _textured(checker(32, 64, 4, (200, 100, 250), (20, 120, 40), 4),
                                                A.PR_MAP_PANORAMIC))
        s.add_sphere((80, 42, 40), 8, _textured(checker(40, 40, 4, (250, 150, 20), (20, 20, 120), 5),
                                                A.PR_MAP_HEMISPHERE))
        s.add_sphere((50, 35, 40), 7, _textured(checker(32, 32, 4, (200, 200, 200), (60, 60, 60), 6),
                                                base=Material.ward((0.2, 0.2, 0.2), (0.6, 0.6, 0.6), 0.1, 0.3)))
        s.add_hemisphere((50, 0.5, 130), 9, _textured(checker(32, 32, 4, (30, 220, 220), (220, 30, 30), 7)))
        s.add_uvplane((10, 0.1, 100), (6, 0, 0), (0, 0, 6), _textured(checker(24, 24, 3, (250, 250, 0), (0, 0, 250),
                                                                              8), repeat=3))
        s.add_sphere((50, 76, 81.6), 5, Material.diffuse((0, 0, 0), (36, 36, 36)))
        s.camera = Camera(position=(50, 52, 220), dir=(0, -0.04, -1), angle=30, width=width, height=height)
        s.settings = RenderSettings(samples=samples, supersamples=supersamples, tent_filter=1, depth=5, nee=1, seed=0)
        return s
    if name in ("ibl_dome", "ibl_nonee"):
        dome = Material.diffuse((0.0, 0.0, 0.0))
        dome.ibl = sky_hdr(32, 64, 11)
        dome.ibl_coef = 1.5
        dome.map_flags = A.PR_MAP_ANGULAR
        s.add_hemisphere((50, 0, 60), 400, dome, normal_inverse=-1)
        floor = Material.diffuse((0.6, 0.6, 0.6))
        floor.ibl = checker(16, 16, 4, (40, 40, 40), (90, 80, 70), 12)
        floor.ibl_coef = 0.2
        s.add_uvplane((-100, 0.01, -100), (0, 0, 15), (15, 0, 0), floor)
        s.add_sphere((25, 14, 60), 14, Material.diffuse((0.7, 0.3, 0.3)))
        s.add_sphere((60, 14, 50), 14, Material.mirror((0.95, 0.95, 0.95)))
        s.add_sphere((85, 10, 90), 10, Material.glass((0.99, 0.99, 0.99)))
        s.add_sphere((40, 6, 100), 6, Material.phong((0.2, 0.5, 0.2), (0.5, 0.5, 0.5), exponent=30.0, roughness=0.3))
        s.add_sphere((70, 60, 70), 4, Material.diffuse((0, 0, 0), (20, 20, 20)))
        s.camera = Camera(position=(50, 40, 220), dir=(0, -0.15, -1), angle=35, width=width, height=height)
        s.settings = RenderSettings(samples=samples, supersamples=supersamples, tent_filter=1, depth=5,
                                    nee=1 if name == "ibl_dome" else 0, seed=0)
        return s
    if name == "ibl_panoramic":
        dome = Material.diffuse((0.0, 0.0, 0.0))
        dome.ibl = checker(32, 64, 8, (120, 160, 250), (250, 220, 180), 21)
        dome.map_flags = A.PR_MAP_PANORAMIC
        s.add_sphere((50, 40, 80), 500, dome, normal_inverse=-1)
        eq = Material.diffuse((0.0, 0.0, 0.0))
        eq.ibl = checker(32, 64, 4, (250, 60, 60), (60, 60, 250), 22)
        eq.map_flags = A.PR_MAP_EQUIRECTANGULAR
        eq.ibl_coef = 0.5
        s.add_sphere((30, 20, 60), 12, eq)
        hm = Material.diffuse((0.0, 0.0, 0.0))
        hm.ibl = checker(32, 32, 4, (60, 250, 60), (250, 250, 60), 23)
        hm.map_flags = A.PR_MAP_HEMISPHERE
        s.add_sphere((70, 20, 60), 12, hm)
        s.add_sphere((50, -100000, 80), 100000, Material.diffuse((0.5, 0.5, 0.5)))
        s.add_sphere((50, 12, 90), 8, Material.mirror((0.9, 0.9, 0.9)))
        s.camera = Camera(position=(50, 40, 220), dir=(0, -0.1, -1), angle=35, width=width, height=height)
        s.settings = RenderSettings(samples=samples, supersamples=supersamples, tent_filter=1, depth=5, nee=1, seed=0)
        return s
    if name in ("bump", "bump_nonee"):
        s.add_sphere((100001, 40.8, 81.6), 100000, Material.diffuse((0.75, 0.25, 0.25)))
        s.add_sphere((-99901, 40.8, 81.6), 100000, Material.diffuse((0.25, 0.25, 0.75)))
        s.add_sphere((50, 40.8, 100000), 100000, Material.diffuse((0.75, 0.75, 0.75)))
        s.add_sphere((50, -99918.4, 81.6), 100000, Material.diffuse((0.75, 0.75, 0.75)))
        floor = Material.diffuse((0.7, 0.7, 0.7))
        floor.bump = bump_map(32, 31, blur=4, amp=60.0)
        floor.repeat = 3
        s.add_uvplane((-20, 0.0, -20), (0, 0, 16), (16, 0, 0), floor)  # spans x, z in [-20, 236]
        ball = Material.diffuse((0.3, 0.7, 0.4))
        ball.bump = bump_map(32, 33)
        s.add_sphere((30, 14, 90), 14, ball)
        ward = Material.ward((0.2, 0.2, 0.3), (0.6, 0.6, 0.5), 0.15, 0.25)
        ward.bump = bump_map(16, 32)
        s.add_sphere((75, 10, 110), 10, ward)
        mir = Material.mirror((0.9, 0.9, 0.9))
        mir.bump = bump_map(16, 34, blur=1)
        s.add_sphere((72, 14, 65), 14, mir)
        tb = _textured(checker(32, 32, 4, (220, 80, 60), (60, 80, 220), 35), repeat=2)
        tb.bump = bump_map(32, 36)
        s.add_sphere((50, 42, 60), 8, tb)
        s.add_sphere((50, 76, 81.6), 5, Material.diffuse((0, 0, 0), (36, 36, 36)))
        s.camera = Camera(position=(50, 52, 220), dir=(0, -0.04, -1), angle=30, width=width, height=height)
        s.settings = RenderSettings(samples=samples, supersamples=supersamples, tent_filter=1, depth=5,
                                    nee=1 if name == "bump" else 0, seed=0)
        return s
    raise KeyError(name)


def one_thread_cases():
    """name -> scene for one-thread renders (bit-exact against the reference)"""
    return {k: build(k, 16, 12, 1, 2) for k in CASES}


def highspp_case(name: str):
    """64 x 48, 64 x 2^2 tent-filtered samples (256 spp) per batch"""
    return build(name, 64, 48, 64, 2)
