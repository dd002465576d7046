"""Wormhole scenes (WormHole.h, scene.cpp:735-925) shared by the golden-vector
generator and the tests: a Dneg wormhole (throat radius rho, length 2a,
lensing width w) between a mouth in front of the camera and one three
million units away, two background images (one per side), objects near both
mouths; renders without next-event estimation and media, as the reference
does for curved-ray scenes.

* 'worm_bg': the two backgrounds only, seen through the throat.
* 'worm_objects': emissive and diffuse spheres on both sides, lit by the
  backgrounds and their own emission.
* 'worm_sign': the final side forced by 'sign -1', non-default map
  coefficients, no image on the far side (its rays end on BACKGROUND)."""
import numpy as np

from prender_gb300.scene import Camera, Material, RenderSettings, Scene

CASES = ["worm_bg", "worm_objects", "worm_sign"]
OUT = (0.0, 0.0, 3.0e6)


def sky(h, w, seed, base):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    img = np.zeros((h, w, 3))
    img[..., 0] = base[0] + 60 * np.sin(x * 6.2832 / w * 4)
    img[..., 1] = base[1] + 60 * np.cos(y * 6.2832 / h * 3)
    img[..., 2] = base[2] + 40 * ((x // 8 + y // 8) % 2)
    img += rng.integers(-10, 11, (h, w, 3))
    return np.clip(img, 0, 255).astype(np.uint8)


def build(name: str, width: int, height: int, samples: int, supersamples: int = 2, max_steps: int = 300) -> Scene:
    s = Scene()
    s.camera = Camera(position=(0.0, 0.5, 12.0), dir=(0.0, -0.02, -1.0), up=(0.0, 1.0, 0.0), angle=60,
                      width=width, height=height)
    s.settings = RenderSettings(samples=samples, supersamples=supersamples, tent_filter=1, depth=4, nee=0, seed=0)
    bg1, bg2 = sky(32, 64, 1, (120, 140, 200)), sky(32, 64, 2, (200, 120, 60))
    if name == "worm_bg":
        s.set_wormhole((0.0, 0.0, 0.0), OUT, rho=1.3, a=0.5, w=0.05, max_steps=max_steps, textures=(bg1, bg2))
        return s
    if name == "worm_objects":
        s.set_wormhole((0.0, 0.0, 0.0), OUT, rho=1.3, a=0.5, w=0.05, max_steps=max_steps, textures=(bg1, bg2),
                       texture_coef=(1.0, 1.5))
        s.add_sphere((3.5, 0.0, -3.0), 1.0, Material.diffuse((0.1, 0.1, 0.1), (2.0, 1.5, 0.5)))
        s.add_sphere((-3.0, -1.5, 1.0), 1.2, Material.diffuse((0.7, 0.7, 0.7)))
        s.add_sphere((OUT[0] + 1.5, OUT[1], OUT[2] - 4.0), 1.0, Material.diffuse((0.1, 0.1, 0.1), (0.5, 2.0, 1.0)))
        s.add_sphere((OUT[0] - 2.0, OUT[1] + 1.0, OUT[2] - 6.0), 1.5, Material.mirror((0.9, 0.9, 0.9)))
        return s
    if name == "worm_sign":
        s.background = (0.1, 0.2, 0.3)
        s.set_wormhole((0.0, 0.0, 0.0), OUT, rho=1.0, a=0.8, w=0.1, max_steps=max_steps, sign=-1,
                       textures=(bg1, None), map_coef=((1.0, 0.2, 2.0, 0.0), (1.0, 0.0, 1.0, 0.0)))
        return s
    raise KeyError(name)


def one_thread_cases():
    """name -> scene for one-thread renders (bit-exact against the reference)"""
    return {k: build(k, 24, 18, 1, 2) for k in CASES}


def highspp_case(name: str):
    """48 x 36, 16 x 2^2 tent-filtered samples (64 spp) per batch"""
    return build(name, 48, 36, 16, 2)
