"""Kerr scenes and rays shared by the golden-vector generator and the tests.

Every case is rebuilt from seeds, so the golden files only hold the rays and
the reference's answers."""
import numpy as np

from prender_gb300 import scenes
from prender_gb300.scene import Material


def _infall_rays(n: int, seed: int) -> np.ndarray:
    # origins 1.2..40 M from the hole (a few inside the horizon), aimed near it
    rng = np.random.default_rng(seed)
    o = rng.normal(size=(n, 3))
    o = o / np.linalg.norm(o, axis=1, keepdims=True) * rng.uniform(1.2, 40.0, (n, 1))
    d = -o + rng.normal(scale=0.3, size=o.shape)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], 1)


def trace_cases():
    """name -> (scene, rays) for the per-ray Kerr trace."""
    out = {}
    s = scenes.kerr_disk(32, 24, a=0.9, max_steps=400)
    out["disk_a09"] = (s, scenes.camera_rays(s))
    s = scenes.kerr_disk(24, 18, a=0.0, max_steps=600)
    s.add_sphere((0.0, 0.0, 0.0), 1.9, Material.diffuse((0.0, 0.0, 0.0), emission=(1.0, 0.0, 0.0)))
    out["core_a0"] = (s, np.concatenate([scenes.camera_rays(s), _infall_rays(64, 1)]))
    s = scenes.kerr_disk(24, 18, a=0.999, max_steps=1500)
    out["disk_a0999"] = (s, np.concatenate([scenes.camera_rays(s), _infall_rays(32, 2)]))
    return out


def render_cases():
    """name -> scene for whole Kerr renders (one thread, bit-exact)."""
    s1 = scenes.kerr_disk(24, 18, a=0.9, max_steps=300, samples=2, supersamples=1)
    s1.background = (0.05, 0.1, 0.2)
    tex = scenes.celestial_texture(64, 32, stars=200, seed=3)
    s2 = scenes.kerr_disk(32, 24, a=0.9, max_steps=300, samples=1, supersamples=1, texture=tex)
    s2.kerr["map_coef"] = (1.0, 0.3, 1.0, -0.7)
    s2.kerr["texture_coef"] = 1.5
    return {"bounce_bg": s1, "texture": s2}


def status_from_reference(obj, hit, rec):
    """The oracle's status codes from the reference harness record: hit flag,
    object id (EVENT_HORIZON = -998, KerrBlackHole.h:19) and whether the
    step loop ran to its end."""
    st = np.full(obj.shape, 4, np.int32)  # left the loop on a step underflow
    st[hit == 1] = 1
    st[obj == -998] = 2
    end = (rec[:, 0] == 1) & (hit == 0) & (obj != -998)
    st[end & (obj >= 0)] = 5
    st[end & (obj < 0)] = 0
    return st


def highspp_case():
    """The textured Kerr render at 256 spp for statistical image parity."""
    tex = scenes.celestial_texture(64, 32, stars=200, seed=3)
    s = scenes.kerr_disk(32, 24, a=0.9, max_steps=300, samples=64, supersamples=2, texture=tex)
    s.kerr["map_coef"] = (1.0, 0.3, 1.0, -0.7)
    s.kerr["texture_coef"] = 1.5
    return s
