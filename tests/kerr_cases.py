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


def disk_scene(width: int, height: int, samples: int = 1, supersamples: int = 1, a: float = 0.9,
               max_steps: int = 600, temperature: bool = False, doppler: float = 0.3, escape: float = 0.0,
               disk_seed: int = 1):
    """The textured accretion disk (disk_map, blackhole_disk 0, a 128 x 128
    procedural disk map, Doppler shift) seen from 30 M, 20 degrees above the
    disk plane, with a plain background (no map: an escape radius does not
    change what an escaped ray returns)."""
    s = scenes.kerr_accretion(a=a, width=width, height=height, max_steps=max_steps, fov=50.0, texture=False,
                              disk_texture=scenes.accretion_texture(128, 128, seed=0), doppler_effect=doppler,
                              disk_temperature=temperature, escape_radius=escape, r_cam=30.0, elevation=20.0,
                              samples=samples, supersamples=supersamples, disk_seed=disk_seed)
    s.background = (0.02, 0.03, 0.05)
    return s


def disk_trace_cases():
    """name -> (scene, rays) for the per-ray trace with the disk's shading."""
    s1 = disk_scene(32, 16)
    s2 = disk_scene(24, 12, a=0.6, temperature=True, doppler=0.6)
    return {"tex_a09": (s1, scenes.camera_rays(s1)), "temp_a06": (s2, scenes.camera_rays(s2))}


def disk_render_cases():
    """name -> scene for one-thread textured-disk renders (bit-exact)."""
    return {"tex": disk_scene(24, 12, samples=2), "temp": disk_scene(16, 8, a=0.6, temperature=True, doppler=0.6)}


def disk_highspp_case():
    """The textured-disk render for statistical image parity (16 batches of
    64 x 2^2 samples); an escape radius keeps the oracle's batches short."""
    return disk_scene(48, 24, samples=64, supersamples=2, escape=60.0)
