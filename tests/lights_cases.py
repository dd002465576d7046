"""Scenes with the reference's other light kinds (light.h:13-74): spot
lights (cone falloff and distance attenuation), parallel lights (uvplane
and sphere emitters whose light travels one way) and infinity lights
(directions with no emitter), shared by the golden-vector generator and
the tests.

Every scene mixes the kinds with an area light registered after them, so
that the registration index the reference keeps per entity differs from
the entity's place in the power-sorted list (the perfect-direction term of
mirrors and glass reads the light kind through that index,
directLight_radiance.h:541), and has diffuse, mirror, glass, Ward and Phong
receivers.  'parallel_nonee' and 'sss_spot' render without next-event
estimation, where the reference still samples the non-area lights
(brdf.h:590-605, Subsurface_Scattering.h:519-535); 'spot_media' is the
reference's own spot-light test set-up (proj/test/CornellBox_spot光源_関与媒質あり.txt:
a cone of 20 degrees with a 10-degree falloff band, 1/d attenuation, a thin
global medium).  'infinity_raw' gives an infinity light the unnormalised
direction of proj/test/san-miguel3b.txt, which the reference uses as it
stands; its shadow rays run along that vector, which the reference's sphere
test takes as unit length, so that case pins the oracle only."""
from prender_gb300 import scenes
from prender_gb300.scene import Camera, Material, Medium, RenderSettings, Scene

CASES = ["spot", "spot_media", "parallel", "parallel_nonee", "infinity", "sss_spot"]
REFERENCE_ONLY = ["infinity_raw"]


def _room(s: Scene) -> None:
    """the sphere Cornell box's walls (proj/test/CornellBox.txt) and receivers"""
    s.add_sphere((100001, 40.8, 81.6), 100000, Material.diffuse((0.75, 0.25, 0.25)))
    s.add_sphere((-99901, 40.8, 81.6), 100000, Material.diffuse((0.25, 0.25, 0.75)))
    s.add_sphere((50, 40.8, 100000), 100000, Material.diffuse((0.75, 0.75, 0.75)))
    s.add_sphere((50, 100000, 81.6), 100000, Material.diffuse((0.75, 0.75, 0.75)))
    s.add_sphere((50, -99918.4, 81.6), 100000, Material.diffuse((0.75, 0.75, 0.75)))
    _receivers(s)


def _receivers(s: Scene) -> None:
    s.add_sphere((65, 20, 20), 20, Material.diffuse((0.25, 0.75, 0.25)))
    s.add_sphere((27, 16.5, 47), 16.5, Material.mirror((0.99, 0.99, 0.99)))
    s.add_sphere((77, 16.5, 78), 16.5, Material.glass((0.99, 0.99, 0.99)))
    s.add_sphere((45, 8, 100), 8, Material.ward((0.1, 0.2, 0.1), (0.6, 0.55, 0.45), alpha_x=0.1, alpha_y=0.3))
    s.add_sphere((20, 7, 95), 7, Material.phong((0.2, 0.2, 0.5), (0.5, 0.5, 0.5), exponent=30.0, roughness=0.3))


def _camera(s: Scene, width, height, samples, supersamples, nee, position=(50, 52, 220), direction=(0, -0.04, -1)):
    s.camera = Camera(position=position, dir=direction, angle=30, width=width, height=height)
    s.settings = RenderSettings(samples=samples, supersamples=supersamples, tent_filter=1, depth=5, nee=nee, seed=0)


def build(name: str, width: int, height: int, samples: int, supersamples: int = 2) -> Scene:
    s = Scene()
    if name in ("spot", "spot_media"):
        if name == "spot":
            s.add_spot_light((40, 78, 70), 1.0, (120, 110, 100), (0.2, -1, 0.1), (35, 15), falloff=2.0,
                             attenuation=(1.0, 0.0, 0.0002))
        else:
            s.add_spot_light((40, 81, 70), 1.0, (400, 400, 400), (0, -1, 0), (20, 10), falloff=0.0,
                             attenuation=(0.0, 1.0, 0.0))
        _room(s)
        s.add_sphere((70, 72, 100), 2.0, Material.diffuse((0, 0, 0), (12, 12, 12)))
        _camera(s, width, height, samples, supersamples, 1)
        if name == "spot_media":
            s.participating_media = 1
            s.medium = Medium(sigma_s_rgb=(0.0015, 0.0015, 0.0015), sigma_a_rgb=(0.0003, 0.0003, 0.0003),
                              phase_g=(0.5, 0.5, 0.5))
            s.settings.media = 1
        return s
    if name in ("parallel", "parallel_nonee"):
        li = s.add_uvplane((40, 81, 70), (5, 0, 0), (0, 0, 5), Material.diffuse((0, 0, 0), (5, 5, 5)))
        s.make_parallel_light(li, (0, -1, 0))
        ls = s.add_sphere((80, 70, 60), 1.5, Material.diffuse((0, 0, 0), (3, 3, 2)))
        s.make_parallel_light(ls, (-0.6, -0.8, 0.0))
        _room(s)
        s.add_sphere((30, 72, 110), 2.0, Material.diffuse((0, 0, 0), (12, 12, 12)))
        _camera(s, width, height, samples, supersamples, 1 if name == "parallel" else 0)
        return s
    if name in ("infinity", "infinity_raw"):
        if name == "infinity":
            s.add_infinity_light((0.0, -0.8, -0.6), (2, 2, 2))
            s.add_infinity_light((0.6, -0.8, 0.0), (1.0, 0.8, 0.6))
        else:
            s.add_infinity_light((1, -1.5, -0.4), (1, 1, 1))
        s.add_sphere((50, -100000, 81.6), 100000, Material.diffuse((0.75, 0.75, 0.75)))  # floor, open sky
        _receivers(s)
        s.add_sphere((80, 30, 60), 3.0, Material.diffuse((0, 0, 0), (10, 10, 10)))
        _camera(s, width, height, samples, supersamples, 1, position=(50, 60, 220), direction=(0, -0.25, -1))
        return s
    if name == "sss_spot":
        s = scenes.sss_cornell(width=width, height=height, samples=samples, supersamples=supersamples, subdiv=3,
                               level=-1)
        s.settings.nee = 0
        s.add_spot_light((50, 70, 70), 1.0, (300, 300, 300), (0, -1, 0), (30, 10), falloff=1.0,
                         attenuation=(1.0, 0.0, 0.0005))
        return s
    raise KeyError(name)


def one_thread_cases():
    """name -> scene for one-thread renders (bit-exact against the reference)"""
    return {k: build(k, 16, 12, 1, 2) for k in CASES + REFERENCE_ONLY}


def highspp_case(name: str):
    """64 x 48, 64 x 2^2 tent-filtered samples (256 spp) per batch"""
    return build(name, 64, 48, 64, 2)
