"""Scenes for primary-sample-space Metropolis light transport
(Render::RunMLT, render.h:363-785), shared by the golden-vector generator
and the tests.

* 'mlt_spheres': the sphere Cornell box (a mirror and a glass ball, a small
  spherical light out of the camera's view) with next-event estimation.
* 'mlt_caustic': the same without next-event estimation, where the glass
  ball's caustic is found by the chains' small steps.
* 'mlt_glossy': a Phong ball, a Ward ball and a textured uvplane floor."""
from prender_gb300 import _abi as A
from prender_gb300 import scenes
from prender_gb300.scene import Material

from texture_cases import checker

CASES = ["mlt_spheres", "mlt_caustic", "mlt_glossy"]
# pinned against the reference on the oracle only: the global medium (HG,
# NEE from medium points) under the Metropolis sampler
ORACLE_CASES = CASES + ["mlt_media"]


def build(name: str, width: int, height: int, chains: int, mutation: float = 2.0, pre_sample: float = 0.4):
    s = scenes.cornell_spheres(width=width, height=height, samples=chains, supersamples=1)
    # the light moves out of the camera's view (above the frustum, near the
    # front): the image is all indirect light, where the chains' local
    # exploration pays; a directly seen emitter would draw a third of the
    # chains' starts onto a few pixels
    light = s.entities[-1]
    light.p = (50.0, 77.0, 150.0)
    light.radius = 4.0
    s.materials[light.material] = Material.diffuse((0, 0, 0), (100, 100, 100))
    st = s.settings
    st.mode = A.PR_MODE_MLT
    st.mutation = mutation
    st.pre_sample = pre_sample
    st.tent_filter = 1
    st.depth = 5
    st.nee = 0 if name == "mlt_caustic" else 1
    if name == "mlt_glossy":
        s.materials[s.entities[-3].material] = Material.phong((0.2, 0.4, 0.2), (0.6, 0.6, 0.6), exponent=30.0,
                                                              roughness=0.3)
        s.materials[s.entities[-2].material] = Material.ward((0.2, 0.2, 0.3), (0.6, 0.5, 0.4), 0.1, 0.3)
        floor = Material.diffuse((0.6, 0.6, 0.6))
        floor.texture = checker(16, 16, 4, (220, 220, 220), (60, 60, 160), 51)
        # a panel 1 above the floor: the radius-1e5 floor sphere's FP32 hit
        # distance at grazing angles is not good to a few hundredths
        s.add_uvplane((2, 1.0, 40), (0, 0, 16), (16, 0, 0), floor)
    elif name == "mlt_media":
        s.participating_media = 1
        s.medium.sigma_s_rgb = (0.004, 0.004, 0.004)
        s.medium.sigma_a_rgb = (0.001, 0.001, 0.001)
        s.medium.phase_g = (0.5, 0.5, 0.5)
        st.media = 1
    elif name not in ("mlt_spheres", "mlt_caustic"):
        raise KeyError(name)
    return s


def one_thread_cases():
    """name -> scene for the reference's one-thread MLT (bit-exact): 32 x 24,
    two chains of 307 seed paths and 1536 mutations each"""
    return {k: build(k, 32, 24, 2) for k in ORACLE_CASES}


ORACLE_TENT_SUBPIXELS = 1 << 16  # the oracle's test-only full 2 x 2 sub-pixel footprint


def pt_settings(s, samples: int = 64):
    """the oracle path tracer's settings for the expectation of an MLT
    scene's image: the tent filter over all 2 x 2 sub-pixels (the footprint
    of generate_new_path; Render::Run's tent fold keeps only sub-pixel 0), no
    luminance clamp"""
    import dataclasses
    return dataclasses.replace(s.settings, mode=A.PR_MODE_MEGAKERNEL, samples=samples, supersamples=2, tent_filter=1,
                               luminance_cutoff=0.0, flags=ORACLE_TENT_SUBPIXELS)


def gpu_case(name: str, seed: int = 0):
    """64 x 48, 16 x 3072 x 32 mutations and 16 x 3072 x 8 bootstrap paths
    (the normalisation b is their mean luminance: a heavy-tailed estimate,
    low in most runs, that a larger bootstrap tightens)"""
    s = build(name, 64, 48, 16, mutation=32.0, pre_sample=8.0)
    s.settings.seed = seed
    return s
