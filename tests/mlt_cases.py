"""Scenes for primary-sample-space Metropolis light transport
(Render::RunMLT, render.h:363-785), shared by the golden-vector generator
and the tests.

* 'mlt_spheres': the sphere Cornell box (a mirror and a glass ball under a
  small area light) with next-event estimation.
* 'mlt_caustic': the same without next-event estimation, where the glass
  ball's caustic is found by the chains' small steps.
* 'mlt_glossy': a Phong ball, a Ward ball and a textured uvplane floor."""
from prender_gb300 import _abi as A
from prender_gb300 import scenes
from prender_gb300.scene import Material

from texture_cases import checker

CASES = ["mlt_spheres", "mlt_caustic", "mlt_glossy"]


def build(name: str, width: int, height: int, chains: int, mutation: float = 2.0, pre_sample: float = 0.4):
    s = scenes.cornell_spheres(width=width, height=height, samples=chains, supersamples=1)
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
        s.add_uvplane((2, 0.05, 40), (0, 0, 16), (16, 0, 0), floor)
    elif name not in ("mlt_spheres", "mlt_caustic"):
        raise KeyError(name)
    return s


def one_thread_cases():
    """name -> scene for the reference's one-thread MLT (bit-exact): 32 x 24,
    two chains of 307 seed paths and 1536 mutations each"""
    return {k: build(k, 32, 24, 2) for k in CASES}
