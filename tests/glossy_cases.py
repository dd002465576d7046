"""Ward and Phong scenes shared by the golden-vector generator and the tests."""
from prender_gb300 import scenes


def one_thread_cases():
    """name -> scene for one-thread renders (bit-exact against the reference)"""
    out = {}
    for mat in ("ward", "phong"):
        for nee in (1, 0):
            sc = scenes.mesh_cornell(width=24, height=18, samples=1, supersamples=2, subdiv=3, material=mat)
            sc.settings.nee = nee
            out[f"{mat}_nee{nee}"] = sc
    return out


def highspp_case(mat: str):
    """64 x 48, 128 x 2^2 tent-filtered samples per batch"""
    return scenes.mesh_cornell(width=64, height=48, samples=128, supersamples=2, subdiv=3, material=mat)
