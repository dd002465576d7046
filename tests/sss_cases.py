"""Subsurface scenes shared by the golden-vector generator and the tests."""
from prender_gb300 import scenes


def l1_cases():
    """name -> scene: level -1 subsurface (dipole or single-scattering walk),
    one sample of 2 x 2 tent-filtered subsamples per pixel"""
    out = {}
    for name, g, nee in (("l1_g0", 0.0, 1), ("l1_g05", 0.5, 1), ("l1_nonee", 0.0, 0)):
        sc = scenes.sss_cornell(width=24, height=18, samples=1, supersamples=2, subdiv=3, level=-1, g=g)
        sc.settings.nee = nee
        out[name] = sc
    return out
