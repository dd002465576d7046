"""Participating-media scenes shared by the golden-vector generator and the
tests: a mesh Cornell box filled with a homogeneous medium (global
SCATTERING / ABSORBING / PAHASE, ParticipatingMediaPrm.h:85-160) over the
range of the batched media workload (sigma_s 0.05 .. 0.5, sigma_a 0.01,
HG g -0.6 .. 0.8), with next-event estimation on and off, one medium whose
coefficients and phase asymmetry differ per channel (scalar sigma_t for
distance sampling, RGB transmittance, the phase channel drawn per vertex),
and the Henyey-Greenstein sampling of the PR_FLAG_HG_CORRECT mode."""
from prender_gb300 import scenes
from prender_gb300 import _abi as A
from prender_gb300.scene import Medium

# name -> (sigma_s, sigma_a, g, nee, flags[, luminance cutoff]); scalars are
# the same on all channels.  The reference clamps each sample's luminance at
# 0.025 x spp (render.h:1375-1384), which in these media scenes removes about
# two thirds of the energy at 256 spp; the '_nocut' cases turn the clamp off
# so the full media estimate is compared as well.
CASES = {
    "g_m06_s005": (0.05, 0.01, -0.6, 1, 0),
    "g_0_s05": (0.5, 0.01, 0.0, 1, 0),
    "g_05_s005_nonee": (0.05, 0.01, 0.5, 0, 0),
    "g_08_s05": (0.5, 0.01, 0.8, 1, 0),
    "g_08_s005_hgc": (0.05, 0.01, 0.8, 1, A.PR_FLAG_HG_CORRECT),
    "rgb": ((0.03, 0.06, 0.12), (0.01, 0.02, 0.005), (0.2, 0.5, -0.3), 1, 0),
    "g_05_s005_nocut": (0.05, 0.01, 0.5, 1, 0, 0.0),
    "g_m06_s05_nocut": (0.5, 0.01, -0.6, 1, 0, 0.0),
}

# the reference has no HG_CORRECT mode: those cases are compared with the
# oracle only (its sampler is checked against the HG distribution itself)
REFERENCE_CASES = [k for k, v in CASES.items() if not v[4]]


def _rgb(x):
    return tuple(float(v) for v in x) if isinstance(x, tuple) else (float(x),) * 3


def build(name: str, width: int, height: int, samples: int, supersamples: int = 2, subdiv: int = 3):
    ss, sa, g, nee, flags = CASES[name][:5]
    s = scenes.media_cornell(width=width, height=height, samples=samples, supersamples=supersamples, subdiv=subdiv)
    s.medium = Medium(sigma_s_rgb=_rgb(ss), sigma_a_rgb=_rgb(sa), phase_g=_rgb(g))
    s.settings.nee = nee
    s.settings.flags = flags
    if len(CASES[name]) > 5:
        s.settings.luminance_cutoff = CASES[name][5]
    return s


def one_thread_cases():
    """name -> scene for one-thread renders (bit-exact against the reference)"""
    return {k: build(k, 16, 12, 1, 2) for k in REFERENCE_CASES}


def root_cases():
    """name -> scene whose camera rays give per-ray radiance() roots"""
    return {k: build(k, 16, 12, 1, 1) for k in ("g_m06_s005", "g_08_s05", "rgb")}


def highspp_case(name: str):
    """64 x 48, 64 x 2^2 tent-filtered samples (256 spp) per batch"""
    return build(name, 64, 48, 64, 2)
