"""Batched media + BSSRDF variants (the uneven-size batch workload at small
sizes) shared by the golden-vector generator and the tests."""
from prender_gb300 import scenes


def one_thread_cases():
    """name -> variant for one-thread renders (bit-exact against the reference)"""
    v = scenes.media_batch(n=2, seed=5, sizes=(16,), samples=1, supersamples=2, subdiv=5)
    for s in v:
        s.camera.height = 12
    return {f"variant{i}": s for i, s in enumerate(v)}


def highspp_variants():
    """three variants at uneven sizes, 64 x 2^2 tent-filtered samples (256 spp) per batch"""
    return scenes.media_batch(n=3, seed=2, sizes=(32, 48, 64), samples=64, supersamples=2, subdiv=5)
