"""Spot, parallel and infinity lights (light.h:13-74) on the GPU against the
oracle, through the C ABI, in both render forms.

The oracle renders every scene of lights_cases bit-exactly like the
reference on one thread (tests/test_oracle_golden.py, lights_render.npz);
its 16 x 256 spp per case (lights_oracle.npz) are the target.  Both sides
are 4096-spp means with measured per-pixel spreads: at most 2 % of pixel
channels beyond 3 sigma, RMSE within 1.3x the noise, image mean within 1 %.
The two forms shade with the same code and streams, so their images also
agree to float summation order."""
import numpy as np
import pytest

from prender_gb300 import gpu
from prender_gb300 import _abi as A

import lights_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g
    g.build_library()
    c = gpu.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("mode", [A.PR_MODE_MEGAKERNEL, A.PR_MODE_WAVEFRONT])
@pytest.mark.parametrize("name", lights_cases.CASES)
def test_light_kinds_match_oracle_statistically(ctx, golden, name, mode):
    s = lights_cases.highspp_case(name)
    s.settings.mode = mode
    ctx.upload(s)
    nb, spp = 16, s.settings.spp
    b = np.stack([ctx.render(s, sample_offset=k * spp).astype(np.float64) for k in range(nb)])
    mean = b.mean(0)
    sd = b.std(0, ddof=1)
    orc = golden["lights_oracle"]
    o_mean = orc[f"{name}_mean"].astype(np.float64)
    o_sd = orc[f"{name}_sd"].astype(np.float64)
    o_nb = int(orc["batches"])
    sigma = np.sqrt(sd ** 2 / nb + o_sd ** 2 / o_nb) + 1e-7
    frac = float((np.abs(mean - o_mean) / sigma > 3.0).mean())
    rmse = float(np.sqrt(((mean - o_mean) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - o_mean.mean()) / o_mean.mean()
    print(f"lights {name} mode {mode}: >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, "
          f"mean rel diff {rel:.4f}")
    assert rel < 0.01
    assert frac < 0.02
    assert rmse < 1.3 * noise


@pytest.mark.parametrize("name", lights_cases.CASES)
def test_light_kinds_wavefront_equals_megakernel(ctx, name):
    """Same shading code and streams in both forms; the two kernels that
    run it here (the megakernel's fuller instantiation, the wavefront's
    extended one) are compiled separately, so their float rounding can
    differ in the last bit, now and then flipping a Russian-roulette or
    branch decision, and these scenes look straight at small bright
    emitters (a spot sphere of emission 120 behind the per-sample clamp),
    where such a sample moves its pixel by up to one clamped sample (0.025
    at 16 spp): 99 % of channels agree to 2e-4, the image means to 1e-3"""
    s = lights_cases.build(name, 48, 36, 4, 2)
    ctx.upload(s)
    s.settings.mode = A.PR_MODE_MEGAKERNEL
    mk = ctx.render(s).astype(np.float64)
    s.settings.mode = A.PR_MODE_WAVEFRONT
    wf = ctx.render(s).astype(np.float64)
    assert mk.mean() > 0
    d = np.abs(wf - mk)
    assert float((d > 2e-4 * np.abs(mk) + 2e-6).mean()) < 0.01
    assert float(d.max()) < 0.03
    assert abs(wf.mean() - mk.mean()) < 1e-3 * mk.mean()

