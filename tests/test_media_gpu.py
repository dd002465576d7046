"""The GPU's participating-media path (homogeneous medium, Henyey-Greenstein
phase) against the oracle, through the C ABI, in both render forms.

The oracle is bit-exact with the reference on one thread for every case
here that the reference has (tests/test_oracle_golden.py, media_render.npz)
and its HG-correct sampler follows the HG distribution; its 16 x 256 spp
per case (media_oracle.npz) are the target.  Both sides are 4096-spp means
with measured per-pixel spreads, so the per-pixel test is symmetric: at most
2 % of pixel channels beyond 3 sigma, RMSE within 1.3x the noise, image mean
within 1 %."""
import numpy as np
import pytest

from prender_gb300 import gpu
from prender_gb300 import _abi as A

import media_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g
    g.build_library()
    c = gpu.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("mode", [A.PR_MODE_MEGAKERNEL, A.PR_MODE_WAVEFRONT])
@pytest.mark.parametrize("name", list(media_cases.CASES))
def test_media_image_matches_oracle_statistically(ctx, golden, name, mode):
    s = media_cases.highspp_case(name)
    s.settings.mode = mode
    ctx.upload(s)
    nb, spp = 16, s.settings.spp
    b = np.stack([ctx.render(s, sample_offset=k * spp).astype(np.float64) for k in range(nb)])
    mean = b.mean(0)
    sd = b.std(0, ddof=1)
    orc = golden["media_oracle"]
    o_mean = orc[f"{name}_mean"].astype(np.float64)
    o_sd = orc[f"{name}_sd"].astype(np.float64)
    o_nb = int(orc["batches"])
    sigma = np.sqrt(sd ** 2 / nb + o_sd ** 2 / o_nb) + 1e-7
    frac = float((np.abs(mean - o_mean) / sigma > 3.0).mean())
    rmse = float(np.sqrt(((mean - o_mean) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - o_mean.mean()) / o_mean.mean()
    print(f"media {name} mode {mode}: >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, "
          f"mean rel diff {rel:.4f}")
    assert rel < 0.01
    assert frac < 0.02
    assert rmse < 1.3 * noise

