"""Primary-sample-space Metropolis light transport on the GPU (PR_MODE_MLT,
Render::RunMLT's estimator as parallel chains) against the oracle.

The oracle's RunMLT is bit-exact with the reference's on one thread
(tests/test_oracle_golden.py, mlt_render.npz); the GPU runs the same
estimator (Kelemen's mutations and weights, b from a bootstrap, p_large
0.5, the tent filter and the 1/4 sensor scale) as 65,536 short chains, so
its image is compared with the value both converge to: the oracle's
path-traced image of the scene without the luminance clamp, 16 x 256 spp
(mlt_oracle.npz).  The GPU side is 8 independent Metropolis renders (16 x
3072 x 32 mutations each), compared on 4 x 4 pixel blocks: their spread
plus the oracle's plus 2 % of the value make sigma: at most 5 % of block
channels beyond 3 sigma, RMSE within 1.5x the noise, image mean within 2 %
or three standard errors of the runs' means (they follow the bootstrap's
heavy-tailed mean luminance)."""
import numpy as np
import pytest

from prender_gb300 import _abi as A
from prender_gb300 import gpu

import mlt_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g
    g.build_library()
    c = gpu.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", mlt_cases.CASES)
def test_mlt_converges_to_the_path_traced_image(ctx, golden, name):
    runs = []
    for k in range(8):
        s = mlt_cases.gpu_case(name, seed=1000 + k)
        ctx.upload(s)
        runs.append(ctx.render(s).astype(np.float64))
    st = ctx.stats()
    assert st["paths"] >= 16 * 3072 * 32 and st["kernel_launches"] >= 4
    # 4 x 4 pixel blocks: a chain's small steps correlate neighbouring
    # pixels and both estimators are heavy-tailed per pixel (caustics, no
    # clamp); block means are compared, with the oracle's block spread from
    # its (independent) pixel spreads
    def blocks(x):
        return x.reshape(x.shape[:-3] + (12, 4, 16, 4, 3)).mean(axis=(-4, -2))
    b = blocks(np.stack(runs))
    mean, sd = b.mean(0), b.std(0, ddof=1)
    orc = golden["mlt_oracle"]
    o_mean = blocks(orc[f"{name}_mean"].astype(np.float64))
    o_sd = np.sqrt(blocks(orc[f"{name}_sd"].astype(np.float64) ** 2) / 16.0)
    o_nb = int(orc["batches"])
    sigma = np.sqrt(sd ** 2 / len(runs) + o_sd ** 2 / o_nb + (0.02 * o_mean) ** 2) + 1e-7
    frac = float((np.abs(mean - o_mean) / sigma > 3.0).mean())
    rmse = float(np.sqrt(((mean - o_mean) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - o_mean.mean()) / o_mean.mean()
    # the image mean follows the bootstrap's mean luminance b, a heavy-tailed
    # estimate: its spread over the runs bounds the mean's agreement too
    rel_sigma = float(np.std([r.mean() for r in runs], ddof=1)) / np.sqrt(len(runs)) / o_mean.mean()
    print(f"mlt {name}: >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, mean rel diff {rel:.4f}, "
          f"{st['paths']} paths in {st['device_ms']:.1f} ms")
    assert rel < max(0.02, 3.0 * rel_sigma)
    assert frac < 0.05
    assert rmse < 1.5 * noise


def test_mlt_refusals(ctx):
    s = mlt_cases.gpu_case("mlt_spheres")
    s.settings.mutation = 0.0
    ctx.upload(s)
    with pytest.raises(gpu.PrenderError):
        ctx.render(s)
    from prender_gb300 import scenes
    s = scenes.sss_cornell(width=16, height=12, samples=1, supersamples=1, subdiv=2)
    s.settings.mode = A.PR_MODE_MLT
    ctx.upload(s)
    with pytest.raises(gpu.PrenderError):
        ctx.render(s)
