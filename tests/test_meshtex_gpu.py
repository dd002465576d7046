"""Smooth and textured meshes and OBJ materials (polygon.h:178-528) on the
GPU against the oracle, through the C ABI, in both render forms.

The oracle renders every scene of meshtex_cases bit-exactly like the
reference on one thread (tests/test_oracle_golden.py, meshtex_render.npz);
its 16 x 256 spp per case (meshtex_oracle.npz) are the target.  Both sides
are 4096-spp means with measured per-pixel spreads (plus 1 % of the value
for texel-edge rounding: the GPU interpolates texture coordinates from float
barycentrics, the oracle from double ones): at most 2 % of pixel channels
beyond 3 sigma, RMSE within 1.3x the noise, image mean within 1 %."""
import numpy as np
import pytest

from prender_gb300 import gpu
from prender_gb300 import _abi as A

import meshtex_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g
    g.build_library()
    c = gpu.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("mode", [A.PR_MODE_MEGAKERNEL, A.PR_MODE_WAVEFRONT])
@pytest.mark.parametrize("name", meshtex_cases.CASES)
def test_mesh_smooth_and_textures_match_oracle_statistically(ctx, golden, name, mode):
    s = meshtex_cases.highspp_case(name)
    s.settings.mode = mode
    ctx.upload(s)
    nb, spp = 16, s.settings.spp
    b = np.stack([ctx.render(s, sample_offset=k * spp).astype(np.float64) for k in range(nb)])
    mean = b.mean(0)
    sd = b.std(0, ddof=1)
    orc = golden["meshtex_oracle"]
    o_mean = orc[f"{name}_mean"].astype(np.float64)
    o_sd = orc[f"{name}_sd"].astype(np.float64)
    o_nb = int(orc["batches"])
    sigma = np.sqrt(sd ** 2 / nb + o_sd ** 2 / o_nb + (0.01 * o_mean) ** 2) + 1e-7
    frac = float((np.abs(mean - o_mean) / sigma > 3.0).mean())
    rmse = float(np.sqrt(((mean - o_mean) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - o_mean.mean()) / o_mean.mean()
    print(f"meshtex {name} mode {mode}: >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, "
          f"mean rel diff {rel:.4f}")
    assert rel < 0.01
    assert frac < 0.02
    assert rmse < 1.3 * noise


def test_smooth_normals_change_the_image(ctx):
    # the same scene with flat normals differs beyond noise on the balls
    s = meshtex_cases.build("smooth", 48, 36, 16, 2)
    ctx.upload(s)
    a = ctx.render(s).astype(np.float64)
    for e in s.entities:
        e.smooth = 0
    ctx.upload(s)
    b = ctx.render(s).astype(np.float64)
    assert np.abs(a - b).mean() > 0.01 * a.mean()


def test_mesh_texture_refusals(ctx):
    s = meshtex_cases.build("mesh_tex", 8, 6, 1, 1)
    s.meshes[-2].uv = None  # the IBL panel without texture coordinates
    s.meshes[-2].face_uv = None
    with pytest.raises(gpu.PrenderError):
        ctx.upload(s)
    s = meshtex_cases.build("mesh_tex", 8, 6, 1, 1)
    s.meshes[-2].uv[0, 0] = 1.5  # outside the image: the reference reads no wrap there
    with pytest.raises(gpu.PrenderError):
        ctx.upload(s)
