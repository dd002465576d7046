"""Batches and the autotuner, through the C ABI.

* pr_render_batch: jobs on different scene objects, cameras and image sizes
  in one captured CUDA graph give the same images as one pr_render_dev per
  job (up to float summation order); a second call with the same shape
  reuses the graph;
* pr_autotune_wavefront: picks a pool size and traversal grid, and the
  wavefront image afterwards is identical to the default configuration's.
"""
import numpy as np
import pytest

from prender_gb300 import _abi as A
from prender_gb300 import gpu, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g
    g.build_library()
    c = gpu.Context(0)
    yield c
    c.close()


def test_batch_matches_single_renders(ctx):
    import torch
    variants = scenes.media_batch(n=6, seed=2, sizes=(48, 64, 96), samples=2, supersamples=2, subdiv=3)
    variants[1] = scenes.cornell_spheres(width=40, height=30, samples=2, supersamples=2)
    variants[2] = scenes.kerr_disk(32, 24, a=0.9, max_steps=300, samples=1, supersamples=2)
    objs = [ctx.scene_object(s) for s in variants]
    outs = [torch.zeros((s.camera.height, s.camera.width, 3), dtype=torch.float32, device="cuda:0") for s in variants]
    for rep in range(2):  # the second call updates the captured graph in place
        ctx.render_batch([(o, out, None, None, 8 * rep) for o, out in zip(objs, outs)])
        torch.cuda.synchronize()
        st = ctx.stats()
        assert st["kernel_launches"] == 2 * len(variants)
        for s, out in zip(variants, outs):
            s.settings.mode = A.PR_MODE_MEGAKERNEL
            ctx.upload(s)
            ref = ctx.render(s, sample_offset=8 * rep)
            got = out.cpu().numpy()
            assert np.isfinite(got).all() and got.mean() > 0
            np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-6)
    for o in objs:
        o.release()


def test_batch_wavefront_jobs_equal_single_wavefront_renders(ctx):
    """Jobs in the wavefront form (one after another on the shared path pool)
    beside plain-form jobs in the same call: each wavefront image equals
    pr_render_dev's wavefront image of the same inputs exactly (fixed-point
    accumulation), subsurface and media scenes included."""
    import torch
    variants = scenes.media_batch(n=4, seed=7, sizes=(40, 56), samples=2, supersamples=2, subdiv=4)
    variants[1].settings.mode = A.PR_MODE_MEGAKERNEL
    for k in (0, 2, 3):
        variants[k].settings.mode = A.PR_MODE_WAVEFRONT
    variants[3] = scenes.mesh_cornell(width=48, height=36, samples=2, supersamples=2, subdiv=4, material="glass")
    variants[3].settings.mode = A.PR_MODE_WAVEFRONT
    objs = [ctx.scene_object(s) for s in variants]
    outs = [torch.zeros((s.camera.height, s.camera.width, 3), dtype=torch.float32, device="cuda:0") for s in variants]
    ctx.render_batch([(o, out, None, None, 4) for o, out in zip(objs, outs)])
    torch.cuda.synchronize()
    for s, out in zip(variants, outs):
        ctx.upload(s)
        ref = ctx.render(s, sample_offset=4)
        got = out.cpu().numpy()
        assert np.isfinite(got).all() and got.mean() > 0
        if s.settings.mode == A.PR_MODE_WAVEFRONT:
            assert np.array_equal(got, ref)
        else:
            np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-6)
    for o in objs:
        o.release()


def test_autotuner_keeps_the_image(ctx):
    s = scenes.mesh_cornell(width=96, height=72, samples=2, supersamples=2, subdiv=5)
    s.settings.mode = A.PR_MODE_WAVEFRONT
    ctx.upload(s)
    before = ctx.render(s)
    t = ctx.autotune(s)
    print("autotuned:", t)
    assert t["slots"] in (1 << 19, 1 << 20, 1 << 21, 1 << 22) and t["trace_blocks_per_sm"] in (4, 8, 16)
    after = ctx.render(s)
    assert np.array_equal(before, after)


def test_batch_of_media_bssrdf_variants_matches_oracle_statistically(ctx, golden):
    """Three variants of the batched workload (global HG medium, 20,480-
    triangle directional-dipole icosphere) at uneven sizes, rendered together
    by pr_render_batch, 16 batches of 256 spp, against the oracle's 16 x 256
    spp per variant (the oracle is bit-exact with the reference on these
    variants, one thread): per-pixel 3 sigma with both sides' spreads, RMSE at
    the noise level, mean within 1 %."""
    import torch
    import batch_cases
    variants = batch_cases.highspp_variants()
    objs = [ctx.scene_object(s) for s in variants]
    outs = [torch.zeros((s.camera.height, s.camera.width, 3), dtype=torch.float32, device="cuda:0") for s in variants]
    nb, spp = 16, variants[0].settings.spp
    acc = [[] for _ in variants]
    for b in range(nb):
        ctx.render_batch([(o, out, None, None, b * spp) for o, out in zip(objs, outs)])
        torch.cuda.synchronize()
        for i, out in enumerate(outs):
            acc[i].append(out.cpu().numpy().astype(np.float64))
    orc = golden["batch_oracle"]
    o_nb = int(orc["batches"])
    for i, s in enumerate(variants):
        bt = np.stack(acc[i])
        mean, sd = bt.mean(0), bt.std(0, ddof=1)
        o_mean = orc[f"v{i}_mean"].astype(np.float64)
        o_sd = orc[f"v{i}_sd"].astype(np.float64)
        sigma = np.sqrt(sd ** 2 / nb + o_sd ** 2 / o_nb) + 1e-7
        frac = float((np.abs(mean - o_mean) / sigma > 3.0).mean())
        rmse = float(np.sqrt(((mean - o_mean) ** 2).mean()))
        noise = float(np.sqrt((sigma ** 2).mean()))
        rel = abs(mean.mean() - o_mean.mean()) / o_mean.mean()
        print(f"batch variant {i} ({s.camera.width}^2): >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, "
              f"mean rel diff {rel:.4f}")
        assert rel < 0.01
        assert frac < 0.02
        assert rmse < 1.3 * noise
    for o in objs:
        o.release()
