"""Path-replay adjoint (pr_render_adjoint) through the C ABI.

* against central finite differences of the GPU's own estimator with common
  random numbers (same seeds, h = 1e-3): colour channels that are not the
  material's largest (so Russian roulette probabilities do not move) and the
  light's emission agree within 1%;
* against the reference algorithm: central differences of the oracle's
  renders (the reference's estimator, its own MT19937-64 streams) of a linear
  image functional agree with the GPU adjoint within their combined
  statistical error;
* cost: one adjoint pass costs at most 3x one forward pass.
"""
import numpy as np
import pytest

from oracle import oracle as O
from prender_gb300 import gpu, scenes

pytestmark = pytest.mark.gpu

H = 1e-3


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g
    g.build_library()
    c = gpu.Context(0)
    yield c
    c.close()


def _scene(albedo=None, emission_scale=1.0, w=32, h=24, samples=16):
    return scenes.diff_cornell(w, h, samples=samples, supersamples=2, subdiv=3, albedo=albedo,
                               emission_scale=emission_scale, seed=3)


def _render(ctx, s):
    ctx.upload(s)
    return ctx.render(s).astype(np.float64)


def test_adjoint_matches_finite_differences(ctx):
    base = _scene()
    alb = np.array([m.color for m in base.materials[:8]], dtype=np.float64)
    # target: the same scene at perturbed albedo (sigma 0.1)
    rng = np.random.default_rng(5)
    target = _render(ctx, _scene(np.clip(alb + rng.normal(0, 0.1, alb.shape), 0.05, 0.95)))
    img = _render(ctx, base)
    n = img.size

    def loss(im):
        return float(((im - target) ** 2).sum() / n)

    dl = (2.0 * (img - target) / n).astype(np.float32)
    ctx.upload(base)
    g = ctx.render_adjoint(dl, base)
    checked = 0
    for m in range(8):
        for c in range(3):
            if c == int(np.argmax(alb[m])):
                continue  # the Russian-roulette probability max(C) moves with this channel
            ap, am = alb.copy(), alb.copy()
            ap[m, c] += H
            am[m, c] -= H
            fd = (loss(_render(ctx, _scene(ap))) - loss(_render(ctx, _scene(am)))) / (2 * H)
            ad = g["color"][m, c]
            print(f"material {m} channel {c}: adjoint {ad:+.6e} fd {fd:+.6e}")
            assert abs(ad - fd) <= 0.01 * abs(fd) + 1e-9, (m, c, ad, fd)
            checked += 1
    assert checked == 16
    # emission scale of the light (material 8)
    fdp = loss(_render(ctx, _scene(alb, emission_scale=1.0 + H)))
    fdm = loss(_render(ctx, _scene(alb, emission_scale=1.0 - H)))
    fd = (fdp - fdm) / (2 * H)
    print(f"emission scale: adjoint {g['emission_scale']:+.6e} fd {fd:+.6e}")
    assert abs(g["emission_scale"] - fd) <= 0.001 * abs(fd)
    # per-material emission gradient of the light, channel sum, equals the scale gradient / 36
    assert abs(g["emission"][8].sum() * 36.0 - g["emission_scale"]) <= 1e-6 * abs(g["emission_scale"])


def test_adjoint_matches_reference_estimator_gradient(ctx):
    # linear functional F = sum(w * image): dF/dC is an expectation, estimated
    # by the GPU adjoint (Philox streams) and by central differences of the
    # oracle (the reference's estimator, common MT19937-64 streams)
    base = _scene(w=24, h=18, samples=32)
    alb = np.array([m.color for m in base.materials[:8]], dtype=np.float64)
    rng = np.random.default_rng(11)
    wgt = rng.uniform(0.0, 1.0, (18, 24, 3))
    ctx.upload(base)
    nb = 8
    grads = []
    for b in range(nb):  # independent sample ranges give the GPU estimate's spread
        grads.append(ctx.render_adjoint(wgt.astype(np.float32), base, sample_offset=b * base.settings.spp)["color"])
    grads = np.array(grads)
    g_mean, g_sd = grads.mean(0), grads.std(0, ddof=1) / np.sqrt(nb)

    def F(a):
        img, _, _ = O.OracleScene(_scene(a, w=24, h=18, samples=32)).render(threads=1)
        return float((wgt * img).sum())

    for m, c in [(0, int(np.argmin(alb[0]))), (2, int(np.argmin(alb[2]))), (5, int(np.argmin(alb[5])))]:
        ap, am = alb.copy(), alb.copy()
        ap[m, c] += H
        am[m, c] -= H
        fd = (F(ap) - F(am)) / (2 * H)
        ad = g_mean[m, c]
        print(f"material {m} channel {c}: GPU adjoint {ad:+.5e} +- {g_sd[m, c]:.1e}, reference FD {fd:+.5e}")
        # the oracle FD has about the spread of one GPU batch (same spp)
        tol = 4.0 * np.sqrt(g_sd[m, c] ** 2 + (g_sd[m, c] * np.sqrt(nb)) ** 2) + 0.02 * abs(fd)
        assert abs(ad - fd) <= tol


def test_adjoint_costs_at_most_three_forward_passes(ctx):
    s = scenes.diff_cornell(256, 256, samples=4, supersamples=2, subdiv=5, seed=1)
    ctx.upload(s)
    img = ctx.render(s)
    ctx.render(s)
    fwd = ctx.stats()["device_ms"]
    dl = np.ones_like(img)
    ctx.render_adjoint(dl, s)
    ctx.render_adjoint(dl, s)
    adj = ctx.stats()["device_ms"]
    print(f"forward {fwd:.2f} ms, adjoint {adj:.2f} ms, ratio {adj / fwd:.2f}")
    assert adj <= 3.0 * fwd


def test_adjoint_rejects_what_it_does_not_cover(ctx):
    s = scenes.media_cornell(width=16, height=12, samples=1, supersamples=1)
    ctx.upload(s)
    with pytest.raises(gpu.PrenderError):
        ctx.render_adjoint(np.zeros((12, 16, 3), np.float32), s)
