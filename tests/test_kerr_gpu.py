"""Kerr geodesic tracer on the GPU (pr_kerr_trace and Kerr renders), through
the C ABI, against the reference's own outputs (golden vectors) and the FP64
oracle.

The kernel runs the reference's FP64 arithmetic in the reference's order
(no FMA contraction); the GPU's sin / cos / acos / atan2 / pow may differ
from the host libm in the last bit, so a ray whose step control sits on a
knife edge may take another step sequence.  Bars: status equal on >= 99.5%
of rays, exit direction within 1e-6 rad on >= 99.5% of the rays that leave
or end on an entity (every ray beyond that bar is counted and printed with
its angle), every ray whose status agrees within 1e-3 rad, hit entities
equal where both hit.
"""
import os

import numpy as np
import pytest

import kerr_cases
from oracle import oracle as O
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


def _angle(a, b):
    a = a / np.linalg.norm(a, axis=1, keepdims=True)
    b = b / np.linalg.norm(b, axis=1, keepdims=True)
    c = np.clip((a * b).sum(1), -1.0, 1.0)
    # small angles: |a x b| is better conditioned than acos
    return np.arctan2(np.linalg.norm(np.cross(a, b), axis=1), c)


def _compare(k, st_ref, dir_ref, ent_ref, label):
    same = k["status"] == st_ref
    # a ray that starts inside the horizon never enters the step loop: the
    # reference records no direction for it
    valid = np.linalg.norm(dir_ref, axis=1) > 0
    assert np.array_equal(valid, np.linalg.norm(k["exit_dir"], axis=1) > 0) or not valid.all()
    ang = np.zeros(len(st_ref))
    ang[valid] = _angle(k["exit_dir"][valid], dir_ref[valid])
    # exit directions of rays that leave (background) or end on an entity;
    # a ray that stalls at the horizon (step underflow) or crosses it has no
    # exit direction, only its status
    out = np.isin(st_ref, (0, 1, 5)) & valid
    frac_dir = float((ang[out] <= 1e-6).mean()) if out.any() else 1.0
    worst = ang[same & out].max() if (same & out).any() else 0.0
    beyond = np.flatnonzero(out & (ang > 1e-6))
    print(f"{label}: status agree {same.mean():.5f}, exit dir <=1e-6 rad {frac_dir:.5f} of {out.sum()} "
          f"({len(beyond)} beyond), max angle (same status) {worst:.3e}, "
          f"median {np.median(ang[out]) if out.any() else 0:.3e}")
    if len(beyond):
        print(f"  beyond 1e-6 rad: angles {np.sort(ang[beyond])[-8:]}, statuses {st_ref[beyond][:8]}")
    assert same.mean() >= 0.995
    assert frac_dir >= 0.995
    assert worst <= 1e-3
    both = same & (st_ref == 1)
    assert np.array_equal(k["hit_entity"][both], ent_ref[both])


@pytest.mark.parametrize("name", sorted(kerr_cases.trace_cases()))
def test_kerr_trace_matches_reference_golden(ctx, golden, name):
    g = golden["kerr_trace"]
    sc, rays = kerr_cases.trace_cases()[name]
    ctx.upload(sc)
    k = ctx.kerr_trace(g[f"{name}_rays"])
    obj, hit, rec = g[f"{name}_obj"], g[f"{name}_hit"], g[f"{name}_rec"]
    st = kerr_cases.status_from_reference(obj, hit, rec)
    _compare(k, st, rec[:, 11:14], obj, name)
    # rays that leave or end on an entity reproduce the reference's step
    # sequence; rays stalling at the horizon are chaotic in their step count
    out = np.isin(st, (0, 1, 5))
    assert (k["steps"][out] == rec[out, 1].astype(np.int32)).mean() >= 0.99
    st_stats = ctx.stats()
    assert st_stats["paths"] == len(rays) and st_stats["kernel_launches"] == 1


@pytest.mark.parametrize("a", [0.6, 0.999])
def test_kerr_lensing_view_matches_oracle(ctx, a):
    # the lensing configuration (camera at r = 6.03 M in the equatorial plane,
    # 60 degree field, disk r 3..15 M) at 96 x 48 rays
    s = scenes.kerr_lensing(a=a, width=96, height=48, max_steps=4000)
    rays = scenes.camera_rays(s)
    ctx.upload(s)
    k = ctx.kerr_trace(rays)
    o = O.OracleScene(s).kerr_trace(rays)
    _compare(k, o["status"], o["exit_dir"], o["hit_entity"], f"lensing a={a}")
    # escaped rays (none at a = 0.6: the view is the hole and the disk):
    # final Boyer-Lindquist r to 1e-7 relative after 4000 steps, angles to 1e-6 rad
    esc = (k["status"] == 0) & (o["status"] == 0)
    if not esc.any():
        return
    kb, ob = k["final_bl"][esc], o["final_bl"][esc]
    assert (np.abs(kb[:, 0] - ob[:, 0]) <= 1e-7 * ob[:, 0]).mean() >= 0.99
    dphi = np.abs((kb[:, 2] - ob[:, 2] + np.pi) % (2 * np.pi) - np.pi)
    assert (np.maximum(np.abs(kb[:, 1] - ob[:, 1]), dphi) <= 1e-6).mean() >= 0.99


@pytest.mark.parametrize("a", [0.6, 0.999])
def test_kerr_lensing_view_512x256_matches_oracle(ctx, a):
    """The same lensing view at 512 x 256 rays (131,072 geodesics of up to
    4000 steps each), FP64 form against the FP64 oracle."""
    s = scenes.kerr_lensing(a=a, width=512, height=256, max_steps=4000)
    rays = scenes.camera_rays(s)
    ctx.upload(s)
    k = ctx.kerr_trace(rays)
    o = O.OracleScene(s).kerr_trace(rays, threads=os.cpu_count() or 1)
    _compare(k, o["status"], o["exit_dir"], o["hit_entity"], f"lensing 512x256 a={a}")
    assert (o["status"] == 1).sum() > 1000  # the disk is in view


def test_kerr_escape_radius_option_matches_oracle(ctx):
    s = scenes.kerr_disk(32, 24, a=0.9, max_steps=4000, escape_radius=200.0)
    rays = scenes.camera_rays(s)
    ctx.upload(s)
    k = ctx.kerr_trace(rays)
    o = O.OracleScene(s).kerr_trace(rays)
    _compare(k, o["status"], o["exit_dir"], o["hit_entity"], "escape_radius 200")
    esc = o["status"] == 0
    assert esc.any() and o["steps"][esc].max() < 4000  # the option ends the escaped rays early


def test_kerr_trace_errors(ctx):
    s = scenes.cornell_spheres(width=16, height=12, samples=1, supersamples=1)
    ctx.upload(s)
    with pytest.raises(gpu.PrenderError):
        ctx.kerr_trace(np.zeros((4, 6)))  # no black hole in the scene
    s = scenes.kerr_disk(8, 6, a=0.9, max_steps=10)
    s.kerr["a"] = 1.0  # |a| must be below M
    with pytest.raises(gpu.PrenderError):
        ctx.upload(s)
    s = scenes.kerr_disk(8, 6, a=0.9, max_steps=10)
    s.settings.nee = 1  # next-event estimation along geodesics is not on this path
    ctx.upload(s)
    with pytest.raises(gpu.PrenderError):
        ctx.render(s)


def _batches(ctx, scene, nb, spp_per_batch):
    return np.stack([ctx.render(scene, sample_offset=b * spp_per_batch).astype(np.float64) for b in range(nb)])


def test_kerr_render_matches_reference_statistically(ctx, golden):
    s = kerr_cases.highspp_case()
    ctx.upload(s)
    ref = golden["kerr_render"]["texture_highspp"]
    nb, spp = 16, s.settings.spp
    b = _batches(ctx, s, nb, spp)
    mean = b.mean(0)
    sd = b.std(0, ddof=1)
    sigma = np.sqrt(sd ** 2 / nb + sd ** 2) + 1e-6
    z = np.abs(mean - ref) / sigma
    frac = float((z > 3.0).mean())
    rmse = float(np.sqrt(((mean - ref) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - ref.mean()) / ref.mean()
    print(f"kerr render: >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, mean rel diff {rel:.4f}")
    assert rel < 0.01
    assert frac < 0.03
    assert rmse < 1.3 * noise


@pytest.mark.parametrize("a", [0.6, 0.999])
def test_kerr_mixed_precision_form_against_fp64(ctx, a):
    """The mixed-precision form (PR_KERR_FP32: the reference's FP64 steps near
    the hole, FP32 h = 2 steps in the far field, captures decided from the
    radial potential) against the FP64 oracle on the lensing view: statuses
    agree (horizon and step underflow are both a capture), hits identical,
    exit directions of escaping rays within 1e-6 rad for 99% of them."""
    s = scenes.kerr_lensing(a=a, width=96, height=48, max_steps=4000)
    rays = scenes.camera_rays(s)
    o = O.OracleScene(s).kerr_trace(rays)
    s.kerr["precision"] = A.PR_KERR_FP32
    ctx.upload(s)
    k = ctx.kerr_trace(rays)
    fast = ctx.stats()
    s.kerr["precision"] = A.PR_KERR_FP64
    ctx.upload(s)
    ctx.kerr_trace(rays)
    exact = ctx.stats()
    cap = lambda st: np.where(np.isin(st, (2, 4)), 2, st)
    same = cap(k["status"]) == cap(o["status"])
    esc = (k["status"] == 0) & (o["status"] == 0)
    hit = (k["status"] == 1) & (o["status"] == 1)
    ang = _angle(k["exit_dir"][esc], o["exit_dir"][esc]) if esc.any() else np.zeros(1)
    print(f"mixed a={a}: status agree {same.mean():.4f}, escaped {esc.sum()}, exit dir median {np.median(ang):.2e} "
          f"p99 {np.quantile(ang, 0.99):.2e} rad; FP64 {exact['device_ms']:.1f} ms / {exact['tri_tests']} RK attempts, "
          f"mixed {fast['device_ms']:.1f} ms / {fast['tri_tests']}")
    assert same.mean() >= 0.995
    assert np.array_equal(k["hit_entity"][hit], o["hit_entity"][hit])
    # near-hole steps run the reference's FP64 formulas, here with FMA contraction
    assert np.abs(k["hit_t"][hit] - o["hit_t"][hit]).max() < 1e-4
    assert (ang <= 1e-6).mean() >= 0.99


def test_kerr_ray_bundle_jacobian_against_central_differences(ctx):
    """d(exit direction)/d(s, t) of the forward-mode dual-number tracer against
    central differences of the FP64 tracer (perturbed initial directions,
    h = 1e-6), for rays that leave the scene; the adjoint form equals w^T J."""
    s = scenes.kerr_disk(24, 18, a=0.9, max_steps=1500)
    rays = scenes.camera_rays(s)
    ctx.upload(s)
    n = rays.shape[0]
    rng = np.random.default_rng(4)
    w = rng.normal(size=(n, 3))
    J = ctx.kerr_sensitivity(rays, cotangent=w)
    d = rays[:, 3:] / np.linalg.norm(rays[:, 3:], axis=1, keepdims=True)
    up = np.where(np.abs(d[:, 2:3]) < 0.9, [[0.0, 0.0, 1.0]], [[1.0, 0.0, 0.0]])
    e1 = np.cross(d, up)
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(e1, d)
    h = 1e-6
    fd = np.empty((n, 3, 2))
    base = ctx.kerr_trace(rays)
    same = base["status"] == 0
    for col, e in enumerate((e1, e2)):
        outs = []
        for sgn in (1.0, -1.0):
            r = rays.copy()
            dd = d + sgn * h * e
            r[:, 3:] = dd / np.linalg.norm(dd, axis=1, keepdims=True)
            outs.append(ctx.kerr_trace(r))
        fd[:, :, col] = (outs[0]["exit_dir"] - outs[1]["exit_dir"]) / (2 * h)
        same &= (outs[0]["status"] == 0) & (outs[1]["status"] == 0)
    ok = (J["status"] == 0) & same
    assert ok.sum() > 100
    rel = np.linalg.norm((J["jac_dir"] - fd)[ok], axis=(1, 2)) / np.linalg.norm(fd[ok], axis=(1, 2))
    print(f"Kerr Jacobian vs central differences over {ok.sum()} rays: median rel {np.median(rel):.2e}, "
          f"p95 {np.quantile(rel, 0.95):.2e}")
    assert np.median(rel) < 1e-4
    assert np.quantile(rel, 0.95) < 1e-2
    assert np.isnan(J["jac_dir"][J["status"] != 0]).all()
    np.testing.assert_allclose(J["grad"][ok], np.einsum("ni,nij->nj", w[ok], J["jac_dir"][ok]), rtol=1e-12, atol=1e-14)


def test_kerr_ray_bundle_jacobian_against_oracle_differences(ctx):
    """The GPU's forward-mode Jacobian against central differences of the
    FP64 oracle (the reference's arithmetic on the CPU) at perturbed initial
    directions, h = 1e-6, for rays that leave the scene in all three traces:
    the derivative of the reference's own map, not of the GPU's tracer."""
    s = scenes.kerr_disk(24, 18, a=0.9, max_steps=1500)
    rays = scenes.camera_rays(s)
    ctx.upload(s)
    n = rays.shape[0]
    J = ctx.kerr_sensitivity(rays)
    d = rays[:, 3:] / np.linalg.norm(rays[:, 3:], axis=1, keepdims=True)
    up = np.where(np.abs(d[:, 2:3]) < 0.9, [[0.0, 0.0, 1.0]], [[1.0, 0.0, 0.0]])
    e1 = np.cross(d, up)
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(e1, d)
    h = 1e-6
    orc = O.OracleScene(s)
    threads = os.cpu_count() or 1
    fd = np.empty((n, 3, 2))
    same = orc.kerr_trace(rays, threads=threads)["status"] == 0
    for col, e in enumerate((e1, e2)):
        outs = []
        for sgn in (1.0, -1.0):
            r = rays.copy()
            dd = d + sgn * h * e
            r[:, 3:] = dd / np.linalg.norm(dd, axis=1, keepdims=True)
            outs.append(orc.kerr_trace(r, threads=threads))
        fd[:, :, col] = (outs[0]["exit_dir"] - outs[1]["exit_dir"]) / (2 * h)
        same &= (outs[0]["status"] == 0) & (outs[1]["status"] == 0)
    ok = (J["status"] == 0) & same
    assert ok.sum() > 100
    rel = np.linalg.norm((J["jac_dir"] - fd)[ok], axis=(1, 2)) / np.linalg.norm(fd[ok], axis=(1, 2))
    print(f"Kerr Jacobian vs oracle central differences over {ok.sum()} rays: median rel {np.median(rel):.2e}, "
          f"p95 {np.quantile(rel, 0.95):.2e}")
    assert np.median(rel) < 1e-4
    assert np.quantile(rel, 0.95) < 1e-2


def test_accretion_disk_shading_matches_oracle(ctx):
    """The textured disk's deterministic branch (circle.h:244-322: ISCO and
    radius cuts, disk-map texel, temperature colours, Doppler shift of colour
    and emission, alpha) at 20,000 points of the disk plane, GPU against the
    oracle: same valid set and texels, values to 1e-9 (CUDA's atan2 / cos /
    sin / pow / exp may differ from the host libm in the last bit)."""
    rng = np.random.default_rng(7)
    r = np.sqrt(rng.uniform(0.0, 16.0 ** 2, 20000))
    ph = rng.uniform(0.0, 2.0 * np.pi, r.shape)
    pts = np.stack([r * np.cos(ph), r * np.sin(ph), np.zeros_like(r)], 1)
    for temperature, doppler, a in ((False, 0.3, 0.9), (True, 0.6, 0.6), (False, 1.0, 0.999)):
        s = kerr_cases.disk_scene(16, 8, a=a, temperature=temperature, doppler=doppler)
        ctx.upload(s)
        g = ctx.kerr_disk_shade(0, pts)
        o = O.OracleScene(s).kerr_disk_shade(0, pts)
        v = o["valid"] == 1
        print(f"disk shade a={a} temperature={temperature}: {v.sum()} valid, max |dcolour| "
              f"{np.abs(g['color'] - o['color']).max():.2e}, max |demission| {np.abs(g['emission'] - o['emission']).max():.2e}")
        assert v.sum() > 2000
        assert np.array_equal(g["valid"], o["valid"])
        assert np.abs(g["color"] - o["color"]).max() < 1e-9
        assert np.abs(g["emission"] - o["emission"]).max() < 1e-9
        assert np.abs(g["alpha"] - o["alpha"]).max() < 1e-9


@pytest.mark.parametrize("precision", [A.PR_KERR_FP64, A.PR_KERR_FP32])
def test_accretion_disk_render_matches_oracle_statistically(ctx, golden, precision):
    """The textured-disk render (alpha test from the GPU's own counter-based
    stream) against the oracle's 16 x 256 spp: per-pixel 3 sigma with both
    sides' spreads, RMSE at the noise level, mean within 1 %."""
    s = kerr_cases.disk_highspp_case()
    s.kerr["precision"] = precision
    ctx.upload(s)
    orc = golden["kerr_disk_oracle"]
    o_mean = orc["mean"].astype(np.float64)
    o_sd = orc["sd"].astype(np.float64)
    o_nb = int(orc["batches"])
    nb, spp = 16, s.settings.spp
    b = _batches(ctx, s, nb, spp)
    mean = b.mean(0)
    sd = b.std(0, ddof=1)
    sigma = np.sqrt(sd ** 2 / nb + o_sd ** 2 / o_nb) + 1e-6
    frac = float((np.abs(mean - o_mean) / sigma > 3.0).mean())
    rmse = float(np.sqrt(((mean - o_mean) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - o_mean.mean()) / o_mean.mean()
    print(f"accretion disk render (precision {precision}): >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise "
          f"{noise:.3e}, mean rel diff {rel:.4f}")
    assert rel < 0.01
    assert frac < 0.02
    assert rmse < 1.3 * noise


def test_accretion_disk_jacobian_is_refused(ctx):
    s = kerr_cases.disk_scene(8, 4)
    ctx.upload(s)
    with pytest.raises(gpu.PrenderError):
        ctx.kerr_sensitivity(scenes.camera_rays(s))
