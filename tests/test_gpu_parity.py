"""GPU parity tests, through the C ABI (ctypes), against the oracle and the
reference-generated golden fixtures.

* closest hits: entity, face id and FP64 distance bit-exact;
* QBVH built by the library equals the reference's;
* images: the GPU estimate (independent counter-based streams) agrees with
  the reference's high-spp render within 3 sigma per pixel for all but a
  small fraction of pixels, and its RMSE is at the noise level.
"""
import numpy as np
import pytest

from oracle import oracle as O
from prender_gb300 import gpu, scenes
from prender_gb300 import _abi as A

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g
    g.build_library()
    c = gpu.Context(0)
    yield c
    c.close()


def test_first_hit_golden_bit_exact(ctx, golden):
    s = scenes.mesh_cornell(width=32, height=24, samples=1, supersamples=2, subdiv=3)
    ctx.upload(s)
    g = golden["mesh_s3_qbvh_firsthit"]
    h = ctx.first_hit(g["rays"])
    assert np.array_equal(h["entity"], g["fh_entity"])
    assert np.array_equal(h["prim"], g["fh_prim"])
    assert np.array_equal(h["t"], g["fh_t"])


def test_qbvh_upload_matches_golden(ctx, golden):
    s = scenes.mesh_cornell(width=32, height=24, samples=1, supersamples=2, subdiv=3)
    ctx.upload(s)
    g = golden["mesh_s3_qbvh_firsthit"]
    q = ctx.qbvh(2)
    assert np.array_equal(q["children"], g["ico_children"])
    assert np.array_equal(q["leaf"], g["ico_leaf"])


def test_first_hit_spheres_bit_exact(ctx):
    s = scenes.cornell_spheres(width=16, height=12)
    ctx.upload(s)
    rays = np.concatenate([scenes.random_rays((2, 1, 1), (98, 80, 170), 20000, seed=11), scenes.camera_rays(s)])
    h = ctx.first_hit(rays)
    o = O.OracleScene(s).first_hit(rays)
    assert np.array_equal(h["entity"], o["entity"])
    assert np.array_equal(h["t"], o["t"])


def test_render_traversal_finds_the_exact_closest_hits(ctx):
    """The renderer's FP32 query runs on its own binned-SAH tree, not the
    reference's QBVH (which the exact path keeps): on the 327,680-triangle
    scene it must find the same entity and face as the exact FP64 first hit,
    up to near-ties at FP32 resolution."""
    s = scenes.mesh_cornell(width=96, height=72, subdiv=7)
    ctx.upload(s)
    rays = np.concatenate([scenes.random_rays((2, 1, 1), (98, 80, 170), 100000, seed=5), scenes.camera_rays(s)])
    e = ctx.first_hit(rays)
    f = ctx.trace_fast(rays)
    same_ent = e["entity"] == f["entity"]
    both = same_ent & (e["entity"] >= 0)
    mesh = both & (e["prim"] >= 0)
    same_prim = (e["prim"][mesh] == f["prim"][mesh]).mean()
    rel = np.abs(f["t"][both] - e["t"][both]) / np.maximum(e["t"][both], 1e-3)
    print(f"render traversal: entity agree {same_ent.mean():.5f}, face agree {same_prim:.5f} of {mesh.sum()}, "
          f"t rel median {np.median(rel):.2e} p99.9 {np.quantile(rel, 0.999):.2e}")
    assert same_ent.mean() >= 0.999
    assert same_prim >= 0.998
    assert np.quantile(rel, 0.999) < 1e-4


def test_first_hit_full_size_mesh_bit_exact(ctx):
    """327,680-triangle displaced icosphere (the mesh Cornell box workload)."""
    s = scenes.mesh_cornell(subdiv=7)
    ctx.upload(s)
    ico = s.meshes[1].vertices
    rays = np.concatenate([scenes.rays_toward(ico, (2, 1, 100), (98, 80, 249), 200000, seed=21),
                           scenes.random_rays((2, 1, 1), (98, 80, 249), 50000, seed=22)])
    h = ctx.first_hit(rays)
    o = O.OracleScene(s).first_hit(rays)
    assert (o["entity"] == 2).sum() > 150000
    assert np.array_equal(h["entity"], o["entity"])
    assert np.array_equal(h["prim"], o["prim"])
    assert np.array_equal(h["t"], o["t"])


def _batches(ctx, scene, nb, spp_per_batch):
    imgs = []
    for b in range(nb):
        imgs.append(ctx.render(scene, sample_offset=b * spp_per_batch).astype(np.float64))
    return np.stack(imgs)


@pytest.mark.parametrize("mode", [A.PR_MODE_MEGAKERNEL, A.PR_MODE_WAVEFRONT])
@pytest.mark.parametrize("name,build,tol_frac", [
    ("spheres_64x48_1024spp", lambda: scenes.cornell_spheres(width=64, height=48, samples=256, supersamples=2), 0.02),
    ("mesh_64x48_512spp", lambda: scenes.mesh_cornell(width=64, height=48, samples=128, supersamples=2, subdiv=3), 0.02),
    ("glass_64x48_512spp", lambda: scenes.mesh_cornell(width=64, height=48, samples=128, supersamples=2, subdiv=3,
                                                       material="glass"), 0.03),
])
def test_image_matches_reference_statistically(ctx, golden, name, build, tol_frac, mode):
    s = build()
    s.settings.mode = mode
    ctx.upload(s)
    ref = golden["render_highspp"][name].astype(np.float64)
    nb = 16
    spp = s.settings.spp
    b = _batches(ctx, s, nb, spp)
    mean = b.mean(0)
    sd_batch = b.std(0, ddof=1)                 # spread of one spp-sample estimate
    sigma = np.sqrt(sd_batch ** 2 / nb + sd_batch ** 2) + 1e-6  # GPU mean + reference (same spp as a batch)
    z = np.abs(mean - ref) / sigma
    frac = float((z > 3.0).mean())
    rmse = float(np.sqrt(((mean - ref) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel_mean = abs(mean.mean() - ref.mean()) / ref.mean()
    print(f"{name} mode {mode}: >3sigma fraction {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, mean rel diff {rel_mean:.4f}")
    assert rel_mean < 0.01
    assert frac < tol_frac
    assert rmse < 1.3 * noise


@pytest.mark.parametrize("mode", [A.PR_MODE_MEGAKERNEL, A.PR_MODE_WAVEFRONT])
def test_subsurface_image_matches_reference_statistically(ctx, golden, mode):
    """Directional-dipole BSSRDF in both forms, 16 x 512 spp.

    Against the oracle's 16 x 512 spp (the oracle is bit-exact with the
    reference on one thread): both sides are 8192-spp means with measured
    per-pixel spreads, so the per-pixel test is symmetric; two halves of the
    oracle's own batches score 0.6-0.7 % beyond 3 sigma.  Against the
    reference's single 512 spp render the subsurface paths' fireflies sit on
    one side: the oracle's 8192-spp mean itself scores 3.2 % of pixels beyond
    3 sigma there (all with the image above the mean), so that comparison is
    bounded at 5 %, with its mean and RMSE held to the usual bars."""
    s = scenes.sss_cornell(width=64, height=48, samples=128, supersamples=2, subdiv=3)
    s.settings.mode = mode
    ctx.upload(s)
    nb, spp = 16, s.settings.spp
    b = _batches(ctx, s, nb, spp)
    mean = b.mean(0)
    sd = b.std(0, ddof=1)
    orc = golden["sss_oracle"]
    o_mean = orc["mean_64x48_8192spp"].astype(np.float64)
    o_sd = orc["sd_64x48_512spp"].astype(np.float64)
    o_nb = int(orc["batches"])
    sigma = np.sqrt(sd ** 2 / nb + o_sd ** 2 / o_nb) + 1e-6
    frac = float((np.abs(mean - o_mean) / sigma > 3.0).mean())
    rmse = float(np.sqrt(((mean - o_mean) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - o_mean.mean()) / o_mean.mean()
    print(f"subsurface vs oracle 8192 spp: >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, "
          f"mean rel diff {rel:.4f}")
    assert rel < 0.01
    assert frac < 0.02
    assert rmse < 1.3 * noise
    ref = golden["sss_render"]["sss_64x48_512spp"].astype(np.float64)
    sigma = np.sqrt(sd ** 2 / nb + sd ** 2) + 1e-6
    frac = float((np.abs(mean - ref) / sigma > 3.0).mean())
    rmse = float(np.sqrt(((mean - ref) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - ref.mean()) / ref.mean()
    print(f"subsurface vs reference 512 spp: >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, "
          f"mean rel diff {rel:.4f}")
    assert rel < 0.01
    assert frac < 0.05
    assert rmse < 1.3 * noise


def test_render_is_deterministic_and_shards_by_sample_offset(ctx):
    s = scenes.mesh_cornell(width=48, height=36, samples=8, supersamples=2, subdiv=3)
    ctx.upload(s)
    a = ctx.render(s)
    b = ctx.render(s)
    assert np.array_equal(a, b)
    # two shards of the same frame (sample ranges [0,16) and [16,32)) sum to it;
    # total_spp keeps the frame's per-sample weight, hence the same clamp
    half = scenes.mesh_cornell(width=48, height=36, samples=4, supersamples=2, subdiv=3).settings
    half.total_spp = s.settings.spp
    h0 = ctx.render(s, settings=half, sample_offset=0)
    h1 = ctx.render(s, settings=half, sample_offset=16)
    np.testing.assert_allclose(h0 + h1, a, rtol=1e-5, atol=1e-7)


def test_device_loop_cap_reports_an_error(ctx):
    s = scenes.cornell_spheres(width=16, height=12, samples=1, supersamples=1)
    ctx.upload(s)
    st = s.settings
    st.max_path_vertices = 1
    with pytest.raises(gpu.PrenderError) as e:
        ctx.render(s, settings=st)
    assert e.value.code == A.PR_E_DEVICE and "loop-cap" in str(e.value)
    st.max_path_vertices = 0
    img = ctx.render(s, settings=st)  # the context stays usable
    assert np.isfinite(img).all()


def test_bad_arguments_are_errors(ctx):
    s = scenes.cornell_spheres(width=16, height=12)
    ctx.upload(s)
    st = s.settings
    st.samples = 0
    with pytest.raises(gpu.PrenderError) as e:
        ctx.render(s, settings=st)
    assert e.value.code == A.PR_E_ARG
    bad = scenes.cornell_spheres()
    bad.entities[0].material = 99
    with pytest.raises(gpu.PrenderError) as e:
        ctx.upload(bad)
    assert e.value.code == A.PR_E_SCENE


@pytest.mark.parametrize("name,build", [
    ("spheres_glass_split", lambda: scenes.cornell_spheres(width=48, height=36, samples=4, supersamples=2)),
    ("mesh_nee", lambda: scenes.mesh_cornell(width=48, height=36, samples=4, supersamples=2, subdiv=4)),
    ("mesh_glass", lambda: scenes.mesh_cornell(width=48, height=36, samples=4, supersamples=2, subdiv=4,
                                               material="glass")),
    ("media_hg", lambda: scenes.media_cornell(width=48, height=36, samples=4, supersamples=2, g=0.5)),
    ("sss_dipole", lambda: scenes.sss_cornell(width=48, height=36, samples=4, supersamples=2, subdiv=3)),
    ("sss_level_minus1", lambda: scenes.sss_cornell(width=48, height=36, samples=4, supersamples=2, subdiv=3,
                                                    level=-1)),
    ("media_bssrdf", lambda: scenes.media_batch(n=1, seed=3, sizes=(48,), samples=4, supersamples=2, subdiv=4)[0]),
])
def test_wavefront_equals_megakernel(ctx, name, build):
    """Both forms shade with the same code and the same per-branch streams, so
    they trace identical paths; only float summation order differs."""
    s = build()
    ctx.upload(s)
    s.settings.mode = A.PR_MODE_MEGAKERNEL
    mk = ctx.render(s)
    s.settings.mode = A.PR_MODE_WAVEFRONT
    wf = ctx.render(s)
    wf2 = ctx.render(s)
    assert np.array_equal(wf, wf2)  # fixed-point accumulation: order-independent
    np.testing.assert_allclose(wf, mk, rtol=2e-4, atol=2e-6)


@pytest.mark.parametrize("mode", [A.PR_MODE_MEGAKERNEL, A.PR_MODE_WAVEFRONT])
def test_subsurface_level_minus1_matches_oracle_statistically(ctx, golden, mode):
    """Level -1 subsurface material (half the accepted entries take the
    dipole, half the single-scattering walk through the object with its two
    radiance bounds) in both forms, 16 x 512 spp, against the oracle's
    16 x 512 spp (the oracle is bit-exact with the reference on one thread)."""
    s = scenes.sss_cornell(width=64, height=48, samples=128, supersamples=2, subdiv=3, level=-1)
    s.settings.mode = mode
    ctx.upload(s)
    nb, spp = 16, s.settings.spp
    b = _batches(ctx, s, nb, spp)
    mean = b.mean(0)
    sd = b.std(0, ddof=1)
    orc = golden["sss_l1_oracle"]
    o_mean = orc["mean_64x48_8192spp"].astype(np.float64)
    o_sd = orc["sd_64x48_512spp"].astype(np.float64)
    o_nb = int(orc["batches"])
    sigma = np.sqrt(sd ** 2 / nb + o_sd ** 2 / o_nb) + 1e-6
    frac = float((np.abs(mean - o_mean) / sigma > 3.0).mean())
    rmse = float(np.sqrt(((mean - o_mean) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - o_mean.mean()) / o_mean.mean()
    print(f"subsurface level -1 vs oracle 8192 spp: >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, "
          f"mean rel diff {rel:.4f}")
    assert rel < 0.01
    assert frac < 0.02
    assert rmse < 1.3 * noise


def test_eight_bit_output_matches_the_reference_formula(ctx, tmp_path):
    """Render::OutputBmp (render.h:1563-1589) with ppm.h's to_int: clamp,
    gamma 1/2.2 (or gamma_offset as the exponent), * 255 + 0.5, truncated;
    bitmap row i = image row H-1-i.  CUDA's pow may differ from the host's
    in the last bit, which moves a value across a .5 boundary at most
    rarely."""
    from prender_gb300.scene import write_bmp
    rng = np.random.default_rng(3)
    img = rng.uniform(-0.2, 1.3, (37, 53, 3)).astype(np.float32)
    img[0, 0] = (0.0, 1.0, np.nan)
    for gamma in (0.0, 0.8):
        g = 1.0 / 2.2 if gamma == 0.0 else gamma
        x = np.clip(img.astype(np.float64), 0.0, 1.0)
        ref = np.floor(np.power(x, g) * 255 + 0.5)
        ref = ref[::-1]
        out = ctx.to_rgb8(img, gamma).astype(np.float64)
        fin = np.isfinite(ref)
        diff = np.abs(out[fin] - ref[fin])
        assert diff.max() <= 1 and (diff > 0).mean() < 1e-3
    write_bmp(str(tmp_path / "out.bmp"), ctx.to_rgb8(img))
    assert (tmp_path / "out.bmp").stat().st_size == 54 + (53 * 3 + 1) * 37
    with pytest.raises(gpu.PrenderError):
        ctx.to_rgb8(img, -1.0)


@pytest.mark.parametrize("mode", [A.PR_MODE_MEGAKERNEL, A.PR_MODE_WAVEFRONT])
@pytest.mark.parametrize("mat", ["ward", "phong"])
def test_glossy_image_matches_oracle_statistically(ctx, golden, mat, mode):
    """Ward (anisotropic) and Phong glossy lobes, 16 x 512 spp, in both forms,
    against the oracle's 16 x 512 spp (bit-exact with the reference on one
    thread): per-pixel 3 sigma with both sides' spreads, RMSE at the noise
    level, image mean within 1 %."""
    import glossy_cases
    s = glossy_cases.highspp_case(mat)
    s.settings.mode = mode
    ctx.upload(s)
    nb, spp = 16, s.settings.spp
    b = _batches(ctx, s, nb, spp)
    mean = b.mean(0)
    sd = b.std(0, ddof=1)
    orc = golden["glossy_oracle"]
    o_mean = orc[f"{mat}_mean"].astype(np.float64)
    o_sd = orc[f"{mat}_sd"].astype(np.float64)
    o_nb = int(orc["batches"])
    sigma = np.sqrt(sd ** 2 / nb + o_sd ** 2 / o_nb) + 1e-6
    frac = float((np.abs(mean - o_mean) / sigma > 3.0).mean())
    rmse = float(np.sqrt(((mean - o_mean) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - o_mean.mean()) / o_mean.mean()
    print(f"{mat} mode {mode}: >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, mean rel diff {rel:.4f}")
    assert rel < 0.01
    assert frac < 0.02
    assert rmse < 1.3 * noise


def test_glossy_materials_are_refused_by_the_adjoint(ctx):
    s = scenes.mesh_cornell(width=16, height=12, samples=1, supersamples=1, subdiv=3, material="ward")
    ctx.upload(s)
    with pytest.raises(gpu.PrenderError):
        ctx.render_adjoint(np.ones((12, 16, 3), np.float32), s)


@pytest.mark.parametrize("mode", [A.PR_MODE_MEGAKERNEL, A.PR_MODE_WAVEFRONT])
@pytest.mark.parametrize("mat", ["diffuse", "glass"])
def test_benchmarked_scene_matches_oracle_statistically(ctx, golden, mat, mode):
    """The benchmarked frame's scene itself -- 12-triangle box, area light,
    327,680-triangle displaced icosphere, diffuse or glass -- at 128 x 96,
    16 x 256 spp, in both forms, against the oracle's 16 x 256 spp (the
    oracle renders through the reference's own QBVH of this mesh)."""
    s = scenes.mesh_cornell(width=128, height=96, samples=64, supersamples=2, subdiv=7, material=mat)
    s.settings.mode = mode
    ctx.upload(s)
    nb, spp = 16, s.settings.spp
    b = _batches(ctx, s, nb, spp)
    mean = b.mean(0)
    sd = b.std(0, ddof=1)
    orc = golden["mesh7_oracle"]
    o_mean = orc[f"{mat}_mean"].astype(np.float64)
    o_sd = orc[f"{mat}_sd"].astype(np.float64)
    o_nb = int(orc["batches"])
    sigma = np.sqrt(sd ** 2 / nb + o_sd ** 2 / o_nb) + 1e-6
    frac = float((np.abs(mean - o_mean) / sigma > 3.0).mean())
    rmse = float(np.sqrt(((mean - o_mean) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - o_mean.mean()) / o_mean.mean()
    print(f"subdiv-7 {mat} mode {mode}: >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, "
          f"mean rel diff {rel:.4f}")
    assert rel < 0.01
    assert frac < 0.02
    assert rmse < 1.3 * noise
