"""The CPU oracle against golden vectors produced by the reference renderer
itself (tests/golden/make_golden.py).  Integer and FP64 results are compared
bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O
from prender_gb300 import scenes


@pytest.fixture(scope="module")
def mesh_s3():
    s = scenes.mesh_cornell(width=32, height=24, samples=1, supersamples=2, subdiv=3)
    return s, O.OracleScene(s)


@pytest.mark.parametrize("ent,prefix", [(0, "box"), (2, "ico")])
def test_qbvh_structure_matches_reference(golden, mesh_s3, ent, prefix):
    g = golden["mesh_s3_qbvh_firsthit"]
    q = mesh_s3[1].qbvh(ent)
    valid = (q["children"] != -1)[:, None, :]
    boxes = np.where(valid, q["boxes"].reshape(-1, 6, 4), np.float32(0)).reshape(-1, 24)
    assert np.array_equal(q["children"], g[f"{prefix}_children"])
    assert np.array_equal(q["axes"], g[f"{prefix}_axes"])
    assert np.array_equal(q["leaf"], g[f"{prefix}_leaf"])
    assert np.array_equal(boxes, g[f"{prefix}_boxes"])


def test_first_hit_bit_exact(golden, mesh_s3):
    g = golden["mesh_s3_qbvh_firsthit"]
    h = mesh_s3[1].first_hit(g["rays"])
    assert np.array_equal(h["entity"], g["fh_entity"])
    assert np.array_equal(h["prim"], g["fh_prim"])
    assert np.array_equal(h["t"], g["fh_t"])
    assert (g["fh_entity"] == 2).sum() > 200  # the rays do reach the icosphere


@pytest.mark.parametrize("name,build", [
    ("spheres", lambda: scenes.cornell_spheres(width=16, height=12, samples=1, supersamples=1)),
    ("mesh_diffuse", lambda: scenes.mesh_cornell(width=16, height=12, samples=1, supersamples=1, subdiv=3)),
    ("mesh_glass", lambda: scenes.mesh_cornell(width=16, height=12, samples=1, supersamples=1, subdiv=3,
                                               material="glass")),
    ("media_g05", lambda: scenes.media_cornell(width=16, height=12, samples=1, supersamples=1, g=0.5)),
])
def test_radiance_roots_bit_exact(golden, name, build):
    g = golden["radiance_roots"]
    sc = build()
    out = O.OracleScene(sc).radiance(g[f"{name}_rays"], 7)
    assert np.array_equal(out, g[f"{name}_rgb"])


@pytest.mark.parametrize("name,build", [
    ("spheres", lambda: scenes.cornell_spheres(width=24, height=18, samples=2, supersamples=2)),
    ("mesh_nee", lambda: scenes.mesh_cornell(width=24, height=18, samples=1, supersamples=2, subdiv=3)),
    ("media_g05", lambda: scenes.media_cornell(width=16, height=12, samples=1, supersamples=2, g=0.5)),
])
def test_render_one_thread_bit_exact(golden, name, build):
    sc = build()
    img, _, _ = O.OracleScene(sc).render(threads=1)
    assert np.array_equal(img, golden["render_1thread"][name])


def test_high_spp_goldens_are_converged(golden):
    # sanity of the statistical fixtures: finite, non-negative, lit
    for k in golden["render_highspp"].files:
        img = golden["render_highspp"][k]
        assert np.isfinite(img).all() and (img >= 0).all() and img.mean() > 1e-3


def test_subsurface_render_one_thread_bit_exact(golden):
    # directional-dipole BSSRDF (level -2): probe rays, dipole, exit NEE,
    # the Fresnel-surface branch and the radiance bounds, against the reference
    sc = scenes.sss_cornell(width=24, height=18, samples=1, supersamples=2, subdiv=3)
    img, _, _ = O.OracleScene(sc).render(threads=1)
    ref = golden["sss_render"]["sss_1thread"]
    assert np.array_equal(img, ref)
    assert ref.mean() > 0


def test_subsurface_oracle_fixture_agrees_with_reference_render(golden):
    # the oracle's 16 x 512 spp subsurface fixture against the reference's own
    # 512 spp render: same mean, RMSE at the noise level (the per-pixel tail
    # is one-sided, reference fireflies, so only the aggregate is bounded here)
    orc = golden["sss_oracle"]
    mean = orc["mean_64x48_8192spp"].astype(np.float64)
    sd = orc["sd_64x48_512spp"].astype(np.float64)
    nb = int(orc["batches"])
    ref = golden["sss_render"]["sss_64x48_512spp"].astype(np.float64)
    sigma = np.sqrt(sd ** 2 / nb + sd ** 2) + 1e-6
    assert abs(mean.mean() - ref.mean()) / ref.mean() < 0.01
    assert np.sqrt(((mean - ref) ** 2).mean()) < 1.3 * np.sqrt((sigma ** 2).mean())


@pytest.mark.parametrize("name", ["l1_g0", "l1_g05", "l1_nonee"])
def test_subsurface_level_minus1_render_one_thread_bit_exact(golden, name):
    # level -1: half the accepted entries take the dipole, half the
    # single-scattering walk radiance_through_media (distance sampling,
    # phase-function retries, exit refraction with next-event samples)
    import sss_cases
    sc = sss_cases.l1_cases()[name]
    img, _, _ = O.OracleScene(sc).render(threads=1)
    ref = golden["sss_l1_render"][name]
    assert np.array_equal(img, ref)
    assert ref.mean() > 0


@pytest.mark.parametrize("name", ["ward_nee1", "ward_nee0", "phong_nee1", "phong_nee0"])
def test_glossy_render_one_thread_bit_exact(golden, name):
    # Ward (anisotropic half-vector sampling, weight (h.i)(h.n)^3 sqrt(o.n / i.n))
    # and Phong (cos^n lobe about the mirror direction, diffuse with
    # probability roughness) with next-event samples evaluated by the lobe
    import glossy_cases
    sc = glossy_cases.one_thread_cases()[name]
    img, _, _ = O.OracleScene(sc).render(threads=1)
    ref = golden["glossy_render"][name]
    assert np.array_equal(img, ref)
    assert ref.mean() > 0


@pytest.mark.parametrize("name", ["spot", "spot_media", "parallel", "parallel_nonee", "infinity", "sss_spot",
                                  "infinity_raw"])
def test_light_kinds_render_one_thread_bit_exact(golden, name):
    # spot (cone falloff, attenuation, the sampled point's cosine), parallel
    # (uvplane and sphere emitters, the plane's own normal by default) and
    # infinity lights (no point drawn, visible iff nothing is hit, a
    # direction used as given), in NEE, the no-NEE sampling of those kinds,
    # media NEE, the perfect-direction term of mirrors and glass through the
    # entity's registration index into the sorted list, and both subsurface
    # exits (the dipole's no-NEE samples at its entry point)
    import lights_cases
    sc = lights_cases.one_thread_cases()[name]
    img, _, _ = O.OracleScene(sc).render(threads=1)
    ref = golden["lights_render"][name]
    assert np.array_equal(img, ref)
    assert ref.mean() > 0


@pytest.mark.parametrize("name", ["tex_maps", "ibl_dome", "ibl_nonee", "ibl_panoramic", "bump", "bump_nonee"])
def test_texture_render_one_thread_bit_exact(golden, name):
    # textures on spheres in every mapping (spherical with repeat,
    # equirectangular, angular, panoramic, hemisphere_map), on a Ward sphere
    # (specular from the texel), a uvplane and a hemisphere; IBL domes from an
    # HDR image (angular map) and bitmaps (panoramic, equirectangular,
    # hemisphere_map, a uvplane) whose hits return their emission; bump maps
    # on diffuse, Ward and mirror surfaces, NEE on and off
    import texture_cases
    sc = texture_cases.one_thread_cases()[name]
    img, _, _ = O.OracleScene(sc).render(threads=1)
    ref = golden["textures_render"][name]
    assert np.array_equal(img, ref)
    assert ref.mean() > 0


@pytest.mark.parametrize("name", ["mlt_spheres", "mlt_caustic", "mlt_glossy", "mlt_media"])
def test_mlt_render_one_thread_bit_exact(golden, name):
    # Render::RunMLT: two Kelemen chains per scene (seed paths, luminance-
    # drawn start, lazy small steps, large steps, the stack a rejection
    # restores, the light choice and surface NEE points from the stream
    # itself), NEE on and off, glossy lobes and a textured floor, the global
    # medium
    import mlt_cases
    sc = mlt_cases.one_thread_cases()[name]
    img = O.OracleScene(sc).render_mlt()
    ref = golden["mlt_render"][name]
    assert np.array_equal(img, ref)
    assert ref.mean() > 0


@pytest.mark.parametrize("name", ["smooth", "smooth_nonee", "mesh_tex", "mesh_tex_nonee", "obj_mtl", "obj_mtl_nonee"])
def test_mesh_smooth_and_texture_render_one_thread_bit_exact(golden, name):
    # 'smooth 1' meshes (vertex normals by the loader's rule and from vn
    # lines, glass, normal -1), textured meshes through vt lines (a texture
    # on diffuse and Phong meshes, an IBL image, a bump map that the mesh
    # hit drops), NEE on and off
    import meshtex_cases
    sc = meshtex_cases.one_thread_cases()[name]
    img, _, _ = O.OracleScene(sc).render(threads=1)
    ref = golden["meshtex_render"][name]
    assert np.array_equal(img, ref)
    assert ref.mean() > 0


@pytest.mark.parametrize("name", ["worm_bg", "worm_objects", "worm_sign"])
def test_wormhole_render_one_thread_bit_exact(golden, name):
    # the Dneg wormhole: both backgrounds seen through the throat, objects
    # near both mouths (emissive, diffuse, mirror), the side forced by 'sign'
    # with non-default map coefficients and no image on the far side
    import wormhole_cases
    sc = wormhole_cases.one_thread_cases()[name]
    img, _, _ = O.OracleScene(sc).render(threads=1)
    ref = golden["wormhole_render"][name]
    assert np.array_equal(img, ref)
    assert ref.mean() > 0


def test_wormhole_trace_threads_agree():
    # per-ray traces are independent: any thread count gives the same rays
    import wormhole_cases
    from prender_gb300 import scenes
    sc = wormhole_cases.build("worm_objects", 16, 12, 1, 1, max_steps=200)
    rays = scenes.camera_rays(sc)
    o = O.OracleScene(sc)
    a, b = o.wormhole_trace(rays, threads=1), o.wormhole_trace(rays, threads=4)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert set(np.unique(a["status"])) <= {0, 1, 3} and (a["status"] == 1).any()


def _media_cases():
    import media_cases
    return media_cases


@pytest.mark.parametrize("name", ["g_m06_s005", "g_0_s05", "g_05_s005_nonee", "g_08_s05", "rgb",
                                  "g_05_s005_nocut", "g_m06_s05_nocut"])
def test_media_render_one_thread_bit_exact(golden, name):
    # participatingMedia_radiance (ParticipatingMedia.h:300-461): scalar
    # sigma_t distance sampling, RGB transmittance, the phase channel drawn
    # per vertex, sampleHG's (g/2) cosine, media NEE -- over g from -0.6 to
    # 0.8, sigma_s 0.05 and 0.5, NEE on and off, and a per-channel medium
    mc = _media_cases()
    sc = mc.one_thread_cases()[name]
    img, _, _ = O.OracleScene(sc).render(threads=1)
    ref = golden["media_render"][f"render_{name}"]
    assert np.array_equal(img, ref)
    assert ref.mean() > 0


@pytest.mark.parametrize("name", ["g_m06_s005", "g_08_s05", "rgb"])
def test_media_radiance_roots_bit_exact(golden, name):
    mc = _media_cases()
    sc = mc.root_cases()[name]
    g = golden["media_render"]
    out = O.OracleScene(sc).radiance(g[f"roots_{name}_rays"], 7)
    assert np.array_equal(out, g[f"roots_{name}_rgb"])


def _hg_cdf(mu, g):
    """CDF of the Henyey-Greenstein cosine, p(mu) = (1-g^2) / (2 (1+g^2-2 g mu)^1.5)"""
    return (1.0 - g * g) / (2.0 * g) * (1.0 / np.sqrt(1.0 + g * g - 2.0 * g * mu) - 1.0 / (1.0 + g))


@pytest.mark.parametrize("g", [-0.6, 0.3, 0.8])
def test_hg_sampling_modes(g):
    """The oracle's sampleHG: with PR_FLAG_HG_CORRECT the cosine to the
    incoming direction follows the HG distribution; the reference's own form
    (sampler.h:55-56, (1.0/2.0*g) read as g/2) gives g^2 times an HG cosine.
    Kolmogorov-Smirnov distance on 200,000 draws each."""
    d = np.array([0.3, -0.5, 0.8])
    d /= np.linalg.norm(d)
    n = 200000
    crit = 1.95 / np.sqrt(n)  # KS at about the 0.1 % level
    cos_c = np.sort(O.sample_hg(g, True, 5, d, n) @ d)
    emp = np.arange(1, n + 1) / n
    assert np.max(np.abs(emp - _hg_cdf(np.clip(cos_c, -1, 1), g))) < crit
    cos_q = np.sort(O.sample_hg(g, False, 5, d, n) @ d)
    assert np.abs(cos_q).max() <= g * g + 1e-9
    assert np.max(np.abs(emp - _hg_cdf(np.clip(cos_q / (g * g), -1, 1), g))) < crit


@pytest.mark.parametrize("name", ["variant0", "variant1"])
def test_batch_variant_render_one_thread_bit_exact(golden, name):
    # the batched workload's variants: a global HG medium around a
    # 20,480-triangle directional-dipole BSSRDF icosphere
    import batch_cases
    sc = batch_cases.one_thread_cases()[name]
    img, _, _ = O.OracleScene(sc).render(threads=1)
    ref = golden["batch_render"][name]
    assert np.array_equal(img, ref)
    assert ref.mean() > 0
