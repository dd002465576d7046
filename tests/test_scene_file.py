"""The scene-file reader (pr_scene_file_load), on the CPU.

* Scene files in the reference's format, written by hand to cover its
  reader's rules (expressions over VAR variables, TARGET_POS, CAMERA_MATRIX,
  transforms, OBJ quads and vertex normals, the global medium, subsurface
  materials, the black hole with textures), read by this library and
  rendered by the oracle, equal bit for bit the reference's own renders of
  the same files (tests/golden/scene_files.npz, made by
  tests/golden/make_golden.py --scene-files-only).
* Scenes built in Python and written with Scene.write_reference read back
  into the same scene description.
* The expression rules, the OBJ face forms, BMP rows and the refusals.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from prender_gb300 import _abi as A
from prender_gb300 import scene_file, scenes
from prender_gb300.scene import write_bmp

HERE = os.path.dirname(os.path.abspath(__file__))
SCENE_DIR = os.path.join(HERE, "golden", "scene_files")
SCENE_FILES = ("spheres_expr", "mesh_obj", "media", "sss", "kerr_disk")


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build_library()
    O.build()


@pytest.mark.parametrize("name", SCENE_FILES)
def test_scene_file_renders_like_the_reference(golden, name):
    s = scene_file.load(os.path.join(SCENE_DIR, name + ".txt"))
    img, _, _ = O.OracleScene(s).render(threads=1)
    ref = golden["scene_files"][name]
    assert ref.mean() > 0
    assert np.array_equal(img, ref)


def _written_cases():
    import glossy_cases
    import kerr_cases
    out = {
        "spheres": scenes.cornell_spheres(width=24, height=18, samples=2, supersamples=2),
        "mesh": scenes.mesh_cornell(width=24, height=18, samples=1, supersamples=2, subdiv=3),
        "media": scenes.media_cornell(width=16, height=12, samples=1, supersamples=2, g=0.5),
        "sss": scenes.sss_cornell(width=16, height=12, samples=1, supersamples=1),
        "sss_l1": scenes.sss_cornell(width=16, height=12, samples=1, supersamples=1, level=-1),
        "kerr_disk": kerr_cases.disk_scene(16, 8, a=0.6, temperature=True, doppler=0.6),
    }
    out.update({"glossy_" + k: v for k, v in glossy_cases.one_thread_cases().items()})
    import lights_cases
    import texture_cases
    out.update({"lights_" + k: v for k, v in lights_cases.one_thread_cases().items()})
    out.update({"tex_" + k: v for k, v in texture_cases.one_thread_cases().items()})
    import wormhole_cases
    out.update(wormhole_cases.one_thread_cases())
    import meshtex_cases
    out.update({"meshtex_" + k: v for k, v in meshtex_cases.one_thread_cases().items()})
    return out


@pytest.mark.parametrize("name", list(_written_cases()))
def test_written_scene_reads_back_the_same(tmp_path, name):
    s = _written_cases()[name]
    back = scene_file.load(s.write_reference(str(tmp_path)))
    assert back.materials == s.materials
    assert back.entities == s.entities
    assert len(back.meshes) == len(s.meshes)
    for a, b in zip(back.meshes, s.meshes):
        assert np.array_equal(a.vertices, b.vertices) and np.array_equal(a.faces, b.faces)
        for f in ("vertex_normals", "face_vn", "uv", "face_uv"):
            x, y = getattr(a, f), getattr(b, f)
            assert (x is None) == (y is None), f
            if x is not None:
                assert np.array_equal(x, y), f
        # a mesh with vn lines gets its face normals from them in the reader
        assert (a.face_normals is None) == (b.vertex_normals is None)
        assert (a.obj_materials is None) == (b.obj_materials is None)
        if b.obj_materials is not None:
            assert np.array_equal(a.face_material, b.face_material)
            for x, y in zip(a.obj_materials, b.obj_materials):
                yc, xc = y.to_c([]), x.to_c([])
                for f in ("diffuse", "specular", "emission", "ward"):
                    assert list(getattr(xc, f)) == list(getattr(yc, f)), f
                for f in ("alpha", "refraction_index", "shininess", "roughness", "reflection", "smooth", "repeat"):
                    assert getattr(xc, f) == getattr(yc, f), f
                assert (x.texture is None) == (y.texture is None)
                if x.texture is not None:
                    assert np.array_equal(np.asarray(x.texture), np.asarray(y.texture))
    assert back.background == tuple(s.background) and back.environment_light == tuple(s.environment_light)
    assert back.participating_media == int(s.participating_media and s.settings.media)
    assert back.medium == s.medium
    c1, c2 = back.camera.to_c(), s.camera.to_c()
    for f, _ in A.pr_camera._fields_:
        assert np.array_equal(np.asarray(getattr(c1, f)), np.asarray(getattr(c2, f))), f
    for f in ("samples", "supersamples", "tent_filter", "depth", "depth_limit", "nee", "sensor_response"):
        assert getattr(back.settings, f) == getattr(s.settings, f), f
    # the reference holds the cut-off in a float
    assert back.settings.luminance_cutoff == float(np.float32(s.settings.luminance_cutoff))
    if s.kerr is not None:
        for k in ("position", "a", "max_steps", "map_coef", "texture_coef", "disk_temperature", "doppler_effect"):
            assert back.kerr[k] == s.kerr[k], k
        assert back.kerr["observer"] == tuple(s.camera.position)
        if s.kerr.get("disk_texture") is not None:
            assert np.array_equal(back.kerr["disk_texture"][:, :, :3], np.asarray(s.kerr["disk_texture"])[:, :, :3])
    if s.wormhole is not None:
        for k in ("in", "out", "rho", "a", "w", "max_steps", "sign", "map_coef", "texture_coef"):
            assert back.wormhole[k] == s.wormhole[k], k
        assert back.wormhole["camera"] == tuple(s.camera.position)
        for a, b in zip(s.wormhole["textures"], back.wormhole["textures"]):
            assert (a is None) == (b is None)
            if a is not None:
                assert np.array_equal(np.asarray(a), b)


@pytest.mark.parametrize("name", ["spot", "spot_media", "parallel", "parallel_nonee", "infinity", "sss_spot",
                                  "infinity_raw"])
def test_light_kind_files_render_like_the_reference(tmp_path, golden, name):
    # the files the reference rendered for lights_render.npz, read by this
    # library's reader (infinity_light, parallel_light(_dir), spot_light,
    # spot_light_dir / _angle / _falloff, spot_attenuation) and rendered by
    # the oracle
    import lights_cases
    sc = lights_cases.one_thread_cases()[name]
    s = scene_file.load(sc.write_reference(str(tmp_path)))
    img, _, _ = O.OracleScene(s).render(threads=1)
    assert np.array_equal(img, golden["lights_render"][name])


@pytest.mark.parametrize("name", ["tex_maps", "ibl_dome", "ibl_nonee", "ibl_panoramic", "bump", "bump_nonee"])
def test_texture_files_render_like_the_reference(tmp_path, golden, name):
    # the files the reference rendered for textures_render.npz (BMP textures,
    # BMP and Radiance HDR IBL images, the mappings, repeat, hemispheres),
    # read by this library's reader and rendered by the oracle
    import texture_cases
    sc = texture_cases.one_thread_cases()[name]
    s = scene_file.load(sc.write_reference(str(tmp_path)))
    for a, b in zip(sc.materials, s.materials):
        for f in ("texture", "ibl", "bump"):
            x, y = getattr(a, f), getattr(b, f)
            assert (x is None) == (y is None)
            if x is not None:
                assert np.asarray(x).dtype == y.dtype and np.array_equal(np.asarray(x), y)
    img, _, _ = O.OracleScene(s).render(threads=1)
    assert np.array_equal(img, golden["textures_render"][name])


@pytest.mark.parametrize("name", ["mlt_spheres", "mlt_caustic", "mlt_glossy", "mlt_media"])
def test_mlt_files_render_like_the_reference(tmp_path, golden, name):
    # the files the reference rendered with RunMLT for mlt_render.npz
    # (metropolisTransport, mutation, pre_sample), read by this library's
    # reader and rendered by the oracle's RunMLT
    import mlt_cases
    sc = mlt_cases.one_thread_cases()[name]
    s = scene_file.load(sc.write_reference(str(tmp_path)))
    assert s.settings.mode == A.PR_MODE_MLT and s.settings.tent_filter == 1
    assert (s.settings.mutation, s.settings.pre_sample) == (sc.settings.mutation, sc.settings.pre_sample)
    img = O.OracleScene(s).render_mlt()
    assert np.array_equal(img, golden["mlt_render"][name])


@pytest.mark.parametrize("name", ["smooth", "smooth_nonee", "mesh_tex", "mesh_tex_nonee", "obj_mtl", "obj_mtl_nonee"])
def test_mesh_texture_files_render_like_the_reference(tmp_path, golden, name):
    # the files the reference rendered for meshtex_render.npz (OBJ vn / vt
    # lines and their face ids, 'smooth 1', textures, IBL images and bump
    # maps on meshes), read by this library's reader and rendered by the oracle
    import meshtex_cases
    sc = meshtex_cases.one_thread_cases()[name]
    s = scene_file.load(sc.write_reference(str(tmp_path)))
    assert [e.smooth for e in s.entities] == [e.smooth for e in sc.entities]
    img, _, _ = O.OracleScene(s).render(threads=1)
    assert np.array_equal(img, golden["meshtex_render"][name])


def test_obj_texture_ids_quads_and_transforms(tmp_path):
    # quads split as (a, b, c), (c, d, a) with their vt and vn ids alike;
    # faces without ids take id 0; vt lines make texture ids, none make none;
    # rotation moves the vn lines with the vertices; a smooth mesh without vn
    # lines under a transform gets the loader's vertex normals, moved
    obj = ("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
           "vn 0 0 1\nvn 0 1 0\nf 1/1/1 2/2/1 3/3/2 4/4/2\nf 1//2 3//1 4//2\n")
    (tmp_path / "q.obj").write_text(obj)
    s = scene_file.load(_scene(tmp_path, "OBJECT\nobjfile q.obj\nsmooth 1\nrotation 90 0 0\n\n"))
    m = s.meshes[0]
    assert m.faces.tolist() == [[0, 1, 2], [2, 3, 0], [0, 2, 3]]
    assert m.face_uv.tolist() == [[0, 1, 2], [2, 3, 0], [0, 0, 0]]
    assert m.face_vn.tolist() == [[0, 0, 1], [1, 1, 0], [1, 0, 1]]
    assert np.allclose(m.vertex_normals[1], (0, 0, 1), atol=1e-6)  # +y turned to +z by 90 degrees about x
    assert s.entities[0].smooth == 1
    (tmp_path / "p.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nf 1 2 3\nf 1 4 2\n")
    s = scene_file.load(_scene(tmp_path, "OBJECT\nobjfile p.obj\nsmooth 1\ntranslate 1 2 3\n\n"))
    m = s.meshes[0]
    assert m.uv is None and m.face_vn.tolist() == m.faces.tolist()
    # vertex 0 joins the faces of normals +z and +y: the mean (0, 1, 1) / 2, normalised
    assert np.allclose(m.vertex_normals[0], (0, 2 ** -0.5, 2 ** -0.5), atol=1e-6)
    (tmp_path / "c.obj").write_text("v 0 0 0 1 0 0\nv 1 0 0 1 0 0\nv 0 1 0 1 0 0\nf 1 2 3\n")
    with pytest.raises(scene_file.SceneFileError, match="vertex colours"):
        scene_file.load(_scene(tmp_path, "OBJECT\nobjfile c.obj\n\n"))


@pytest.mark.parametrize("name", ["worm_bg", "worm_objects", "worm_sign"])
def test_wormhole_files_render_like_the_reference(tmp_path, golden, name):
    # the files the reference rendered for wormhole_render.npz (the WORMHOLE
    # block: in, out, Rho, a, W, sign, geodesics_max_length, both background
    # BMPs with their map_coef / coef lines), read by this library's reader
    # and rendered by the oracle
    import wormhole_cases
    sc = wormhole_cases.one_thread_cases()[name]
    s = scene_file.load(sc.write_reference(str(tmp_path)))
    img, _, _ = O.OracleScene(s).render(threads=1)
    assert np.array_equal(img, golden["wormhole_render"][name])


def test_wormhole_placed_along_the_camera(tmp_path):
    # without 'in' / 'out' the 'in' mouth sits dist along the camera
    # direction and 'out' at the origin (scene_env.h:2100-2110); the block's
    # geodesics_max_length is the black hole's setting too
    s = scene_file.load(_scene(tmp_path, "CAMERA_POS\n0 0 10\n\nCAMERA_DIR\n0 0 -2\n\n"
                                         "WORMHOLE\ndist 25\nRho 2\nsign -1\ngeodesics_max_length 500\n"
                                         "map_coef2 1 0.5 2 0\ncoef1 3\nunknown 1\n\n"))
    w = s.wormhole
    assert w["in"] == (0.0, 0.0, -15.0) and w["out"] == (0.0, 0.0, 0.0)
    assert w["rho"] == 2.0 and w["a"] == 0.5 and w["w"] == 0.05 and w["sign"] == -1 and w["max_steps"] == 500
    assert w["map_coef"] == ((1.0, 0.0, 1.0, 0.0), (1.0, 0.5, 2.0, 0.0)) and w["texture_coef"] == (3.0, 1.0)
    assert w["camera"] == (0.0, 0.0, 10.0)
    assert "skipped in WORMHOLE: unknown 1" in s.file_warnings


def test_hdr_reader_rows_and_values(tmp_path):
    # HDRImage::load_unsafe: byte * 2^(e - 128) / 256 per channel, file row y
    # is image row H - 1 - y; IBL_Color(i, j) reads image row i
    from prender_gb300.scene import hdr_rgbe, rgbe_values, write_hdr
    rng = np.random.default_rng(5)
    q = np.concatenate([rng.integers(0, 256, (9, 200, 3)), rng.integers(100, 160, (9, 200, 1))], 2).astype(np.uint8)
    q[0, 0] = (0, 0, 0, 0)
    vals = rgbe_values(q)
    write_hdr(str(tmp_path / "i.hdr"), hdr_rgbe(vals)[::-1])
    body = f"IMAGE\n8 6\n\nOBJECT\nsphere 0 0 0 1\ncolor 0 0 0\nreflection diffuse\nibl_texture {tmp_path / 'i.hdr'}\n\n"
    s = scene_file.load(_scene(tmp_path, body))
    assert s.materials[0].ibl.dtype == np.float32 and np.array_equal(s.materials[0].ibl, vals)


@pytest.mark.parametrize("body,code,msg", [
    ("disk 0 10 0 1\nnormal 0 -1 0\ntexture TEX\n", A.PR_E_UNSUPPORTED, "spheres, hemispheres, uvplanes and meshes"),
    ("objfile OBJ\ntexture TEX\n", A.PR_E_UNSUPPORTED, "needs texture coordinates"),
    ("sphere 0 10 0 1\nemission 1 1 1\nibl_texture TEX\n", A.PR_E_UNSUPPORTED, "IBL image"),
    ("hemisphere 0 10 0 1\nemission 1 1 1\n", A.PR_E_UNSUPPORTED, "hemispheres that emit"),
])
def test_textures_refused_where_not_rendered(tmp_path, body, code, msg):
    from prender_gb300 import gpu
    from prender_gb300.scene import _write_bmp24
    _write_bmp24(str(tmp_path / "t.bmp"), np.full((4, 4, 3), 200, np.uint8))
    body = body.replace("TEX", str(tmp_path / "t.bmp"))
    from prender_gb300.scenes import icosphere
    v, f = icosphere(1)  # a mesh without vt lines
    (tmp_path / "m.obj").write_text("".join("v %r %r %r\n" % tuple(map(float, x)) for x in v) +
                                    "".join("f %d %d %d\n" % tuple(int(i) + 1 for i in x) for x in f))
    body = body.replace("OBJ", str(tmp_path / "m.obj"))
    text = "IMAGE\n8 6\n\nOBJECT\n" + body + "color 0 0 0\nreflection diffuse\n\n"
    s = scene_file.load(_scene(tmp_path, text))
    with pytest.raises(gpu.PrenderError) as e:
        gpu.check_scene(s)
    assert str(code) in str(e.value) and msg in str(e.value)


@pytest.mark.parametrize("body,code,msg", [
    ("uvplane 0 10 0\nU 1 0 0\nV 0 0 1\nspot_light 1\n", A.PR_E_UNSUPPORTED, "spot lights are spheres"),
    ("sphere 0 10 0 1\nparallel_light 1\nspot_light 1\n", A.PR_E_UNSUPPORTED, "either a parallel or a spot"),
    ("sphere 0 10 0 1\nparallel_light 1\n", A.PR_E_SCENE, "parallel_light_dir"),
    ("disk 0 10 0 1\nnormal 0 -1 0\nparallel_light 1\nparallel_light_dir 0 -1 0\n", A.PR_E_UNSUPPORTED,
     "parallel disk"),
    ("infinity_light 0 0 0\n", A.PR_E_SCENE, "infinity light needs a direction"),
])
def test_light_kinds_refused_where_the_reference_reads_garbage(tmp_path, body, code, msg):
    """A spot light's centre is read as a sphere's whatever its shape, a
    parallel sphere without a direction shoots zero-length shadow rays, a
    disk's sampling is undefined (circle.h:110-134): pr_scene_check refuses
    them on the host, as an upload would"""
    from prender_gb300 import gpu
    text = ("IMAGE\n8 6\n\nOBJECT\n" + body + "emission 1 1 1\ncolor 0 0 0\nreflection diffuse\n\n"
            "OBJECT\nsphere 0 0 0 1\ncolor 0.5 0.5 0.5\nreflection diffuse\n\n")
    s = scene_file.load(_scene(tmp_path, text))
    with pytest.raises(gpu.PrenderError) as e:
        gpu.check_scene(s)
    assert str(code) in str(e.value) and msg in str(e.value)


def test_light_kind_fields_read_from_the_file(tmp_path):
    text = ("IMAGE\n8 6\n\nOBJECT\ninfinity_light 1 -1.5 -0.4\nemission 1 1 1\ncolor 0 0 0\n"
            "reflection diffuse\n\nOBJECT\nsphere 40 81 70 1\nemission 50 50 50\ncolor 0 0 0\n"
            "reflection diffuse\nspot_light 1\nspot_light_angle 20 10\nspot_light_dir 0 -2 0\n"
            "spot_light_falloff 0.5\nspot_attenuation 0 1 0\n\nOBJECT\nuvplane 0 10 0\nU 5 0 0\nV 0 0 5\n"
            "emission 5 5 5\ncolor 0 0 0\nreflection diffuse\nparallel_light 1\n\n")
    s = scene_file.load(_scene(tmp_path, text))
    inf, spot, par = s.entities
    assert inf.type == A.PR_ENT_INF_LIGHT and inf.light_dir == (1.0, -1.5, -0.4)  # as given
    assert spot.spot_light == 1 and spot.light_dir == (0.0, -1.0, 0.0)  # normalised
    assert spot.spot_angle == (20.0, 10.0) and spot.spot_falloff == 0.5 and spot.spot_attenuation == (0.0, 1.0, 0.0)
    assert par.parallel_light == 1 and par.light_dir == (0.0, 0.0, 0.0)  # the plane's normal, taken at upload
    assert par.spot_attenuation == (0.0, 0.0, 1.0)  # the parser's default
    from prender_gb300 import gpu
    gpu.check_scene(s)


def _scene(tmp_path, body, name="s.txt"):
    p = tmp_path / name
    p.write_text(body)
    return str(p)


def _screen(tmp_path, text):
    return scene_file.load(_scene(tmp_path, f"SCREEN\n{text}\n")).camera.screen


def _gamma(tmp_path, text, pre=""):
    return scene_file.load(_scene(tmp_path, f"{pre}gamma_offset\n{text}\n")).gamma_offset


def test_values_split_at_blanks_before_operands(tmp_path):
    assert _screen(tmp_path, "1 -2 3") == (1.0, -2.0, 3.0)
    assert _screen(tmp_path, "1 - 2 3") == (1.0, -2.0, 3.0)
    assert _screen(tmp_path, "1+2 3*4 (5)") == (3.0, 12.0, 5.0)


@pytest.mark.parametrize("text,value", [
    ("010", 8.0), ("0x1f", 31.0), ("0t15", 15.0), ("0b2:101", 5.0), ("0.5", 0.5), ("1.5e2", 150.0),
    ("2e-1", 0.2), ("2^3^2", 512.0), ("-2^2", 4.0), ("7%4", 3.0), ("-7%4", 1.0), ("10/4*2", 5.0),
    ("1-2-3", -4.0), ("sqrt(16)+floor(2.7)+ceil(0.2)", 7.0), ("pow(2,10)", 1024.0), ("atan2(0,1)", 0.0),
    ("sind(90)", 1.0), ("datan2(1,1)", 45.0), ("pi", np.pi), ("e", np.e),
])
def test_expression_values(tmp_path, text, value):
    assert _gamma(tmp_path, text) == pytest.approx(value, rel=1e-15, abs=1e-15)


def test_literals_accumulate_digits_and_divide_once(tmp_path):
    # every digit into one double, one division by 10^(fraction digits)
    assert _gamma(tmp_path, "0.123456789") == 123456789.0 / 1e9
    assert _gamma(tmp_path, "12.5e3") == 125.0 / 10.0 * 1000.0


def test_variables_first_definition_holds(tmp_path):
    pre = "VAR A\n2\n\nVAR B\nA*3\n\nVAR A\n100\n\n"
    assert _gamma(tmp_path, "A+B", pre) == 8.0


def test_environment_references(tmp_path, monkeypatch):
    monkeypatch.setenv("PR_TEST_GAMMA", "1.5*2")
    assert _gamma(tmp_path, "%PR_TEST_GAMMA%") == 3.0
    monkeypatch.delenv("PR_TEST_GAMMA")
    assert _gamma(tmp_path, "%PR_TEST_GAMMA%") == 0.0


@pytest.mark.parametrize("body,msg", [
    ("gamma_offset\n1 2\n", "unexpected text"),
    ("gamma_offset\nZZ\n", "unknown name"),
    ("gamma_offset\n(1 + 2)\n", "expected ')'"),
    ("SCREEN\n1 2\n", "expected a number"),
    ("OBJECT\nsphere 0 0 0 1\ncolor 1 1\n\n", "expected a number"),
    ("OBJECT\nsphere 0 0 0 1\nward_brdf 0.75 0.5 0.5\n\n", "expected a number"),
])
def test_bad_values_are_errors_with_the_line(tmp_path, body, msg):
    with pytest.raises(scene_file.SceneFileError) as e:
        scene_file.load(_scene(tmp_path, body))
    assert msg in str(e.value) and "s.txt:" in str(e.value)


@pytest.mark.parametrize("body", [
    "OBJECT\nsphere 0 0 0 1\nMATERIAL_SYMBOL\nKetchup\n\n",
    "OBJECT\nsphere 0 0 0 1\nreflection reflection1\n1 2 3 4 5 6\n\n",
    "OBJECT\nplane 0 0 0\nnormal 0 1 0\n\n",
    "OBJECT\nuvplane 0 0 0\nU 1 0 0\nV 0 1 0\nrotation 0 10 0\n\n",
    "OBJECT\ndisk 0 0 0 1\nnormal 0 1 0\ntranslate 1 0 0\n\n",
    "OBJECT\nsphere 0 0 0 1\nreflection reflection\nreflection Subsurface_Scattering\n\n",
    "LENS\n0.5 100\n",
    "energyRedistributionPathTracing\n1\n",
    "BLACKHOLE\ninitial_condition 1\n\n",
])
def test_features_not_rendered_here_are_refused(tmp_path, body):
    with pytest.raises(scene_file.SceneFileError):
        scene_file.load(_scene(tmp_path, body))


def test_switched_off_features_are_accepted(tmp_path):
    s = scene_file.load(_scene(tmp_path, "LENS\n0 100\n\nmetropolisTransport\n0\n\n"
                                         "OBJECT\nsphere 0 0 0 1\nparallel_light 0\nsmooth 0\nback 0\n\n"))
    assert len(s.entities) == 1


def test_missing_files_are_errors(tmp_path):
    with pytest.raises(scene_file.SceneFileError, match="cannot open"):
        scene_file.load(str(tmp_path / "none.txt"))
    with pytest.raises(scene_file.SceneFileError, match="cannot open"):
        scene_file.load(_scene(tmp_path, "OBJECT\nobjfile nowhere.obj\n\n"))


def test_defaults_and_line_rules(tmp_path):
    body = ("# one comment line before a keyword is skipped\n"
            "IMAGE\n#a comment in place of the value is skipped too\n64 32\n\n"
            "CAMERA_POS\n1 2 3\n\nCAMERA_DIR\n0 0 -2\n\n"
            "PAHASE 0.1 0.2 0.3\n\n"
            "SCATTERING\n9\n0.1 0.2 0.3\n\n"
            "THREAD\n8\n\nOUTPUT\nx.bmp\n\nunknown_keyword\n\n"
            "OBJECT\nsphere 1 2 3 4\nPAHASE 0.5 0.6 0.7\nnormal -1\n\n"
            "OBJECT\ndisk2 0 0 0 5 1\nnormal 0 0 1\nblackhole_disk 2\n\n"
            "OBJECT\ndisk 0 0 0 5\nnormal 0 0 1\n\n")
    s = scene_file.load(_scene(tmp_path, body.replace("\n", "\r\n")))
    assert (s.camera.width, s.camera.height) == (64, 32)
    assert s.camera.dir == (0.0, 0.0, -1.0) and s.camera.position == (1.0, 2.0, 3.0)
    assert s.medium.phase_g == (0.1, 0.2, 0.3)
    assert s.medium.sigma_s_rgb == (0.1, 0.2, 0.3)
    assert s.settings.samples == 8 and s.settings.supersamples == 2 and s.settings.depth == 8
    assert s.settings.media == 0
    assert "unknown_keyword" in s.file_warnings
    m = s.materials[0]
    assert m.medium.phase_g == (0.5, 0.5, 0.7)  # an OBJECT block keeps x for y
    assert s.entities[0].p == (0.5, 0.6, 0.7)   # and the line moves the sphere's centre
    assert s.entities[0].normal_inverse == -1
    assert s.entities[1].blackhole_disk == 2 and s.entities[2].blackhole_disk == 2
    assert s.entities[1].radius_inner == 1.0


def test_camera_angle_and_target(tmp_path):
    s = scene_file.load(_scene(tmp_path, "SCREEN\n1 1 40\n\nCAMERA_ANGLE\n30\n\n"
                                         "CAMERA_POS\n0 0 0\n\nTARGET_POS\n3 0 4\n\n"))
    w = 2.0 * 40.0 * np.tan(30.0 * (np.pi / 180.0) / 2.0)
    assert s.camera.screen[0] == w and s.camera.screen[1] == w
    assert s.camera.dir == pytest.approx((0.6, 0.0, 0.8), abs=1e-15)


def test_black_hole_placed_along_the_camera(tmp_path):
    s = scene_file.load(_scene(tmp_path, "CAMERA_POS\n0 0 10\n\nCAMERA_DIR\n0 0 -1\n\n"
                                         "BLACKHOLE\ndist 25\nangular_momentum 0.5\ncoef 2\n\n"))
    assert s.kerr["position"] == (0.0, 0.0, -15.0)
    assert s.kerr["a"] == 0.5 and s.kerr["texture_coef"] == 2.0 and s.kerr["max_steps"] == 10000


def _obj_scene(tmp_path, obj, extra=""):
    (tmp_path / "m.obj").write_text(obj)
    return scene_file.load(_scene(tmp_path, f"OBJECT\nobjfile m.obj\n{extra}\n"))


def test_obj_quads_split_as_the_reference(tmp_path):
    obj = "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\n  v 0 0 1\nf 1 2 3 4\nf 1/1 2/1 5/1\nf 2//1 3//1 5//1\n"
    s = _obj_scene(tmp_path, obj)
    m = s.meshes[0]
    assert m.vertices.shape == (5, 3)
    assert m.faces.tolist() == [[0, 1, 2], [2, 3, 0], [0, 1, 4], [1, 2, 4]]
    assert m.face_normals is None  # no vertex normals: the loader's rule at upload


def test_obj_vertex_normals_give_the_face_normal(tmp_path):
    obj = ("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nvn 1 0 0\nvn 0 1 0\nvn 0 0 1\n"
           "f 1//1 2//2 3//3\nf 2 4 3\n")
    fn = _obj_scene(tmp_path, obj).meshes[0].face_normals
    # the mean in float (sum in float, / 3 in double), then divided by the
    # length of its float square sum
    c = np.float32(1.0 / 3.0)
    sq = np.float32(np.float32(c * c) + np.float32(c * c)) + np.float32(c * c)
    assert fn[0].tolist() == [float(np.float32(float(c) / np.sqrt(float(sq))))] * 3
    # a face without normal numbers takes normal 1 for all three (the reference's zeroed ids)
    assert fn[1].tolist() == [1.0, 0.0, 0.0]


def test_obj_materials_are_read_as_the_loader_reads_them(tmp_path):
    # LoadMTLFile's first-character dispatch: Kd / Ks, d, Tr, Ni / Ns and the
    # '#' extensions; '#REFLECTION 2' with Ni 0 sets 1.5 and '#REFLECTION 1'
    # the roughness 0; usemtl takes the last material of a name, ignoring
    # case; faces before any usemtl (or after an unknown name) get none
    (tmp_path / "m.mtl").write_text(
        "newmtl red\n  Kd 1 0 0\nKs 0.5 0.5 0.5\nd 1\nNs 12\n#ROUGHNESS 0.4\n#REFLECTION 1\n"
        "newmtl Glass\nTr 0\n#REFLECTION 2\n#SMOOTH 0\n#REPEAT 3\n#EMISSION 1 2 3\n#WARD 0.1 0.2\n"
        "newmtl red\nKd 0 1 0\n#COLOR 0 0 1\n#SMOOTH 1\n")
    obj = ("mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nf 1 2 3\nusemtl RED\nf 2 4 3\n"
           "usemtl glass\nf 1 2 4 3\nusemtl nothing\nf 1 3 4\n")
    s = _obj_scene(tmp_path, obj)
    m = s.meshes[0]
    assert m.face_material.tolist() == [-1, 2, 1, 1, -1]
    red0, glass, red1 = m.obj_materials
    assert tuple(red0.diffuse) == (1.0, 0.0, 0.0) and tuple(red0.specular) == (0.5, 0.5, 0.5)
    assert red0.alpha == 1.0 and red0.shininess == 12.0 and red0.reflection == 1 and red0.roughness == 0.0
    assert glass.alpha == 1.0 and glass.reflection == 2 and glass.refraction_index == 1.5 and glass.smooth == 2
    assert glass.repeat == 3 and tuple(glass.emission) == (1.0, 2.0, 3.0) and tuple(glass.ward) == (
        float(np.float32(0.1)), float(np.float32(0.2)))
    assert tuple(red1.diffuse) == (0.0, 0.0, 1.0) and red1.smooth == 1 and red1.reflection == -1


def test_obj_material_refusals(tmp_path):
    from prender_gb300 import gpu
    (tmp_path / "m.mtl").write_text("newmtl half\nKd 1 0 0\nd 0.5\n")
    s = _obj_scene(tmp_path, "mtllib m.mtl\nusemtl half\nv 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nf 1 2 3\nf 2 4 3\n"
                             "f 1 2 4\nf 1 3 4\nf 1 4 2\n")
    with pytest.raises(gpu.PrenderError, match="alpha"):
        gpu.check_scene(s)


def test_mesh_transforms_move_vertices_in_float_steps(tmp_path):
    obj = "v 1 0 0\nv 0 1 0\nv 0 0 1\nv 1 1 1\nf 1 2 3\nf 2 3 4\n"
    m = _obj_scene(tmp_path, obj, "scale 2 3 4\ntranslate 1 1 1\n").meshes[0]
    assert m.vertices.tolist() == [[3, 1, 1], [1, 4, 1], [1, 1, 5], [3, 4, 5]]
    assert m.face_normals is not None and np.allclose(np.linalg.norm(m.face_normals, axis=1), 1.0, atol=1e-6)


def _bmp_scene(tmp_path, data, name="t.bmp"):
    (tmp_path / name).write_bytes(data)
    return scene_file.load(_scene(tmp_path, f"BLACKHOLE\naccretion_disk_texture {name}\nbackground_texture {name}\n\n"))


def _bmp32(w, h, px, top_down=False):
    hdr = bytearray(54)
    hdr[0:2] = b"BM"
    hdr[10:14] = (54).to_bytes(4, "little")
    hdr[14:18] = (40).to_bytes(4, "little")
    hdr[18:22] = w.to_bytes(4, "little")
    hdr[22:26] = (-h if top_down else h).to_bytes(4, "little", signed=True)
    hdr[26:28] = (1).to_bytes(2, "little")
    hdr[28:30] = (32).to_bytes(2, "little")
    return bytes(hdr) + bytes(px)


def test_bmp_rows_and_alpha(tmp_path):
    tex = np.arange(2 * 3 * 3, dtype=np.uint8).reshape(2, 3, 3) * 7
    write_bmp(str(tmp_path / "a.bmp"), tex)
    s = _bmp_scene(tmp_path, (tmp_path / "a.bmp").read_bytes())
    assert np.array_equal(s.kerr["texture"], tex)
    assert np.array_equal(s.kerr["disk_texture"][:, :, :3], tex) and (s.kerr["disk_texture"][:, :, 3] == 255).all()
    # 32-bit, stored bottom-up: row 0 of the file is cell row 0
    px = [10, 20, 30, 40, 50, 60, 70, 80]  # B G R A per pixel, 2 x 1
    s = _bmp_scene(tmp_path, _bmp32(1, 2, px))
    assert s.kerr["disk_texture"].tolist() == [[[30, 20, 10, 40]], [[70, 60, 50, 80]]]
    # stored top-down (negative height): the rows reverse
    s = _bmp_scene(tmp_path, _bmp32(1, 2, px, top_down=True))
    assert s.kerr["disk_texture"].tolist() == [[[70, 60, 50, 80]], [[30, 20, 10, 40]]]
    # all-zero alpha reads as opaque
    s = _bmp_scene(tmp_path, _bmp32(1, 2, [1, 2, 3, 0, 4, 5, 6, 0]))
    assert (s.kerr["disk_texture"][:, :, 3] == 255).all()
    with pytest.raises(scene_file.SceneFileError, match="BMP"):
        _bmp_scene(tmp_path, b"GIF89a" + bytes(100))
