"""Scenes read from the reference's scene files (pr_scene_file_load),
uploaded and traced on the GPU: closest hits bit-exact against the oracle
(transformed meshes, OBJ quads, faces with their own normals), and renders
that agree with the oracle's statistically."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from prender_gb300 import gpu, scene_file, scenes

pytestmark = pytest.mark.gpu

SCENE_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scene_files")


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g
    g.build_library()
    O.build()
    c = gpu.Context(0)
    yield c
    c.close()


def _load(name):
    return scene_file.load(os.path.join(SCENE_DIR, name + ".txt"))


@pytest.mark.parametrize("name", ["spheres_expr", "mesh_obj", "media", "sss"])
def test_scene_file_closest_hits_bit_exact(ctx, name):
    s = _load(name)
    ctx.upload(s)
    rays = np.concatenate([scenes.random_rays((2, 1, 1), (98, 80, 170), 20000, seed=3), scenes.camera_rays(s)])
    h = ctx.first_hit(rays)
    o = O.OracleScene(s).first_hit(rays)
    assert np.array_equal(h["entity"], o["entity"])
    assert np.array_equal(h["prim"], o["prim"])
    assert np.array_equal(h["t"], o["t"])


@pytest.mark.parametrize("name", ["spheres_expr", "mesh_obj", "media", "sss"])
def test_scene_file_render_matches_oracle_statistically(ctx, name):
    # 16 independent 1024-spp GPU frames against one 1024-spp oracle frame:
    # the GPU mean carries sd / 4, the oracle frame sd, where sd is the
    # spread of a 1024-spp frame measured over the GPU frames
    s = _load(name)
    s.settings.samples, s.settings.supersamples = 256, 2
    nb, spp = 16, s.settings.spp
    ctx.upload(s)
    b = np.stack([ctx.render(s, sample_offset=k * spp).astype(np.float64) for k in range(nb)])
    mean = b.mean(0)
    sd = b.std(0, ddof=1)
    # one oracle thread: the oracle's rows then draw from fixed streams, so
    # the comparison is the same on every run
    ref, _, _ = O.OracleScene(s).render(threads=1)
    sigma = np.sqrt(sd ** 2 / nb + sd ** 2) + 1e-6
    z = np.abs(mean - ref) / sigma
    frac = float((z > 3.0).mean())
    rmse = float(np.sqrt(((mean - ref) ** 2).mean()))
    noise = float(np.sqrt((sigma ** 2).mean()))
    rel = abs(mean.mean() - ref.mean()) / ref.mean()
    print(f"{name}: >3 sigma {frac:.4f}, rmse {rmse:.3e} vs noise {noise:.3e}, mean rel diff {rel:.4f}")
    assert rel < 0.03
    assert frac < 0.03
    assert rmse < 1.3 * noise
