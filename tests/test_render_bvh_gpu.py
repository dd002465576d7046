"""The GPU builder of the render path's trees (pr_render_bvh_export with
on_gpu = 1, used by pr_scene_upload for meshes of 4096 faces and more)
against the host builder: the same split decisions, so the 80-byte wide
nodes are equal byte for byte and every leaf holds the same faces (their
order within a leaf may differ).  The traversal parity tests then cover
the GPU-built trees as well, since every scene with a large mesh uses them."""
import time

import numpy as np
import pytest

from prender_gb300 import gpu, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g
    g.build_library()
    c = gpu.Context(0)
    yield c
    c.close()


def _soup(n, seed):
    """n triangles of widely varying size and aspect, scattered in a box"""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0, 100, (n, 1, 3))
    size = np.exp(rng.uniform(np.log(0.01), np.log(10.0), (n, 1, 1)))
    v = (c + rng.normal(0, 1, (n, 3, 3)) * size).astype(np.float32).reshape(-1, 3)
    return v, np.arange(3 * n, dtype=np.int32).reshape(n, 3)


def _leaves(tree):
    out = []
    for row in tree["nodes"]:
        tri_base = int(row[20:24].view(np.int32)[0])
        for m in row[24:32]:
            if m:
                cnt, off = bin(int(m) >> 5).count("1"), int(m) & 31
                out.append(tuple(sorted(tree["tri_faces"][tri_base + off:tri_base + off + cnt])))
    return out


@pytest.mark.parametrize("name", ["box", "ico_subdiv5", "ico_subdiv7", "soup_60k"])
def test_gpu_build_equals_host_build(ctx, name):
    if name == "box":
        v, f = scenes.box_mesh((1, 0, 0), (99, 81.6, 250))
    elif name.startswith("ico"):
        v, f = scenes.displaced_icosphere(int(name[-1]), (50, 24, 70), 20.0, amp=0.05, seed=0)
    else:
        v, f = _soup(60000, 7)
    h = ctx.render_bvh(v, f, on_gpu=False)
    t0 = time.perf_counter()
    g = ctx.render_bvh(v, f, on_gpu=True)
    gpu_s = time.perf_counter() - t0
    print(f"{name}: {len(f)} faces, {len(h['nodes'])} wide nodes, GPU build + host collapse {gpu_s * 1e3:.1f} ms")
    assert np.array_equal(h["nodes"], g["nodes"])
    assert sorted(g["tri_faces"].tolist()) == list(range(len(f)))
    assert _leaves(h) == _leaves(g)


def test_upload_of_the_benchmarked_scene_is_fast(ctx):
    """The 327,680-triangle scene uploads with its render tree built on the
    GPU and the reference-layout QBVH left for the exact path's first use."""
    s = scenes.mesh_cornell(width=64, height=48, subdiv=7)
    ctx.upload(s)  # the first upload pays the CUDA module loads
    t0 = time.perf_counter()
    ctx.upload(s)
    up = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx.first_hit(scenes.camera_rays(s))  # builds the deferred QBVH
    fh = time.perf_counter() - t0
    print(f"upload {up * 1e3:.1f} ms, first exact query (deferred QBVH build) {fh * 1e3:.1f} ms")
    assert up < 0.25
