"""CPU checks of the C ABI library: it loads, exports every entry point that
include/*.h declares, its struct layouts match the ctypes mirror, and its
host-side QBVH build equals the reference's (golden fixture).  No compute
call needs a GPU here."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from prender_gb300 import _abi as A
from prender_gb300 import _lib, gpu, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build_library()
    return _lib.load()


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(pr_\w+)\s*\(", src))
    return names


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 12
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_lib.EXPORTS) >= names


def test_struct_layouts_match(lib):
    structs = [A.pr_medium, A.pr_material, A.pr_entity, A.pr_mesh, A.pr_kerr, A.pr_scene_desc, A.pr_camera,
               A.pr_render_params, A.pr_render_stats]
    for i, s in enumerate(structs):
        assert lib.pr_abi_sizeof(i) == C.sizeof(s), s.__name__
    assert lib.pr_abi_sizeof(9) == C.sizeof(A.pr_job)
    assert lib.pr_abi_version() == 8


def test_no_gpu_context_is_an_error_not_a_fallback(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    st = C.c_int(0)
    h = lib.pr_create(0, C.byref(st))
    assert not h and st.value in (A.PR_E_CUDA, A.PR_E_ARG)


@pytest.mark.parametrize("mesh_index,prefix", [(0, "box"), (1, "ico")])
def test_host_qbvh_build_matches_reference(golden, lib, mesh_index, prefix):
    s = scenes.mesh_cornell(width=32, height=24, samples=1, supersamples=2, subdiv=3)
    m = s.meshes[mesh_index]
    q = gpu.qbvh_build_host(m.vertices, m.faces)
    g = golden["mesh_s3_qbvh_firsthit"]
    valid = (q["children"] != -1)[:, None, :]
    boxes = np.where(valid, q["boxes"].reshape(-1, 6, 4), np.float32(0)).reshape(-1, 24)
    assert np.array_equal(q["children"], g[f"{prefix}_children"])
    assert np.array_equal(q["axes"], g[f"{prefix}_axes"])
    assert np.array_equal(q["leaf"], g[f"{prefix}_leaf"])
    assert np.array_equal(boxes, g[f"{prefix}_boxes"])


def test_host_qbvh_rejects_bad_input(lib):
    v = np.zeros((3, 3), np.float32)
    with pytest.raises(_lib.PrenderError):
        gpu.qbvh_build_host(v, np.array([[0, 1, 5]], np.int32))
