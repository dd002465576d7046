"""pr_render_dev_noalloc: the allocation-free render entry point.

It exists for callers that may not allocate device memory while they render
(a frame loop that cannot absorb the device-wide synchronisation cudaMalloc
may cause, or a host whose device memory is all owned by its own pool).  Its scratch is a static device array shared by all calls, so
this file checks, through the C ABI, that two calls in a row each give the
same image as pr_render_dev, and that a failed call leaves nothing behind
for the next one.  The file is named to run last, so a failure here comes
after every other test has run; it also passes when run on its own.
"""
import ctypes as C

import numpy as np
import pytest

from prender_gb300 import _abi as A
from prender_gb300 import gpu, scenes

pytestmark = pytest.mark.gpu


def _render(L, fn, ctx, cam, prm, offset):
    import torch
    out = torch.full((cam.height, cam.width, 3), float("nan"), dtype=torch.float32, device="cuda:0")
    rc = fn(ctx.h, C.byref(cam), C.byref(prm), C.c_void_p(out.data_ptr()), offset, 0)
    torch.cuda.synchronize()
    return rc, out.cpu().numpy()


def test_noalloc_matches_pr_render_dev_twice():
    import __graft_entry__ as g
    g.build_library()
    ctx = gpu.Context(0)
    L = ctx.L
    s = scenes.mesh_cornell(width=64, height=48, samples=4, supersamples=2, subdiv=3)
    s.settings.mode = A.PR_MODE_MEGAKERNEL
    ctx.upload(s)
    cam, prm = s.camera.to_c(), s.settings.to_c()
    for call, offset in enumerate((0, 16)):
        rc0, ref = _render(L, L.pr_render_dev, ctx, cam, prm, offset)
        assert rc0 == 0, L.pr_last_error(ctx.h).decode()
        rc1, got = _render(L, L.pr_render_dev_noalloc, ctx, cam, prm, offset)
        assert rc1 == 0, L.pr_last_error(ctx.h).decode()
        assert np.isfinite(got).all() and got.mean() > 0, f"call {call}"
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-7, err_msg=f"call {call}")
    ctx.close()


def test_noalloc_clears_its_error_word_and_rejects_oversize_images():
    import __graft_entry__ as g
    g.build_library()
    ctx = gpu.Context(0)
    L = ctx.L
    s = scenes.cornell_spheres(width=32, height=24, samples=1, supersamples=2)
    ctx.upload(s)
    cam = s.camera.to_c()
    bad = s.settings.to_c()
    bad.max_path_vertices = 1  # every path hits the device-side cap
    rc, _ = _render(L, L.pr_render_dev_noalloc, ctx, cam, bad, 0)
    assert rc == A.PR_E_DEVICE and b"loop-cap" in L.pr_last_error(ctx.h)
    good = s.settings.to_c()
    rc, got = _render(L, L.pr_render_dev_noalloc, ctx, cam, good, 0)
    assert rc == 0, L.pr_last_error(ctx.h).decode()
    rc0, ref = _render(L, L.pr_render_dev, ctx, cam, good, 0)
    assert rc0 == 0
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-7)
    # beyond the stated maximum (1,398,080 pixels) the call is refused
    big = s.camera
    big.width, big.height = 2048, 1024
    bcam = big.to_c()
    import torch
    out = torch.empty((1, 1, 3), dtype=torch.float32, device="cuda:0")
    rc = L.pr_render_dev_noalloc(ctx.h, C.byref(bcam), C.byref(good), C.c_void_p(out.data_ptr()), 0, 0)
    assert rc == A.PR_E_ARG and b"exceeds" in L.pr_last_error(ctx.h)
    # a missing parameter block is an argument error, as for pr_render_dev
    rc = L.pr_render_dev_noalloc(ctx.h, C.byref(cam), None, C.c_void_p(out.data_ptr()), 0, 0)
    assert rc == A.PR_E_ARG
    ctx.close()


def test_noalloc_large_image_with_fewer_chunks_agrees_to_rounding():
    """At 1024 x 768 pr_render_dev sums each pixel's samples in two chunks
    whose partial images do not both fit in the static array; this entry
    point then sums them in one.  Same samples, other float summation order:
    equal to rounding, on two calls in a row."""
    import __graft_entry__ as g
    g.build_library()
    ctx = gpu.Context(0)
    L = ctx.L
    s = scenes.mesh_cornell(width=1024, height=768, samples=1, supersamples=2, subdiv=3)
    s.settings.mode = A.PR_MODE_MEGAKERNEL
    ctx.upload(s)
    cam, prm = s.camera.to_c(), s.settings.to_c()
    for call, offset in enumerate((0, 4)):
        rc0, ref = _render(L, L.pr_render_dev, ctx, cam, prm, offset)
        assert rc0 == 0, L.pr_last_error(ctx.h).decode()
        rc1, got = _render(L, L.pr_render_dev_noalloc, ctx, cam, prm, offset)
        assert rc1 == 0, L.pr_last_error(ctx.h).decode()
        assert np.isfinite(got).all() and got.mean() > 0, f"call {call}"
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-7, err_msg=f"call {call}")
    ctx.close()
