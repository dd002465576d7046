"""HDR output (Render::OutputHdr, render.h:1649-1667; HDRImage, hdr.h:15-246):
the Radiance RGBE pixels from the GPU (pr_image_to_rgbe) and the file framing
of scene.write_hdr against the file the reference itself wrote for a seeded
image (tests/golden/hdr_output.npz: black pixels, values below the 1e-32
cut, exact powers of two, scanlines wider than one 127-byte run)."""
import os

import numpy as np
import pytest

from prender_gb300.scene import write_hdr


def rgbe_restated(img: np.ndarray) -> np.ndarray:
    """HDRPixel (hdr.h:30-44) in numpy: d = max(r, g, b) in double, zero at or
    below 1e-32, else m 2^e = d and channel c -> (unsigned char)(c m 256 / d),
    exponent e + 128"""
    x = img.astype(np.float64)
    d = x.max(axis=2)
    m, e = np.frexp(d)
    ok = d > 1e-32
    sc = np.where(ok, m * 256.0 / np.where(ok, d, 1.0), 0.0)
    q = np.zeros(img.shape[:2] + (4,), np.uint8)
    q[..., :3] = (x * sc[..., None]).astype(np.uint8)
    q[..., 3] = np.where(ok, e + 128, 0)
    return q


def _file_bytes(tmp_path, q):
    p = os.path.join(str(tmp_path), "out.hdr")
    write_hdr(p, q)
    return np.frombuffer(open(p, "rb").read(), np.uint8)


def test_writer_reproduces_the_reference_file(golden, tmp_path):
    g = golden["hdr_output"]
    assert np.array_equal(_file_bytes(tmp_path, rgbe_restated(g["image"])), g["hdr"])


@pytest.mark.gpu
def test_gpu_rgbe_reproduces_the_reference_file(golden, tmp_path):
    import __graft_entry__ as ge
    from prender_gb300 import gpu
    ge.build_library()
    ctx = gpu.Context(0)
    g = golden["hdr_output"]
    q = ctx.to_rgbe(g["image"])
    assert np.array_equal(q, rgbe_restated(g["image"]))
    assert np.array_equal(_file_bytes(tmp_path, q), g["hdr"])
    ctx.close()
