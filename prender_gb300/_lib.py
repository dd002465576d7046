"""Loads libprender_gpu.so (the C ABI of include/prender_gpu.h) via ctypes.

The library is the product: there is no CPU fallback.  If it is missing the
import fails loudly with the build command to run.
"""
import ctypes as C
import os

from . import _abi as A

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libprender_gpu.so")

# every entry point declared in include/prender_gpu.h
EXPORTS = (
    "pr_create", "pr_destroy", "pr_last_error", "pr_abi_version", "pr_abi_sizeof",
    "pr_scene_upload", "pr_scene_check", "pr_qbvh_info", "pr_qbvh_export", "pr_qbvh_build_host", "pr_render_bvh_export",
    "pr_first_hit", "pr_first_hit_dev", "pr_trace_fast", "pr_render", "pr_render_dev", "pr_render_dev_noalloc", "pr_last_render_stats",
    "pr_kerr_trace", "pr_kerr_trace_dev", "pr_wormhole_trace", "pr_wormhole_trace_dev", "pr_render_adjoint", "pr_render_adjoint_dev",
    "pr_last_kernel_times", "pr_kerr_sensitivity", "pr_kerr_sensitivity_adjoint", "pr_kerr_disk_shade", "pr_image_to_rgb8", "pr_image_to_rgb8_dev", "pr_image_to_rgbe", "pr_image_to_rgbe_dev", "pr_autotune_wavefront",
    "pr_scene_create", "pr_scene_release", "pr_render_batch",
    "pr_scene_file_load", "pr_scene_file_desc", "pr_scene_file_camera", "pr_scene_file_warnings", "pr_scene_file_free",
)

_lib = None


class PrenderError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"prender_gpu error {code}: {msg}")
        self.code = code


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with "
                          f"`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    L.pr_create.restype = vp
    L.pr_create.argtypes = [C.c_int, C.POINTER(C.c_int)]
    L.pr_destroy.argtypes = [vp]
    L.pr_last_error.restype = C.c_char_p
    L.pr_last_error.argtypes = [vp]
    L.pr_abi_sizeof.restype = C.c_size_t
    L.pr_abi_sizeof.argtypes = [C.c_int]
    L.pr_scene_upload.argtypes = [vp, vp]
    L.pr_scene_check.argtypes = [vp, vp, C.c_int]
    L.pr_qbvh_info.argtypes = [vp, C.c_int, vp, vp]
    L.pr_qbvh_export.argtypes = [vp, C.c_int, vp, vp, vp, vp]
    L.pr_qbvh_build_host.argtypes = [vp, i32, vp, i32, vp, vp, vp, vp, vp, vp]
    L.pr_first_hit.argtypes = [vp, vp, i64, vp, vp, vp]
    L.pr_first_hit_dev.argtypes = [vp, vp, i64, vp, vp, vp]
    L.pr_trace_fast.argtypes = [vp, vp, i64, vp, vp, vp]
    L.pr_render.argtypes = [vp, vp, vp, vp, C.c_uint64, C.c_int]
    L.pr_render_dev.argtypes = [vp, vp, vp, vp, C.c_uint64, C.c_int]
    L.pr_render_dev_noalloc.argtypes = [vp, vp, vp, vp, C.c_uint64, C.c_int]
    L.pr_render_bvh_export.argtypes = [vp, vp, C.c_int, vp, i64, vp, i64, vp, vp]
    L.pr_image_to_rgbe.argtypes = [vp, vp, i32, i32, vp]
    L.pr_image_to_rgbe_dev.argtypes = [vp, vp, i32, i32, vp]
    L.pr_last_render_stats.argtypes = [vp, C.POINTER(A.pr_render_stats)]
    L.pr_kerr_trace.argtypes = [vp, vp, i64, vp, vp, vp, vp, vp, vp]
    L.pr_kerr_trace_dev.argtypes = [vp, vp, i64, vp, vp, vp, vp, vp, vp]
    L.pr_wormhole_trace.argtypes = [vp, vp, i64, vp, vp, vp, vp, vp]
    L.pr_wormhole_trace_dev.argtypes = [vp, vp, i64, vp, vp, vp, vp, vp]
    L.pr_render_adjoint.argtypes = [vp, vp, vp, vp, C.c_uint64, vp, vp, vp]
    L.pr_render_adjoint_dev.argtypes = [vp, vp, vp, vp, C.c_uint64, vp, vp]
    L.pr_last_kernel_times.argtypes = [vp, vp, vp, C.c_int]
    L.pr_kerr_sensitivity.argtypes = [vp, vp, i64, vp, vp, vp, vp]
    L.pr_kerr_sensitivity_adjoint.argtypes = [vp, vp, i64, vp, vp, vp]
    L.pr_kerr_disk_shade.argtypes = [vp, C.c_int, vp, i64, vp, vp, vp, vp]
    L.pr_image_to_rgb8.argtypes = [vp, vp, C.c_int32, C.c_int32, C.c_double, vp]
    L.pr_image_to_rgb8_dev.argtypes = [vp, vp, C.c_int32, C.c_int32, C.c_double, vp]
    L.pr_autotune_wavefront.argtypes = [vp, vp, vp, vp, vp, vp]
    L.pr_scene_create.restype = vp
    L.pr_scene_create.argtypes = [vp, vp, C.POINTER(C.c_int)]
    L.pr_scene_release.argtypes = [vp, vp]
    L.pr_render_batch.argtypes = [vp, C.c_int, vp]
    L.pr_scene_file_load.restype = vp
    L.pr_scene_file_load.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
    L.pr_scene_file_desc.restype = vp
    L.pr_scene_file_desc.argtypes = [vp]
    L.pr_scene_file_camera.argtypes = [vp, vp, vp, vp]
    L.pr_scene_file_warnings.restype = C.c_char_p
    L.pr_scene_file_warnings.argtypes = [vp]
    L.pr_scene_file_free.argtypes = [vp]
    _lib = L
    return L
