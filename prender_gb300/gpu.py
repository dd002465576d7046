"""Python host side of the GPU renderer: a thin wrapper over the C ABI that
mirrors the reference's driver sequence (SceneEnv::Load -> CreateEntList ->
Render::Run, main.cpp:21-229) so user code and tests read like the
reference's own flow:

    ctx = Context(0)
    ctx.upload(scene)             # SceneEnv::Load + CreateEntList + QBVH build
    img = ctx.render(scene)       # Render::Run -> accumulated image (H, W, 3)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from ._lib import PrenderError, load  # noqa: F401


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def qbvh_build_host(vertices: np.ndarray, faces: np.ndarray) -> dict:
    """Reference-layout QBVH of one mesh, built on the host (no GPU)."""
    L = load()
    v = np.ascontiguousarray(vertices, dtype=np.float32)
    f = np.ascontiguousarray(faces, dtype=np.int32)
    nn, nl = C.c_int64(0), C.c_int64(0)
    rc = L.pr_qbvh_build_host(_p(v), v.shape[0], _p(f), f.shape[0], C.byref(nn), C.byref(nl),
                              None, None, None, None)
    if rc != 0:
        raise PrenderError(rc, "QBVH build rejected the mesh")
    boxes = np.empty((nn.value, 24), np.float32)
    children = np.empty((nn.value, 4), np.int64)
    axes = np.empty((nn.value, 3), np.int32)
    leaf = np.empty(nl.value, np.int32)
    rc = L.pr_qbvh_build_host(_p(v), v.shape[0], _p(f), f.shape[0], None, None, _p(boxes), _p(children),
                              _p(axes), _p(leaf))
    if rc != 0:
        raise PrenderError(rc, "QBVH build failed")
    return dict(boxes=boxes, children=children, axes=axes, leaf=leaf)


def check_scene(scene) -> None:
    """The checks of a scene upload, on the host (no GPU): raises
    PrenderError with pr_scene_upload's status and reason."""
    L = load()
    desc = scene.to_desc()
    msg = C.create_string_buffer(512)
    rc = L.pr_scene_check(desc.ptr(), msg, 512)
    if rc != 0:
        raise PrenderError(rc, msg.value.decode(errors="replace"))


class Context:
    """One GPU context (pr_ctx)."""

    def __init__(self, device: int = 0):
        self.L = load()
        st = C.c_int(0)
        self.h = self.L.pr_create(device, C.byref(st))
        if not self.h:
            raise PrenderError(st.value, f"pr_create({device}) failed (no usable CUDA device?)")
        self._desc = None
        self.scene = None

    def close(self):
        if getattr(self, "h", None):
            self.L.pr_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc: int):
        if rc != 0:
            raise PrenderError(rc, self.L.pr_last_error(self.h).decode())

    # ---- scene ----
    def upload(self, scene) -> None:
        self._desc = scene.to_desc()
        self._check(self.L.pr_scene_upload(self.h, C.byref(self._desc.desc)))
        self.scene = scene

    def qbvh(self, entity: int) -> dict:
        nn, nl = C.c_int64(0), C.c_int64(0)
        self._check(self.L.pr_qbvh_info(self.h, entity, C.byref(nn), C.byref(nl)))
        boxes = np.empty((nn.value, 24), np.float32)
        children = np.empty((nn.value, 4), np.int64)
        axes = np.empty((nn.value, 3), np.int32)
        leaf = np.empty(nl.value, np.int32)
        self._check(self.L.pr_qbvh_export(self.h, entity, _p(boxes), _p(children), _p(axes), _p(leaf)))
        return dict(boxes=boxes, children=children, axes=axes, leaf=leaf)

    # ---- queries ----
    def first_hit(self, rays: np.ndarray) -> dict:
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        n = rays.shape[0]
        ent = np.empty(n, np.int32)
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float64)
        self._check(self.L.pr_first_hit(self.h, _p(rays), n, _p(ent), _p(prim), _p(t)))
        return dict(entity=ent, prim=prim, t=t)

    def trace_fast(self, rays: np.ndarray) -> dict:
        """The renderer's FP32 closest-hit query on the same batch."""
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        n = rays.shape[0]
        ent = np.empty(n, np.int32)
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float64)
        self._check(self.L.pr_trace_fast(self.h, _p(rays), n, _p(ent), _p(prim), _p(t)))
        return dict(entity=ent, prim=prim, t=t)

    def render_adjoint(self, dl_drgb: np.ndarray, scene=None, settings=None, camera=None,
                       sample_offset: int = 0) -> dict:
        """Path-replay adjoint of render(): dLoss/d(material colour) and
        dLoss/d(material emission), (n_materials, 3) each, and dLoss/d(scale)
        of all emission, for dl_drgb = dLoss/d(image) of the image render()
        returned with the same scene, settings, camera and sample_offset."""
        scene = scene or self.scene
        cam = (camera or scene.camera).to_c()
        prm = (settings or scene.settings).to_c()
        g = np.ascontiguousarray(dl_drgb, dtype=np.float32)
        if g.shape != (cam.height, cam.width, 3):
            raise ValueError("dl_drgb must have the image's shape (H, W, 3)")
        n = len(scene.materials)
        d_color = np.zeros((n, 3))
        d_em = np.zeros((n, 3))
        d_scale = C.c_double(0.0)
        self._check(self.L.pr_render_adjoint(self.h, C.byref(cam), C.byref(prm), _p(g), sample_offset,
                                             _p(d_color), _p(d_em), C.byref(d_scale)))
        return dict(color=d_color, emission=d_em, emission_scale=d_scale.value)

    def scene_object(self, scene) -> "SceneObject":
        """An uploaded scene independent of upload() (for render_batch)."""
        return SceneObject(self, scene)

    def render_batch(self, jobs) -> None:
        """Renders (scene_object, out_tensor, settings, camera, sample_offset)
        jobs as one captured CUDA graph; out_tensor is a CUDA float32 tensor
        (H, W, 3) per job (any object with data_ptr())."""
        arr = (A.pr_job * len(jobs))()
        for j, job in enumerate(jobs):
            so, out = job[0], job[1]
            settings = job[2] if len(job) > 2 and job[2] is not None else so.scene.settings
            camera = job[3] if len(job) > 3 and job[3] is not None else so.scene.camera
            arr[j].scene = so.h
            arr[j].camera = camera.to_c()
            arr[j].params = settings.to_c()
            arr[j].rgb_dev = out.data_ptr()
            arr[j].sample_offset = job[4] if len(job) > 4 else 0
            arr[j].accumulate = 0
        self._check(self.L.pr_render_batch(self.h, len(jobs), arr))

    def render_bvh(self, vertices: np.ndarray, faces: np.ndarray, on_gpu: bool) -> dict:
        """The render path's tree of one mesh from the host or the GPU builder
        (pr_render_bvh_export): nodes as raw 80-byte records (uint8, n x 80)
        and the face id of each triangle slot."""
        v = np.ascontiguousarray(vertices, dtype=np.float32)
        f = np.ascontiguousarray(faces, dtype=np.int32)
        m = A.pr_mesh()
        m.n_vertices, m.n_faces = v.shape[0], f.shape[0]
        m.vertices = v.ctypes.data_as(C.POINTER(C.c_float))
        m.faces = f.ctypes.data_as(C.POINTER(C.c_int32))
        m.face_normals = None
        nn, nt = C.c_int64(0), C.c_int64(0)
        self._check(self.L.pr_render_bvh_export(self.h, C.byref(m), int(on_gpu), None, 0, None, 0, C.byref(nn),
                                                C.byref(nt)))
        nodes = np.zeros((nn.value, 80), np.uint8)
        tri = np.zeros(nt.value, np.int32)
        self._check(self.L.pr_render_bvh_export(self.h, C.byref(m), int(on_gpu), _p(nodes), nn.value, _p(tri),
                                                nt.value, C.byref(nn), C.byref(nt)))
        return dict(nodes=nodes, tri_faces=tri)

    def autotune(self, scene=None, settings=None, camera=None) -> dict:
        """Picks the wavefront pool size and traversal grid for this context
        by timing short frames of the scene (pr_autotune_wavefront)."""
        scene = scene or self.scene
        cam = (camera or scene.camera).to_c()
        prm = (settings or scene.settings).to_c()
        sl, bps, ms = C.c_int32(0), C.c_int32(0), C.c_double(0.0)
        self._check(self.L.pr_autotune_wavefront(self.h, C.byref(cam), C.byref(prm), C.byref(sl), C.byref(bps),
                                                 C.byref(ms)))
        return dict(slots=sl.value, trace_blocks_per_sm=bps.value, frame_ms=ms.value)

    def kerr_trace(self, rays: np.ndarray) -> dict:
        """The Kerr branch of intersect_scene per ray (FP64 geodesics);
        status 0 background, 1 entity hit, 2 event horizon, 4 step underflow,
        5 entity ahead of the last step."""
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        n = rays.shape[0]
        out = dict(status=np.empty(n, np.int32), final_bl=np.empty((n, 3)), exit_dir=np.empty((n, 3)),
                   steps=np.empty(n, np.int32), hit_entity=np.empty(n, np.int32), hit_t=np.empty(n))
        self._check(self.L.pr_kerr_trace(self.h, _p(rays), n, _p(out["status"]), _p(out["final_bl"]),
                                         _p(out["exit_dir"]), _p(out["steps"]), _p(out["hit_entity"]),
                                         _p(out["hit_t"])))
        return out

    def wormhole_trace(self, rays: np.ndarray) -> dict:
        """The wormhole branch of intersect_scene__ per ray (FP64 geodesics);
        status 1 entity hit, 0 background 1, 3 background 2."""
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        n = rays.shape[0]
        out = dict(status=np.empty(n, np.int32), final_y=np.empty((n, 3)), exit_dir=np.empty((n, 3)),
                   steps=np.empty(n, np.int32), hit_entity=np.empty(n, np.int32))
        self._check(self.L.pr_wormhole_trace(self.h, _p(rays), n, _p(out["status"]), _p(out["final_y"]),
                                             _p(out["exit_dir"]), _p(out["steps"]), _p(out["hit_entity"])))
        return out

    def kerr_sensitivity(self, rays: np.ndarray, basis: np.ndarray | None = None,
                         cotangent: np.ndarray | None = None) -> dict:
        """Ray-bundle Jacobian of the Kerr map: d(exit direction)/d(s, t)
        (n, 3, 2) and d(final theta, phi)/d(s, t) (n, 2, 2) for rays that
        leave the scene (NaN otherwise); with a cotangent (n, 3), also the
        adjoint product grad = w^T J (n, 2)."""
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        n = rays.shape[0]
        b = None if basis is None else np.ascontiguousarray(basis, dtype=np.float64).reshape(n, 6)
        out = dict(status=np.empty(n, np.int32), jac_dir=np.empty((n, 3, 2)), jac_bl=np.empty((n, 2, 2)))
        self._check(self.L.pr_kerr_sensitivity(self.h, _p(rays), n, _p(b), _p(out["status"]), _p(out["jac_dir"]),
                                               _p(out["jac_bl"])))
        if cotangent is not None:
            w = np.ascontiguousarray(cotangent, dtype=np.float64).reshape(n, 3)
            g = np.empty((n, 2))
            self._check(self.L.pr_kerr_sensitivity_adjoint(self.h, _p(rays), n, _p(b), _p(w), _p(g)))
            out["grad"] = g
        return out

    def to_rgb8(self, image: np.ndarray, gamma_offset: float = 0.0) -> np.ndarray:
        """Render::OutputBmp's 8-bit conversion of an (H, W, 3) float image in
        pr_render's row order; returns (H, W, 3) uint8 rows as the bitmap's
        cell(i, j) holds them (write with scene.write_bmp)."""
        img = np.ascontiguousarray(image, dtype=np.float32)
        h, w = img.shape[0], img.shape[1]
        out = np.empty((h, w, 3), np.uint8)
        self._check(self.L.pr_image_to_rgb8(self.h, _p(img), w, h, float(gamma_offset), _p(out)))
        return out

    def to_rgbe(self, image: np.ndarray) -> np.ndarray:
        """Render::OutputHdr's Radiance RGBE pixels of an (H, W, 3) float image
        in pr_render's row order; returns (H, W, 4) uint8, scanline r = image
        row r (write with scene.write_hdr)."""
        img = np.ascontiguousarray(image, dtype=np.float32)
        h, w = img.shape[0], img.shape[1]
        out = np.empty((h, w, 4), np.uint8)
        self._check(self.L.pr_image_to_rgbe(self.h, _p(img), w, h, _p(out)))
        return out

    def kerr_disk_shade(self, entity: int, points: np.ndarray) -> dict:
        """The accretion disk's texture / temperature / Doppler shading at
        world points of disk entity (no alpha test): valid, colour,
        emission, alpha."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        n = pts.shape[0]
        out = dict(valid=np.empty(n, np.int32), color=np.empty((n, 3)), emission=np.empty((n, 3)),
                   alpha=np.empty(n))
        self._check(self.L.pr_kerr_disk_shade(self.h, int(entity), _p(pts), n, _p(out["valid"]), _p(out["color"]),
                                              _p(out["emission"]), _p(out["alpha"])))
        return out

    def render(self, scene=None, settings=None, camera=None, sample_offset: int = 0,
               accumulate: np.ndarray | None = None) -> np.ndarray:
        """Render::Run: returns the (H, W, 3) float32 image in the reference's
        row order (row 0 = image index 0, i.e. the bottom scan line)."""
        scene = scene or self.scene
        cam = (camera or scene.camera).to_c()
        prm = (settings or scene.settings).to_c()
        if accumulate is not None:
            out = np.ascontiguousarray(accumulate, dtype=np.float32)
        else:
            out = np.empty((cam.height, cam.width, 3), np.float32)
        self._check(self.L.pr_render(self.h, C.byref(cam), C.byref(prm), _p(out), sample_offset,
                                     1 if accumulate is not None else 0))
        return out

    def stats(self) -> dict:
        s = A.pr_render_stats()
        self._check(self.L.pr_last_render_stats(self.h, C.byref(s)))
        return dict(paths=s.paths, segments=s.segments, nodes_visited=s.nodes_visited, tri_tests=s.tri_tests,
                    device_ms=s.device_ms, kernel_launches=s.kernel_launches)


class SceneObject:
    """A scene uploaded as its own object (pr_scene_create)."""

    def __init__(self, ctx: "Context", scene):
        self.ctx = ctx
        self.scene = scene
        self._desc = scene.to_desc()
        st = C.c_int(0)
        self.h = ctx.L.pr_scene_create(ctx.h, self._desc.ptr(), C.byref(st))
        if not self.h:
            raise PrenderError(st.value, f"pr_scene_create failed: {ctx.L.pr_last_error(ctx.h).decode()}")

    def release(self):
        if self.h:
            self.ctx.L.pr_scene_release(self.ctx.h, self.h)
            self.h = None
