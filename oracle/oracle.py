"""ctypes binding of the CPU restatement (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU
baseline leg of bench.py, never by the product package.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "prender_ref")

_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB) or _stale():
        subprocess.run(["bash", os.path.join(HERE, "build_oracle.sh")], check=True, capture_output=True)
    return LIB


def _stale() -> bool:
    t = os.path.getmtime(LIB)
    for f in ("prender_oracle.cpp", "oracle_math.h"):
        p = os.path.join(HERE, f)
        if os.path.exists(p) and os.path.getmtime(p) > t:
            return True
    return os.path.getmtime(os.path.join(HERE, "..", "include", "prender_gpu.h")) > t


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.oracle_scene_create.restype = vp
        L.oracle_scene_create.argtypes = [vp, C.POINTER(C.c_int), C.c_char_p, C.c_int]
        L.oracle_scene_destroy.argtypes = [vp]
        L.oracle_qbvh_info.argtypes = [vp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.oracle_qbvh_export.argtypes = [vp, C.c_int, vp, vp, vp, vp]
        L.oracle_first_hit.argtypes = [vp, vp, C.c_int64, vp, vp, vp, vp, vp, vp, vp]
        L.oracle_radiance.argtypes = [vp, vp, C.c_int64, C.c_uint64, vp, vp]
        L.oracle_render.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp]
        L.oracle_render_rows.argtypes = [vp, vp, vp, C.c_int, vp, C.c_int, vp, vp, vp]
        L.oracle_light_count.argtypes = [vp]
        L.oracle_kerr_trace.argtypes = [vp, vp, C.c_int64, vp, vp, vp, vp, vp, vp, vp, vp]
        L.oracle_render_mlt.argtypes = [vp, vp, vp, C.c_double, C.c_double, vp]
        L.oracle_wormhole_trace.argtypes = [vp, C.c_int, vp, C.c_int64, vp, vp, vp, vp, vp]
        L.oracle_kerr_trace_threads.argtypes = [vp, C.c_int, vp, C.c_int64, vp, vp, vp, vp, vp, vp, vp, vp]
        L.oracle_kerr_disk_shade.argtypes = [vp, C.c_int, vp, C.c_int64, vp, vp, vp, vp]
        L.oracle_sample_hg.argtypes = [C.c_double, C.c_int, C.c_uint64, vp, C.c_int64, vp]
        _lib = L
    return _lib


def sample_hg(g: float, correct: bool, seed: int, raydir, n: int) -> np.ndarray:
    """n scattering directions of sampleHG about raydir (n x 3)"""
    d = np.ascontiguousarray(raydir, dtype=np.float64)
    out = np.empty((n, 3), np.float64)
    assert lib().oracle_sample_hg(float(g), int(bool(correct)), int(seed), _p(d), int(n), _p(out)) == 0
    return out


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


class OracleScene:
    def __init__(self, scene):
        self.scene = scene
        self._desc = scene.to_desc()
        st = C.c_int(0)
        err = C.create_string_buffer(512)
        self.h = lib().oracle_scene_create(C.addressof(self._desc.desc), C.byref(st), err, 512)
        if not self.h:
            raise RuntimeError(f"oracle scene rejected ({st.value}): {err.value.decode()}")

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_scene_destroy(self.h)
            self.h = None

    def first_hit(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        n = rays.shape[0]
        ent = np.empty(n, np.int32)
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float64)
        pos = np.empty((n, 3), np.float64)
        nrm = np.empty((n, 3), np.float64)
        nodes = C.c_uint64(0)
        tris = C.c_uint64(0)
        rc = lib().oracle_first_hit(self.h, _p(rays), n, _p(ent), _p(prim), _p(t), _p(pos), _p(nrm),
                                    C.byref(nodes), C.byref(tris))
        assert rc == 0, rc
        return dict(entity=ent, prim=prim, t=t, pos=pos, normal=nrm, nodes=nodes.value, tri_tests=tris.value)

    def qbvh(self, entity: int):
        nn, nl = C.c_int64(0), C.c_int64(0)
        assert lib().oracle_qbvh_info(self.h, entity, C.byref(nn), C.byref(nl)) == 0
        boxes = np.empty((nn.value, 24), np.float32)
        children = np.empty((nn.value, 4), np.int64)
        axes = np.empty((nn.value, 3), np.int32)
        leaf = np.empty(nl.value, np.int32)
        assert lib().oracle_qbvh_export(self.h, entity, _p(boxes), _p(children), _p(axes), _p(leaf)) == 0
        return dict(boxes=boxes, children=children, axes=axes, leaf=leaf)

    def render(self, threads: int = 1, row0: int = 0, row1: int = 0, settings=None):
        cam = self.scene.camera.to_c()
        prm = (settings or self.scene.settings).to_c()
        img = np.zeros((cam.height, cam.width, 3), np.float64)
        secs = C.c_double(0)
        segs = C.c_uint64(0)
        rc = lib().oracle_render(self.h, C.byref(cam), C.byref(prm), threads, row0, row1, _p(img),
                                 C.byref(secs), C.byref(segs))
        assert rc == 0, rc
        return img, secs.value, segs.value

    def render_mlt(self, settings=None):
        """Render::RunMLT on one thread (the reference's chains in order);
        settings.samples chains of settings.mutation / pre_sample per pixel."""
        st = settings or self.scene.settings
        cam = self.scene.camera.to_c()
        prm = st.to_c()
        img = np.zeros((cam.height, cam.width, 3), np.float64)
        rc = lib().oracle_render_mlt(self.h, C.byref(cam), C.byref(prm), float(st.mutation), float(st.pre_sample),
                                     _p(img))
        assert rc == 0, rc
        return img

    def render_rows(self, rows, threads: int = 1, settings=None):
        """Render::Run over the given image rows only (the rest stays zero)."""
        cam = self.scene.camera.to_c()
        prm = (settings or self.scene.settings).to_c()
        r = np.ascontiguousarray(rows, dtype=np.int32)
        img = np.zeros((cam.height, cam.width, 3), np.float64)
        secs = C.c_double(0)
        segs = C.c_uint64(0)
        rc = lib().oracle_render_rows(self.h, C.byref(cam), C.byref(prm), threads, _p(r), int(r.size), _p(img),
                                      C.byref(secs), C.byref(segs))
        assert rc == 0, rc
        return img, secs.value, segs.value

    def radiance(self, rays: np.ndarray, seed: int, settings=None):
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        prm = (settings or self.scene.settings).to_c()
        out = np.empty((rays.shape[0], 3), np.float64)
        assert lib().oracle_radiance(self.h, _p(rays), rays.shape[0], seed, C.byref(prm), _p(out)) == 0
        return out

    def kerr_trace(self, rays: np.ndarray, threads: int = 1):
        """Kerr branch of intersect_scene per ray; status 0 background,
        1 entity hit, 2 event horizon, 4 step underflow, 5 entity ahead of the
        last step; with the hit point's colour and emission (the accretion
        disk rewrites them, drawing its alpha test from the scene stream
        seeded with the black hole's disk_seed, one stream over the rays).
        threads > 1 traces in parallel where no such disk is in the scene."""
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        n = rays.shape[0]
        out = dict(status=np.empty(n, np.int32), final_bl=np.empty((n, 3)), exit_dir=np.empty((n, 3)),
                   steps=np.empty(n, np.int32), hit_entity=np.empty(n, np.int32), hit_t=np.empty(n),
                   hit_color=np.empty((n, 3)), hit_emission=np.empty((n, 3)))
        rc = lib().oracle_kerr_trace_threads(self.h, int(threads), _p(rays), n, _p(out["status"]), _p(out["final_bl"]),
                                     _p(out["exit_dir"]), _p(out["steps"]), _p(out["hit_entity"]),
                                     _p(out["hit_t"]), _p(out["hit_color"]), _p(out["hit_emission"]))
        assert rc == 0, rc
        return out

    def wormhole_trace(self, rays: np.ndarray, threads: int = 1):
        """The wormhole branch of intersect_scene per ray: status 1 entity
        hit, 0 background 1 (l >= 0), 3 background 2; final (l, theta, phi)
        with the angles of the last polyline direction, that direction,
        steps, hit entity"""
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        n = rays.shape[0]
        out = dict(status=np.empty(n, np.int32), final_y=np.empty((n, 3)), exit_dir=np.empty((n, 3)),
                   steps=np.empty(n, np.int32), hit_entity=np.empty(n, np.int32))
        rc = lib().oracle_wormhole_trace(self.h, int(threads), _p(rays), n, _p(out["status"]), _p(out["final_y"]),
                                         _p(out["exit_dir"]), _p(out["steps"]), _p(out["hit_entity"]))
        assert rc == 0, rc
        return out

    def kerr_disk_shade(self, entity: int, points: np.ndarray):
        """The accretion disk's texture / temperature / Doppler shading at
        world points of disk entity (no alpha test): valid, colour,
        emission, alpha."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        n = pts.shape[0]
        out = dict(valid=np.empty(n, np.int32), color=np.empty((n, 3)), emission=np.empty((n, 3)),
                   alpha=np.empty(n))
        rc = lib().oracle_kerr_disk_shade(self.h, int(entity), _p(pts), n, _p(out["valid"]), _p(out["color"]),
                                          _p(out["emission"]), _p(out["alpha"]))
        assert rc == 0, rc
        return out


def reference_available() -> bool:
    return os.path.exists(REF_BIN)
