"""Generates the golden fixtures in tests/golden/ by running the reference
renderer itself (Sanaxen/prender, compiled by oracle/build_ref.sh).

Run from the repository root in a container where the reference sources are
mounted:

    python tests/golden/make_golden.py [REFERENCE_ROOT]

Each fixture stores the synthetic inputs (scene parameters, rays) together
with the reference's outputs, so the tests need neither the reference nor
its build on the machine that runs them.

    python tests/golden/make_golden.py --sss-oracle

writes sss_oracle.npz from the oracle alone (no reference build needed);
--disk-oracle, --sss-l1-oracle, --glossy-oracle, --media-oracle,
--mesh7-oracle, --batch-oracle and --lights-oracle write kerr_disk_oracle.npz,
sss_l1_oracle.npz, glossy_oracle.npz, media_oracle.npz, mesh7_oracle.npz,
batch_oracle.npz and lights_oracle.npz the same way; --media-only,
--batch-only and --lights-only write the reference's own one-thread media,
batch-variant and light-kind renders, --hdr-only its Render::OutputHdr file
of a seeded image; --textures-only and --textures-oracle do the same for the
texture and image-based-lighting scenes (textures_render.npz,
textures_oracle.npz); --wormhole-only writes the reference's one-thread
wormhole renders (wormhole_render.npz), --wormhole-oracle the oracle's
16 batches of each wormhole scene (wormhole_oracle.npz); --meshtex-only and
--meshtex-oracle do the same for smooth and textured meshes
(meshtex_render.npz, meshtex_oracle.npz); --mlt-only writes the reference's
one-thread Metropolis renders (mlt_render.npz), --mlt-oracle the oracle's
path-traced expectation of the GPU Metropolis scenes (mlt_oracle.npz).
--scene-files-only writes the meshes and textures that the scene files in
scene_files/ name, and scene_files.npz from the reference's renders of them.
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from prender_gb300 import scenes  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "prender_ref")


def run_ref(args, cwd, threads=1, scene_seed=1):
    # PRENDER_SCENE_RAND_SEED: the harness reseeds the scene's own generator
    # (the accretion disk's alpha test), which the reference seeds from the clock
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), PRENDER_SCENE_RAND_SEED=str(scene_seed))
    r = subprocess.run([REF_BIN] + args, cwd=cwd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"reference failed: {args}\n{r.stderr[-2000:]}")
    return r.stdout


def ref_qbvh(path, ent, d):
    run_ref(["qbvh", path, str(ent), os.path.join(d, "q.bin")], d)
    b = open(os.path.join(d, "q.bin"), "rb").read()
    nn, nl = struct.unpack("qq", b[:16])
    rec = np.dtype([("boxes", "<f4", 24), ("ch", "<u8", 4), ("ax", "<i4", 3)])
    nodes = np.frombuffer(b[16:16 + nn * rec.itemsize], dtype=rec)
    leaf = np.frombuffer(b[16 + nn * rec.itemsize:], dtype="<i4").copy()
    children = nodes["ch"].view(np.int64).copy()
    boxes = nodes["boxes"].reshape(nn, 6, 4).copy()
    # slots with an invalid child carry uninitialised boxes in the reference
    boxes = np.where((children == -1)[:, None, :], np.float32(0), boxes).reshape(nn, 24)
    return dict(boxes=boxes, children=children, axes=nodes["ax"].copy(), leaf=leaf)


def ref_firsthit(path, rays, d):
    rays.astype(np.float64).tofile(os.path.join(d, "rays.f64"))
    run_ref(["firsthit", path, os.path.join(d, "rays.f64"), os.path.join(d, "fh.bin")], d)
    rec = np.dtype([("ent", "<i4"), ("prim", "<i4"), ("t", "<f8"), ("pn", "<f8", 6)])
    fh = np.fromfile(os.path.join(d, "fh.bin"), dtype=rec)
    return dict(entity=fh["ent"].copy(), prim=fh["prim"].copy(), t=fh["t"].copy())


def ref_radiance(path, rays, seed, d):
    rays.astype(np.float64).tofile(os.path.join(d, "rays.f64"))
    run_ref(["radiance", path, os.path.join(d, "rays.f64"), os.path.join(d, "rad.f64"), str(seed)], d)
    return np.fromfile(os.path.join(d, "rad.f64")).reshape(-1, 3)


def ref_render(path, shape, d, threads=1):
    out = run_ref(["render", path, os.path.join(d, "img.f64")], d, threads)
    return np.fromfile(os.path.join(d, "img.f64")).reshape(shape[1], shape[0], 3), out.strip().splitlines()[-1]


def ref_kerr(path, rays, d):
    """harness record per ray: object id, hit flag, 16 doubles (loop ended,
    steps, y[6], org2, dir2, hit distance, 0), hit colour and emission"""
    rays.astype(np.float64).tofile(os.path.join(d, "rays.f64"))
    run_ref(["kerr", path, os.path.join(d, "rays.f64"), os.path.join(d, "k.bin")], d)
    rec = np.dtype([("obj", "<i4"), ("hit", "<i4"), ("rec", "<f8", 16), ("col", "<f8", 3), ("em", "<f8", 3)])
    k = np.fromfile(os.path.join(d, "k.bin"), dtype=rec)
    return dict(obj=k["obj"].copy(), hit=k["hit"].copy(), rec=k["rec"].copy(), col=k["col"].copy(),
                em=k["em"].copy())


def kerr_golden(d):
    sys.path.insert(0, os.path.dirname(HERE))
    import kerr_cases
    out = {}
    for name, (sc, rays) in kerr_cases.trace_cases().items():
        dd = os.path.join(d, "k_" + name)
        os.makedirs(dd)
        r = ref_kerr(sc.write_reference(dd), rays, dd)
        out[f"{name}_rays"] = rays
        out.update({f"{name}_{k}": v for k, v in r.items()})
    np.savez_compressed(os.path.join(HERE, "kerr_trace.npz"), **out)
    imgs = {}
    for name, sc in kerr_cases.render_cases().items():
        dd = os.path.join(d, "kr_" + name)
        os.makedirs(dd)
        img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
        imgs[name] = img
        print("kerr", name, info)
    sc = kerr_cases.highspp_case()
    dd = os.path.join(d, "kr_highspp")
    os.makedirs(dd)
    img, info = ref_render(sc.write_reference(dd, threads=os.cpu_count()), (sc.camera.width, sc.camera.height), dd,
                           threads=os.cpu_count())
    imgs["texture_highspp"] = img.astype(np.float32)
    print("kerr texture_highspp", info)
    np.savez_compressed(os.path.join(HERE, "kerr_render.npz"), **imgs)


def disk_golden(d):
    """textured accretion disk under the black hole: per-ray traces with the
    hit point's colour and emission, one-thread renders (the harness seeds
    the scene's alpha-test generator with the scenes' disk_seed, 1)"""
    sys.path.insert(0, os.path.dirname(HERE))
    import kerr_cases
    out = {}
    for name, (sc, rays) in kerr_cases.disk_trace_cases().items():
        dd = os.path.join(d, "kd_" + name)
        os.makedirs(dd)
        r = ref_kerr(sc.write_reference(dd), rays, dd)
        out[f"{name}_rays"] = rays
        out.update({f"{name}_{k}": v for k, v in r.items()})
    for name, sc in kerr_cases.disk_render_cases().items():
        dd = os.path.join(d, "kdr_" + name)
        os.makedirs(dd)
        img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
        out[f"render_{name}"] = img
        print("disk", name, info)
    np.savez_compressed(os.path.join(HERE, "kerr_disk.npz"), **out)


def disk_oracle_golden(nb=16):
    """16 independent renders of the textured-disk high-spp case by the
    oracle (pinned to the reference by kerr_disk.npz): per-pixel mean and
    standard deviation for the GPU's statistical parity."""
    sys.path.insert(0, os.path.dirname(HERE))
    import kerr_cases
    from oracle import oracle as O
    sc = kerr_cases.disk_highspp_case()
    imgs = []
    for k in range(nb):
        sc.settings.seed = 100 + k
        sc.kerr["disk_seed"] = 1000 + k
        img, _, _ = O.OracleScene(sc).render(threads=os.cpu_count())
        imgs.append(img)
    b = np.stack(imgs)
    np.savez_compressed(os.path.join(HERE, "kerr_disk_oracle.npz"), mean=b.mean(0).astype(np.float32),
                        sd=b.std(0, ddof=1).astype(np.float32), batches=np.int32(nb))
    print("disk oracle batches", nb)


def sss_golden(d):
    """subsurface (directional dipole) renders: one thread bit-exact, and a
    high-spp image for the GPU's statistical parity"""
    out = {}
    sc = scenes.sss_cornell(width=24, height=18, samples=1, supersamples=2, subdiv=3)
    dd = os.path.join(d, "s_1t")
    os.makedirs(dd)
    img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
    out["sss_1thread"] = img
    print("sss 1thread", info)
    sc = scenes.sss_cornell(width=64, height=48, samples=128, supersamples=2, subdiv=3)
    dd = os.path.join(d, "s_hi")
    os.makedirs(dd)
    img, info = ref_render(sc.write_reference(dd, threads=os.cpu_count()), (sc.camera.width, sc.camera.height), dd,
                           threads=os.cpu_count())
    out["sss_64x48_512spp"] = img.astype(np.float32)
    print("sss highspp", info)
    np.savez_compressed(os.path.join(HERE, "sss_render.npz"), **out)


def sss_l1_golden(d):
    """level -1 subsurface renders by the reference, one thread (bit-exact)"""
    sys.path.insert(0, os.path.dirname(HERE))
    import sss_cases
    out = {}
    for name, sc in sss_cases.l1_cases().items():
        dd = os.path.join(d, "s_" + name)
        os.makedirs(dd)
        img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
        out[name] = img
        print("sss", name, info)
    np.savez_compressed(os.path.join(HERE, "sss_l1_render.npz"), **out)


def glossy_golden(d):
    """Ward and Phong renders by the reference, one thread (bit-exact)"""
    sys.path.insert(0, os.path.dirname(HERE))
    import glossy_cases
    out = {}
    for name, sc in glossy_cases.one_thread_cases().items():
        dd = os.path.join(d, "g_" + name)
        os.makedirs(dd)
        img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
        out[name] = img
        print("glossy", name, info)
    np.savez_compressed(os.path.join(HERE, "glossy_render.npz"), **out)


def glossy_oracle_golden(nb=16):
    """16 independent 512-spp renders of each glossy scene by the oracle:
    per-pixel mean and standard deviation for the GPU's statistical parity"""
    sys.path.insert(0, os.path.dirname(HERE))
    import glossy_cases
    from oracle import oracle as O
    out = {}
    for mat in ("ward", "phong"):
        sc = glossy_cases.highspp_case(mat)
        imgs = []
        for k in range(nb):
            sc.settings.seed = 100 + k
            img, _, _ = O.OracleScene(sc).render(threads=os.cpu_count())
            imgs.append(img)
        b = np.stack(imgs)
        out[f"{mat}_mean"] = b.mean(0).astype(np.float32)
        out[f"{mat}_sd"] = b.std(0, ddof=1).astype(np.float32)
    out["batches"] = np.int32(nb)
    np.savez_compressed(os.path.join(HERE, "glossy_oracle.npz"), **out)
    print("glossy oracle batches", nb)


def sss_oracle_golden(nb=16, level=-2):
    """16 independent 512-spp renders of the 64x48 subsurface scene by the
    oracle (pinned bit-exact to the reference by the one-thread fixtures):
    per-pixel mean and standard deviation, the symmetric high-spp target for
    the GPU's statistical parity.  Needs no reference build."""
    from oracle import oracle as O
    sc = scenes.sss_cornell(width=64, height=48, samples=128, supersamples=2, subdiv=3, level=level)
    imgs = []
    for k in range(nb):
        sc.settings.seed = 100 + k
        img, _, _ = O.OracleScene(sc).render(threads=os.cpu_count())
        imgs.append(img)
    b = np.stack(imgs)
    name = "sss_oracle.npz" if level == -2 else "sss_l1_oracle.npz"
    np.savez_compressed(os.path.join(HERE, name), mean_64x48_8192spp=b.mean(0).astype(np.float32),
                        sd_64x48_512spp=b.std(0, ddof=1).astype(np.float32), batches=np.int32(nb))
    print("sss oracle batches", nb, "level", level)


def media_golden(d):
    """participating-media renders by the reference, one thread (bit-exact),
    and per-ray radiance() roots, over the media cases' sigma_s, g and NEE"""
    sys.path.insert(0, os.path.dirname(HERE))
    import media_cases
    out = {}
    for name, sc in media_cases.one_thread_cases().items():
        dd = os.path.join(d, "m_" + name)
        os.makedirs(dd)
        img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
        out[f"render_{name}"] = img
        print("media", name, info)
    for name, sc in media_cases.root_cases().items():
        dd = os.path.join(d, "mr_" + name)
        os.makedirs(dd)
        r = scenes.camera_rays(sc)
        out[f"roots_{name}_rays"] = r
        out[f"roots_{name}_rgb"] = ref_radiance(sc.write_reference(dd), r, 7, dd)
    np.savez_compressed(os.path.join(HERE, "media_render.npz"), **out)


def media_oracle_golden(nb=16):
    """16 independent 256-spp renders of each media case by the oracle
    (pinned bit-exact to the reference by media_render.npz; its HG-correct
    sampler by the HG distribution): per-pixel mean and spread"""
    sys.path.insert(0, os.path.dirname(HERE))
    import media_cases
    from oracle import oracle as O
    out = {}
    for name in media_cases.CASES:
        sc = media_cases.highspp_case(name)
        imgs = []
        for k in range(nb):
            sc.settings.seed = 100 + k
            img, _, _ = O.OracleScene(sc).render(threads=os.cpu_count())
            imgs.append(img)
        b = np.stack(imgs)
        out[f"{name}_mean"] = b.mean(0).astype(np.float32)
        out[f"{name}_sd"] = b.std(0, ddof=1).astype(np.float32)
        print("media oracle", name, float(b.mean()))
    out["batches"] = np.int32(nb)
    np.savez_compressed(os.path.join(HERE, "media_oracle.npz"), **out)


def hdr_golden(d):
    """Render::OutputHdr of a seeded image by the reference: the image (float32,
    as pr_render returns it) and the file's bytes"""
    rng = np.random.default_rng(11)
    w, h = 300, 23  # wider than one 127-byte literal run, two bytes of width
    img = np.exp(rng.uniform(np.log(1e-6), np.log(50.0), (h, w, 3))).astype(np.float32)
    img[0, :5] = 0.0                   # black
    img[1, :3] = (1e-33, 0.0, 0.0)     # below the 1e-32 cut
    img[2, :4] = (1.0, 0.5, 0.25)      # exact powers of two
    img[3, :2] = (255.9, 1.0, 0.001)
    sc = scenes.cornell_spheres(width=w, height=h, samples=1, supersamples=1)
    p = sc.write_reference(d)
    img.astype(np.float64).reshape(-1, 3).tofile(os.path.join(d, "img.f64"))
    run_ref(["hdr", p, os.path.join(d, "img.f64"), os.path.join(d, "out.hdr")], d)
    data = np.frombuffer(open(os.path.join(d, "out.hdr"), "rb").read(), np.uint8)
    np.savez_compressed(os.path.join(HERE, "hdr_output.npz"), image=img, hdr=data)
    print("hdr bytes", data.size)


def batch_golden(d):
    """media + BSSRDF batch variants rendered by the reference, one thread (bit-exact)"""
    sys.path.insert(0, os.path.dirname(HERE))
    import batch_cases
    out = {}
    for name, sc in batch_cases.one_thread_cases().items():
        dd = os.path.join(d, "b_" + name)
        os.makedirs(dd)
        img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
        out[name] = img
        print("batch", name, info)
    np.savez_compressed(os.path.join(HERE, "batch_render.npz"), **out)


def batch_oracle_golden(nb=16):
    """16 independent 256-spp renders of each high-spp batch variant by the
    oracle: per-pixel mean and spread"""
    sys.path.insert(0, os.path.dirname(HERE))
    import batch_cases
    from oracle import oracle as O
    out = {}
    for i, sc in enumerate(batch_cases.highspp_variants()):
        o = O.OracleScene(sc)
        imgs = []
        for k in range(nb):
            sc.settings.seed = 100 + k
            img, _, _ = o.render(threads=os.cpu_count(), settings=sc.settings)
            imgs.append(img)
        b = np.stack(imgs)
        out[f"v{i}_mean"] = b.mean(0).astype(np.float32)
        out[f"v{i}_sd"] = b.std(0, ddof=1).astype(np.float32)
        print("batch oracle", i, sc.camera.width, float(b.mean()))
    out["batches"] = np.int32(nb)
    np.savez_compressed(os.path.join(HERE, "batch_oracle.npz"), **out)


def lights_golden(d):
    """spot / parallel / infinity light scenes rendered by the reference, one thread (bit-exact)"""
    sys.path.insert(0, os.path.dirname(HERE))
    import lights_cases
    out = {}
    for name, sc in lights_cases.one_thread_cases().items():
        dd = os.path.join(d, "l_" + name)
        os.makedirs(dd)
        img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
        out[name] = img
        print("lights", name, info, float(img.mean()))
    np.savez_compressed(os.path.join(HERE, "lights_render.npz"), **out)


def lights_oracle_golden(nb=16):
    """16 independent 256-spp renders of each light-kind scene by the
    oracle (pinned bit-exact to the reference by lights_render.npz):
    per-pixel mean and spread"""
    sys.path.insert(0, os.path.dirname(HERE))
    import lights_cases
    from oracle import oracle as O
    out = {}
    for name in lights_cases.CASES:
        sc = lights_cases.highspp_case(name)
        o = O.OracleScene(sc)
        imgs = []
        for k in range(nb):
            sc.settings.seed = 100 + k
            img, _, _ = o.render(threads=os.cpu_count(), settings=sc.settings)
            imgs.append(img)
        b = np.stack(imgs)
        out[f"{name}_mean"] = b.mean(0).astype(np.float32)
        out[f"{name}_sd"] = b.std(0, ddof=1).astype(np.float32)
        print("lights oracle", name, float(b.mean()))
    out["batches"] = np.int32(nb)
    np.savez_compressed(os.path.join(HERE, "lights_oracle.npz"), **out)


def textures_golden(d):
    """texture and IBL scenes rendered by the reference, one thread (bit-exact)"""
    sys.path.insert(0, os.path.dirname(HERE))
    import texture_cases
    out = {}
    for name, sc in texture_cases.one_thread_cases().items():
        dd = os.path.join(d, "t_" + name)
        os.makedirs(dd)
        img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
        out[name] = img
        print("textures", name, info, float(img.mean()))
    np.savez_compressed(os.path.join(HERE, "textures_render.npz"), **out)


def meshtex_golden(d):
    """smooth and textured meshes rendered by the reference, one thread (bit-exact)"""
    sys.path.insert(0, os.path.dirname(HERE))
    import meshtex_cases
    out = {}
    for name, sc in meshtex_cases.one_thread_cases().items():
        dd = os.path.join(d, "m_" + name)
        os.makedirs(dd)
        img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
        out[name] = img
        print("meshtex", name, info, float(img.mean()))
    np.savez_compressed(os.path.join(HERE, "meshtex_render.npz"), **out)


def mlt_golden(d):
    """Metropolis (RunMLT) renders by the reference, one thread (bit-exact)"""
    sys.path.insert(0, os.path.dirname(HERE))
    import mlt_cases
    out = {}
    for name, sc in mlt_cases.one_thread_cases().items():
        dd = os.path.join(d, "l_" + name)
        os.makedirs(dd)
        img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
        out[name] = img
        print("mlt", name, info, float(img.mean()))
    np.savez_compressed(os.path.join(HERE, "mlt_render.npz"), **out)


def mlt_oracle_golden(nb=16):
    """16 independent 256-spp path-traced renders (no luminance clamp) of each
    Metropolis scene by the oracle: the expectation the Metropolis image
    converges to, per-pixel mean and spread"""
    sys.path.insert(0, os.path.dirname(HERE))
    import mlt_cases
    from oracle import oracle as O
    out = {}
    for name in mlt_cases.CASES:
        sc = mlt_cases.gpu_case(name)
        o = O.OracleScene(sc)
        st = mlt_cases.pt_settings(sc)
        imgs = []
        for k in range(nb):
            st.seed = 100 + k
            img, _, _ = o.render(threads=os.cpu_count(), settings=st)
            imgs.append(img)
        b = np.stack(imgs)
        out[f"{name}_mean"] = b.mean(0).astype(np.float32)
        out[f"{name}_sd"] = b.std(0, ddof=1).astype(np.float32)
        print("mlt oracle", name, float(b.mean()))
    out["batches"] = np.int32(nb)
    np.savez_compressed(os.path.join(HERE, "mlt_oracle.npz"), **out)


def meshtex_oracle_golden(nb=16):
    """16 independent 256-spp renders of each smooth / textured mesh scene
    by the oracle (pinned bit-exact to the reference by meshtex_render.npz):
    per-pixel mean and spread"""
    sys.path.insert(0, os.path.dirname(HERE))
    import meshtex_cases
    from oracle import oracle as O
    out = {}
    for name in meshtex_cases.CASES:
        sc = meshtex_cases.highspp_case(name)
        o = O.OracleScene(sc)
        imgs = []
        for k in range(nb):
            sc.settings.seed = 100 + k
            img, _, _ = o.render(threads=os.cpu_count(), settings=sc.settings)
            imgs.append(img)
        b = np.stack(imgs)
        out[f"{name}_mean"] = b.mean(0).astype(np.float32)
        out[f"{name}_sd"] = b.std(0, ddof=1).astype(np.float32)
        print("meshtex oracle", name, float(b.mean()))
    out["batches"] = np.int32(nb)
    np.savez_compressed(os.path.join(HERE, "meshtex_oracle.npz"), **out)


def textures_oracle_golden(nb=16):
    """16 independent 256-spp renders of each texture scene by the oracle
    (pinned bit-exact to the reference by textures_render.npz): per-pixel
    mean and spread"""
    sys.path.insert(0, os.path.dirname(HERE))
    import texture_cases
    from oracle import oracle as O
    out = {}
    for name in texture_cases.CASES:
        sc = texture_cases.highspp_case(name)
        o = O.OracleScene(sc)
        imgs = []
        for k in range(nb):
            sc.settings.seed = 100 + k
            img, _, _ = o.render(threads=os.cpu_count(), settings=sc.settings)
            imgs.append(img)
        b = np.stack(imgs)
        out[f"{name}_mean"] = b.mean(0).astype(np.float32)
        out[f"{name}_sd"] = b.std(0, ddof=1).astype(np.float32)
        print("textures oracle", name, float(b.mean()))
    out["batches"] = np.int32(nb)
    np.savez_compressed(os.path.join(HERE, "textures_oracle.npz"), **out)


def wormhole_oracle_golden(nb=16):
    """16 independent 64-spp renders of each wormhole scene by the oracle
    (pinned bit-exact to the reference by wormhole_render.npz): per-pixel
    mean and spread"""
    sys.path.insert(0, os.path.dirname(HERE))
    import wormhole_cases
    from oracle import oracle as O
    out = {}
    for name in wormhole_cases.CASES:
        sc = wormhole_cases.highspp_case(name)
        o = O.OracleScene(sc)
        imgs = []
        for k in range(nb):
            sc.settings.seed = 100 + k
            img, _, _ = o.render(threads=os.cpu_count(), settings=sc.settings)
            imgs.append(img)
        b = np.stack(imgs)
        out[f"{name}_mean"] = b.mean(0).astype(np.float32)
        out[f"{name}_sd"] = b.std(0, ddof=1).astype(np.float32)
        print("wormhole oracle", name, float(b.mean()))
    out["batches"] = np.int32(nb)
    np.savez_compressed(os.path.join(HERE, "wormhole_oracle.npz"), **out)


def wormhole_golden(d):
    """wormhole scenes rendered by the reference, one thread (bit-exact)"""
    sys.path.insert(0, os.path.dirname(HERE))
    import wormhole_cases
    out = {}
    for name, sc in wormhole_cases.one_thread_cases().items():
        dd = os.path.join(d, "w_" + name)
        os.makedirs(dd)
        img, info = ref_render(sc.write_reference(dd), (sc.camera.width, sc.camera.height), dd, threads=1)
        out[name] = img
        print("wormhole", name, info, float(img.mean()))
    np.savez_compressed(os.path.join(HERE, "wormhole_render.npz"), **out)


def mesh7_oracle_golden(nb=16):
    """The benchmarked scene itself (327,680-triangle displaced icosphere,
    diffuse and glass) at 128 x 96, 16 independent 256-spp renders by the
    oracle: per-pixel mean and spread"""
    from oracle import oracle as O
    out = {}
    for mat in ("diffuse", "glass"):
        sc = scenes.mesh_cornell(width=128, height=96, samples=64, supersamples=2, subdiv=7, material=mat)
        o = O.OracleScene(sc)
        imgs = []
        for k in range(nb):
            sc.settings.seed = 100 + k
            img, _, _ = o.render(threads=os.cpu_count(), settings=sc.settings)
            imgs.append(img)
        b = np.stack(imgs)
        out[f"{mat}_mean"] = b.mean(0).astype(np.float32)
        out[f"{mat}_sd"] = b.std(0, ddof=1).astype(np.float32)
        print("mesh subdiv 7 oracle", mat, float(b.mean()))
    out["batches"] = np.int32(nb)
    np.savez_compressed(os.path.join(HERE, "mesh7_oracle.npz"), **out)


SCENE_DIR = os.path.join(HERE, "scene_files")
SCENE_FILES = ("spheres_expr", "mesh_obj", "media", "sss", "kerr_disk")


def _grid(o, u, v, n):
    """(n+1)^2 vertices of the parallelogram o + s u + t v"""
    o, u, v = (np.asarray(x, dtype=np.float64) for x in (o, u, v))
    return [o + u * (i / n) + v * (j / n) for j in range(n + 1) for i in range(n + 1)]


def _quads(base, n):
    """vertex numbers (1-based) of the n x n cells of a grid starting at base"""
    for j in range(n):
        for i in range(n):
            a = base + j * (n + 1) + i
            yield a, a + 1, a + n + 2, a + n + 1


def write_scene_assets():
    """The OBJ meshes and BMP textures that the scene files in scene_files/
    name: a room whose walls are quads and triangles, a cube whose faces use
    every face form of the OBJ reader (v, v/vt, v//vn, v/vt/vn; three and
    four vertices) with vertex normals, and two small textures."""
    out = ["# walls of a room: quads (floor, ceiling) and triangles (back, left, right)"]
    walls = [((0, 0, 170), (100, 0, 0), (0, 0, -170), "q"), ((0, 81.6, 0), (100, 0, 0), (0, 0, 170), "q"),
             ((0, 0, 0), (100, 0, 0), (0, 81.6, 0), "t"), ((0, 0, 170), (0, 0, -170), (0, 81.6, 0), "t"),
             ((100, 0, 0), (0, 0, 170), (0, 81.6, 0), "t")]
    n, faces, nv = 4, [], 0
    for o, u, v, kind in walls:
        for p in _grid(o, u, v, n):
            out.append("v %.6g %.6g %.6g" % tuple(p))
        for a, b, c, d in _quads(nv + 1, n):
            faces += [f"f {a} {b} {c} {d}"] if kind == "q" else [f"f {a} {b} {c}", f"f {c} {d} {a}"]
        nv += (n + 1) ** 2
    with open(os.path.join(SCENE_DIR, "room.obj"), "w", newline="\n") as fh:
        fh.write("\n".join(out + faces) + "\n")
    # a cube [-1, 1]^3; vn 1 is the normal that the faces without normal
    # numbers fall back on (outward for +z, inward for -z), vn 2..7 the
    # outward normals
    out = ["# a cube written with every face form", "vt 0 0", "vn 0 0 1"]
    sides = [((1, -1, 1), (0, 0, -2), (0, 2, 0), (1, 0, 0), "vn4"), ((-1, -1, -1), (0, 0, 2), (0, 2, 0), (-1, 0, 0), "vn4"),
             ((-1, 1, 1), (2, 0, 0), (0, 0, -2), (0, 1, 0), "vtn4"), ((-1, -1, -1), (2, 0, 0), (0, 0, 2), (0, -1, 0), "vtn3"),
             ((-1, -1, 1), (2, 0, 0), (0, 2, 0), (0, 0, 1), "vt4"), ((1, -1, -1), (-2, 0, 0), (0, 2, 0), (0, 0, -1), "v3")]
    n, faces, nv = 3, [], 0
    for k, (o, u, v, nrm, kind) in enumerate(sides):
        out.append("vn %g %g %g" % nrm)
        for p in _grid(o, u, v, n):
            out.append("v %.6g %.6g %.6g" % tuple(p))
        ni = k + 2
        for a, b, c, d in _quads(nv + 1, n):
            if kind == "vn4":
                faces.append(f"f {a}//{ni} {b}//{ni} {c}//{ni} {d}//{ni}")
            elif kind == "vtn4":
                faces.append(f"f {a}/1/{ni} {b}/1/{ni} {c}/1/{ni} {d}/1/{ni}")
            elif kind == "vtn3":
                faces += [f"f {a}/1/{ni} {b}/1/{ni} {c}/1/{ni}", f"f {c}/1/{ni} {d}/1/{ni} {a}/1/{ni}"]
            elif kind == "vt4":
                faces.append(f"f {a}/1 {b}/1 {c}/1 {d}/1")
            else:
                faces += [f"f {a} {b} {c}", f"f {c} {d} {a}"]
        nv += (n + 1) ** 2
    with open(os.path.join(SCENE_DIR, "cube_vn.obj"), "w", newline="\n") as fh:
        fh.write("\n".join(out + faces) + "\n")
    from prender_gb300.scene import write_bmp
    rng = np.random.default_rng(7)
    y, x = np.mgrid[0:16, 0:32]
    sky = np.stack([x * 8, y * 16, (x + y) * 5], axis=2) + rng.integers(0, 8, (16, 32, 3))
    write_bmp(os.path.join(SCENE_DIR, "sky.bmp"), np.clip(sky, 0, 255).astype(np.uint8))
    y, x = np.mgrid[0:32, 0:32]
    disk = np.stack([255 - x * 4, 128 + (y % 8) * 12, x * y // 5], axis=2) + rng.integers(0, 16, (32, 32, 3))
    write_bmp(os.path.join(SCENE_DIR, "disk.bmp"), np.clip(disk, 0, 255).astype(np.uint8))


def scene_files_golden(d):
    """One-thread renders by the reference of the scene files in
    scene_files/, read by the reference's own SceneEnv::Load (run from a
    copy of that folder, so the files they name resolve there)"""
    import shutil
    write_scene_assets()
    work = os.path.join(d, "scene_files")  # the reference writes dumps beside its working folder
    shutil.copytree(SCENE_DIR, work)
    out = {}
    for name in SCENE_FILES:
        path = os.path.join(work, name + ".txt")
        img_path = os.path.join(d, name + ".f64")
        info = run_ref(["render", path, img_path], work, 1).strip().splitlines()[-1]
        w, h = _image_size(path)
        out[name] = np.fromfile(img_path).reshape(h, w, 3)
        print("scene file", name, info)
    np.savez_compressed(os.path.join(HERE, "scene_files.npz"), **out)


def _image_size(path):
    lines = open(path).read().splitlines()
    w, h = lines[lines.index("IMAGE") + 1].split()
    return int(w), int(h)


KNOWN_FLAGS = {"--kerr-only", "--disk-only", "--sss-only", "--sss-l1-only", "--glossy-only", "--sss-oracle",
               "--sss-l1-oracle", "--disk-oracle", "--glossy-oracle", "--scene-files-only", "--media-only",
               "--media-oracle", "--mesh7-oracle", "--batch-only", "--batch-oracle", "--hdr-only",
               "--lights-only", "--lights-oracle", "--textures-only", "--textures-oracle", "--wormhole-only",
               "--wormhole-oracle", "--meshtex-only", "--meshtex-oracle",
               "--mlt-only", "--mlt-oracle"}


def main():
    bad = [a for a in sys.argv[1:] if a.startswith("--") and a not in KNOWN_FLAGS]
    if bad:
        sys.exit(f"unknown option(s) {bad}; known: {sorted(KNOWN_FLAGS)}")
    if "--media-oracle" in sys.argv:
        media_oracle_golden()
        return
    if "--lights-oracle" in sys.argv:
        lights_oracle_golden()
        return
    if "--textures-oracle" in sys.argv:
        textures_oracle_golden()
        return
    if "--wormhole-oracle" in sys.argv:
        wormhole_oracle_golden()
        return
    if "--meshtex-oracle" in sys.argv:
        meshtex_oracle_golden()
        return
    if "--mlt-oracle" in sys.argv:
        mlt_oracle_golden()
        return
    if "--mesh7-oracle" in sys.argv:
        mesh7_oracle_golden()
        return
    if "--batch-oracle" in sys.argv:
        batch_oracle_golden()
        return
    if "--sss-oracle" in sys.argv:
        sss_oracle_golden()
        return
    if "--sss-l1-oracle" in sys.argv:
        sss_oracle_golden(level=-1)
        return
    if "--glossy-oracle" in sys.argv:
        glossy_oracle_golden()
        return
    if "--disk-oracle" in sys.argv:
        disk_oracle_golden()
        return
    if not os.path.exists(REF_BIN):
        args = [a for a in sys.argv[1:] if not a.startswith("--")]
        ref = args[0] if args else "/root/reference"
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), ref], check=True)
    if "--scene-files-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            scene_files_golden(d)
        return
    if "--kerr-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            kerr_golden(d)
        return
    if "--media-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            media_golden(d)
        return
    if "--wormhole-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            wormhole_golden(d)
        return
    if "--meshtex-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            meshtex_golden(d)
        return
    if "--mlt-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            mlt_golden(d)
        return
    if "--textures-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            textures_golden(d)
        return
    if "--lights-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            lights_golden(d)
        return
    if "--hdr-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            hdr_golden(d)
        return
    if "--batch-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            batch_golden(d)
        return
    if "--disk-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            disk_golden(d)
        return
    if "--sss-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            sss_golden(d)
        return
    if "--glossy-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            glossy_golden(d)
        return
    if "--sss-l1-only" in sys.argv:
        with tempfile.TemporaryDirectory() as d:
            sss_l1_golden(d)
        return
    with tempfile.TemporaryDirectory() as d:
        kerr_golden(d)
        disk_golden(d)
        sss_golden(d)
        sss_l1_golden(d)
        glossy_golden(d)
        scene_files_golden(d)
        # -- QBVH structure + first hits on the subdiv-3 mesh Cornell box
        s = scenes.mesh_cornell(width=32, height=24, samples=1, supersamples=2, subdiv=3)
        p = s.write_reference(d)
        q0, q2 = ref_qbvh(p, 0, d), ref_qbvh(p, 2, d)
        rays = np.concatenate([scenes.random_rays((2, 1, 1), (98, 80, 249), 4096, seed=1), scenes.camera_rays(s)])
        fh = ref_firsthit(p, rays, d)
        np.savez_compressed(os.path.join(HERE, "mesh_s3_qbvh_firsthit.npz"), rays=rays,
                            **{f"box_{k}": v for k, v in q0.items()}, **{f"ico_{k}": v for k, v in q2.items()},
                            **{f"fh_{k}": v for k, v in fh.items()})
        # -- per-ray radiance() roots from one MT19937-64 stream
        cases = {
            "spheres": scenes.cornell_spheres(width=16, height=12, samples=1, supersamples=1),
            "mesh_diffuse": scenes.mesh_cornell(width=16, height=12, samples=1, supersamples=1, subdiv=3),
            "mesh_glass": scenes.mesh_cornell(width=16, height=12, samples=1, supersamples=1, subdiv=3,
                                              material="glass"),
            "media_g05": scenes.media_cornell(width=16, height=12, samples=1, supersamples=1, g=0.5),
        }
        rad = {}
        for name, sc in cases.items():
            dd = os.path.join(d, name)
            os.makedirs(dd)
            pp = sc.write_reference(dd)
            r = scenes.camera_rays(sc)
            rad[f"{name}_rays"] = r
            rad[f"{name}_rgb"] = ref_radiance(pp, r, 7, dd)
        np.savez_compressed(os.path.join(HERE, "radiance_roots.npz"), **rad)
        # -- whole Render::Run images, one thread (bit-exact) -----------
        imgs = {}
        for name, sc in {
            "spheres": scenes.cornell_spheres(width=24, height=18, samples=2, supersamples=2),
            "mesh_nee": scenes.mesh_cornell(width=24, height=18, samples=1, supersamples=2, subdiv=3),
            "media_g05": scenes.media_cornell(width=16, height=12, samples=1, supersamples=2, g=0.5),
        }.items():
            dd = os.path.join(d, "r_" + name)
            os.makedirs(dd)
            pp = sc.write_reference(dd)
            img, info = ref_render(pp, (sc.camera.width, sc.camera.height), dd, threads=1)
            imgs[name] = img
            print(name, info)
        np.savez_compressed(os.path.join(HERE, "render_1thread.npz"), **imgs)
        # -- high-spp reference images for statistical image parity ------
        hi = {}
        for name, sc in {
            "spheres_64x48_1024spp": scenes.cornell_spheres(width=64, height=48, samples=256, supersamples=2),
            "mesh_64x48_512spp": scenes.mesh_cornell(width=64, height=48, samples=128, supersamples=2, subdiv=3),
            "glass_64x48_512spp": scenes.mesh_cornell(width=64, height=48, samples=128, supersamples=2, subdiv=3,
                                                      material="glass"),
        }.items():
            dd = os.path.join(d, "h_" + name)
            os.makedirs(dd)
            pp = sc.write_reference(dd, threads=os.cpu_count())
            img, info = ref_render(pp, (sc.camera.width, sc.camera.height), dd, threads=os.cpu_count())
            hi[name] = img.astype(np.float32)
            print(name, info)
        np.savez_compressed(os.path.join(HERE, "render_highspp.npz"), **hi)


if __name__ == "__main__":
    main()
