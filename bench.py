"""Benchmark: Mpaths/s of the radiance estimator on the triangle-mesh Cornell
box (1024x768, 64 spp tent-filtered, NEE, 327,680-triangle displaced
icosphere) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
                    [--mode megakernel] [--small]

A step is one full frame (W*H*spp camera paths).  Under torchrun (N>1) each
rank renders its own disjoint sample range of the same frame (weak scaling,
no collective on the data path); value = all ranks' paths / max-over-ranks
time.  Rank 0 prints one JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpaths/s on 1 GB300 at matched RMSE, wavefront vs plain; adjoint/forward cost"
# bytes a traversal reads per node visit / triangle test / ray (see the roofline below)
B_NODE, B_TRI, B_RAY = 80.0, 48.0, 64.0


def baseline_metric():
    try:
        with open(os.path.join(ROOT, "BASELINE.json")) as f:
            return json.load(f).get("metric", METRIC)
    except OSError:
        return METRIC


def workload(small: bool, profile: bool = False):
    from prender_gb300 import scenes
    if profile:
        s = scenes.mesh_cornell(width=512, height=384, samples=4, supersamples=2, subdiv=7)
        name = "mesh_cornell_512x384_16spp_subdiv7"
    elif small:
        s = scenes.mesh_cornell(width=256, height=192, samples=4, supersamples=2, subdiv=5)
        name = "mesh_cornell_256x192_16spp_subdiv5"
    else:
        s = scenes.mesh_cornell(width=1024, height=768, samples=16, supersamples=2, subdiv=7)
        name = "mesh_cornell_1024x768_64spp_subdiv7"
    return s, name


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return

        def rd():
            for line in self.proc.stdout:
                self.rows.append([x.strip() for x in line.split(",")])

        self.thread = threading.Thread(target=rd, daemon=True)
        self.thread.start()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def sample_rows(height: int, rows: int):
    """rows image rows spread evenly over the frame (every k-th row, the
    first at k / 2), so the CPU sample sees walls, floor, light and mesh in
    the frame's own proportions"""
    rows = max(1, min(rows, height))
    step = height / rows
    return [int(step * i + step / 2) for i in range(rows)]


def cpu_baseline(scene, rows: int, threads: int):
    """The oracle port on the host cores over a bounded sample of rows spread
    over the whole frame."""
    from oracle import oracle as O
    o = O.OracleScene(scene)
    rl = sample_rows(scene.camera.height, rows)
    t0 = time.perf_counter()
    _, secs, _ = o.render_rows(rl, threads=threads)
    wall = time.perf_counter() - t0
    paths = len(rl) * scene.camera.width * scene.settings.spp
    return paths / secs / 1e6, secs, wall, paths


def sample_desc(scene, rows: int) -> str:
    H = scene.camera.height
    rl = sample_rows(H, rows)
    return (f"{len(rl)} rows spread over the frame (every {H / len(rl):g}th row of {H}) x "
            f"{scene.camera.width} px x {scene.settings.spp} spp")


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    scene, name = workload(args.small)
    threads = os.cpu_count() or 1
    rows = max(1, int(args.ref_rows))
    vals = []
    for i in range(args.warmup + args.steps):
        v, secs, _, paths = cpu_baseline(scene, rows, threads)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    sample = sample_desc(scene, rows) + " per step"
    line = {
        "impl": "reference", "metric": baseline_metric(), "value": round(value, 4), "unit": "Mpaths/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * rows * scene.camera.width * scene.settings.spp / (value * 1e6), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": name, "sample": sample},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mpaths/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__ as g
    g.build_library()
    from prender_gb300 import gpu
    scene, name = workload(args.small, args.profile)
    W, H, spp = scene.camera.width, scene.camera.height, scene.settings.spp
    ctx = gpu.Context(local)
    t0 = time.perf_counter()
    ctx.upload(scene)
    upload_s = time.perf_counter() - t0
    import ctypes as C
    from prender_gb300 import _abi as A
    scene.settings.mode = A.PR_MODE_WAVEFRONT if args.mode == "wavefront" else A.PR_MODE_MEGAKERNEL
    cam, prm = scene.camera.to_c(), scene.settings.to_c()
    out = torch.empty((H, W, 3), dtype=torch.float32, device=f"cuda:{local}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")  # > L2 (129 MB)
    L = ctx.L

    def step(i):
        off = (rank + ws * i) * spp  # disjoint sample ranges per rank and step
        rc = L.pr_render_dev(ctx.h, C.byref(cam), C.byref(prm), C.c_void_p(out.data_ptr()), off, 0)
        if rc != 0:
            raise RuntimeError(L.pr_last_error(ctx.h).decode())
        return ctx.stats()

    def timed(nsteps, first):
        walls, kern, st = [], [], None
        for i in range(nsteps):
            flush.zero_()
            torch.cuda.synchronize()
            if dist:
                dist.barrier()
            t0 = time.perf_counter()
            st = step(first + i)
            torch.cuda.synchronize()
            walls.append(time.perf_counter() - t0)
            kern.append(st["device_ms"] / 1e3)
        return walls, kern, st

    tuned = None
    if args.autotune and args.mode == "wavefront":
        tuned = ctx.autotune(scene)  # pool size and traversal grid for this scene, kept by the context
    for i in range(args.warmup):
        step(i)
    clk = ClockSampler(local)
    clk.start()
    walls, kern, st = timed(args.steps, args.warmup)
    clocks = clk.stop()
    ms = 1e3 * statistics.mean(walls)
    kern_s = statistics.mean(kern)
    # the other form on the same frames, for the wavefront-vs-plain ratio
    other = None
    if not args.single_mode:
        prm_main = prm
        prm = scene.settings.to_c()
        prm.mode = A.PR_MODE_MEGAKERNEL if prm_main.mode == A.PR_MODE_WAVEFRONT else A.PR_MODE_WAVEFRONT
        for i in range(1):
            step(i)
        w2, k2, st2 = timed(max(1, min(args.steps, 3)), args.warmup)
        other = {"mode": "megakernel" if prm.mode == A.PR_MODE_MEGAKERNEL else "wavefront",
                 "mpaths_per_s": round(W * H * spp / statistics.mean(w2) / 1e6, 3),
                 "ms_per_step": round(1e3 * statistics.mean(w2), 3), "segments_per_step": st2["segments"]}
        prm = prm_main
    if dist:
        t = torch.tensor([ms, kern_s], device=f"cuda:{local}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, kern_s = float(t[0]), float(t[1])
    paths = W * H * spp
    value = ws * paths / (ms / 1e3) / 1e6

    # e2e through the C ABI with a host image buffer (camera + parameters in,
    # image out, copies inside the timed region)
    host = np.empty((H, W, 3), np.float32)
    e2e = []
    for i in range(max(2, min(args.steps, 4))):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.render(scene, sample_offset=(rank + ws * (1000 + i)) * spp, accumulate=None)
        e2e.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * statistics.mean(e2e)
    if dist:
        t = torch.tensor([e2e_ms], device=f"cuda:{local}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t[0])
    e2e_val = ws * paths / (e2e_ms / 1e3) / 1e6
    del host

    # per-kernel split of one more frame: the host-driven loop times every
    # launch with CUDA events on the render stream (same kernels and work)
    kernel_ms = None
    if args.mode == "wavefront":
        os.environ["PR_WF_HOST_LOOP"] = "1"
        try:
            step(args.warmup + args.steps)
            torch.cuda.synchronize()
            kms = (C.c_double * 4)()
            shc = (C.c_ulonglong * 3)()
            L.pr_last_kernel_times(ctx.h, kms, shc, 4)
            st_split = ctx.stats()
            kernel_ms = {"shade": kms[0], "extend": kms[1], "shadow": kms[2], "control": kms[3],
                         "iterations": None, "shadow_rays": shc[0], "shadow_nodes": shc[1], "shadow_tris": shc[2],
                         "segments": st_split["segments"], "nodes": st_split["nodes_visited"],
                         "tris": st_split["tri_tests"]}
        finally:
            del os.environ["PR_WF_HOST_LOOP"]

    # the same frame with the glass icosphere (the workload names diffuse and
    # glass), both forms, after the headline measurement
    glass = None
    if not args.small and not args.profile and not args.no_glass:
        from prender_gb300 import scenes as SC
        gs = SC.mesh_cornell(width=W, height=H, samples=16, supersamples=2, subdiv=7, material="glass")
        ctx.upload(gs)
        glass = {}
        for mname, mval in (("wavefront", A.PR_MODE_WAVEFRONT), ("megakernel", A.PR_MODE_MEGAKERNEL)):
            gp = gs.settings.to_c()
            gp.mode = mval
            gcam = gs.camera.to_c()
            ts = []
            for i in range(3 if mval == A.PR_MODE_WAVEFRONT else 2):
                flush.zero_()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                rc = L.pr_render_dev(ctx.h, C.byref(gcam), C.byref(gp), C.c_void_p(out.data_ptr()),
                                     (rank + ws * (2000 + i)) * spp, 0)
                torch.cuda.synchronize()
                if rc != 0:
                    raise RuntimeError(L.pr_last_error(ctx.h).decode())
                ts.append(time.perf_counter() - t0)
            gst = ctx.stats()
            t = statistics.mean(ts[1:])  # the first frame builds the glass scene's pool and graph
            glass[mname] = {"mpaths_per_s": round(paths / t / 1e6, 3), "ms_per_step": round(1e3 * t, 3),
                            "segments_per_step": int(gst["segments"])}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    # roofline of the dominant kernel: algorithmic bytes of its traversal,
    # B = 80 N_node + 48 N_tri + 64 per ray (one 80-byte compressed 8-wide
    # node per visit, three 16-byte vertex records per triangle test, ray
    # record in and hit record out), N_node and N_tri counted by the kernel
    # itself on this frame, over its own device time
    segs = st["segments"]
    peak, peak_kind = measured_peak_hbm()
    if kernel_ms:
        dom = max(("extend", "shadow"), key=lambda k: kernel_ms[k])  # the traversal kernels (wf_shade: path state)
        if dom == "shadow":
            nodes, tris, rays = kernel_ms["shadow_nodes"], kernel_ms["shadow_tris"], kernel_ms["shadow_rays"]
        else:
            nodes = kernel_ms["nodes"] - kernel_ms["shadow_nodes"]
            tris = kernel_ms["tris"] - kernel_ms["shadow_tris"]
            rays = kernel_ms["segments"] - kernel_ms["shadow_rays"]
        alg_bytes = B_NODE * nodes + B_TRI * tris + B_RAY * rays
        achieved = alg_bytes / (kernel_ms[dom] / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": f"wf_{dom}", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": None, "peak_kind": peak_kind,
                "kernel_share": round(kernel_ms[dom] / sum(kernel_ms[k] for k in ("shade", "extend", "shadow",
                                                                                   "control")), 4),
                "kernel_ms_per_frame": {k: round(kernel_ms[k], 3) for k in ("shade", "extend", "shadow", "control")},
                "kernel_rays_per_frame": int(rays), "kernel_nodes_per_frame": int(nodes),
                "kernel_tris_per_frame": int(tris),
                "note": "algorithmic traversal bytes of the dominant kernel (80 B per wide-node visit, 48 B per "
                        "triangle test, 64 B per ray) over its CUDA-event time; the scene (~26 MB) is "
                        "L2-resident, so DRAM traffic is far below these bytes"}
        prof = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(prof):
            try:
                with open(prof) as f:
                    tr = json.load(f).get(f"wf_{dom}")
                if tr and rays:
                    # DRAM bytes per ray from an ncu capture of the same kernel, times this frame's rays per launch
                    iters = max(1, int(st_split.get("kernel_launches", 4) // 4))
                    roof["traffic"] = round(tr["dram_bytes_per_ray"] * rays / iters, 1)
                    roof["traffic_source"] = tr.get("source")
            except (OSError, ValueError, KeyError):
                pass
    else:
        alg_bytes = B_NODE * st["nodes_visited"] + B_TRI * st["tri_tests"] + B_RAY * segs + 12.0 * st["paths"]
        achieved = alg_bytes / (st["device_ms"] / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": "pt_megakernel", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": None, "peak_kind": peak_kind,
                "note": "algorithmic traversal bytes of the frame; scene (~28 MB) is L2-resident"}
    adjoint = None
    if not args.no_adjoint:
        adjoint = adjoint_cost(ctx, local, args.small)
    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        threads = os.cpu_count() or 1
        rows = max(1, int(args.ref_rows))
        v, secs, wall, npaths = cpu_baseline(scene, rows, threads)
        cpu = {"value": round(v, 4), "unit": "Mpaths/s", "cores": threads, "kind": "port",
               "sample": sample_desc(scene, rows) + f" ({npaths} paths, {secs:.1f} s)"}
    line = {
        "metric": baseline_metric(), "value": round(value, 3), "unit": "Mpaths/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": name, "width": W, "height": H, "spp": spp, "triangles": int(scene.meshes[1].faces.shape[0]),
                   "nee": 1, "mode": args.mode, "other_form": other, "l2": "flushed between steps (256 MB write)",
                   "paths_per_step": paths, "segments_per_step": segs, "kernel_ms_per_step": round(kern_s * 1e3, 3),
                   "scene_upload_s": round(upload_s, 3), "autotuned": tuned, "glass_icosphere": glass},
        "e2e": {"value": round(e2e_val, 3), "unit": "Mpaths/s",
                "h2d_bytes_per_step": C.sizeof(cam) + C.sizeof(prm), "d2h_bytes_per_step": W * H * 3 * 4},
        "gpu_launches": int(st["kernel_launches"]) * args.steps,
        "roofline": roof,
        "adjoint": adjoint,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


def adjoint_cost(ctx, device: int, small: bool, reps: int = 3):
    """The metric's second half on the differentiable-render workload: mesh
    Cornell box 512^2, 64 spp (16 x 2^2 tent-filtered), eight Lambertian
    materials with RGB albedo U(0.1, 0.9) plus the light's emission scale as
    parameters; L2 loss to a target rendered at parameters perturbed by
    N(0, 0.1^2).  Device time of one forward frame (plain form, which the
    adjoint replays, and the wavefront form) against one path-replay adjoint
    pass through pr_render_adjoint_dev."""
    import ctypes as C
    import torch
    from prender_gb300 import _abi as A
    from prender_gb300 import scenes
    side = 128 if small else 512
    s = scenes.diff_cornell(side, side, samples=16, supersamples=2, subdiv=5, seed=0)
    alb = np.random.default_rng(0).uniform(0.1, 0.9, (8, 3))  # diff_cornell's own draw for seed 0
    pert = np.random.default_rng(1)
    tgt = scenes.diff_cornell(side, side, samples=16, supersamples=2, subdiv=5, seed=0,
                              albedo=np.clip(alb + pert.normal(0.0, 0.1, alb.shape), 0.0, 1.0),
                              emission_scale=1.0 + float(pert.normal(0.0, 0.1)))
    dev = f"cuda:{device}"
    L = ctx.L
    target = torch.empty((side, side, 3), dtype=torch.float32, device=dev)
    img = torch.empty_like(target)
    cam = s.camera.to_c()

    def render(out, mode, off=0):
        prm = s.settings.to_c()
        prm.mode = mode
        rc = L.pr_render_dev(ctx.h, C.byref(cam), C.byref(prm), C.c_void_p(out.data_ptr()), off, 0)
        if rc != 0:
            raise RuntimeError(L.pr_last_error(ctx.h).decode())
        return ctx.stats()["device_ms"]

    ctx.upload(tgt)
    render(target, A.PR_MODE_MEGAKERNEL, off=1 << 20)
    ctx.upload(s)
    fwd = [render(img, A.PR_MODE_MEGAKERNEL) for _ in range(reps + 1)][1:]
    fwd_wf = [render(img, A.PR_MODE_WAVEFRONT) for _ in range(reps + 1)][1:]
    render(img, A.PR_MODE_MEGAKERNEL)
    dl = (2.0 * (img - target)).contiguous()
    n_mat = len(s.materials)
    d_color = torch.zeros((n_mat, 3), dtype=torch.float64, device=dev)
    d_em = torch.zeros((n_mat, 3), dtype=torch.float64, device=dev)
    prm = s.settings.to_c()
    adj = []
    for _ in range(reps + 1):
        rc = L.pr_render_adjoint_dev(ctx.h, C.byref(cam), C.byref(prm), C.c_void_p(dl.data_ptr()), 0,
                                     C.c_void_p(d_color.data_ptr()), C.c_void_p(d_em.data_ptr()))
        if rc != 0:
            raise RuntimeError(L.pr_last_error(ctx.h).decode())
        adj.append(ctx.stats()["device_ms"])
    adj = adj[1:]
    f, fw, a = statistics.median(fwd), statistics.median(fwd_wf), statistics.median(adj)
    loss = float(((img - target) ** 2).sum())
    return {"workload": f"diff_cornell_{side}x{side}_64spp_8materials_subdiv5", "paths": side * side * 64,
            "forward_ms": round(f, 3), "forward_wavefront_ms": round(fw, 3), "adjoint_ms": round(a, 3),
            "ratio": round(a / f, 3), "ratio_vs_wavefront": round(a / fw, 3), "loss": loss,
            "grad_norm": float(torch.linalg.norm(d_color).item()),
            "note": "device time per pass (CUDA events on the render stream), median of "
                    f"{reps}; ratio = adjoint / forward of the plain form the adjoint replays"}


def kerr_jobs(n_jobs: int, width: int, height: int, precision: int):
    """The Kerr lensing workload: n_jobs scenes alternating spin 0.6 / 0.999,
    each seen from its own azimuth around the hole (camera at Boyer-Lindquist
    r = 6.03 M in the disk plane, 60 degree field), textured accretion disk
    r 3..15 M with Doppler shading, procedural celestial sphere."""
    import math
    from prender_gb300 import scenes
    from prender_gb300.scene import Camera
    out = []
    for j in range(n_jobs):
        a = 0.6 if j % 2 == 0 else 0.999
        s = scenes.kerr_accretion(a=a, width=width, height=height, max_steps=4000, precision=precision)
        ph = 2.0 * math.pi * (j // 2) / max(1, n_jobs // 2)
        d = math.sqrt(6.03 * 6.03 + a * a)
        s.camera = Camera(position=(round(d * math.sin(ph), 12), round(-d * math.cos(ph), 12), 0.0),
                          dir=(round(-math.sin(ph), 12), round(math.cos(ph), 12), 0.0), up=(0.0, 0.0, 1.0),
                          width=width, height=height, angle=60.0)
        out.append(s)
    return out


def run_kerr(args):
    """Kerr lensing renders: one step = n_jobs cameras / spins of 2048 x 1024
    rays, one sample each, as one pr_render_batch launch (the mixed-precision
    form); the reference-arithmetic FP64 form is timed on one job beside it."""
    import torch
    import __graft_entry__ as g
    g.build_library()
    from prender_gb300 import gpu
    from prender_gb300 import _abi as A
    W, H = (512, 256) if args.small else (2048, 1024)
    n_jobs = args.kerr_jobs
    torch.cuda.set_device(0)
    ctx = gpu.Context(0)
    jobs_s = kerr_jobs(n_jobs, W, H, A.PR_KERR_FP32)
    objs = [ctx.scene_object(s) for s in jobs_s]
    outs = [torch.empty((H, W, 3), dtype=torch.float32, device="cuda:0") for _ in range(n_jobs)]

    def step(i):
        ctx.render_batch([(objs[j], outs[j], None, None, i) for j in range(n_jobs)])
        return ctx.stats()

    for i in range(args.warmup):
        step(i)
    clk = ClockSampler(0)
    clk.start()
    walls, dev, st = [], [], None
    for i in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = step(args.warmup + i)
        torch.cuda.synchronize()
        walls.append(time.perf_counter() - t0)
        dev.append(st["device_ms"])
    clocks = clk.stop()
    paths = n_jobs * W * H
    ms = 1e3 * statistics.mean(walls)
    value = paths / (ms / 1e3) / 1e6
    # the FP64 form (the reference's arithmetic in its order) on job 1 (a = 0.999) and job 0 (a = 0.6)
    fp64 = {}
    for j in (0, 1):
        s = kerr_jobs(2, W, H, A.PR_KERR_FP64)[j]
        ctx.upload(s)
        ctx.render(s)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.render(s)
        wall = time.perf_counter() - t0
        st64 = ctx.stats()
        fp64[f"a{s.kerr['a']}"] = {"mpaths_per_s": round(W * H / wall / 1e6, 4), "ms": round(1e3 * wall, 1),
                                  "rk_attempts": int(st64["tri_tests"]), "device_ms": round(st64["device_ms"], 1)}
    # FP64 form roofline: about 630 flops per RK45 attempt (Cash-Karp step
    # with five geodesic evaluations), against GB300's FP64 pipe
    # (2 DFMA / clock / SM x 152 SMs x 2.07 GHz x 2 flops = 1.26 TFLOP/s)
    f = fp64["a0.999"]
    achieved = 630.0 * f["rk_attempts"] / (f["device_ms"] / 1e3) / 1e12
    line = {
        "metric": "Mpaths/s, Kerr geodesic renders", "value": round(value, 4), "unit": "Mpaths/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"kerr_lensing_{W}x{H}_x{n_jobs}_accretion_disk", "jobs_per_launch": n_jobs,
                   "spins": [0.6, 0.999], "max_steps": 4000, "precision": "mixed (PR_KERR_FP32)",
                   "rk_attempts_per_step": int(st["tri_tests"]), "steps_accepted_per_step": int(st["nodes_visited"]),
                   "fp64_form_one_job": fp64},
        "roofline": {"bound": "fp64", "kernel": "kerr_render_kernel (FP64 form, a = 0.999)",
                     "achieved": round(achieved, 4), "peak": 1.26, "unit": "TFLOP/s",
                     "frac": round(achieved / 1.26, 4), "peak_kind": "nominal FP64 pipe",
                     "note": "630 flops per RK45 attempt"},
        "clocks": clocks,
    }
    print(json.dumps(line))
    for o in objs:
        o.release()
    ctx.close()
    return 0


def run_curved_or_mlt(args):
    """Two non-headline workloads, one JSON line each:
    mlt: Metropolis light transport (PR_MODE_MLT) of the sphere Cornell box,
    256 x 192, 16 x W H x 16 mutations and 16 x W H x 0.4 bootstrap paths
    per step; Mpaths/s counts proposals and bootstrap paths; the CPU baseline
    is the oracle's RunMLT (the reference's sequential chains) on one thread.
    wormhole: a wormhole render (objects on both sides), 512 x 384, 4 tent
    samples per pixel, geodesics of up to 300 FP64 Cash-Karp steps each."""
    import torch
    import __graft_entry__ as g
    g.build_library()
    from prender_gb300 import gpu, scenes
    from prender_gb300 import _abi as A
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    torch.cuda.set_device(0)
    ctx = gpu.Context(0)
    if args.workload == "mlt":
        s = scenes.cornell_spheres(width=256, height=192, samples=16, supersamples=1)
        s.settings.mode = A.PR_MODE_MLT
        s.settings.mutation, s.settings.pre_sample, s.settings.nee = 16.0, 0.4, 1
        name = "cornell_spheres_256x192_mlt_16x16_mutations_per_pixel"
    else:
        import wormhole_cases
        s = wormhole_cases.build("worm_objects", 512, 384, 1, 2, max_steps=300)
        name = "wormhole_objects_512x384_4spp_300_steps"
    ctx.upload(s)
    for i in range(args.warmup):
        ctx.render(s, sample_offset=i)
    clk = ClockSampler(0)
    clk.start()
    walls, paths, launches = [], 0, 0
    for i in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.render(s, sample_offset=args.warmup + i)
        torch.cuda.synchronize()
        walls.append(time.perf_counter() - t0)
        st = ctx.stats()
        paths, launches = st["paths"], st["kernel_launches"]
    clocks = clk.stop()
    ms = 1e3 * statistics.mean(walls)
    cpu = None
    if args.workload == "mlt":
        from oracle import oracle as O
        O.build()
        small = scenes.cornell_spheres(width=64, height=48, samples=2, supersamples=1)
        small.settings.mode = A.PR_MODE_MLT
        small.settings.mutation, small.settings.pre_sample, small.settings.nee = 16.0, 0.4, 1
        t0 = time.perf_counter()
        O.OracleScene(small).render_mlt()
        wall = time.perf_counter() - t0
        n = 2 * int(64 * 48 * 16) + 2 * int(64 * 48 * 0.4)
        cpu = {"value": round(n / wall / 1e6, 5), "unit": "Mpaths/s", "cores": 1, "kind": "port",
               "sample": "oracle RunMLT, 64 x 48, 2 chains x (1228 seeds + 49152 mutations), one thread"}
    line = {
        "metric": "Mpaths/s, " + ("Metropolis light transport" if args.workload == "mlt" else "wormhole geodesic renders"),
        "value": round(paths / (ms / 1e3) / 1e6, 4), "unit": "Mpaths/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if args.workload == "mlt" else "f64", "data": "synthetic",
        "config": {"workload": name, "paths_per_step": int(paths), "gpu_launches": int(launches)},
        "cpu_baseline": cpu, "clocks": clocks,
    }
    print(json.dumps(line))
    ctx.close()
    return 0


def run_batch(args):
    """The media + BSSRDF batch: 32 Cornell variants (global HG medium with
    sigma_s U(0.05, 0.5), sigma_a 0.01, g U(-0.6, 0.8); a 20,480-triangle
    directional-dipole icosphere) at uneven square sizes 128^2 .. 1024^2,
    64 spp, all 32 jobs in one pr_render_batch call per step, in the form
    --mode names (wavefront: jobs one after another on the shared pool;
    megakernel: one captured graph)."""
    import torch
    import __graft_entry__ as g
    g.build_library()
    from prender_gb300 import gpu, scenes
    torch.cuda.set_device(0)
    ctx = gpu.Context(0)
    n = 8 if args.small else 32
    sizes = (32, 64, 96, 128, 192, 256) if args.small else (128, 256, 384, 512, 768, 1024)
    jobs_s = scenes.media_batch(n=n, seed=0, sizes=sizes)
    from prender_gb300 import _abi as A
    form = A.PR_MODE_WAVEFRONT if args.mode == "wavefront" else A.PR_MODE_MEGAKERNEL
    for s in jobs_s:
        s.settings.mode = form
    t0 = time.perf_counter()
    objs = [ctx.scene_object(s) for s in jobs_s]
    upload_s = time.perf_counter() - t0
    outs = [torch.empty((s.camera.height, s.camera.width, 3), dtype=torch.float32, device="cuda:0") for s in jobs_s]
    paths = sum(s.camera.width * s.camera.height * s.settings.spp for s in jobs_s)

    def step(i):
        ctx.render_batch([(objs[j], outs[j], None, None, i * jobs_s[j].settings.spp) for j in range(n)])
        return ctx.stats()

    tuned = None
    if form == A.PR_MODE_WAVEFRONT and args.autotune:
        ctx.upload(jobs_s[0])
        tuned = ctx.autotune(jobs_s[0])  # the pool for these scenes (kept by the context)
    for i in range(args.warmup):
        step(i)
    clk = ClockSampler(0)
    clk.start()
    walls, dev, st = [], [], None
    for i in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = step(args.warmup + i)
        torch.cuda.synchronize()
        walls.append(time.perf_counter() - t0)
        dev.append(st["device_ms"])
    clocks = clk.stop()
    ms = 1e3 * statistics.mean(walls)
    line = {
        "metric": "Mpaths/s, media + BSSRDF batch (32 jobs per call)", "value": round(paths / (ms / 1e3) / 1e6, 4),
        "unit": "Mpaths/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"media_bssrdf_batch_{n}_jobs", "jobs": n,
                   "sizes": [s.camera.width for s in jobs_s], "spp": jobs_s[0].settings.spp,
                   "paths_per_step": paths, "segments_per_step": int(st["segments"]),
                   "kernel_launches_per_step": int(st["kernel_launches"]), "scene_upload_s": round(upload_s, 3),
                   "form": "wavefront (jobs one after another on the shared path pool)" if form == A.PR_MODE_WAVEFRONT
                   else "plain (all jobs in one captured graph)", "autotuned": tuned},
        "clocks": clocks,
    }
    print(json.dumps(line))
    for o in objs:
        o.release()
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--mode", default="wavefront", choices=["wavefront", "megakernel"])
    ap.add_argument("--single-mode", action="store_true", help="do not also time the other render form")
    ap.add_argument("--small", action="store_true")
    ap.add_argument("--profile", action="store_true", help="full scene, 256x192x16spp image (ncu captures)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint/forward cost measurement")
    ap.add_argument("--no-glass", action="store_true", help="skip the glass-icosphere frames")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default wavefront pool size and traversal grid")
    ap.add_argument("--ref-rows", type=int, default=48)
    ap.add_argument("--workload", default="mesh", choices=["mesh", "kerr", "batch", "mlt", "wormhole"],
                    help="kerr: the Kerr lensing renders; batch: the media + BSSRDF batch; mlt: Metropolis light "
                         "transport; wormhole: wormhole renders (none of them the headline workload)")
    ap.add_argument("--kerr-jobs", type=int, default=16)
    args = ap.parse_args()
    if args.workload == "kerr":
        return run_kerr(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload in ("mlt", "wormhole"):
        return run_curved_or_mlt(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
