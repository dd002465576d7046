"""The multi-GPU path's host logic on CPU: two gloo ranks each render their
sample range of a frame and all-reduce the images; the result equals one
process rendering all samples.  The per-sample renderer here is a CPU
stand-in with the GPU path's contract (each camera sample a deterministic
function of its index, weighted 1 / total_spp)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from prender_gb300 import shard


def _samples(offset, count, total, shape=(6, 8, 3)):
    out = np.zeros(shape, np.float64)
    for k in range(offset, offset + count):
        rng = np.random.default_rng(1000 + k)  # sample k of every pixel
        out += rng.random(shape) / total
    return out.astype(np.float32)


def _worker(rank, world, port, spp, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        img = shard.render_sharded(lambda off, total: _samples(off, spp, total), spp)
        q.put((rank, img))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_ranges():
    assert shard.shard(0, 2, 16) == (0, 32)
    assert shard.shard(1, 2, 16) == (16, 32)
    with pytest.raises(ValueError):
        shard.shard(2, 2, 16)
    # samples 4 on a 2x2 supersampling grid are 16 camera samples per pixel
    from prender_gb300.scene import RenderSettings
    st = RenderSettings(samples=4, supersamples=2)
    assert shard.shard_settings(1, 2, st) == (16, 32)


def test_two_gloo_ranks_equal_one_process():
    spp, world = 8, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, spp, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    full = _samples(0, world * spp, world * spp)
    for r in range(world):
        np.testing.assert_allclose(got[r], full, rtol=1e-5, atol=1e-6)
