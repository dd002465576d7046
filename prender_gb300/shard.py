"""Multi-GPU sharding of one frame by sample range.

The reference splits a frame by image rows across MPI ranks and gathers the
rows (render.h:1181-1198, :1411-1449).  Here each rank renders every pixel
for its own range of camera samples -- rank r of W takes samples
[r * spp, (r + 1) * spp) of a frame of W * spp -- with `total_spp` set to the
whole frame so each sample keeps the frame's weight (the luminance clamp
depends on it, render.h:1375).  The counter-based streams make the union of
the shards the same samples a single GPU would render; the one exchange is a
sum of the float images (an all-reduce; gloo on CPU, NCCL on GPUs).
"""
from __future__ import annotations

from typing import Callable

import numpy as np


def shard(rank: int, world: int, spp: int):
    """(sample_offset, total_spp) of rank's shard of a frame of world * spp samples.

    spp counts camera samples per pixel as the renderer draws them:
    samples * supersamples^2 of pr_render_params (Render::Run folds the
    supersampling grid and the tent filter into the sample count,
    render.h:1133-1138) -- not the 'samples' field alone.  shard_settings()
    derives it from the render parameters."""
    if not (0 <= rank < world) or spp <= 0:
        raise ValueError("bad shard")
    return rank * spp, world * spp


def shard_settings(rank: int, world: int, settings):
    """(sample_offset, total_spp) of rank's shard when every rank renders with
    these RenderSettings (its samples * supersamples^2 camera samples per pixel)."""
    return shard(rank, world, settings.samples * settings.supersamples * settings.supersamples)


def render_sharded(render: Callable[[int, int], np.ndarray], spp: int, group=None) -> np.ndarray:
    """Renders this rank's shard with render(sample_offset, total_spp) and sums
    the images over the process group; every rank returns the frame."""
    import torch
    import torch.distributed as dist
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    off, total = shard(rank, world, spp)
    img = np.ascontiguousarray(render(off, total), dtype=np.float32)
    if world == 1:
        return img
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.from_numpy(img).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()
