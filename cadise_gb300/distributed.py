"""Multi-GPU rendering of one frame: one process per GPU.

Path samples are independent and keyed by (seed, scene, pixel, sample), so
rank r of R renders the sample indices `sample_range(spp, r, R)` into its
own FP64 film with no communication; the only exchange is one sum of the
films when a single image is wanted (`merge_films`, an all-reduce over
torch.distributed - NCCL on GPUs, gloo on CPUs).  Because every sample index
is rendered exactly once by exactly one rank, the merged film equals the
single-GPU film of all samples up to the order of the FP64 additions.
"""
from __future__ import annotations

from typing import Tuple

import numpy as np


def sample_range(spp: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous share [first, first + count) of `spp` samples for `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(spp, world)
    first = rank * base + min(rank, extra)
    count = base + (1 if rank < extra else 0)
    return first, count


def merge_films(sum_rgb: np.ndarray, sum_sq: np.ndarray, count: np.ndarray, group=None, device=None):
    """All-reduce (sum) the three FP64 film arrays in place across ranks."""
    import torch
    import torch.distributed as dist
    flat = np.concatenate([sum_rgb.reshape(-1), sum_sq.reshape(-1), count.reshape(-1)])
    t = torch.from_numpy(flat)
    if device is not None:
        t = t.to(device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    out = t.cpu().numpy()
    n1, n2 = sum_rgb.size, sum_sq.size
    sum_rgb.reshape(-1)[:] = out[:n1]
    sum_sq.reshape(-1)[:] = out[n1:n1 + n2]
    count.reshape(-1)[:] = out[n1 + n2:]
    return sum_rgb, sum_sq, count


def render_frame(ctx, sid: int, spp: int, seed: int, rank: int, world: int, mode=None, group=None, device=None):
    """Render this rank's share of the frame on its GPU and merge the films."""
    from . import CGPU_MODE_WAVEFRONT
    first, count = sample_range(spp, rank, world)
    ctx.film_clear(sid)
    if count:
        ctx.render([sid], first, count, seed, mode=CGPU_MODE_WAVEFRONT if mode is None else mode)
    s, q, n = ctx.film_read(sid)
    if world > 1:
        merge_films(s, q, n, group=group, device=device)
    return s, q, n
