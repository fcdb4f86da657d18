"""Replica parallelism of the render call across processes (one GPU each).

Paths are independent, so N GPUs render the same film from disjoint ranges of
sample indices: every rank's per-(pixel, sample) PCG streams are the ones a
single GPU would draw for those samples, and the image is the sum of the ranks'
films divided by the total sample count. The only exchange is that sum, done on
the host (films are small next to the work that fills them); nothing on the
data path waits for another rank. Timings are reduced with a max over ranks.

Used by bench.py (N > 1) and by applications that split a render over several
processes; the collectives go through ``torch.distributed`` on CPU tensors, so
any backend with CPU support (gloo) carries them.
"""
from __future__ import annotations

from typing import Tuple

import numpy as np


def sample_range(rank: int, world: int, spp: int, first: int = 0) -> Tuple[int, int]:
    """(first sample, sample count) of `rank` when `spp` samples starting at
    `first` are split as evenly as possible over `world` ranks (the first
    spp % world ranks take one more)."""
    if world < 1 or not 0 <= rank < world or spp < 0:
        raise ValueError("need 0 <= rank < world and spp >= 0")
    base, extra = divmod(spp, world)
    begin = first + rank * base + min(rank, extra)
    return begin, base + (1 if rank < extra else 0)


def reduce_film(film: np.ndarray, group=None) -> np.ndarray:
    """Sum of every rank's film (radiance sums [H, W, 3]), accumulated in FP64 and
    returned to every rank as float32."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(film, dtype=np.float64))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy().astype(np.float32)


def max_over_ranks(value: float, group=None) -> float:
    """The largest of the ranks' values (the job's time is its slowest rank's)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def render_replica(render, rank: int, world: int, spp: int, first: int = 0, group=None) -> np.ndarray:
    """Runs ``render(sample_begin, sample_count) -> film sums`` on this rank's range
    and returns the summed film of all ranks (every rank receives it)."""
    begin, count = sample_range(rank, world, spp, first)
    film = render(begin, count)
    return reduce_film(film, group)
