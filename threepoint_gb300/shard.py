"""Multi-GPU form of the batched <Map^3> evaluation: one process per GPU.

Every (cosmology, theta-triplet) integral is independent and every cosmology's
tables are read-only, so ranks take contiguous blocks of the cosmology list
and evaluate them with no communication; the only collective is the host-side
gather of the finished result blocks to rank 0 (torch.distributed
gather_object: works on gloo and NCCL process groups). This is the reference's
one-cosmology-per-process use (interface.cu:150-244, one MapMapMap per triplet)
spread over processes.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """[lo, hi) of rank's contiguous block of n items; block sizes differ by
    at most one, lower ranks take the larger blocks."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError("need 0 <= rank < world and n >= 0")
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def gather_blocks(block: np.ndarray, lo: int, n_total: int, group=None):
    """Gather every rank's (lo, block) to rank 0 and assemble the rows in
    global order; returns the full array on rank 0 and None elsewhere."""
    import torch.distributed as dist

    if not dist.is_initialized():
        return block
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    parts = [None] * world if rank == 0 else None
    dist.gather_object((lo, block), parts, dst=0, group=group)
    if rank != 0:
        return None
    shape = None
    for _, b in parts:
        if b is not None and len(b):
            shape = b.shape[1:]
            dtype = b.dtype
            break
    if shape is None:
        return np.zeros((n_total,) + tuple(block.shape[1:]), dtype=block.dtype)
    out = np.empty((n_total,) + tuple(shape), dtype=dtype)
    seen = np.zeros(n_total, dtype=bool)
    for lo_r, b in parts:
        out[lo_r:lo_r + len(b)] = b
        seen[lo_r:lo_r + len(b)] = True
    if not seen.all():
        raise RuntimeError("gathered blocks do not cover every cosmology")
    return out


def map3_sharded(cosmologies: Sequence, evaluate: Callable[[Sequence, int], np.ndarray], group=None):
    """Evaluate this rank's block of cosmologies with evaluate(block, lo) ->
    array [len(block), ...] and gather all blocks to rank 0 (None elsewhere).
    With no initialised process group this is a single-process call."""
    import torch.distributed as dist

    if dist.is_initialized():
        rank, world = dist.get_rank(group), dist.get_world_size(group)
    else:
        rank, world = 0, 1
    lo, hi = shard_range(len(cosmologies), rank, world)
    block = np.asarray(evaluate(cosmologies[lo:hi], lo))
    return gather_blocks(block, lo, len(cosmologies), group)


def context_evaluator(ctx, nz, thetas, batch: int = 64, precision: int = 1, **kw):
    """evaluate(block, lo) for map3_sharded on one GPU context: the block's
    cosmologies in batches of `batch`, all triplets each, through
    Context.map3_batch."""
    th = np.asarray(thetas, dtype=np.float64).reshape(-1, 3)

    def evaluate(block, lo):
        out = np.zeros((len(block), len(th)))
        for s in range(0, len(block), batch):
            part = list(block[s:s + batch])
            ctx.set_cosmologies(part, nz)
            out[s:s + len(part)] = ctx.map3_batch(th, precision=precision, **kw)
        return out

    return evaluate
