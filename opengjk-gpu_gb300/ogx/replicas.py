"""Data-parallel replicas: one process per GPU, each with the whole body pool and a
contiguous range of the pairs.

Pairs are independent, so a batch shards by pair ranges with no collective in the
compute (the reference runs one GPU; this is how the same batch spreads over several).
Ranges are balanced by work, measured as n1 + n2 per pair (the points both bodies
contribute to every support scan).  Results are gathered to every rank (or kept where
they were computed) with one all-gather per output array.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(counts: np.ndarray, pairs: np.ndarray, world: int) -> np.ndarray:
    """Boundaries b[0] = 0 <= b[1] <= ... <= b[world] = npairs: rank r takes pairs
    [b[r], b[r+1]), ranges balanced by the summed points of both bodies."""
    if world < 1:
        raise ValueError("world must be >= 1")
    n = int(pairs.shape[0])
    w = counts[pairs[:, 0]].astype(np.int64) + counts[pairs[:, 1]]
    c = np.concatenate([[0], np.cumsum(w)])
    targets = c[-1] * np.arange(world + 1) / world
    b = np.searchsorted(c, targets, side="left").clip(0, n)
    b[0], b[-1] = 0, n
    return np.maximum.accumulate(b)


def shard(counts: np.ndarray, pairs: np.ndarray, world: int, rank: int) -> tuple[int, int]:
    b = shard_bounds(counts, pairs, world)
    return int(b[rank]), int(b[rank + 1])


def all_gather_rows(local: np.ndarray, bounds: np.ndarray, group=None) -> np.ndarray:
    """Concatenate every rank's rows (rank order) on every rank with torch.distributed
    (any backend; CPU tensors for gloo).  `bounds` from shard_bounds gives each rank's
    row count, so ranks may hold different numbers of rows."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    sizes = np.diff(bounds)
    m = int(sizes.max()) if sizes.size else 0
    flat = np.ascontiguousarray(local).view(np.uint8).reshape(local.shape[0], -1)
    width = flat.shape[1] if flat.ndim == 2 and flat.shape[0] else np.dtype(local.dtype).itemsize * int(
        np.prod(local.shape[1:]))
    buf = torch.zeros((m, width), dtype=torch.uint8)
    if local.shape[0]:
        buf[: local.shape[0]] = torch.from_numpy(flat)
    outs = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(outs, buf, group=group)
    rows = [o[: int(sizes[r])].numpy() for r, o in enumerate(outs)]
    joined = np.concatenate(rows, axis=0)
    return joined.view(local.dtype).reshape((-1,) + local.shape[1:])
