"""Host-side packing of bodies into the engine's padded SoA pool layout.

Body b occupies 3 * n4 floats starting at float offset 4 * quad[b]:
x[0..n4), y[0..n4), z[0..n4), with n4 = n rounded up to a multiple of 4.  Padding
points repeat point 0 (a support scan never picks them: ties go to the lower index).
The same layout is produced on the device by ogx_pool_upload / ogx_pool_load_device.
"""
from __future__ import annotations

import numpy as np


def layout(counts: np.ndarray):
    """(quad offsets uint32, total floats) for bodies with `counts` points."""
    counts = np.asarray(counts, dtype=np.int64)
    if counts.size and counts.min() < 1:
        raise ValueError("every body needs at least one point")
    nq = 3 * ((counts + 3) // 4)
    quad = np.zeros(counts.shape[0], dtype=np.int64)
    np.cumsum(nq[:-1], out=quad[1:])
    total = int(4 * nq.sum())
    if total // 4 >= 2 ** 32:
        raise ValueError("pool too large for 32-bit quad offsets")
    return quad.astype(np.uint32), total


def pack(coords: np.ndarray, counts: np.ndarray):
    """AoS points (bodies concatenated) -> (pool float32, quad uint32)."""
    coords = np.ascontiguousarray(coords, dtype=np.float32).reshape(-1, 3)
    counts = np.asarray(counts, dtype=np.int64)
    quad, total = layout(counts)
    pool = np.empty(total, dtype=np.float32)
    n4 = 4 * ((counts + 3) // 4)
    body = np.repeat(np.arange(counts.shape[0]), n4)
    start = np.repeat(np.cumsum(n4) - n4, n4)
    local = np.arange(int(n4.sum())) - start          # slot within the body
    src_off = np.zeros(counts.shape[0], dtype=np.int64)
    np.cumsum(counts[:-1], out=src_off[1:])
    src = src_off[body] + np.where(local < counts[body], local, 0)
    base = 4 * quad.astype(np.int64)[body]
    for c in range(3):
        pool[base + c * n4[body] + local] = coords[src, c]
    return pool, quad
