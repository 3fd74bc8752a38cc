"""Python mirror of OpenGJK-GPU's host API (GJK/gpu/openGJK.h, examples/gpu/example.h)
over the engine's reference-compatible C entry points (ogx_compute_*, ...).

Polytopes are ``gkPolytope`` descriptor arrays (``POLYTOPE_DTYPE``: numpoints + a pointer
to xyz-interleaved float32 coordinates), exactly what the reference's functions take;
results are ``gkSimplex`` arrays (``SIMPLEX_DTYPE``), distances and normals.  Output
conventions are the reference's: distance >= 0 when separated, 0 when GJK encloses the
origin, -depth after EPA; witnesses in simplex["witnesses"].
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import POLYTOPE_DTYPE, SIMPLEX_DTYPE, check

_P = ctypes.c_void_p
_I = ctypes.c_int
SIGNATURES = {
    "ogx_compute_minimum_distance": (_I, [_I, _P, _P, _P, _P]),
    "ogx_compute_collision_information": (_I, [_I, _P, _P, _P, _P, _P]),
    "ogx_compute_gjk_epa": (_I, [_I, _P, _P, _P, _P, _P]),
    "ogx_compute_collision_information_witnesses": (_I, [_I, _P, _P, _P, _P, _P, _P, _P]),
    "ogx_allocate_and_copy_device_arrays": (_I, [_I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "ogx_compute_minimum_distance_device": (_I, [_I, _P, _P, _P, _P]),
    "ogx_compute_epa_device": (_I, [_I, _P, _P, _P, _P, _P]),
    "ogx_copy_results_from_device": (_I, [_I, _P, _P, _P, _P]),
    "ogx_free_device_arrays": (_I, [_P, _P, _P, _P, _P, _P]),
    "ogx_allocate_epa_device_arrays": (_I, [_I, _P, _P, _P]),
    "ogx_copy_epa_results_from_device": (_I, [_I, _P, _P, _P, _P, _P, _P]),
    "ogx_free_epa_device_arrays": (_I, [_P, _P, _P]),
    "ogx_allocate_indexed_device": (_I, [_I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "ogx_free_indexed_device": (_I, [_P, _P, _P, _P, _P, _P]),
    "ogx_upload_pairs_device": (_I, [_I, _P, _P]),
    "ogx_compute_minimum_distance_indexed": (_I, [_I, _I, _P, _P, _P, _P]),
    "ogx_compute_minimum_distance_indexed_device": (_I, [_I, _P, _P, _P, _P]),
    "ogx_compute_epa_indexed": (_I, [_I, _I, _P, _P, _P, _P, _P]),
    "ogx_compute_epa_indexed_device": (_I, [_I, _P, _P, _P, _P, _P]),
    "ogx_compute_gjk_epa_indexed": (_I, [_I, _I, _P, _P, _P, _P, _P]),
    "ogx_compat_last_gpu_ms": (ctypes.c_float, []),
}

_lib_ref = None


def lib():
    global _lib_ref
    if _lib_ref is None:
        L = _lib.load()
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib_ref = L
    return _lib_ref


class Polytopes:
    """A gkPolytope descriptor array over host coordinates (kept alive here)."""

    def __init__(self, coords: np.ndarray, counts: np.ndarray, offsets: np.ndarray | None = None):
        self.coords = np.ascontiguousarray(coords, dtype=np.float32).reshape(-1, 3)
        counts = np.asarray(counts, dtype=np.int32)
        if offsets is None:
            offsets = np.zeros(counts.shape[0], dtype=np.int64)
            np.cumsum(counts[:-1], out=offsets[1:])
        self.desc = np.zeros(counts.shape[0], dtype=POLYTOPE_DTYPE)
        self.desc["numpoints"] = counts
        self.desc["coord"] = self.coords.ctypes.data + 12 * np.asarray(offsets, dtype=np.uint64)

    def __len__(self):
        return int(self.desc.shape[0])

    @property
    def ptr(self) -> int:
        return self.desc.ctypes.data

    def take(self, idx) -> "Polytopes":
        p = Polytopes.__new__(Polytopes)
        p.coords = self.coords
        p.desc = np.ascontiguousarray(self.desc[idx])
        return p


def from_batch(batch):
    """(bd1, bd2) descriptor arrays of a workloads.Batch's pairs, and the pool's."""
    pool = Polytopes(batch.coords, batch.counts, batch.offsets)
    return pool.take(batch.pairs[:, 0]), pool.take(batch.pairs[:, 1]), pool


def _out(n, normals=True):
    return (np.zeros(n, SIMPLEX_DTYPE), np.zeros(n, np.float32),
            np.zeros((n, 3), np.float32) if normals else None)


def _ptr(a):
    return None if a is None else a.ctypes.data


def compute_minimum_distance(bd1: Polytopes, bd2: Polytopes):
    """GJK::GPU::computeDistances / compute_minimum_distance(n, ...)."""
    n = len(bd1)
    smp, dist, _ = _out(n, False)
    check(lib().ogx_compute_minimum_distance(n, bd1.ptr, bd2.ptr, _ptr(smp), _ptr(dist)))
    return smp, dist


def compute_gjk_epa(bd1: Polytopes, bd2: Polytopes):
    """GJK::GPU::computeGJKAndEPA / compute_gjk_epa."""
    n = len(bd1)
    smp, dist, nrm = _out(n)
    check(lib().ogx_compute_gjk_epa(n, bd1.ptr, bd2.ptr, _ptr(smp), _ptr(dist), _ptr(nrm)))
    return smp, dist, nrm


def compute_epa(bd1: Polytopes, bd2: Polytopes, simplices, distances, with_normals=True):
    """GJK::GPU::computeEPA / computeCollisionInformation(n, ...): updates simplices and
    distances in place, returns the normals (or None)."""
    n = len(bd1)
    nrm = np.zeros((n, 3), np.float32) if with_normals else None
    check(lib().ogx_compute_collision_information(n, bd1.ptr, bd2.ptr, _ptr(simplices), _ptr(distances),
                                                  _ptr(nrm)))
    return nrm


def compute_collision_information(bd1: Polytopes, bd2: Polytopes, simplices, distances):
    """GJK::GPU::computeCollisionInformation (README.md:39-46 form): witnesses as n x 3."""
    n = len(bd1)
    w1 = np.zeros((n, 3), np.float32)
    w2 = np.zeros((n, 3), np.float32)
    nrm = np.zeros((n, 3), np.float32)
    check(lib().ogx_compute_collision_information_witnesses(n, bd1.ptr, bd2.ptr, _ptr(simplices),
                                                            _ptr(distances), _ptr(w1), _ptr(w2), _ptr(nrm)))
    return w1, w2, nrm


def compute_gjk_epa_indexed(pool: Polytopes, pairs: np.ndarray):
    pairs = np.ascontiguousarray(pairs, dtype=np.int32)
    n = pairs.shape[0]
    smp, dist, nrm = _out(n)
    check(lib().ogx_compute_gjk_epa_indexed(len(pool), n, pool.ptr, pairs.ctypes.data, _ptr(smp), _ptr(dist),
                                            _ptr(nrm)))
    return smp, dist, nrm


def compute_minimum_distance_indexed(pool: Polytopes, pairs: np.ndarray):
    pairs = np.ascontiguousarray(pairs, dtype=np.int32)
    n = pairs.shape[0]
    smp, dist, _ = _out(n, False)
    check(lib().ogx_compute_minimum_distance_indexed(len(pool), n, pool.ptr, pairs.ctypes.data, _ptr(smp),
                                                     _ptr(dist)))
    return smp, dist


def last_gpu_ms() -> float:
    """GJK::GPU::timer().getGpuElapsedTimeForPreviousOperation()."""
    return float(lib().ogx_compat_last_gpu_ms())
