"""The FP64 drop-in (*_f64 entry points: the reference built with USE_32BITS off,
gkFloat = double, 48-byte gkPolytope, 184-byte gkSimplex) on the FP64 plain-GJK
workload -- 1,000 pairs of 32-point spheres, radius U[0.5, 2], centres U[-5, 5]^3,
coordinates in double -- through the C ABI, against the FP64 oracle on the same double
inputs: verdicts exact outside the contact band, separated distances within 1e-5
relative, depths within 1e-4; plus the known answers through the FP64 calls.  The
engine's search runs on the inputs rounded to float; separated pairs are finished in
FP64 on the double inputs (exact supports and Minkowski points), so the distance carries
no input rounding."""
import ctypes
import os

import numpy as np
import pytest

import parity
from ogx import _lib, workloads as W

pytestmark = pytest.mark.gpu

POLY64 = np.dtype([("numpoints", "<i4"), ("s", "<f8", (3,)), ("s_idx", "<i4"), ("coord", "<u8")], align=True)
SMP64 = np.dtype([("nvrtx", "<i4"), ("vrtx", "<f8", (4, 3)), ("vrtx_idx", "<i4", (4, 2)),
                  ("witnesses", "<f8", (2, 3))], align=True)


def test_fp64_layouts():
    assert POLY64.itemsize == 48 and SMP64.itemsize == 184


def _lib64():
    L = _lib.load()
    P, I = ctypes.c_void_p, ctypes.c_int
    for name, args in (("ogx_compute_gjk_epa_f64", [I, P, P, P, P, P]),
                       ("ogx_compute_minimum_distance_f64", [I, P, P, P, P]),
                       ("ogx_compute_gjk_epa_indexed_f64", [I, I, P, P, P, P, P])):
        fn = getattr(L, name)
        fn.restype = ctypes.c_int
        fn.argtypes = args
    return L


def _desc(coords64, offsets, counts, idx):
    d = np.zeros(len(idx), POLY64)
    d["numpoints"] = counts[idx]
    d["coord"] = coords64.ctypes.data + 24 * offsets[idx].astype(np.uint64)
    return d


@pytest.mark.parametrize("seed", [1, 4, 7])
def test_fp64_plain_workload_parity(engine, orc, seed):
    L = _lib64()
    b = W.plain(seed=seed, n_pairs=1000, dtype=np.float64)
    c64 = np.ascontiguousarray(b.coords)
    d1 = _desc(c64, b.offsets, b.counts, b.pairs[:, 0])
    d2 = _desc(c64, b.offsets, b.counts, b.pairs[:, 1])
    n = b.n_pairs
    smp, dist, nrm = np.zeros(n, SMP64), np.zeros(n), np.zeros((n, 3))
    P = ctypes.c_void_p
    _lib.check(L.ogx_compute_gjk_epa_f64(n, P(d1.ctypes.data), P(d2.ctypes.data), P(smp.ctypes.data),
                                         P(dist.ctypes.data), P(nrm.ctypes.data)))
    o = orc.run(c64, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64")
    s = parity.pair_scale(b)
    band = np.abs(o["dist"]) <= parity.BAND * s
    col64 = o["epa_exit"] > 0
    col = dist <= 0
    assert np.all((col == col64) | band)
    sep = ~col & ~col64 & ~band
    rel = np.abs(dist[sep] - o["dist"][sep]) / o["dist"][sep]
    assert rel.max() <= parity.REL, rel.max()
    con = col & col64 & ~band
    assert np.all(np.abs(dist[con] - o["dist"][con]) <= parity.ABS4)
    nerr = np.linalg.norm(nrm[sep] - o["normal"][sep], axis=1)
    assert nerr.max() <= parity.ABS4, nerr.max()
    # GJK alone through the FP64 call gives the same separated distances
    smp2, dist2 = np.zeros(n, SMP64), np.zeros(n)
    _lib.check(L.ogx_compute_minimum_distance_f64(n, P(d1.ctypes.data), P(d2.ctypes.data), P(smp2.ctypes.data),
                                                  P(dist2.ctypes.data)))
    assert np.array_equal(dist2[sep], dist[sep])
    # and the indexed FP64 call over the whole pool
    pool = _desc(c64, b.offsets, b.counts, np.arange(b.n_bodies))
    pairs = np.ascontiguousarray(b.pairs, np.int32)
    smp3, dist3, nrm3 = np.zeros(n, SMP64), np.zeros(n), np.zeros((n, 3))
    _lib.check(L.ogx_compute_gjk_epa_indexed_f64(b.n_bodies, n, P(pool.ctypes.data), P(pairs.ctypes.data),
                                                 P(smp3.ctypes.data), P(dist3.ctypes.data), P(nrm3.ctypes.data)))
    assert np.array_equal(dist3, dist) and np.array_equal(nrm3, nrm)


def test_fp64_known_answers(engine):
    """README.md:111-115 and 131-137 through the FP64 calls, on the double inputs."""
    L = _lib64()
    P = ctypes.c_void_p
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "usage_gjk.npz"))
    c64 = np.ascontiguousarray(z["coords"], np.float64)
    d1 = _desc(c64, z["offsets"], z["counts"], np.array([0]))
    d2 = _desc(c64, z["offsets"], z["counts"], np.array([1]))
    smp, dist = np.zeros(1, SMP64), np.zeros(1)
    _lib.check(L.ogx_compute_minimum_distance_f64(1, P(d1.ctypes.data), P(d2.ctypes.data), P(smp.ctypes.data),
                                                  P(dist.ctypes.data)))
    assert f"{dist[0]:.6f}" == "3.653650"
    assert [f"{x:.6f}" for x in smp["witnesses"][0, 0]] == ["1.025173", "1.490318", "0.255463"]
    cubes = np.concatenate([W.cube(), W.rotated_cube()]).astype(np.float64)
    off, cnt = np.array([0, 8]), np.array([8, 8], np.int32)
    d1, d2 = _desc(cubes, off, cnt, np.array([0])), _desc(cubes, off, cnt, np.array([1]))
    smp, dist, nrm = np.zeros(1, SMP64), np.zeros(1), np.zeros((1, 3))
    _lib.check(L.ogx_compute_gjk_epa_f64(1, P(d1.ctypes.data), P(d2.ctypes.data), P(smp.ctypes.data),
                                         P(dist.ctypes.data), P(nrm.ctypes.data)))
    assert abs(dist[0] + 1.5) < 1e-4 and np.allclose(nrm[0], [1, 0, 0], atol=1e-4)
