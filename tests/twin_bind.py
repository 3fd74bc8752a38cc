"""ctypes binding of the host test build of the engine's per-pair code
(tests/twin/libogx_twin.so).  Test infrastructure only."""
import ctypes
import os

import numpy as np

from ogx import _lib
from ogx import pool as P

HERE = os.path.dirname(os.path.abspath(__file__))
_lib_twin = ctypes.CDLL(os.path.join(HERE, "twin", "libogx_twin.so"))
_lib_twin.twin_run.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_void_p] + \
    [ctypes.c_void_p] * 5 + [ctypes.c_int]
_lib_twin.twin_config.argtypes = [ctypes.c_int, ctypes.c_void_p]
_lib_twin.twin_run_posed.argtypes = _lib_twin.twin_run.argtypes + [ctypes.c_void_p]
_lib_twin.twin_pose_points.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4


def config(reference=False, **kw):
    c = _lib.Config()
    _lib_twin.twin_config(int(reference), ctypes.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def pose_points(counts, local, xf):
    """World points of the fused-transform pipeline: pose_point of every body point."""
    counts = np.ascontiguousarray(counts, np.int32)
    local = np.ascontiguousarray(local, np.float32)
    xf = np.ascontiguousarray(xf, np.float32)
    out = np.empty_like(local)
    _lib_twin.twin_pose_points(int(counts.shape[0]), counts.ctypes.data, local.ctypes.data, xf.ctypes.data,
                               out.ctypes.data)
    return out


def run(b, mode=2, cfg=None, threads=8, xf=None):
    """xf: poses (B, 12) to run the posed pipeline on b's points taken as body frames."""
    pool, quad = P.pack(b.coords, b.counts)
    n = b.n_pairs
    dist = np.zeros(n, np.float32)
    smp = np.zeros(n, _lib.SIMPLEX_DTYPE)
    nrm = np.zeros((n, 3), np.float32)
    st = np.zeros(n, np.int32)
    it = np.zeros((n, 2), np.int32)
    cfg = cfg or config()
    pairs = np.ascontiguousarray(b.pairs, np.int32)
    cnt = np.ascontiguousarray(b.counts, np.int32)
    xfa = None if xf is None else np.ascontiguousarray(xf, np.float32)
    rc = _lib_twin.twin_run_posed(n, pool.ctypes.data, quad.ctypes.data, cnt.ctypes.data, pairs.ctypes.data, mode,
                                  ctypes.byref(cfg), dist.ctypes.data, smp.ctypes.data, nrm.ctypes.data,
                                  st.ctypes.data, it.ctypes.data, threads,
                                  None if xfa is None else xfa.ctypes.data)
    assert rc == 0
    return {"dist": dist, "simplex": smp, "normal": nrm, "status": st, "iters": it}
