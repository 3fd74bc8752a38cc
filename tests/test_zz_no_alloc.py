"""ogx_gjk_epa_noalloc: the entry point that allocates no device memory (for callers
that must not allocate at query time -- inside an application-owned device-memory arena,
in allocation-free real-time loops).  Called twice in a row through
the C ABI, it must agree with the regular ogx_gjk_epa within the parity tolerances.
This file is collected last so that a failure here stops a `-x` run only after every
other test has run."""
import ctypes

import numpy as np
import pytest

import parity
from ogx import _lib, workloads as W

pytestmark = pytest.mark.gpu


def test_noalloc_matches_regular_entry_point_twice(engine):
    import torch
    L = _lib.load()
    fn = L.ogx_gjk_epa_noalloc
    P = ctypes.c_void_p
    fn.restype = ctypes.c_int
    fn.argtypes = [P, P, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P, P]

    b = W.powerlaw(seed=77, n_pairs=6000)
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, b.counts)
    pool.upload(b.coords)
    pairs = torch.from_numpy(np.ascontiguousarray(b.pairs)).cuda()
    ref = engine.run(ctx, pool, pairs, engine.MODE_GJK_EPA).to_host()
    ctx.synchronize()
    d_points, d_bodies = pool.device_layout()

    for call in range(2):
        out = engine.Results(b.n_pairs, pairs.device)
        ctx.stream.wait_stream(torch.cuda.current_stream())  # zero-filled outputs are ready
        rc = fn(P(d_points), P(d_bodies), b.n_bodies, b.n_pairs, P(pairs.data_ptr()), P(out.simplex.data_ptr()),
                P(out.dist.data_ptr()), P(out.normal.data_ptr()), P(out.status.data_ptr()), None,
                P(ctx.stream.cuda_stream))
        assert rc == 0, L.ogx_last_error()
        ctx.synchronize()
        got = out.to_host()
        d, dr = got["dist"].astype(np.float64), ref["dist"].astype(np.float64)
        scale = parity.pair_scale(b)
        sep = (dr > parity.BAND * scale) & (d > 0)
        assert np.all(np.abs(d[sep] - dr[sep]) <= parity.REL * dr[sep]), f"call {call}: distance"
        con = (dr < 0) & (d < 0)
        assert np.all(np.abs(d[con] - dr[con]) <= parity.ABS4), f"call {call}: depth"
        assert np.mean(np.sign(d) == np.sign(dr)) > 0.999, f"call {call}: verdicts"
        nerr = np.linalg.norm(got["normal"][con] - ref["normal"][con], axis=1)
        assert np.mean(nerr <= parity.ABS4) > 0.995, f"call {call}: normals"


def test_noalloc_rejects_oversized_batch(engine):
    L = _lib.load()
    fn = L.ogx_gjk_epa_noalloc
    P = ctypes.c_void_p
    fn.restype = ctypes.c_int
    fn.argtypes = [P, P, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P, P]
    dummy = ctypes.c_int(0)
    p = ctypes.addressof(dummy)
    rc = fn(P(p), P(p), 2, 16385, P(p), P(p), P(p), P(p), None, None, None)
    assert rc == -5 and b"at most 16384" in L.ogx_last_error()
