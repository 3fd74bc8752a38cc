"""ogx_gjk_epa_noalloc: the GJK + EPA entry point that allocates no device memory.

Some callers cannot call cudaMalloc at query time: a physics or rendering loop whose
device memory is one arena it owns, a real-time tick that cannot take the allocator's
latency, a plugin whose host application forbids it to allocate.  This entry point keeps
the pipeline's work lists in a static device array instead.

It runs the same per-pair code as the regular entry point with other kernel variants (one
pair per warp, the sub-distance decision tree instead of the table, capacity spills
restarted at full capacity instead of resumed), all of which give the same bits.  So it
is checked, twice in a row through the C ABI, at its largest batch (16384 pairs), for bit
identity with the regular entry point on every output, and against the FP64 oracle under
every parity rule.  The regular engine's work counters on the same batch show that the
spill passes ran.

This file is collected last, so a failure here stops a `-x` run only after every other
test has run."""
import ctypes

import numpy as np
import pytest

import parity
from ogx import _lib, workloads as W

pytestmark = pytest.mark.gpu

MAX_PAIRS = 16384


def _fn():
    L = _lib.load()
    fn = L.ogx_gjk_epa_noalloc
    P = ctypes.c_void_p
    fn.restype = ctypes.c_int
    fn.argtypes = [P, P, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P, P]
    return L, fn


def _join(a, b):
    """One batch holding the bodies and pairs of a and then b."""
    off = a.coords.shape[0]
    pairs = np.concatenate([a.pairs, b.pairs + a.n_bodies]).astype(np.int32)
    return W.Batch(np.concatenate([a.coords, b.coords]), np.concatenate([a.offsets, b.offsets + off]),
                   np.concatenate([a.counts, b.counts]), pairs, "stress+powerlaw")


def test_noalloc_matches_regular_entry_point_twice(engine, orc):
    import torch
    L, fn = _fn()
    P = ctypes.c_void_p
    # near-touching pairs, boxes and thin disks (FP64 refinement, certified re-runs, late
    # contacts) plus power-law pairs up to 1024 points (small-capacity spills)
    b = _join(W.stress(seed=91, n_pairs=MAX_PAIRS // 2), W.powerlaw(seed=92, n_pairs=MAX_PAIRS // 2))
    assert b.n_pairs == MAX_PAIRS
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, b.counts)
    pool.upload(b.coords)
    pairs = torch.from_numpy(np.ascontiguousarray(b.pairs)).cuda()
    ref = engine.run(ctx, pool, pairs, engine.MODE_GJK_EPA).to_host()
    ctx.synchronize()
    work = ctx.work_counts()
    assert work["epa_spill"] > 0, work  # contacts re-run at full capacity on this batch
    d_points, d_bodies = pool.device_layout()
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64", threads=16)
    parity.assert_parity(parity.check(b, ref, o, label="regular"), max_witness_mismatch_frac=2e-3)

    for call in range(2):
        out = engine.Results(b.n_pairs, pairs.device)
        ctx.stream.wait_stream(torch.cuda.current_stream())  # zero-filled outputs are ready
        rc = fn(P(d_points), P(d_bodies), b.n_bodies, b.n_pairs, P(pairs.data_ptr()), P(out.simplex.data_ptr()),
                P(out.dist.data_ptr()), P(out.normal.data_ptr()), P(out.status.data_ptr()), None,
                P(ctx.stream.cuda_stream))
        assert rc == 0, L.ogx_last_error()
        ctx.synchronize()
        got = out.to_host()
        for k in ("dist", "normal", "status"):
            assert np.array_equal(got[k], ref[k]), f"call {call}: {k}"
        assert got["simplex"].tobytes() == ref["simplex"].tobytes(), f"call {call}: simplex"
        parity.assert_parity(parity.check(b, got, o, label=f"noalloc call {call}"), max_witness_mismatch_frac=2e-3)


def test_noalloc_rejects_oversized_batch(engine):
    L, fn = _fn()
    P = ctypes.c_void_p
    dummy = ctypes.c_int(0)
    p = ctypes.addressof(dummy)
    rc = fn(P(p), P(p), 2, MAX_PAIRS + 1, P(p), P(p), P(p), P(p), None, None, None)
    assert rc == _lib.ERR_CAPACITY and b"at most 16384" in L.ogx_last_error()
