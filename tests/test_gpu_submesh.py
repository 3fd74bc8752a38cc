"""Bodies made of several convex parts: body pairs expand to part pairs in the reference's
order (a-major), GJK+EPA runs on the part pairs, and the per-body-pair reduction gives the
smallest part-pair distance -- checked against numpy and the FP64 oracle."""
import numpy as np
import pytest

import parity
from ogx import workloads as W

pytestmark = pytest.mark.gpu


def test_expand_and_reduce(engine, orc):
    import torch
    rng = np.random.default_rng(3)
    parts = W.ellipsoid(seed=13, n_pairs=1500)          # 3000 convex parts
    nb = 700                                             # bodies of 1-8 parts
    cnt = rng.integers(1, 9, nb)
    cnt[-1] = 3000 - cnt[:-1].sum() if cnt[:-1].sum() < 3000 else 1
    cnt = cnt[np.cumsum(cnt) <= 3000]
    nb = cnt.shape[0]
    first = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int32)
    cnt = cnt.astype(np.int32)
    bp = np.stack([rng.integers(0, nb, 2000), rng.integers(0, nb, 2000)], 1).astype(np.int32)
    bp[5] = [nb + 3, 0]                                  # invalid body: no parts
    ref = []
    for i, (a, b) in enumerate(bp):
        if 0 <= a < nb and 0 <= b < nb:
            ref += [(first[a] + x, first[b] + y) for x in range(cnt[a]) for y in range(cnt[b])]
    ref = np.array(ref, np.int32)
    ctx = engine.Context(0)
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    sub, owner, off = engine.expand_submesh_pairs(ctx, d(bp), d(first), d(cnt), max_sub_pairs=len(ref) + 10)
    ctx.synchronize()
    assert np.array_equal(sub.cpu().numpy(), ref)
    offs = off.cpu().numpy()
    assert offs[-1] == len(ref) and np.all(np.diff(offs) >= 0)
    own = owner.cpu().numpy()
    assert np.all(own == np.repeat(np.arange(len(bp)), np.diff(offs)))
    # narrow phase on the part pairs, reduction per body pair
    pool = engine.Pool(ctx, parts.counts)
    pool.upload(parts.coords)
    res = engine.run(ctx, pool, sub.contiguous(), engine.MODE_GJK_EPA)
    best, arg = engine.reduce_submesh_pairs(ctx, off, res.dist, max_sub_pairs=len(ref) + 10)
    ctx.synchronize()
    dist = res.dist.cpu().numpy()
    b_host = np.array([dist[offs[i]:offs[i + 1]].min() if offs[i + 1] > offs[i] else np.inf
                       for i in range(len(bp))], np.float32)
    assert np.array_equal(best.cpu().numpy(), b_host)
    assert arg.cpu().numpy()[5] == -1
    # the part pairs themselves meet the parity rules
    pb = W.Batch(parts.coords, parts.offsets, parts.counts, ref, "parts")
    o = orc.run(pb.coords, pb.offsets, pb.counts, pb.pairs, mode=orc.MODE_GJK_EPA, precision="f64", threads=16)
    rep = parity.check(pb, res.to_host(), o, label="parts")
    parity.assert_parity(rep, max_witness_mismatch_frac=2e-3)
