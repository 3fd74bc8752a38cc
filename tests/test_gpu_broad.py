"""Device broad phase (ogx_broadphase) against a brute-force box-overlap test on the host:
the same pair set, each pair once, sorted by (i, j), for any cell size."""
import numpy as np
import pytest

from ogx import workloads as W

pytestmark = pytest.mark.gpu


def _boxes(world, counts, margin):
    off = np.concatenate([[0], np.cumsum(counts)[:-1]])
    lo = np.minimum.reduceat(world, off, axis=0).astype(np.float32) - np.float32(margin)
    hi = np.maximum.reduceat(world, off, axis=0).astype(np.float32) + np.float32(margin)
    return lo, hi


def _brute(lo, hi):
    n = lo.shape[0]
    out = []
    for i in range(n - 1):
        ok = np.all((np.maximum(lo[i], lo[i + 1:]) <= np.minimum(hi[i], hi[i + 1:])), axis=1)
        j = np.flatnonzero(ok) + i + 1
        out.append(np.stack([np.full(j.size, i), j], 1))
    return np.concatenate(out).astype(np.int32) if out else np.zeros((0, 2), np.int32)


@pytest.mark.parametrize("cell,margin", [(4.0, 0.0), (2.0, 0.25), (20.0, 0.5)])
def test_broadphase_matches_brute_force(engine, cell, margin):
    sc = W.serving_scene(seed=8, n_bodies=3000, half=20.0)
    world = sc.world(sc.transforms(3))
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, sc.counts)
    pool.upload(world)
    br = engine.Broad(ctx, 3000)
    pairs, count, flags = br.run(pool, cell, margin, max_pairs=200_000)
    lo, hi = _boxes(world, sc.counts, margin)
    ref = _brute(lo, hi)
    assert flags == 0
    assert count == ref.shape[0] > 100
    assert np.array_equal(pairs.cpu().numpy(), ref)
    # capacity: the count still reports every pair, the first max_pairs are written
    part, count2, _ = br.run(pool, cell, margin, max_pairs=50)
    assert count2 == count and part.shape[0] == 50
    br.close()


def test_broadphase_feeds_gjk(engine, orc):
    """Broad phase -> GJK/EPA on the device, compared with the oracle on the same pairs."""
    import parity
    sc = W.serving_scene(seed=9, n_bodies=2000, half=15.0)
    world = sc.world(sc.transforms(1))
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, sc.counts)
    pool.upload(world)
    br = engine.Broad(ctx, 2000)
    pairs, count, flags = br.run(pool, 4.0, 0.1, max_pairs=100_000)
    res = engine.run(ctx, pool, pairs.contiguous(), engine.MODE_GJK_EPA).to_host()
    ctx.synchronize()
    b = W.Batch(world, sc.offsets, sc.counts, pairs.cpu().numpy(), "broad")
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64", threads=16)
    rep = parity.check(b, res, o, label="broad")
    parity.assert_parity(rep, max_witness_mismatch_frac=2e-3)
    assert rep["contacts"] > 10
