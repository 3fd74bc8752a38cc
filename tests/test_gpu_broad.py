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


def reference_sphere_pairs(sph, cell, boundary, grid):
    """The reference's broad-phase pairs restated on the host
    (visualization/integrate_final_gjk.cu:467-570): a sphere's cell is
    floor((p + boundary) / cell) per axis clamped to [0, grid); i < j pair when their
    cells are neighbours (at most one apart on every axis) and
    fx*fx + fy*fy + fz*fz < (r_i + r_j)^2, all in FP32 in that order."""
    p = sph[:, :3].astype(np.float32)
    r = sph[:, 3].astype(np.float32)
    c = np.clip(np.floor((p + np.float32(boundary)) / np.float32(cell)), 0, grid - 1).astype(np.int64)
    out = []
    for i in range(len(p) - 1):
        j = np.arange(i + 1, len(p))
        near = np.all(np.abs(c[j] - c[i]) <= 1, axis=1)
        f = p[i] - p[j]
        d2 = (f[:, 0] * f[:, 0] + f[:, 1] * f[:, 1]) + f[:, 2] * f[:, 2]
        rs = r[i] + r[j]
        k = j[near & (d2 < rs * rs)]
        out.append(np.stack([np.full(k.size, i), k], 1))
    return np.concatenate(out).astype(np.int32)


@pytest.mark.parametrize("cell,boundary,grid", [(4.0, 20.0, 10), (1.5, 20.0, 27), (6.0, 12.0, 4)])
def test_sphere_broadphase_matches_reference_semantics(engine, cell, boundary, grid):
    """ogx_broadphase_spheres gives the reference's pair set: the same cells (clamped at
    the grid's edge, so spheres outside the box share the edge cells), the same 27-cell
    neighbourhood (pairs whose centres are more than a cell apart are missed, as there,
    when the cell is small against the radii), the same FP32 overlap test."""
    import torch
    rng = np.random.default_rng(int(cell * 10) + grid)
    n = 4000
    pos = rng.uniform(-1.15 * boundary, 1.15 * boundary, size=(n, 3))
    rad = rng.uniform(0.2, 1.6, size=(n, 1))
    sph = np.concatenate([pos, rad], axis=1).astype(np.float32)
    ref = reference_sphere_pairs(sph, cell, boundary, grid)
    assert len(ref) > 100
    ctx = engine.Context(0)
    br = engine.Broad(ctx, n)
    pairs, count = br.run_spheres(torch.from_numpy(sph).cuda(), cell, boundary, grid, max_pairs=4 * len(ref))
    ctx.synchronize()
    assert count == len(ref)
    assert np.array_equal(pairs.cpu().numpy(), ref)  # both sorted by (i, j)
