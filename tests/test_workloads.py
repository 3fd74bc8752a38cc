import numpy as np

from ogx import pool as P
from ogx import workloads as W


def test_seeded_and_shaped():
    a = W.ellipsoid(seed=1, n_pairs=2000)
    b = W.ellipsoid(seed=1, n_pairs=2000)
    assert np.array_equal(a.coords, b.coords)
    assert a.counts.min() >= 8 and a.counts.max() <= 256
    c = W.powerlaw(seed=1, n_pairs=20000)
    assert c.counts.min() >= 4 and c.counts.max() <= 1024
    assert 55 < c.counts.mean() < 75  # E[n] = 64 for p(n) ~ n^-1.5 on [4, 1024]
    p = W.plain(seed=1, n_pairs=100)
    assert np.all(p.counts == 32)
    assert np.abs(p.coords).max() <= 7.0  # centres in [-5, 5]^3, radius <= 2


def test_about_half_overlap(orc):
    for gen in (W.ellipsoid, W.powerlaw):
        b = gen(seed=7, n_pairs=6000)
        o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK, precision="f64", threads=8)
        frac = np.mean(o["nvrtx"] == 4)
        assert 0.44 < frac < 0.56, frac


def test_stress_gaps_are_exact(orc):
    b = W.stress(seed=2, n_pairs=300)
    kind, gap = b.meta["kind"], b.meta["gap"]
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK, precision="f64")
    sel = kind == 0  # near-touching ellipsoids: distance is the drawn gap up to FP32 rounding
    assert np.all(np.abs(o["dist"][sel] - gap[sel]) <= 2e-6)


def test_pool_layout():
    b = W.from_bodies([np.arange(15, dtype=np.float32).reshape(5, 3), np.ones((2, 3), np.float32)])
    pool, quad = P.pack(b.coords, b.counts)
    assert quad.tolist() == [0, 6]
    x = pool[0:8]
    assert x.tolist() == [0, 3, 6, 9, 12, 0, 0, 0]      # padding repeats point 0
    assert pool[8:16].tolist() == [1, 4, 7, 10, 13, 1, 1, 1]
    assert pool[24:28].tolist() == [1, 1, 1, 1]


def test_serving_scene():
    sc = W.serving_scene(seed=3, n_bodies=500)
    assert sc.counts.min() >= 8 and sc.counts.max() <= 512
    R, p = sc.poses(7)
    assert np.abs(np.einsum("bij,bkj->bik", R, R) - np.eye(3)).max() < 1e-12
    assert np.all(np.abs(p) <= sc.half + 1e-9)
    xf = sc.transforms(7)
    assert xf.shape == (500, 12) and xf.dtype == np.float32
    w = sc.world(xf)
    # the world formula in float64, one rounding
    b = np.repeat(np.arange(500), sc.counts)
    m = xf.astype(np.float64)[b]
    x = sc.local.astype(np.float64)
    ref = ((m[:, 0] * x[:, 0] + m[:, 1] * x[:, 1]) + m[:, 2] * x[:, 2]) + m[:, 9]
    assert np.array_equal(w[:, 0], ref.astype(np.float32))
    pairs = sc.candidate_pairs(7, 1500)
    assert pairs.shape == (1500, 2) and np.all(pairs[:, 0] < pairs[:, 1])
    assert len({tuple(q) for q in pairs}) == 1500
    sizes = W.tick_sizes(1, 1000)
    assert sizes.min() >= 1000 and sizes.max() <= 200_000
    t = W.poisson_arrivals(1, 20000, 500.0)
    assert abs(np.diff(t).mean() - 1 / 500.0) < 1e-4
