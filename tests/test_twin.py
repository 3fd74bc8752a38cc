"""The engine's per-pair GJK/EPA code (host build of the same source as the CUDA
kernels, one lane per team) against the FP64 oracle, with the tolerances of
tests/parity.py.  Checks the algorithm on a CPU-only machine; the GPU tests check the
kernels."""
import numpy as np
import pytest

import parity
from ogx import workloads as W


@pytest.mark.parametrize("gen,n", [(W.plain, 2000), (W.ellipsoid, 4000), (W.powerlaw, 4000)],
                         ids=["plain", "ellipsoid", "powerlaw"])
def test_engine_algorithm_vs_oracle(orc, twin, gen, n):
    b = gen(seed=31, n_pairs=n)
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64", threads=8)
    r = twin.run(b)
    rep = parity.check(b, r, o, label=b.name)
    parity.assert_parity(rep, max_witness_mismatch_frac=2e-3)


def test_reference_tolerances_close_to_reference_fp32(orc, twin):
    """With the reference's FP32 constants the engine agrees with the reference FP32
    CPU path within the reference's own CPU-vs-GPU tolerance (examples/main.cpp:184-188)."""
    b = W.ellipsoid(seed=32, n_pairs=3000)
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f32")
    r = twin.run(b, cfg=twin.config(reference=True))
    diff = np.abs(r["dist"] - o["dist"])
    assert np.mean(diff <= 1e-3) > 0.995


def test_default_beats_reference_fp32_accuracy(orc, twin):
    """Against the FP64 oracle, the engine's default mode is more accurate than the
    reference's FP32 path on the same inputs (the reference stops at eps*1e4)."""
    b = W.ellipsoid(seed=33, n_pairs=3000)
    o64 = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK, precision="f64")
    o32 = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK, precision="f32")
    r = twin.run(b, mode=1)
    sep = (o64["nvrtx"] < 4) & (o64["dist"] > 1e-3)
    e_ref = np.abs(o32["dist"][sep] - o64["dist"][sep]) / o64["dist"][sep]
    e_us = np.abs(r["dist"][sep] - o64["dist"][sep]) / o64["dist"][sep]
    assert e_us.max() <= 1e-5 < e_ref.max()


def test_posed_pipeline_vs_oracle(orc, twin):
    """The fused-transform pipeline (bodies in their own frame, each pose applied as the
    points are read, support scans on the direction rotated into the body frame) against
    the FP64 oracle on the same world points (pose_point of every body point), and
    against the world-frame pipeline on those points."""
    scene = W.serving_scene(seed=41, n_bodies=2000)
    xf = scene.transforms(3)
    pairs = scene.candidate_pairs(3, 6000)
    world = twin.pose_points(scene.counts, scene.local, xf)
    bw = W.Batch(world, scene.offsets, scene.counts, pairs, "serving")
    bl = W.Batch(scene.local, scene.offsets, scene.counts, pairs, "serving")
    o = orc.run(bw.coords, bw.offsets, bw.counts, bw.pairs, mode=orc.MODE_GJK_EPA, precision="f64", threads=8)
    posed = twin.run(bl, xf=xf)
    parity.assert_parity(parity.check(bw, posed, o, label="posed"), max_witness_mismatch_frac=2e-3)
    plain = twin.run(bw)
    assert np.array_equal(posed["dist"] < 0, plain["dist"] < 0)
    close = np.abs(posed["dist"].astype(np.float64) - plain["dist"]) <= 1e-5 * np.maximum(1, np.abs(plain["dist"]))
    assert close.all()
    # the posed points themselves: R p + t within FP32 rounding of the FP64 product
    body = np.repeat(np.arange(scene.n_bodies), scene.counts)
    m = xf.astype(np.float64)[body]
    p = scene.local.astype(np.float64)
    exact = np.stack([(m[:, 3 * r:3 * r + 3] * p).sum(1) + m[:, 9 + r] for r in range(3)], axis=1)
    assert np.abs(world - exact).max() <= 4e-7 * np.abs(exact).max()
