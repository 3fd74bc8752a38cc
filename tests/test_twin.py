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
