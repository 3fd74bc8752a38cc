"""The CPU oracle: pinned to the reference's golden vectors and known answers, and
(where the reference sources are present) bit-identical to the reference's own build."""
import json
import os

import numpy as np
import pytest

from ogx import workloads as W

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FIELDS = ("dist", "wit", "normal", "vrtx", "idx", "nvrtx")


def load_set(name):
    z = np.load(os.path.join(GOLD, f"{name}.npz"))
    b = W.Batch(z["coords"], z["offsets"], z["counts"], z["pairs"], name)
    return b, z


def same(x, y):
    if x.dtype.kind == "f":
        return np.all((x == y) | (np.isnan(x) & np.isnan(y)))
    return np.all(x == y)


@pytest.mark.parametrize("name", ["usage_gjk", "usage_epa", "set_plain", "set_ellipsoid",
                                  "set_powerlaw", "set_stress"])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_matches_golden(orc, name, prec):
    b, z = load_set(name)
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision=prec)
    for f in FIELDS:
        assert same(o[f], z[f"{prec}_{f}"]), f


def test_golden_fixtures_were_checked_against_reference_build():
    with open(os.path.join(GOLD, "manifest.json")) as f:
        m = json.load(f)
    assert len(m["checked_bit_identical_to_reference_build"]) == 12


def test_gjk_known_answer(orc):
    """examples/usage/userP.dat / userQ.dat: README.md:113-114 prints
    distance 3.653650, witnesses (1.025173, 1.490318, 0.255463) and the negation."""
    b, _ = load_set("usage_gjk")
    for prec in ("f32", "f64"):
        o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK, precision=prec)
        assert f"{o['dist'][0]:.6f}" == "3.653650"
        assert [f"{x:.6f}" for x in o["wit"][0, 0]] == ["1.025173", "1.490318", "0.255463"]
        assert [f"{x:.6f}" for x in o["wit"][0, 1]] == ["-1.025173", "-1.490318", "-0.255463"]


def test_epa_known_answer(orc):
    """Cube vs cube rotated 45 deg about x, y, z and shifted +1 in x
    (examples/usage/EPAUsage.cpp): README.md:133-136 prints depth 1.500000, witnesses
    (1, 0.5, 0.707107) / (-0.5, 0.5, 0.707107), normal (1, -0, 0).  The FP64 oracle
    reproduces it; the FP32 CPU build ends GJK with a 3-point simplex whose growth finds
    no new point, so it reports depth 0 (a property of the reference's FP32 path)."""
    b, _ = load_set("usage_epa")
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64")
    assert f"{-o['dist'][0]:.6f}" == "1.500000"
    assert [f"{x:.6f}" for x in o["wit"][0, 0]] == ["1.000000", "0.500000", "0.707107"]
    assert [f"{x:.6f}" for x in o["wit"][0, 1]] == ["-0.500000", "0.500000", "0.707107"]
    assert [f"{abs(x):.6f}" for x in o["normal"][0]] == ["1.000000", "0.000000", "0.000000"]
    o32 = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f32")
    assert abs(o32["dist"][0]) < 1e-6


def _cubes(offset, half=1.0):
    return W.from_bodies([W.cube(half), W.cube(half) + np.float32(offset)])


def test_reference_hand_cases(orc):
    """Range checks of the reference's EPATesting (examples/gpu/example.cu:385-897)."""
    # overlapping unit cubes offset by 1: depth in (0.8, 1.2)   (example.cu:450)
    o = orc.run(*_args(_cubes([1.0, 0, 0])), mode=orc.MODE_GJK_EPA, precision="f64")
    assert 0.8 < -o["dist"][0] < 1.2
    # touching: 0 <= d < 0.01                                     (example.cu:515)
    o = orc.run(*_args(_cubes([2.0, 0, 0])), mode=orc.MODE_GJK_EPA, precision="f64")
    assert 0.0 <= o["dist"][0] < 0.01
    # cubes of half-size 1 whose faces are 3 apart: 2.9 < d < 3.1, nvrtx < 4 (example.cu:580)
    o = orc.run(*_args(_cubes([5.0, 0, 0])), mode=orc.MODE_GJK_EPA, precision="f64")
    assert 2.9 < o["dist"][0] < 3.1 and o["nvrtx"][0] < 4


def _args(b):
    return b.coords, b.offsets, b.counts, b.pairs


@pytest.mark.skipif(not __import__("oracle.orc", fromlist=["x"]).ref_available(),
                    reason="reference build (oracle/_ref) not present on this machine")
@pytest.mark.parametrize("gen", [W.plain, W.ellipsoid, W.powerlaw, W.stress])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_bit_identical_to_reference_build(orc, gen, prec):
    b = gen(seed=77, n_pairs=1500)
    o = orc.run(*_args(b), mode=orc.MODE_GJK_EPA, precision=prec, threads=4)
    r = orc.run_reference(*_args(b), mode=orc.MODE_GJK_EPA, precision=prec)
    for f in FIELDS:
        assert same(o[f], r[f]), f


def test_oracle_threads_identical(orc):
    b = W.ellipsoid(seed=5, n_pairs=3000)
    a = orc.run(*_args(b), precision="f64", threads=1)
    c = orc.run(*_args(b), precision="f64", threads=8)
    for f in FIELDS:
        assert same(a[f], c[f])


def test_epa_only_mode_equals_fused(orc):
    b = W.ellipsoid(seed=6, n_pairs=500)
    fused = orc.run(*_args(b), mode=orc.MODE_GJK_EPA, precision="f64")
    g = orc.run(*_args(b), mode=orc.MODE_GJK, precision="f64")
    e = orc.run(*_args(b), mode=orc.MODE_EPA, precision="f64", results=g.copy())
    for f in FIELDS:
        assert same(fused[f], e[f]), f


def test_oracle_rejects_bad_mode(orc):
    b = W.plain(n_pairs=2)
    with pytest.raises(RuntimeError):
        orc.run(*_args(b), mode=9)
