"""GPU engine (through the C ABI) against the FP64 oracle and the host build of the
same per-pair code.  Tolerances: tests/parity.py."""
import numpy as np
import pytest

import parity
from ogx import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = ["set_plain", "set_ellipsoid", "set_powerlaw"]


def _golden(name):
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz"))
    b = W.Batch(z["coords"], z["offsets"], z["counts"], z["pairs"], name)
    o = np.zeros(b.n_pairs, dtype=__import__("oracle.orc", fromlist=["x"]).RESULT_DTYPE)
    for f in o.dtype.names:
        o[f] = z[f"f64_{f}"]
    return b, o


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_sets(engine, name):
    b, o = _golden(name)
    res = engine.query(b, engine.MODE_GJK_EPA)
    rep = parity.check(b, res, o, label=name)
    parity.assert_parity(rep)


@pytest.mark.parametrize("gen,n", [(W.plain, 1000), (W.ellipsoid, 20000), (W.powerlaw, 20000)],
                         ids=["plain_1k_fp64cfg", "ellipsoid_20k", "powerlaw_20k"])
def test_workloads_vs_oracle(engine, orc, gen, n):
    b = gen(n_pairs=n)
    res = engine.query(b, engine.MODE_GJK_EPA)
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64", threads=16)
    rep = parity.check(b, res, o, label=b.name)
    print(rep)
    parity.assert_parity(rep, max_witness_mismatch_frac=2e-3)


def test_gpu_matches_host_build(engine, twin):
    """Same per-pair code on the GPU (teams of 4-32 lanes) and on the CPU (one lane):
    identical arithmetic, so results agree to the last bit except for rare ties."""
    b = W.powerlaw(seed=21, n_pairs=5000)
    g = engine.query(b, engine.MODE_GJK_EPA)
    h = twin.run(b)
    same_d = g["dist"] == h["dist"]
    assert same_d.mean() > 0.995, same_d.mean()
    close = np.abs(g["dist"].astype(np.float64) - h["dist"]) <= 1e-6 * np.maximum(1, np.abs(h["dist"]))
    assert close.mean() > 0.999


def test_gjk_only_mode(engine, orc):
    b = W.ellipsoid(seed=22, n_pairs=3000)
    res = engine.query(b, engine.MODE_GJK)
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK, precision="f64")
    sep = (o["nvrtx"] < 4) & (o["dist"] > 1e-4)
    d = res["dist"].astype(np.float64)
    rel = np.abs(d[sep] - o["dist"][sep]) / o["dist"][sep]
    assert rel.max() <= parity.REL
    enclosed = o["nvrtx"] == 4
    assert np.all(res["simplex"]["nvrtx"][enclosed] == 4)
    assert np.all(d[enclosed] == 0.0)


def _variant_columns(ctx):
    """For each bucket, the (lanes, blocks) variants the library accepts for it."""
    from ogx import _lib
    cols = {"gjk": [[] for _ in range(7)], "epa": [[] for _ in range(7)]}
    for kind in ("gjk", "epa"):
        for b in range(7):
            for L in (1, 2, 4, 8, 16, 32):
                for K in (0, 1, 2, 4, 4 << 8, 5 << 8, 1 + (5 << 8), 2 + (5 << 8), 2 + (4 << 8),
                          (4 << 8) + (2 << 16), (4 << 8) + (3 << 16), (4 << 8) + (4 << 16),
                          (4 << 8) + (8 << 16)):
                    try:
                        ctx.set_kernel_choice(kind, b, L, K)
                    except _lib.OgxError:
                        continue
                    cols[kind][b].append((L, K))
    return cols


def test_every_variant_matches_host_build(engine, twin):
    """The autotuner may pick any compiled variant for a bucket: each one must give the
    host build's results (ranked slot order makes EPA independent of the team width)."""
    import torch
    b = W.powerlaw(seed=23, n_pairs=6000)
    h = twin.run(b)
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, b.counts)
    pool.upload(b.coords)
    pairs = torch.from_numpy(np.ascontiguousarray(b.pairs)).cuda()
    cols = _variant_columns(ctx)
    width = max(len(c) for kind in cols.values() for c in kind)
    tried = set()
    for i in range(width):
        for kind in ("gjk", "epa"):
            for bk in range(7):
                c = cols[kind][bk]
                if c:
                    L, K = c[min(i, len(c) - 1)]
                    ctx.set_kernel_choice(kind, bk, L, K)
                    tried.add((kind, bk, L, K))
        g = engine.run(ctx, pool, pairs, engine.MODE_GJK_EPA).to_host()
        same = g["dist"] == h["dist"]
        assert same.mean() > 0.995, (i, ctx.kernel_choice(), same.mean())
        close = np.abs(g["dist"].astype(np.float64) - h["dist"]) <= 1e-6 * np.maximum(1, np.abs(h["dist"]))
        assert close.mean() > 0.999, (i, ctx.kernel_choice())
    assert len(tried) >= 20


def _stress_report(b, res, o):
    """Per-kind, per-output errors of the engine against the FP64 oracle on the stress
    workload (kind 0 near-touching ellipsoids, 1 boxes face to face, 2 boxes edge to
    edge, 3 thin near-coplanar disks)."""
    out = {}
    names = {0: "near_touching_ellipsoids", 1: "boxes_face", 2: "boxes_edge", 3: "thin_disks"}
    kind = b.meta["kind"]
    for k, name in names.items():
        s = np.flatnonzero(kind == k)
        sub = b.subset(s)
        rr = {key: res[key][s] for key in ("dist", "simplex", "normal", "status")}
        rep = parity.check(sub, rr, o[s], label=name)
        # normals that miss the oracle's: the depth along them against the oracle's depth
        d, d64 = rr["dist"].astype(np.float64), o["dist"][s]
        both = (d < 0) & (d64 < 0) & (np.abs(d64) > parity.BAND * parity.pair_scale(sub))
        nerr = np.linalg.norm(rr["normal"][both].astype(np.float64) - o["normal"][s][both], axis=1)
        rep["normal_within_1e-4_frac"] = float(np.mean(nerr <= parity.ABS4)) if nerr.size else 1.0
        gaps = []
        for i in np.flatnonzero(both)[nerr > parity.ABS4]:
            A, B = sub.body(sub.pairs[i, 0]).astype(np.float64), sub.body(sub.pairs[i, 1]).astype(np.float64)
            n = rr["normal"][i].astype(np.float64)
            n /= np.linalg.norm(n)
            gaps.append((A @ n).max() - (B @ n).min() + d64[i])
        rep["other_normal_depth_excess_max"] = float(max(gaps)) if gaps else 0.0
        out[name] = rep
    return out


def test_stress_200k_error_report(engine, orc):
    """Mixed-precision stress set at its full size (200k pairs): error of every output
    against the FP64 oracle, per kind, and every parity rule for every kind -- the
    1e-4-thick near-coplanar disks included: a thin contact's FP32 convergence is checked
    with exact supports along its face's FP64 plane, and a face hop to a neighbour more
    than 1e-5 rad off is refused by the FP32 pass, which runs the contact again certified
    (the report gives how far the depth along each normal that differs from the oracle's
    is from the oracle's depth)."""
    import json
    import os
    b = W.stress(seed=9, n_pairs=200_000)
    res = engine.query(b, engine.MODE_GJK_EPA)
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64", threads=16)
    rep = _stress_report(b, res, o)
    print("STRESS_REPORT " + json.dumps(rep))
    out_dir = os.environ.get("OGX_PARITY_REPORT_DIR")
    if out_dir:  # the report of this run, for the measurement summaries
        os.makedirs(out_dir, exist_ok=True)
        with open(os.path.join(out_dir, "parity_stress_200k.json"), "w") as f:
            json.dump({"workload": "stress_200k", "report": rep}, f, indent=1)
    for name, r in rep.items():
        assert r["verdict_mismatch"] == 0 and r["band_abs_violations"] == 0, (name, r)
        assert r["sep_rel_violations"] == 0, (name, r)
        parity.assert_parity(r, max_witness_mismatch_frac=2e-3)
