"""Parity at the benchmark's full sizes: the 1M-pair power-law batch (vertex counts
p(n) ~ n^-1.5 on [4, 1024]) and the 100k-pair ellipsoid batch (log-uniform 8-256), every
pair against the FP64 oracle under the rules of tests/parity.py, and every pair's
witnesses certified on its own: for a contact, w0 - w1 = depth * n and both witnesses on
their bodies' supporting planes normal to n; for a separated pair, |w1 - w0| = d and both
witnesses on the supporting planes normal to the distance vector.  Plus determinism and
batch independence at that size."""
import os

import numpy as np
import pytest

import parity
from ogx import workloads as W

pytestmark = pytest.mark.gpu

ABS4 = parity.ABS4


def support_extremes(b, rows, n, chunk=100_000):
    """max over body A of <a, n> and min over body B of <b, n> (FP64) for pairs `rows`."""
    hi = np.empty(len(rows))
    lo = np.empty(len(rows))
    for s in range(0, len(rows), chunk):
        r = rows[s:s + chunk]
        nn = n[s:s + chunk]
        for col, out, red in ((0, hi, np.maximum), (1, lo, np.minimum)):
            bodies = b.pairs[r, col]
            cnt = b.counts[bodies].astype(np.int64)
            first = np.cumsum(cnt) - cnt
            pts = np.repeat(b.offsets[bodies].astype(np.int64), cnt) + (np.arange(cnt.sum()) - np.repeat(first, cnt))
            dots = np.einsum("ij,ij->i", b.coords[pts].astype(np.float64), np.repeat(nn, cnt, axis=0))
            out[s:s + chunk] = red.reduceat(dots, first)
    return hi, lo


def certify_witnesses(b, res, o):
    """Counts of pairs whose witnesses fail the invariants above."""
    d = res["dist"].astype(np.float64)
    w = res["simplex"]["witnesses"].astype(np.float64)
    col = (res["status"] & 8) != 0
    out = {}
    c = np.flatnonzero(col)
    n = res["normal"][c].astype(np.float64)
    depth = -d[c]
    incons = np.linalg.norm((w[c, 0] - w[c, 1]) - depth[:, None] * n, axis=1)
    hi, lo = support_extremes(b, c, n)
    ga = np.einsum("ij,ij->i", w[c, 0], n) - hi
    gb = lo - np.einsum("ij,ij->i", w[c, 1], n)
    out["contacts"] = int(c.size)
    out["contact_inconsistent"] = int(np.sum(incons > ABS4 * np.maximum(1.0, depth)))
    out["contact_off_support"] = int(np.sum((np.abs(ga) > ABS4) | (np.abs(gb) > ABS4)))
    # separated pairs outside the contact band; the distance vector's direction is the
    # engine's normal (computed from the closest point -v itself, so it resolves tiny
    # distances, which the difference of two FP32 witnesses does not)
    band = np.abs(o["dist"]) <= parity.BAND * parity.pair_scale(b)
    s = np.flatnonzero(~col & ~band & (o["epa_exit"] <= 0))
    dirn = res["normal"][s].astype(np.float64)
    dirn /= np.maximum(np.linalg.norm(dirn, axis=1, keepdims=True), 1e-300)
    length = np.abs(np.linalg.norm(w[s, 1] - w[s, 0], axis=1) - d[s])
    hi, lo = support_extremes(b, s, dirn)
    ga = np.einsum("ij,ij->i", w[s, 0], dirn) - hi
    gb = lo - np.einsum("ij,ij->i", w[s, 1], dirn)
    out["separated"] = int(s.size)
    out["sep_length_off"] = int(np.sum(length > ABS4 * np.maximum(1.0, d[s])))
    out["sep_off_support"] = int(np.sum((np.abs(ga) > ABS4) | (np.abs(gb) > ABS4)))
    return out


@pytest.mark.parametrize("name", ["powerlaw_1M", "ellipsoid_100k"])
def test_full_size_parity(engine, orc, name):
    if name == "powerlaw_1M":
        b = W.powerlaw(seed=1000, n_pairs=1_000_000)  # the benchmark's own batch
    else:
        b = W.ellipsoid(seed=2, n_pairs=100_000)
    res = engine.query(b, engine.MODE_GJK_EPA)
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64",
                threads=os.cpu_count() or 1)
    rep = parity.check(b, res, o, label=name, witness_sample=5000)
    cert = certify_witnesses(b, res, o)
    print(f"\n{name}: {rep}\n{name} witnesses: {cert}")
    out_dir = os.environ.get("OGX_PARITY_REPORT_DIR")
    if out_dir:  # the report of this run, for the measurement summaries
        import json
        os.makedirs(out_dir, exist_ok=True)
        with open(os.path.join(out_dir, f"parity_{name}.json"), "w") as f:
            json.dump({"workload": name, "report": rep, "witness_certificates": cert}, f, indent=1)
    parity.assert_parity(rep, max_witness_mismatch_frac=2e-3)
    assert cert["contact_inconsistent"] == 0 and cert["contact_off_support"] == 0, cert
    assert cert["sep_length_off"] == 0 and cert["sep_off_support"] == 0, cert
    # the same batch again, and a random tenth of it alone: identical bits
    again = engine.query(b, engine.MODE_GJK_EPA)
    for k in ("dist", "normal", "status"):
        assert np.array_equal(res[k], again[k]), k
    sub = np.sort(np.random.default_rng(5).choice(b.n_pairs, b.n_pairs // 10, replace=False))
    part = engine.query(b.subset(sub), engine.MODE_GJK_EPA)
    assert np.array_equal(part["dist"], res["dist"][sub])
    assert np.array_equal(part["normal"], res["normal"][sub])
    assert np.array_equal(part["simplex"]["witnesses"], res["simplex"]["witnesses"][sub])
