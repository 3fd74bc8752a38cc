"""Regenerate the golden fixtures in this directory (run from the repository root).

Inputs:
  * examples/usage/userP.dat, userQ.dat of the reference (its GJK known-answer example,
    expected output in its README.md:111-115) -- read from the reference checkout;
  * the cube / rotated-cube pair of the reference's EPA example
    (examples/usage/EPAUsage.cpp:46-84, expected output README.md:131-137), rebuilt by
    ogx.workloads.cube / rotated_cube;
  * small seeded batches of every workload generator.
Outputs: the CPU oracle's FP32 and FP64 results.  When the reference's own CPU build
is present (oracle/_ref, compiled by `make -C oracle ref`), every output is first
checked to be bit-identical to it; the fixture records whether that check ran.
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "opengjk-gpu_gb300"))
from ogx import workloads as W  # noqa: E402
from oracle import orc  # noqa: E402

REF = os.environ.get("REFERENCE_DIR", os.path.normpath(os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "..", "reference")))
OUT = os.path.dirname(os.path.abspath(__file__))


def read_dat(path):
    with open(path) as f:
        n = int(f.readline())
        pts = [list(map(float, f.readline().split())) for _ in range(n)]
    return np.array(pts, dtype=np.float32)


def oracle_all(b, checked):
    res = {}
    for prec in ("f32", "f64"):
        o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision=prec)
        if orc.ref_available():
            r = orc.run_reference(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision=prec)
            for f in ("dist", "wit", "normal", "vrtx", "idx", "nvrtx"):
                x, y = o[f], r[f]
                same = (x == y) | (np.isnan(x) & np.isnan(y)) if x.dtype.kind == "f" else (x == y)
                assert np.all(same), f"oracle differs from the reference build in {f} ({b.name}, {prec})"
            checked.append(f"{b.name}/{prec}")
        res[prec] = o
    return res


def save(name, b, res, extra=None):
    arrays = dict(coords=b.coords, offsets=b.offsets, counts=b.counts, pairs=b.pairs)
    for prec, o in res.items():
        for f in o.dtype.names:
            arrays[f"{prec}_{f}"] = o[f]
    if extra:
        arrays.update(extra)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **arrays)


def main():
    orc.build()
    orc.build_ref(REF)
    checked = []
    P = read_dat(os.path.join(REF, "examples", "usage", "userP.dat"))
    Q = read_dat(os.path.join(REF, "examples", "usage", "userQ.dat"))
    b = W.from_bodies([P, Q], name="usage_gjk")
    save("usage_gjk", b, oracle_all(b, checked))
    b = W.from_bodies([W.cube(), W.rotated_cube()], name="usage_epa")
    save("usage_epa", b, oracle_all(b, checked))
    sets = [
        ("plain", W.plain(seed=101, n_pairs=100)),
        ("ellipsoid", W.ellipsoid(seed=102, n_pairs=100)),
        ("powerlaw", W.powerlaw(seed=103, n_pairs=100)),
        ("stress", W.stress(seed=104, n_pairs=90)),
    ]
    for name, b in sets:
        b.name = name
        save(f"set_{name}", b, oracle_all(b, checked))
    with open(os.path.join(OUT, "manifest.json"), "w") as f:
        json.dump({"checked_bit_identical_to_reference_build": checked,
                   "generator": "tests/golden/make_golden.py"}, f, indent=1)
    print("golden fixtures written; reference check ran for", len(checked), "sets")


if __name__ == "__main__":
    main()
