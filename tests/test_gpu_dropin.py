"""The drop-in as a caller of the reference uses it: C++ programs written against the
reference's headers (include "examples/gpu/example.h", "GJK/common.h"), built with g++
against include/compat + libogx.so in both precisions, run on the GPU.

tests/dropin/known_answers.cpp reproduces the reference's two usage examples -- the GJK
distance and witnesses of examples/usage/userP.dat / userQ.dat (README.md:111-115) and
the EPA depth, witnesses and normal of a unit cube against the cube rotated 45 degrees
about x, y and z (README.md:131-137) -- and runs the facade's EPA checks;
tests/dropin/api_crosscheck.cpp checks the high-level, indexed, indexed-device and fused
calls against each other and calls made from four host threads at once."""
import os
import re
import subprocess

import numpy as np
import pytest

from ogx import workloads as W

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = [f"-I{os.path.join(ROOT, 'include', 'compat')}", f"-I{os.path.join(ROOT, 'include')}"]
PRECISIONS = {"fp32": [], "fp64": ["-DOGX_GKFLOAT_DOUBLE"]}


def _build(tmp_path, name, prec):
    from ogx import build
    libdir = os.path.dirname(build.build())
    exe = str(tmp_path / f"{name}_{prec}")
    r = subprocess.run(["g++", "-std=c++17", "-O2", *PRECISIONS[prec], *INC,
                        os.path.join(ROOT, "tests", "dropin", f"{name}.cpp"), f"-L{libdir}", "-logx",
                        f"-Wl,-rpath,{libdir}", "-pthread", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


def _write_body(path, pts):
    pts = np.asarray(pts, np.float64).reshape(-1, 3)
    with open(path, "w") as f:
        f.write(f"{len(pts)}\n")
        for p in pts:
            f.write(f"{p[0]:.9g} {p[1]:.9g} {p[2]:.9g}\n")


def _numbers(line):
    return [float(x) for x in re.findall(r"-?\d+\.\d+", line)]


@pytest.mark.parametrize("prec", sorted(PRECISIONS))
def test_usage_known_answers(tmp_path, engine, prec):
    z = np.load(os.path.join(ROOT, "tests", "golden", "usage_gjk.npz"))
    P = z["coords"][z["offsets"][0]:z["offsets"][0] + z["counts"][0]]
    Q = z["coords"][z["offsets"][1]:z["offsets"][1] + z["counts"][1]]
    files = [str(tmp_path / f) for f in ("P.txt", "Q.txt", "cube.txt", "rot.txt")]
    for f, pts in zip(files, (P, Q, W.cube(), W.rotated_cube())):
        _write_body(f, pts)
    r = subprocess.run([_build(tmp_path, "known_answers", prec), *files], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = r.stdout.splitlines()
    # README.md:111-115, printed with %f as the reference's example prints them
    assert out[0] == "Distance between bodies 3.653650", out
    assert out[1] == "Witnesses: (1.025173, 1.490318, 0.255463) and (-1.025173, -1.490318, -0.255463)", out
    # README.md:131-137 (the reference's FP32 build does not reach these; the FP64 oracle
    # and this engine do): depth 1.5 along +x
    depth = _numbers(out[2])[0]
    w1, w2, n = _numbers(out[3]), _numbers(out[4]), _numbers(out[5])
    assert abs(depth - 1.5) < 1e-4, out
    assert np.allclose(w1, [1.0, 0.5, 0.707107], atol=1e-4), out
    assert np.allclose(w2, [-0.5, 0.5, 0.707107], atol=1e-4), out
    assert np.allclose(n, [1.0, 0.0, 0.0], atol=1e-4), out
    assert "EPA tests: 4 of 4 passed" in r.stdout, r.stdout


@pytest.mark.parametrize("prec", sorted(PRECISIONS))
def test_api_crosscheck(tmp_path, engine, prec):
    r = subprocess.run([_build(tmp_path, "api_crosscheck", prec)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0 and "FAIL" not in r.stdout and "0 failure(s)" in r.stdout, r.stdout + r.stderr
    assert r.stdout.count("PASS") >= (8 if prec == "fp32" else 7)
