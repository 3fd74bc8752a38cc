"""The drop-in headers as a caller of the reference uses them (builds only; no GPU here).

include/opengjk_gpu.hpp compiles on its own in both precisions; the test callers in
tests/dropin/ build against include/compat + libogx.so; and where the reference's sources
are present, its own unmodified callers -- examples/usage/GJKUsage.c,
examples/usage/EPAUsage.cpp and examples/main.cpp (with the reference's CPU code for its
GJK::CPU half) -- compile and link against the drop-in instead of the reference's GPU
library.  Two portability slips of those files under g++ on Linux are met by a prelude
that changes no line of them: EPAUsage.cpp names a variable M_PI, which glibc's math.h
defines as a macro (the prelude undefines it after including math.h), and main.cpp calls
memcpy without including string.h (the prelude includes it)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = [f"-I{os.path.join(ROOT, 'include', 'compat')}", f"-I{os.path.join(ROOT, 'include')}"]
REF = os.environ.get("REFERENCE_DIR", os.path.normpath(os.path.join(ROOT, "..", "reference")))
PRECISIONS = {"fp32": [], "fp64": ["-DOGX_GKFLOAT_DOUBLE"]}


@pytest.fixture(scope="module")
def libdir():
    from ogx import build
    return os.path.dirname(build.build())


def _gxx(args, cwd):
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wno-unused-but-set-variable", *args],
                       cwd=cwd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


@pytest.mark.parametrize("prec", sorted(PRECISIONS))
def test_shim_header_compiles_alone(tmp_path, prec):
    src = tmp_path / "one.cpp"
    src.write_text('#include "opengjk_gpu.hpp"\nint main() { return sizeof(gkSimplex) > 0 ? 0 : 1; }\n')
    _gxx([*PRECISIONS[prec], *INC, "-fsyntax-only", str(src)], tmp_path)


@pytest.mark.parametrize("prec", sorted(PRECISIONS))
def test_dropin_callers_build(tmp_path, libdir, prec):
    for name in ("known_answers", "api_crosscheck"):
        _gxx([*PRECISIONS[prec], *INC, os.path.join(ROOT, "tests", "dropin", f"{name}.cpp"), f"-L{libdir}",
              "-logx", "-pthread", "-o", str(tmp_path / name)], tmp_path)


def _prelude(tmp_path):
    p = tmp_path / "prelude.h"
    p.write_text("#include <math.h>\n#include <string.h>\n#undef M_PI\n")
    return ["-include", str(p)]


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "examples", "usage", "GJKUsage.c")),
                    reason="the reference's sources are not present")
@pytest.mark.parametrize("prec", sorted(PRECISIONS))
def test_reference_usage_examples_build(tmp_path, libdir, prec):
    for src in ("GJKUsage.c", "EPAUsage.cpp"):
        _gxx(["-x", "c++", *_prelude(tmp_path), *PRECISIONS[prec], *INC,
              os.path.join(REF, "examples", "usage", src), "-x", "none", f"-L{libdir}", "-logx",
              "-o", str(tmp_path / src.split(".")[0])], tmp_path)


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "examples", "main.cpp")),
                    reason="the reference's sources are not present")
def test_reference_driver_builds(tmp_path, libdir):
    cuda_inc = "/usr/local/cuda/include"
    cuda_lib = "/usr/local/cuda/lib64"
    if not os.path.isdir(cuda_inc) or shutil.which("g++") is None:
        pytest.skip("CUDA headers not present")
    objs = []
    # the reference's CPU half (GJK::CPU), compiled where it lies, for the driver's link
    for src in ("examples/cpu/example.cpp", "GJK/cpu/openGJK.c", "GJK/cpu/EPA.c"):
        o = str(tmp_path / (os.path.basename(src) + ".o"))
        r = subprocess.run(["g++", "-x", "c++", "-c", "-O1", "-w", "-include", "string.h", f"-I{REF}",
                            f"-I{cuda_inc}", os.path.join(REF, src), "-o", o], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        objs.append(o)
    main_o = str(tmp_path / "main.o")
    _gxx(["-x", "c++", "-c", *_prelude(tmp_path), *INC, f"-I{REF}", f"-I{cuda_inc}",
          os.path.join(REF, "examples", "main.cpp"), "-o", main_o], tmp_path)
    _gxx([main_o, *objs, f"-L{libdir}", "-logx", f"-L{cuda_lib}", "-lcudart", "-o", str(tmp_path / "driver")],
         tmp_path)
