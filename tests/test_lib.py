"""The C-ABI library: it builds for sm_103a, loads, exports every function declared in
include/*.h, and fails loudly (no CPU fallback) when no GPU is usable."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(ogx_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from ogx import build, _lib
    build.build()
    return _lib.load()


def test_builds_for_sm103a(lib):
    from ogx import build
    assert any("arch=compute_103a,code=sm_103a" in a for a in build.ARCH)
    assert os.path.exists(build.LIB_PATH)


def test_exports_every_declared_function(lib):
    decl = declared_functions()
    assert len(decl) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (ogx_\w+)", out))
    missing = [d for d in decl if d not in exported]
    assert not missing, missing


def test_config_and_status_without_gpu(lib):
    from ogx import _lib
    c = _lib.default_config()
    assert c.flags & _lib.FLAG_FP64_POLISH and c.gjk_max_iter >= 25
    r = _lib.reference_config()
    assert r.gjk_max_iter == 25 and r.epa_max_iter == 64 and r.flags == _lib.FLAG_REFERENCE_TOL
    assert lib.ogx_status_string(-1) == b"invalid argument"
    assert b"sm_103a" in lib.ogx_version()


def test_no_cpu_fallback():
    """On a machine without a usable GPU the engine refuses to run."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ogx import _lib, engine
    with pytest.raises(_lib.OgxError):
        engine.Context(0)
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.ogx_ctx_create(0, None, None, ctypes.byref(h)) == -4
