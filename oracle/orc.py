"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only the test-suite, the smoke check and the benchmark's CPU-baseline leg use this
module.  It loads ``oracle/liborc.so`` (the restatement of the reference CPU
GJK/EPA, built from ``oracle/orc.c`` by ``make -C oracle``) and, when present,
``oracle/_ref/libref_f{32,64}.so`` (the reference's own CPU sources compiled in
place, used to check the restatement bit for bit).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc.so")
REF_DIR = os.path.join(HERE, "_ref")

MODE_GJK, MODE_GJK_EPA, MODE_EPA = 1, 2, 3

# epa_exit codes
EPA_SKIPPED, EPA_CONVERGED, EPA_DUPLICATE, EPA_ITER_CAP, EPA_TOUCH, EPA_STALLED = range(6)

RESULT_DTYPE = np.dtype(
    [
        ("dist", "<f8"),
        ("wit", "<f8", (2, 3)),
        ("normal", "<f8", (3,)),
        ("vrtx", "<f8", (4, 3)),
        ("idx", "<i4", (4, 2)),
        ("nvrtx", "<i4"),
        ("gjk_iters", "<i4"),
        ("epa_iters", "<i4"),
        ("epa_exit", "<i4"),
    ],
    align=True,
)


class _Config(ctypes.Structure):
    _fields_ = [
        ("eps_rel", ctypes.c_double),
        ("eps_tot", ctypes.c_double),
        ("gjk_max_iter", ctypes.c_int32),
        ("epa_tol", ctypes.c_double),
        ("epa_max_iter", ctypes.c_int32),
    ]


def build(force: bool = False) -> None:
    """Compile liborc.so (and the reference build when its sources are present)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "liborc.so"], check=True)


def reference_dir() -> str:
    """The reference checkout: $REFERENCE_DIR, else a sibling of this repository."""
    return os.environ.get("REFERENCE_DIR", os.path.normpath(os.path.join(HERE, "..", "..", "reference")))


def build_ref(ref_dir: str | None = None) -> bool:
    """Compile the reference's own CPU GJK/EPA into oracle/_ref (validation only)."""
    ref_dir = ref_dir or reference_dir()
    if not os.path.isdir(os.path.join(ref_dir, "GJK", "cpu")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={ref_dir}"], check=True)
    return True


_lib = None


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB_PATH)
        for name in ("orc_run_f32", "orc_run_f64"):
            fn = getattr(lib, name)
            fn.restype = ctypes.c_int
            fn.argtypes = [
                ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
            ]
        _lib = lib
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def run(coords, offsets, counts, pairs, *, mode=MODE_GJK_EPA, precision="f64", threads=1,
        eps_rel=0.0, eps_tot=0.0, gjk_max_iter=0, epa_tol=0.0, epa_max_iter=0,
        results: np.ndarray | None = None) -> np.ndarray:
    """Run the oracle over a pool of bodies and a pair list.

    coords: (P, 3) float32 points of all bodies; offsets/counts: first point and
    point count per body; pairs: (N, 2) body indices.  precision "f64" widens the
    FP32 coordinates exactly to double (the parity oracle); float64 coordinates given
    with "f64" are used as they are (inputs of FP64 callers); "f32" is the reference's
    shipped precision.  Zero tolerances select the reference constants.
    """
    lib = _load()
    given64 = precision == "f64" and np.asarray(coords).dtype == np.float64
    if given64:
        c64 = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
    coords = np.ascontiguousarray(coords, dtype=np.float32).reshape(-1, 3)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
    n = pairs.shape[0]
    if results is None:
        results = np.zeros(n, dtype=RESULT_DTYPE)
    cfg = _Config(eps_rel, eps_tot, gjk_max_iter, epa_tol, epa_max_iter)
    if precision == "f64":
        c = c64 if given64 else coords.astype(np.float64)
        fn = lib.orc_run_f64
    elif precision == "f32":
        c = coords
        fn = lib.orc_run_f32
    else:
        raise ValueError(precision)
    rc = fn(n, _ptr(c), _ptr(offsets), _ptr(counts), _ptr(pairs), mode, ctypes.addressof(cfg),
            _ptr(results), int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle returned {rc}")
    return results


_ref_libs: dict = {}


def ref_available() -> bool:
    return all(os.path.exists(os.path.join(REF_DIR, f"libref_{p}.so")) for p in ("f32", "f64"))


def run_reference(coords, offsets, counts, pairs, *, mode=MODE_GJK_EPA, precision="f64",
                  results: np.ndarray | None = None) -> np.ndarray:
    """Run the reference's own CPU GJK/EPA (compiled into oracle/_ref)."""
    if precision not in _ref_libs:
        lib = ctypes.CDLL(os.path.join(REF_DIR, f"libref_{precision}.so"))
        lib.ref_run.restype = ctypes.c_int
        lib.ref_run.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_void_p]
        _ref_libs[precision] = lib
    lib = _ref_libs[precision]
    coords = np.ascontiguousarray(coords, dtype=np.float32).reshape(-1, 3)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
    n = pairs.shape[0]
    if results is None:
        results = np.zeros(n, dtype=RESULT_DTYPE)
    c = coords.astype(np.float64) if precision == "f64" else coords
    rc = lib.ref_run(n, _ptr(c), _ptr(offsets), _ptr(counts), _ptr(pairs), mode, _ptr(results))
    if rc != 0:
        raise RuntimeError(f"reference returned {rc}")
    return results
