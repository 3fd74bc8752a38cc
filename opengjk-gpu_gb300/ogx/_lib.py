"""ctypes loader of the engine's C ABI (``libogx.so``, declared in include/ogx.h).

The library is the only compute path: if it cannot be loaded, or no usable GPU is
present, every call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIB_PATH

OGX_OK = 0
ERRORS = {
    -1: "OGX_ERR_INVALID",
    -2: "OGX_ERR_CUDA",
    -3: "OGX_ERR_NOMEM",
    -4: "OGX_ERR_NO_DEVICE",
    -5: "OGX_ERR_CAPACITY",
    -6: "OGX_ERR_BUSY",
}
ERR_BUSY = -6
ERR_CAPACITY = -5

FLAG_FP64_ESCALATE = 1
FLAG_FP64_POLISH = 2
FLAG_REFERENCE_TOL = 4

# per-pair status bits
PAIR_GJK_CAP = 1
PAIR_GJK_ESCALATED = 2
PAIR_POLISHED = 4
PAIR_EPA_RUN = 8
PAIR_EPA_CONVERGED = 16
PAIR_EPA_DUPLICATE = 32
PAIR_EPA_CAP = 64
PAIR_EPA_TOUCH = 128
PAIR_EPA_TOPOLOGY = 256
PAIR_EPA_CAPACITY = 512
PAIR_EPA_ESCALATED = 1024
PAIR_EPA_CERTIFIED = 2048
PAIR_BAD_INPUT = 16384

# gkSimplex, FP32 layout of the reference (GJK/common.h:84-89): 108 bytes
SIMPLEX_DTYPE = np.dtype([
    ("nvrtx", "<i4"),
    ("vrtx", "<f4", (4, 3)),
    ("vrtx_idx", "<i4", (4, 2)),
    ("witnesses", "<f4", (2, 3)),
])
assert SIMPLEX_DTYPE.itemsize == 108

# gkPolytope (GJK/common.h:68-78) on LP64: 32 bytes
POLYTOPE_DTYPE = np.dtype({
    "names": ["numpoints", "s", "s_idx", "coord"],
    "formats": ["<i4", ("<f4", (3,)), "<i4", "<u8"],
    "offsets": [0, 4, 16, 24],
    "itemsize": 32,
})


class OgxError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{ERRORS.get(status, status)}: {message}")
        self.status = status


class BodyState(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("pos", "quat", "vel", "ang", "inv_mass", "inv_inertia")]


class ResponseParams(ctypes.Structure):
    _fields_ = [("contact_eps", ctypes.c_float), ("baumgarte", ctypes.c_float), ("restitution", ctypes.c_float),
                ("restitution_threshold", ctypes.c_float)]


class Config(ctypes.Structure):
    _fields_ = [
        ("gjk_eps_rel", ctypes.c_float),
        ("gjk_eps_tot", ctypes.c_float),
        ("gjk_noise", ctypes.c_float),
        ("gjk_max_iter", ctypes.c_int),
        ("epa_tol", ctypes.c_float),
        ("epa_rel", ctypes.c_float),
        ("epa_vis", ctypes.c_float),
        ("epa_max_iter", ctypes.c_int),
        ("flags", ctypes.c_int),
        ("polish_rel", ctypes.c_float),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_P = ctypes.c_void_p
_I = ctypes.c_int
# name -> (restype, argtypes)
SIGNATURES = {
    "ogx_config_default": (_I, [_P]),
    "ogx_config_reference": (_I, [_P]),
    "ogx_status_string": (ctypes.c_char_p, [_I]),
    "ogx_last_error": (ctypes.c_char_p, []),
    "ogx_version": (ctypes.c_char_p, []),
    "ogx_ctx_create": (_I, [_I, _P, _P, _P]),
    "ogx_ctx_destroy": (_I, [_P]),
    "ogx_ctx_set_config": (_I, [_P, _P]),
    "ogx_ctx_get_config": (_I, [_P, _P]),
    "ogx_ctx_set_stream": (_I, [_P, _P]),
    "ogx_ctx_stream": (_P, [_P]),
    "ogx_ctx_synchronize": (_I, [_P]),
    "ogx_ctx_last_launches": (_I, [_P]),
    "ogx_ctx_set_timing": (_I, [_P, _I]),
    "ogx_ctx_kernel_times": (_I, [_P, _P, _P, _I]),
    "ogx_ctx_set_stage_timeline": (_I, [_P, _I]),
    "ogx_ctx_stage_timeline": (_I, [_P, _P, _P, _I]),
    "ogx_ctx_work_counts": (_I, [_P, _P, _I]),
    "ogx_ctx_get_kernel_choice": (_I, [_P, _I, _I, _P, _P]),
    "ogx_ctx_set_kernel_choice": (_I, [_P, _I, _I, _I, _I]),
    "ogx_autotune": (_I, [_P, _P, _I, _P, _I]),
    "ogx_pool_create": (_I, [_P, _I, _P, _P]),
    "ogx_pool_destroy": (_I, [_P]),
    "ogx_pool_num_bodies": (_I, [_P]),
    "ogx_pool_num_points": (ctypes.c_int64, [_P]),
    "ogx_pool_upload": (_I, [_P, _P, _P]),
    "ogx_pool_load_device": (_I, [_P, _P, _P]),
    "ogx_pool_device_layout": (_I, [_P, _P, _P]),
    "ogx_gjk": (_I, [_P, _P, _I, _P, _P, _P, _P]),
    "ogx_gjk_epa": (_I, [_P, _P, _I, _P, _P, _P, _P, _P]),
    "ogx_epa": (_I, [_P, _P, _I, _P, _P, _P, _P, _P]),
    "ogx_broad_create": (_I, [_P, _I, _P]),
    "ogx_broadphase": (_I, [_P, _P, ctypes.c_float, ctypes.c_float, _I, _P, _P]),
    "ogx_broadphase_spheres": (_I, [_P, _P, _I, ctypes.c_float, ctypes.c_float, _I, _I, _P, _P]),
    "ogx_broad_destroy": (_I, [_P]),
    "ogx_gjk_epa_streamed": (_I, [_P, _P, _P, _I, _P, _P, _P, _P, _P, _I]),
    "ogx_gjk_epa_streamed_ranges": (_I, [_P, _P, _P, _I, _P, _P, _P, _P, _P, _P, _I, _I]),
    "ogx_ctx_stream_timeline": (_I, [_P, _P, _I]),
    "ogx_contact_response": (_I, [_P, _I, _P, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "ogx_expand_submesh_pairs": (_I, [_P, _I, _P, _I, _P, _P, _I, _P, _P, _P]),
    "ogx_reduce_submesh_pairs": (_I, [_P, _I, _P, _I, _P, _P, _P]),
    "ogx_graph_create": (_I, [_P, _P, _I, _P, _P, _P, _P, _P, _I, _P]),
    "ogx_graph_launch": (_I, [_P]),
    "ogx_graph_kernel_launches": (_I, [_P]),
    "ogx_graph_destroy": (_I, [_P]),
}

_lib = None


def load(path: str | None = None):
    """Load libogx.so (build it first with ogx.build.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OgxError(-4, f"engine library not built: {path} is missing (run ogx.build.build())")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _lib = lib
    return lib


def check(status: int):
    if status != OGX_OK:
        msg = load().ogx_last_error()
        raise OgxError(status, msg.decode() if msg else "")
    return status


def default_config() -> Config:
    c = Config()
    check(load().ogx_config_default(ctypes.byref(c)))
    return c


def reference_config() -> Config:
    c = Config()
    check(load().ogx_config_reference(ctypes.byref(c)))
    return c
