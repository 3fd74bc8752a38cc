"""ogx -- batched GJK distance and EPA penetration on GB300 (sm_103a).

Host side of the engine: ``build`` compiles libogx.so, ``engine`` wraps the C ABI
(contexts, device pools, batched queries), ``refapi`` mirrors the reference's
GJK::GPU / openGJK.h host API on top of it, ``workloads`` generates seeded inputs.
"""
from . import _lib, build, pool, workloads  # noqa: F401
from ._lib import OgxError, SIMPLEX_DTYPE, POLYTOPE_DTYPE, default_config, reference_config  # noqa: F401

__all__ = ["OgxError", "SIMPLEX_DTYPE", "POLYTOPE_DTYPE", "default_config", "reference_config",
           "build", "pool", "workloads"]
