"""The reference's own GPU kernels ("plain form" baseline) -- measurement infrastructure.

The cubin `oracle/_ref/plain_form_sm103a.cubin` is the reference's GJK/gpu/openGJK.cu
(FP32 as shipped) compiled for sm_103a from the reference sources where they lie
(`make -C oracle plain`); it is not part of this repository's history and holds device
code only.  This module loads it through the CUDA driver API and launches the
reference's indexed kernels exactly as its fused indexed call does
(GJK/gpu/openGJK.cu:3274-3310): simplices zeroed, then
`compute_minimum_distance_indexed_kernel` with 256 threads per block and 8 threads per
pair (:3124-3140), then `compute_epa_kernel_indexed_kernel` with 4 pairs of 32 threads
per block and 4 x sizeof(EPAPolytope) bytes of dynamic shared memory (:3143-3160).

Used by the GPU tests (the plain form against the reference's CPU code) and by
bench.py's baseline leg; never by the engine.  Device memory comes from torch.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "plain_form_sm103a.cubin")

# mangled names of the reference's kernels (GJK/gpu/openGJK.cu:1451, :2759)
GJK_KERNEL = b"_Z39compute_minimum_distance_indexed_kernelPK10gkPolytopePK15gkCollisionPairP9gkSimplexPfi"
EPA_KERNEL = b"_Z33compute_epa_kernel_indexed_kernelPK10gkPolytopePK15gkCollisionPairP9gkSimplexPfS7_i"

# launch shapes of the reference (GJK/gpu/openGJK.cu:43-44, 53-61)
THREADS_PER_GJK = 8
GJK_BLOCK = 256
EPA_PAIRS_PER_BLOCK = 4
EPA_BLOCK = EPA_PAIRS_PER_BLOCK * 32
# sizeof(EPAPolytope) in FP32 (GJK/gpu/openGJK.cu:1486-1501): vertices 132 x 12 B,
# vertex indices 132 x 8 B, num_vertices 4 B, 128 faces of 56 B, max_face_index 4 B
EPA_POLYTOPE_BYTES = 132 * 12 + 132 * 8 + 4 + 128 * 56 + 4

# gkPolytope in FP32 (GJK/common.h:68-80): int numpoints; float s[3]; int s_idx;
# float* coord (8-byte aligned) -> 32 bytes
POLYTOPE_DTYPE = np.dtype({"names": ["numpoints", "s", "s_idx", "coord"],
                           "formats": [np.int32, (np.float32, 3), np.int32, np.uint64],
                           "offsets": [0, 4, 16, 24], "itemsize": 32})
SIMPLEX_BYTES = 108  # gkSimplex in FP32 (GJK/common.h:86-91)


def available() -> bool:
    return os.path.isfile(CUBIN)


class _Driver:
    def __init__(self):
        self.lib = ctypes.CDLL("libcuda.so.1")

    def __call__(self, name, *args):
        rc = getattr(self.lib, name)(*args)
        if rc != 0:
            msg = ctypes.c_char_p()
            self.lib.cuGetErrorString(rc, ctypes.byref(msg))
            raise RuntimeError(f"{name} failed: {rc} {msg.value.decode() if msg.value else ''}")


class PlainForm:
    """The reference's indexed GJK and EPA kernels over one resident set of bodies."""

    def __init__(self, device: int = 0):
        import torch
        if not available():
            raise FileNotFoundError(f"{CUBIN} is missing (make -C oracle plain on a host with the reference)")
        self.torch = torch
        self.device = torch.device("cuda", device)
        torch.empty(1, device=self.device)  # torch's (primary) context is current
        self.cu = _Driver()
        ctx = ctypes.c_void_p()
        self.cu("cuCtxGetCurrent", ctypes.byref(ctx))
        if not ctx.value:
            dev = ctypes.c_int()
            self.cu("cuDeviceGet", ctypes.byref(dev), device)
            self.cu("cuDevicePrimaryCtxRetain", ctypes.byref(ctx), dev)
            self.cu("cuCtxSetCurrent", ctx)
        self.module = ctypes.c_void_p()
        self.cu("cuModuleLoad", ctypes.byref(self.module), CUBIN.encode())
        self.f_gjk = ctypes.c_void_p()
        self.f_epa = ctypes.c_void_p()
        self.cu("cuModuleGetFunction", ctypes.byref(self.f_gjk), self.module, GJK_KERNEL)
        self.cu("cuModuleGetFunction", ctypes.byref(self.f_epa), self.module, EPA_KERNEL)
        self.polytopes = None
        self.coords = None

    def load(self, coords_dev, offsets: np.ndarray, counts: np.ndarray):
        """Body descriptors over device xyz `coords_dev` (float32 [P, 3], contiguous):
        body b has counts[b] points starting at point offsets[b]."""
        torch = self.torch
        assert coords_dev.dtype == torch.float32 and coords_dev.is_contiguous()
        self.coords = coords_dev
        d = np.zeros(len(counts), POLYTOPE_DTYPE)
        d["numpoints"] = counts
        d["coord"] = np.uint64(coords_dev.data_ptr()) + 12 * np.asarray(offsets[:len(counts)], np.uint64)
        host = torch.from_numpy(d.view(np.uint8).copy())
        self.polytopes = host.to(self.device)
        return self

    def run(self, pairs_dev, out: dict | None = None) -> dict:
        """GJK then EPA over `pairs_dev` (int32 [n, 2] on the device) on torch's current
        stream; returns device tensors simplex (uint8 [n, 108]), dist [n], normal [n, 3]."""
        torch = self.torch
        n = int(pairs_dev.shape[0])
        if out is None:
            out = {"simplex": torch.empty((n, SIMPLEX_BYTES), dtype=torch.uint8, device=self.device),
                   "dist": torch.empty(n, dtype=torch.float32, device=self.device),
                   "normal": torch.empty((n, 3), dtype=torch.float32, device=self.device)}
        if n == 0:
            return out
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        out["simplex"].zero_()
        P = ctypes.c_void_p
        gjk_args = [P(self.polytopes.data_ptr()), P(pairs_dev.data_ptr()), P(out["simplex"].data_ptr()),
                    P(out["dist"].data_ptr()), ctypes.c_int(n)]
        epa_args = gjk_args[:4] + [P(out["normal"].data_ptr()), ctypes.c_int(n)]
        pairs_per_block = GJK_BLOCK // THREADS_PER_GJK
        self._launch(self.f_gjk, (n + pairs_per_block - 1) // pairs_per_block, GJK_BLOCK, 0, stream, gjk_args)
        self._launch(self.f_epa, (n + EPA_PAIRS_PER_BLOCK - 1) // EPA_PAIRS_PER_BLOCK, EPA_BLOCK,
                     EPA_PAIRS_PER_BLOCK * EPA_POLYTOPE_BYTES, stream, epa_args)
        return out

    def _launch(self, f, grid, block, smem, stream, args):
        params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        self.cu("cuLaunchKernel", f, ctypes.c_uint(grid), ctypes.c_uint(1), ctypes.c_uint(1),
                ctypes.c_uint(block), ctypes.c_uint(1), ctypes.c_uint(1), ctypes.c_uint(smem), stream,
                params, None)

    def close(self):
        if self.module is not None and self.module.value:
            self.cu("cuModuleUnload", self.module)
            self.module = None
