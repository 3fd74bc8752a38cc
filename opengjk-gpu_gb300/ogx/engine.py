"""Python host side of the engine API: contexts, device pools and batched queries.

Device buffers are torch CUDA tensors (torch is only the allocator and stream
provider here); every computation is a call into libogx.so.
"""
from __future__ import annotations

import atexit
import ctypes
import sys
import weakref

import numpy as np

from . import _lib
from ._lib import SIMPLEX_DTYPE, check

MODE_GJK, MODE_GJK_EPA, MODE_EPA = 1, 2, 3

# Engine objects still open at exit are closed by an atexit hook (pools, graphs and
# broad-phase objects before their contexts), while the CUDA runtime and torch are still
# intact; objects that are garbage-collected during interpreter shutdown are left to the
# process exit.  The C objects refer to their context, so a context closes its children
# first, and a child whose context is already closed is not destroyed again.
_live_pools: "weakref.WeakSet" = weakref.WeakSet()
_live_ctxs: "weakref.WeakSet" = weakref.WeakSet()


@atexit.register
def _close_all():
    for p in list(_live_pools):
        try:
            p.close()
        except Exception:
            pass
    for c in list(_live_ctxs):
        try:
            c.close()
        except Exception:
            pass


def _torch():
    import torch
    return torch


class Context:
    """One engine instance on one GPU, bound to a torch CUDA stream (default: a stream of
    its own).  `run` orders the engine's work after the caller's current torch stream and
    makes that stream wait for it, so results behave like any other torch op's."""

    def __init__(self, device: int = 0, config: _lib.Config | None = None, stream=None):
        torch = _torch()
        if not torch.cuda.is_available():
            raise _lib.OgxError(-4, "no CUDA device visible")
        self.lib = _lib.load()
        self.device = device
        torch.cuda.set_device(device)
        if stream is None or stream.cuda_stream == 0:
            # the C API reads a NULL stream as "create one"; keep the stream visible here
            stream = torch.cuda.Stream(device)
        self.stream = stream
        h = ctypes.c_void_p()
        cfgp = ctypes.byref(config) if config is not None else None
        check(self.lib.ogx_ctx_create(device, cfgp, ctypes.c_void_p(stream.cuda_stream), ctypes.byref(h)))
        self.handle = h
        _live_ctxs.add(self)

    def close(self):
        if self.handle:
            for p in list(_live_pools):  # pools, graphs, broad phases cannot outlive it
                if p.ctx is self:
                    p.close()
            self.lib.ogx_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass

    @property
    def config(self) -> _lib.Config:
        c = _lib.Config()
        check(self.lib.ogx_ctx_get_config(self.handle, ctypes.byref(c)))
        return c

    @config.setter
    def config(self, c: _lib.Config):
        check(self.lib.ogx_ctx_set_config(self.handle, ctypes.byref(c)))

    def set_stream(self, stream):
        self.stream = stream
        check(self.lib.ogx_ctx_set_stream(self.handle, ctypes.c_void_p(stream.cuda_stream)))

    def synchronize(self):
        check(self.lib.ogx_ctx_synchronize(self.handle))

    @property
    def last_launches(self) -> int:
        return int(self.lib.ogx_ctx_last_launches(self.handle))

    def set_timing(self, on: bool = True):
        check(self.lib.ogx_ctx_set_timing(self.handle, int(on)))

    def kernel_times(self) -> list:
        """[(kernel name, ms)] of the last batched call (needs set_timing(True))."""
        names = (ctypes.c_char_p * 32)()
        ms = (ctypes.c_float * 32)()
        n = self.lib.ogx_ctx_kernel_times(self.handle, names, ms, 32)
        if n < 0:
            raise _lib.OgxError(-2, "kernel timing failed")
        return [(names[i].decode(), float(ms[i])) for i in range(n)]

    def set_stage_timeline(self, on: bool = True):
        check(self.lib.ogx_ctx_set_stage_timeline(self.handle, int(bool(on))))

    def stage_timeline(self) -> list:
        """[(stage, ms from the call's start)] of the last concurrent call (needs
        set_stage_timeline(True))."""
        names = (ctypes.c_char_p * 40)()
        ms = (ctypes.c_float * 40)()
        n = self.lib.ogx_ctx_stage_timeline(self.handle, names, ms, 40)
        if n < 0:
            raise _lib.OgxError(-2, "stage timeline failed")
        return [(names[i].decode(), float(ms[i])) for i in range(n)]

    def kernel_choice(self) -> dict:
        """{"gjk": [(lanes, blocks)] * 7, "epa": [...]} per size bucket."""
        out = {}
        for kind, name in ((0, "gjk"), (1, "epa")):
            row = []
            for b in range(7):
                L, K = ctypes.c_int(), ctypes.c_int()
                check(self.lib.ogx_ctx_get_kernel_choice(self.handle, kind, b, ctypes.byref(L), ctypes.byref(K)))
                row.append((L.value, K.value))
            out[name] = row
        return out

    def set_kernel_choice(self, kind: str, bucket: int, lanes: int, blocks: int):
        check(self.lib.ogx_ctx_set_kernel_choice(self.handle, 0 if kind == "gjk" else 1, bucket, lanes, blocks))

    def autotune(self, pool, pairs_dev, reps: int = 2):
        """Pick the fastest kernel variant per bucket on this batch (synchronous)."""
        check(self.lib.ogx_autotune(self.handle, pool.handle, int(pairs_dev.shape[0]),
                                    ctypes.c_void_p(pairs_dev.data_ptr()), int(reps)))
        return self.kernel_choice()

    def work_counts(self) -> dict:
        c = (ctypes.c_int32 * 21)()
        n = self.lib.ogx_ctx_work_counts(self.handle, c, 21)
        if n != 21:
            raise _lib.OgxError(-2, "work counts unavailable")
        return {"gjk": list(c[0:7]), "epa": list(c[7:14]), "polish": int(c[14]), "refine": int(c[15]),
                "refine_full": int(c[16]) + int(c[18]), "refine_full_warp": int(c[18]),
                "epa_spill": int(c[17]), "epa_late": int(c[19]), "epa_resumed": min(int(c[20]), 4096)}


class Pool:
    """Device-resident polytope pool (padded SoA layout)."""

    def __init__(self, ctx: Context, counts):
        self.ctx = ctx
        counts = np.ascontiguousarray(counts, dtype=np.int32)
        self.counts = counts
        h = ctypes.c_void_p()
        check(ctx.lib.ogx_pool_create(ctx.handle, int(counts.shape[0]), counts.ctypes.data, ctypes.byref(h)))
        self.handle = h
        _live_pools.add(self)

    @property
    def num_bodies(self) -> int:
        return int(self.ctx.lib.ogx_pool_num_bodies(self.handle))

    @property
    def num_points(self) -> int:
        return int(self.ctx.lib.ogx_pool_num_points(self.handle))

    def upload(self, coords):
        """coords: host (numpy, or pinned torch CPU tensor) float32 xyz of all bodies."""
        torch = _torch()
        if isinstance(coords, torch.Tensor):
            assert coords.device.type == "cpu" and coords.dtype == torch.float32 and coords.is_contiguous()
            ptr = coords.data_ptr()
            self._keep = coords
        else:
            arr = np.ascontiguousarray(coords, dtype=np.float32)
            ptr = arr.ctypes.data
            self._keep = arr
        check(self.ctx.lib.ogx_pool_upload(self.ctx.handle, self.handle, ctypes.c_void_p(ptr)))

    def load_device(self, coords_dev):
        """coords_dev: torch CUDA float32 tensor, xyz of all bodies (AoS)."""
        assert coords_dev.is_cuda and coords_dev.dtype == _torch().float32 and coords_dev.is_contiguous()
        check(self.ctx.lib.ogx_pool_load_device(self.ctx.handle, self.handle, ctypes.c_void_p(coords_dev.data_ptr())))

    def device_layout(self):
        pts, bodies = ctypes.c_void_p(), ctypes.c_void_p()
        check(self.ctx.lib.ogx_pool_device_layout(self.handle, ctypes.byref(pts), ctypes.byref(bodies)))
        return pts.value, bodies.value

    def close(self):
        if self.handle and self.ctx.handle:
            self.ctx.lib.ogx_pool_destroy(self.handle)
        self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


class Results:
    """Device outputs of one batched call (torch CUDA tensors)."""

    def __init__(self, n: int, device, with_normals: bool = True):
        torch = _torch()
        self.n = n
        self.simplex = torch.zeros((n, 27), dtype=torch.int32, device=device)  # 108 B per pair
        self.dist = torch.zeros(n, dtype=torch.float32, device=device)
        self.normal = torch.zeros((n, 3), dtype=torch.float32, device=device) if with_normals else None
        self.status = torch.zeros(n, dtype=torch.int32, device=device)

    def to_host(self) -> dict:
        smp = self.simplex.cpu().numpy().view(SIMPLEX_DTYPE).reshape(self.n)
        out = {
            "dist": self.dist.cpu().numpy(),
            "simplex": smp,
            "status": self.status.cpu().numpy(),
        }
        out["normal"] = self.normal.cpu().numpy() if self.normal is not None else None
        return out


def run(ctx: Context, pool: Pool, pairs_dev, mode: int = MODE_GJK_EPA, out: Results | None = None) -> Results:
    """Batched query over device pairs (int32 [n, 2] CUDA tensor)."""
    torch = _torch()
    assert pairs_dev.is_cuda and pairs_dev.dtype == torch.int32 and pairs_dev.is_contiguous()
    n = int(pairs_dev.shape[0])
    if out is None:
        out = Results(n, pairs_dev.device, with_normals=(mode != MODE_GJK))
    cur = torch.cuda.current_stream(pairs_dev.device)
    if cur != ctx.stream:
        ctx.stream.wait_stream(cur)  # inputs and output buffers are ready
    P = ctypes.c_void_p
    args = [ctx.handle, pool.handle, n, P(pairs_dev.data_ptr()), P(out.simplex.data_ptr()), P(out.dist.data_ptr())]
    if mode == MODE_GJK:
        check(ctx.lib.ogx_gjk(*args, P(out.status.data_ptr())))
    elif mode == MODE_GJK_EPA:
        check(ctx.lib.ogx_gjk_epa(*args, P(out.normal.data_ptr()), P(out.status.data_ptr())))
    elif mode == MODE_EPA:
        check(ctx.lib.ogx_epa(*args, P(out.normal.data_ptr()), P(out.status.data_ptr())))
    else:
        raise ValueError(mode)
    if cur != ctx.stream:
        cur.wait_stream(ctx.stream)  # later torch work sees the results
    return out


def streamed(ctx: Context, pool: Pool, coords, pairs, out: dict | None = None, chunks: int = 8,
             bounds=None, lanes: int = 0) -> dict:
    """Host-to-host GJK + EPA (ogx_gjk_epa_streamed): uploads `coords` (all bodies' xyz)
    and `pairs` in chunks, overlapping the copies with the kernels; synchronous.
    coords / pairs: numpy arrays or pinned torch CPU tensors; `out`: dict of host arrays
    (simplex, dist, normal, status) to fill, allocated if None.  `bounds` (ascending pair
    indices from 0 to n) gives the pieces explicitly (ogx_gjk_epa_streamed_ranges), with
    up to `lanes` pieces computing side by side (0 = default)."""
    def ptr(x):
        return x.data_ptr() if hasattr(x, "data_ptr") else x.ctypes.data
    n = int(pairs.shape[0])
    if out is None:
        out = {"simplex": np.zeros(n, SIMPLEX_DTYPE), "dist": np.zeros(n, np.float32),
               "normal": np.zeros((n, 3), np.float32), "status": np.zeros(n, np.int32)}
    P = ctypes.c_void_p
    args = (ctx.handle, pool.handle, P(ptr(coords)), n, P(ptr(pairs)), P(ptr(out["simplex"])),
            P(ptr(out["dist"])), P(ptr(out["normal"])), P(ptr(out["status"])))
    if bounds is None:
        check(ctx.lib.ogx_gjk_epa_streamed(*args, int(chunks)))
    else:
        b = np.ascontiguousarray(bounds, dtype=np.int32)
        check(ctx.lib.ogx_gjk_epa_streamed_ranges(*args, P(b.ctypes.data), int(b.shape[0]) - 1, int(lanes)))
    return out


def contact_response(ctx: Context, state: dict, pairs_dev, res: Results, baumgarte: float = 0.2,
                     restitution: float = 0.5, restitution_threshold: float = 1.0,
                     contact_eps: float = 1.1920929e-07) -> dict:
    """Collision response (ogx_contact_response) from a GJK+EPA result: `state` holds
    CUDA float32 tensors pos [n,3], quat [n,4] (x,y,z,w), vel [n,3], ang [n,3],
    inv_mass [n], inv_inertia [n,3]; returns new vel, ang, pos tensors."""
    torch = _torch()
    n = int(state["pos"].shape[0])
    st = _lib.BodyState(*(state[k].data_ptr() for k in ("pos", "quat", "vel", "ang", "inv_mass", "inv_inertia")))
    prm = _lib.ResponseParams(contact_eps, baumgarte, restitution, restitution_threshold)
    out = {k: torch.empty((n, 3), dtype=torch.float32, device=state["pos"].device) for k in ("vel", "ang", "pos")}
    cur = torch.cuda.current_stream(pairs_dev.device)
    if cur != ctx.stream:
        ctx.stream.wait_stream(cur)
    P = ctypes.c_void_p
    check(ctx.lib.ogx_contact_response(ctx.handle, n, ctypes.byref(st), int(pairs_dev.shape[0]),
                                       P(pairs_dev.data_ptr()), P(res.dist.data_ptr()), P(res.normal.data_ptr()),
                                       P(res.simplex.data_ptr()), ctypes.byref(prm), P(out["vel"].data_ptr()),
                                       P(out["ang"].data_ptr()), P(out["pos"].data_ptr())))
    if cur != ctx.stream:
        cur.wait_stream(ctx.stream)
    return out


def expand_submesh_pairs(ctx: Context, body_pairs_dev, first_part_dev, part_count_dev, max_sub_pairs: int):
    """Body pairs -> part pairs (ogx_expand_submesh_pairs): returns (part pairs [m, 2],
    owner body pair [m], offsets [n + 1]) as CUDA tensors; waits for the total."""
    torch = _torch()
    n = int(body_pairs_dev.shape[0])
    dev = body_pairs_dev.device
    sub = torch.empty((max(max_sub_pairs, 1), 2), dtype=torch.int32, device=dev)
    owner = torch.empty(max(max_sub_pairs, 1), dtype=torch.int32, device=dev)
    off = torch.empty(n + 1, dtype=torch.int32, device=dev)
    cur = torch.cuda.current_stream(dev)
    if cur != ctx.stream:
        ctx.stream.wait_stream(cur)
    P = ctypes.c_void_p
    check(ctx.lib.ogx_expand_submesh_pairs(ctx.handle, n, P(body_pairs_dev.data_ptr()), int(first_part_dev.shape[0]),
                                           P(first_part_dev.data_ptr()), P(part_count_dev.data_ptr()),
                                           int(max_sub_pairs), P(sub.data_ptr()), P(owner.data_ptr()),
                                           P(off.data_ptr())))
    if cur != ctx.stream:
        cur.wait_stream(ctx.stream)
    total = int(off[n].item())
    m = min(total, max_sub_pairs)
    return sub[:m], owner[:m], off


def reduce_submesh_pairs(ctx: Context, offsets_dev, sub_dist_dev, max_sub_pairs: int):
    """Per body pair: (smallest part-pair distance, its part-pair index) CUDA tensors."""
    torch = _torch()
    n = int(offsets_dev.shape[0]) - 1
    best = torch.empty(max(n, 1), dtype=torch.float32, device=offsets_dev.device)
    arg = torch.empty(max(n, 1), dtype=torch.int32, device=offsets_dev.device)
    cur = torch.cuda.current_stream(offsets_dev.device)
    if cur != ctx.stream:
        ctx.stream.wait_stream(cur)
    P = ctypes.c_void_p
    check(ctx.lib.ogx_reduce_submesh_pairs(ctx.handle, n, P(offsets_dev.data_ptr()), int(max_sub_pairs),
                                           P(sub_dist_dev.data_ptr()), P(best.data_ptr()), P(arg.data_ptr())))
    if cur != ctx.stream:
        cur.wait_stream(ctx.stream)
    return best[:n], arg[:n]


def stream_timeline(ctx: Context) -> np.ndarray:
    """[chunks, 5] ms of the last streamed call made with timing on: body upload end, pair
    upload end, kernels start, kernels end, download end."""
    n = ctx.lib.ogx_ctx_stream_timeline(ctx.handle, None, 0)
    buf = (ctypes.c_float * max(n, 1))()
    ctx.lib.ogx_ctx_stream_timeline(ctx.handle, buf, n)
    return np.array(buf[:n], np.float32).reshape(-1, 5)


class Graph:
    """One call captured as a CUDA graph (ogx_graph_*): `launch()` replays the whole
    pipeline on the context's stream with one launch.  The pair and output buffers are
    fixed at capture; their contents may change between launches."""

    def __init__(self, ctx: Context, pool: Pool, pairs_dev, mode: int = MODE_GJK_EPA, out: Results | None = None):
        torch = _torch()
        assert pairs_dev.is_cuda and pairs_dev.dtype == torch.int32 and pairs_dev.is_contiguous()
        self.ctx, self.pool, self.pairs = ctx, pool, pairs_dev
        n = int(pairs_dev.shape[0])
        self.out = out if out is not None else Results(n, pairs_dev.device, with_normals=(mode != MODE_GJK))
        torch.cuda.current_stream(pairs_dev.device).synchronize()
        P = ctypes.c_void_p
        h = ctypes.c_void_p()
        nrm = P(self.out.normal.data_ptr()) if self.out.normal is not None else None
        check(ctx.lib.ogx_graph_create(ctx.handle, pool.handle, n, P(pairs_dev.data_ptr()),
                                       P(self.out.simplex.data_ptr()), P(self.out.dist.data_ptr()), nrm,
                                       P(self.out.status.data_ptr()), int(mode), ctypes.byref(h)))
        self.handle = h
        _live_pools.add(self)

    @property
    def kernel_launches(self) -> int:
        return int(self.ctx.lib.ogx_graph_kernel_launches(self.handle))

    def launch(self) -> Results:
        torch = _torch()
        cur = torch.cuda.current_stream(self.pairs.device)
        if cur != self.ctx.stream:
            self.ctx.stream.wait_stream(cur)
        check(self.ctx.lib.ogx_graph_launch(self.handle))
        if cur != self.ctx.stream:
            cur.wait_stream(self.ctx.stream)
        return self.out

    def close(self):
        if self.handle and self.ctx.handle:
            self.ctx.lib.ogx_graph_destroy(self.handle)
        self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


class Broad:
    """Device broad phase (ogx_broadphase): the pairs of a pool's bodies whose boxes
    (grown by `margin`) overlap, each once, sorted, on the device."""

    def __init__(self, ctx: Context, max_bodies: int):
        self.ctx = ctx
        h = ctypes.c_void_p()
        check(ctx.lib.ogx_broad_create(ctx.handle, int(max_bodies), ctypes.byref(h)))
        self.handle = h
        _live_pools.add(self)
        self._result = _torch().zeros(2, dtype=_torch().int32, device=f"cuda:{ctx.device}")

    def run(self, pool: Pool, cell: float, margin: float = 0.0, max_pairs: int = 1 << 20, pairs_dev=None):
        """Returns (pairs int32 [n, 2] CUDA tensor, total count, error flags); waits for
        the count."""
        torch = _torch()
        if pairs_dev is None:
            pairs_dev = torch.empty((max_pairs, 2), dtype=torch.int32, device=f"cuda:{self.ctx.device}")
        cur = torch.cuda.current_stream(pairs_dev.device)
        if cur != self.ctx.stream:
            self.ctx.stream.wait_stream(cur)
        check(self.ctx.lib.ogx_broadphase(self.handle, pool.handle, float(cell), float(margin), int(max_pairs),
                                          ctypes.c_void_p(pairs_dev.data_ptr()),
                                          ctypes.c_void_p(self._result.data_ptr())))
        if cur != self.ctx.stream:
            cur.wait_stream(self.ctx.stream)
        count, flags = (int(x) for x in self._result.cpu().tolist())
        return pairs_dev[:min(count, max_pairs)], count, flags

    def run_spheres(self, spheres_dev, cell: float, boundary: float, grid_size: int, max_pairs: int = 1 << 20):
        """The reference's bounding-sphere pairs (ogx_broadphase_spheres): spheres_dev is a
        float32 [n, 4] CUDA tensor (x, y, z, radius).  Returns (pairs int32 [n, 2] CUDA
        tensor sorted by (i, j), total count)."""
        torch = _torch()
        assert spheres_dev.is_cuda and spheres_dev.dtype == torch.float32 and spheres_dev.is_contiguous()
        pairs_dev = torch.empty((max(max_pairs, 1), 2), dtype=torch.int32, device=spheres_dev.device)
        cur = torch.cuda.current_stream(spheres_dev.device)
        if cur != self.ctx.stream:
            self.ctx.stream.wait_stream(cur)
        check(self.ctx.lib.ogx_broadphase_spheres(self.handle, ctypes.c_void_p(spheres_dev.data_ptr()),
                                                  int(spheres_dev.shape[0]), ctypes.c_float(cell),
                                                  ctypes.c_float(boundary), int(grid_size), int(max_pairs),
                                                  ctypes.c_void_p(pairs_dev.data_ptr()),
                                                  ctypes.c_void_p(self._result.data_ptr())))
        if cur != self.ctx.stream:
            cur.wait_stream(self.ctx.stream)
        count = int(self._result.cpu()[0])
        return pairs_dev[:min(count, max_pairs)], count

    def close(self):
        if self.handle and self.ctx.handle:
            self.ctx.lib.ogx_broad_destroy(self.handle)
        self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def query(batch, mode: int = MODE_GJK_EPA, config: _lib.Config | None = None, device: int = 0) -> dict:
    """One-shot convenience: upload a workloads.Batch, run, return host numpy results."""
    torch = _torch()
    ctx = Context(device, config)
    pool = Pool(ctx, batch.counts)
    pool.upload(batch.coords)
    pairs = torch.from_numpy(np.ascontiguousarray(batch.pairs, dtype=np.int32)).to(f"cuda:{device}")
    res = run(ctx, pool, pairs, mode)
    ctx.synchronize()
    out = res.to_host()
    out["launches"] = ctx.last_launches
    pool.close()
    ctx.close()
    return out
