"""Python handle on the engine's serving loop (ogx_server_* in include/ogx.h).

A server keeps the bodies on the GPU in their own frame, takes pose updates
(``set_transforms``, one version per tick) and pair requests (``submit``), admits
queued requests as device slots and the in-flight pair budget allow, runs them
concurrently and returns each request's results and its submit-to-done latency.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

P = ctypes.c_void_p


class ServerConfig(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_int), ("slot_pairs", ctypes.c_int), ("max_pairs_in_flight", ctypes.c_int),
                ("world_slots", ctypes.c_int), ("warm_start", ctypes.c_int), ("warm_capacity_log2", ctypes.c_int),
                ("max_bytes_in_flight", ctypes.c_int64), ("fused_transform", ctypes.c_int)]


def _bind(lib):
    if getattr(lib, "_ogx_server_bound", False):
        return
    I64 = ctypes.c_int64
    lib.ogx_server_config_default.restype = None
    lib.ogx_server_config_default.argtypes = [P]
    lib.ogx_server_create.restype = ctypes.c_int
    lib.ogx_server_create.argtypes = [ctypes.c_int, P, P, ctypes.c_int, P, P, P]
    lib.ogx_server_destroy.restype = ctypes.c_int
    lib.ogx_server_destroy.argtypes = [P]
    lib.ogx_server_set_transforms.restype = ctypes.c_int
    lib.ogx_server_set_transforms.argtypes = [P, P, ctypes.POINTER(I64)]
    lib.ogx_server_submit.restype = ctypes.c_int
    lib.ogx_server_submit.argtypes = [P, I64, ctypes.c_int, P, P, P, P, P, ctypes.POINTER(I64)]
    lib.ogx_server_submit_broadphase.restype = ctypes.c_int
    lib.ogx_server_submit_broadphase.argtypes = [P, I64, ctypes.c_float, ctypes.c_float, ctypes.c_int, P, P, P, P,
                                                 P, P, ctypes.POINTER(I64)]
    lib.ogx_server_poll.restype = ctypes.c_int
    lib.ogx_server_poll.argtypes = [P, I64, ctypes.POINTER(ctypes.c_int)]
    lib.ogx_server_wait.restype = ctypes.c_int
    lib.ogx_server_wait.argtypes = [P, I64, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
    lib.ogx_server_wait_phases.restype = ctypes.c_int
    lib.ogx_server_wait_phases.argtypes = [P, I64, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double)]
    lib.ogx_server_admission.restype = ctypes.c_int
    lib.ogx_server_admission.argtypes = [P] + [ctypes.POINTER(I64)] * 4
    lib.ogx_server_world_layout.restype = ctypes.c_int
    lib.ogx_server_world_layout.argtypes = [P, I64, ctypes.POINTER(P), ctypes.POINTER(P)]
    lib._ogx_server_bound = True


def _pinned(nbytes: int):
    """Page-locked host buffer (torch's caching pinned allocator) and its numpy view."""
    import torch
    t = torch.empty(max(nbytes, 16), dtype=torch.uint8, pin_memory=True)
    return t, t.numpy()[:nbytes]


_SET_FIELDS = (("dist", np.float32, ()), ("simplex", None, ()), ("normal", np.float32, (3,)),
               ("status", np.int32, ()), ("pairs", np.int32, (2,)))


class _ResultSets:
    """Page-locked result arrays for requests of up to `cap` pairs, kept and handed out
    again when a request is released, so that a running server allocates no pinned
    memory per request (pinning tens of MB takes milliseconds)."""

    def __init__(self, cap: int):
        self.cap = cap
        self.free = []

    def new(self, n: int) -> dict:
        out = {}
        for name, dtype, tail in _SET_FIELDS:
            dt = np.dtype(_lib.SIMPLEX_DTYPE if dtype is None else dtype)
            shape = (n,) + tail
            t, raw = _pinned(int(np.prod(shape)) * dt.itemsize)
            out[name] = (t, raw.view(dt).reshape(shape))
        t, raw = _pinned(8)
        out["count"] = (t, raw.view(np.int32))
        return out

    def take(self, n: int) -> tuple[dict, bool]:
        if n > self.cap:
            return self.new(n), False
        try:  # list.pop is atomic: submit and release may run on different threads
            return self.free.pop(), True
        except IndexError:
            return self.new(self.cap), True


class Request:
    """Host result arrays of one submitted request (filled when it completes).  They are
    page-locked, so the device writes them directly.  ``release()`` hands them back to
    the server for later requests; without it they are freed with the request."""

    def __init__(self, ticket: int, pairs: np.ndarray | None, n: int, bufs: dict, pool: _ResultSets | None):
        self.ticket = ticket
        self._set = bufs
        self._pool = pool
        self.dist = bufs["dist"][1][:n]
        self.simplex = bufs["simplex"][1][:n]
        self.normal = bufs["normal"][1][:n]
        self.status = bufs["status"][1][:n]
        self.pairs = pairs
        self.latency_ms = None
        self.phases_ms = None
        self.count = None  # broad-phase requests: [pairs found, error flags]
        self.done = False

    def release(self):
        """Give the result arrays back to the server (after wait()); the request's arrays,
        and any view of them, must not be used afterwards."""
        if not self.done:
            raise RuntimeError("release() before the request was waited for")
        if self._pool is not None and self._set is not None:
            self._pool.free.append(self._set)
        self._set = None
        self.dist = self.simplex = self.normal = self.status = self.pairs = self.count = None

    def results(self) -> dict:
        n = self.n_run
        return {"dist": self.dist[:n], "simplex": self.simplex[:n], "normal": self.normal[:n],
                "status": self.status[:n]}

    @property
    def n_run(self) -> int:
        """Pairs the request ran (for broad-phase requests: min(found, capacity))."""
        if self.count is None:
            return int(self.dist.shape[0])
        return int(min(self.count[0], self.dist.shape[0]))


class Server:
    def __init__(self, counts, local_xyz, config: _lib.Config | None = None, device: int = 0, slots: int = 4,
                 slot_pairs: int = 262144, max_pairs_in_flight: int = 1 << 20, world_slots: int = 4,
                 warm_start: bool = True, warm_capacity_log2: int = 22, result_sets: int | None = None,
                 fused_transform: bool = False, max_bytes_in_flight: int = 0):
        """`result_sets` page-locked result sets of `slot_pairs` pairs are allocated up
        front (default 2 x slots) and recycled by Request.release().  `fused_transform`:
        keep no world copies, the kernels apply the poses as they read the points.
        `max_bytes_in_flight`: admission budget in device bytes (0: half the free memory)."""
        self.lib = _lib.load()
        _bind(self.lib)
        sc = ServerConfig()
        self.lib.ogx_server_config_default(ctypes.byref(sc))
        sc.slots, sc.slot_pairs, sc.max_pairs_in_flight = slots, slot_pairs, max_pairs_in_flight
        sc.world_slots, sc.warm_start, sc.warm_capacity_log2 = world_slots, int(warm_start), warm_capacity_log2
        sc.fused_transform = int(fused_transform)
        sc.max_bytes_in_flight = int(max_bytes_in_flight)
        self.counts = np.ascontiguousarray(counts, np.int32)
        local = np.ascontiguousarray(local_xyz, np.float32)
        h = P()
        rc = self.lib.ogx_server_create(device, ctypes.byref(config) if config is not None else None,
                                        ctypes.byref(sc), int(self.counts.shape[0]), self.counts.ctypes.data,
                                        local.ctypes.data, ctypes.byref(h))
        _lib.check(rc)
        self.handle = h
        self._live = {}
        self._sets = _ResultSets(slot_pairs)
        for _ in range(2 * slots if result_sets is None else result_sets):
            self._sets.free.append(self._sets.new(slot_pairs))

    def set_transforms(self, xf: np.ndarray) -> int:
        xf = np.ascontiguousarray(xf, np.float32)
        assert xf.shape == (self.counts.shape[0], 12)
        v = ctypes.c_int64()
        _lib.check(self.lib.ogx_server_set_transforms(self.handle, xf.ctypes.data, ctypes.byref(v)))
        return v.value

    def submit(self, version: int, pairs: np.ndarray) -> Request:
        pairs = np.ascontiguousarray(pairs, np.int32)
        n = int(pairs.shape[0])
        t = ctypes.c_int64()
        bufs, pooled = self._sets.take(n)
        req = Request(0, pairs, n, bufs, self._sets if pooled else None)
        self._refused(req, self.lib.ogx_server_submit(self.handle, int(version), n, pairs.ctypes.data,
                                                      req.simplex.ctypes.data, req.dist.ctypes.data,
                                                      req.normal.ctypes.data, req.status.ctypes.data,
                                                      ctypes.byref(t)))
        req.ticket = t.value
        self._live[req.ticket] = req  # the arrays must outlive the request
        return req

    def submit_broadphase(self, version: int, cell: float, margin: float = 0.0, max_pairs: int = 262144) -> Request:
        """Pairs from the device broad phase of the version's world copy (boxes grown by
        `margin` that overlap), then GJK + EPA on them.  req.pairs[:req.n_run] are the
        pairs run, req.count[0] the number found."""
        t = ctypes.c_int64()
        bufs, pooled = self._sets.take(max_pairs)
        req = Request(0, None, max_pairs, bufs, self._sets if pooled else None)
        req.pairs = bufs["pairs"][1][:max_pairs]
        req.count = bufs["count"][1]
        self._refused(req, self.lib.ogx_server_submit_broadphase(
            self.handle, int(version), float(cell), float(margin), int(max_pairs), req.pairs.ctypes.data,
            req.count.ctypes.data, req.simplex.ctypes.data, req.dist.ctypes.data, req.normal.ctypes.data,
            req.status.ctypes.data, ctypes.byref(t)))
        req.ticket = t.value
        self._live[req.ticket] = req
        return req

    @staticmethod
    def _refused(req: Request, rc: int):
        """A submit the server refused: its result set goes back to the pool, then raise."""
        if rc != 0:
            req.done = True
            req.release()
        _lib.check(rc)

    def done(self, req: Request) -> bool:
        d = ctypes.c_int()
        _lib.check(self.lib.ogx_server_poll(self.handle, req.ticket, ctypes.byref(d)))
        return bool(d.value)

    def wait(self, req: Request, timeout_s: float = 60.0) -> Request:
        """Block until the request is done; sets req.latency_ms (submit to results in host
        memory) and req.phases_ms (queued, host staging, device, rest)."""
        lat = ctypes.c_double()
        ph = (ctypes.c_double * 4)()
        rc = self.lib.ogx_server_wait_phases(self.handle, req.ticket, float(timeout_s), ctypes.byref(lat), ph)
        if rc != _lib.ERR_BUSY:
            # done or failed: the device no longer writes the arrays (a timed-out request
            # stays registered, its arrays alive)
            self._live.pop(req.ticket, None)
            req.done = True
        _lib.check(rc)
        req.latency_ms = lat.value
        req.phases_ms = tuple(ph)
        return req

    def admission(self) -> dict:
        """Admission budgets (pairs, device bytes), bytes per pair, peak bytes in flight."""
        v = [ctypes.c_int64() for _ in range(4)]
        _lib.check(self.lib.ogx_server_admission(self.handle, *[ctypes.byref(x) for x in v]))
        return dict(zip(("max_pairs_in_flight", "max_bytes_in_flight", "bytes_per_pair", "peak_bytes_in_flight"),
                        (x.value for x in v)))

    def world_layout(self, version: int):
        pts, bodies = P(), P()
        _lib.check(self.lib.ogx_server_world_layout(self.handle, int(version), ctypes.byref(pts),
                                                    ctypes.byref(bodies)))
        return pts.value, bodies.value

    def close(self):
        if self.handle:
            self.lib.ogx_server_destroy(self.handle)
            self.handle = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
