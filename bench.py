#!/usr/bin/env python3
"""Benchmark: batched GJK+EPA pairs/s on one GB300 (FP32 bulk, FP64 where needed).

Workload (default): 1,000,000 pairs in one batch; vertex counts from a discrete power
law p(n) ~ n^-1.5 on [4, 1024]; points uniform on random ellipsoids (semi-axes
U[0.3, 2], uniform rotation); centres placed so that about half the pairs overlap.
Seeded synthetic data (no dataset exists for this benchmark).

One step = one pass of the whole pipeline (bin, GJK, EPA on the contacts, FP64 polish)
over the batch.  `value` is measured with inputs resident in HBM (the pool is 1.5 GB,
larger than L2, so no flush is needed between steps); `e2e` repeats the step through
the C ABI with host buffers: pinned host points + pairs copied in, results copied out.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

# more hardware work queues than the runtime's default 8, so that the streamed call's
# lanes and their per-bucket streams do not serialise (read when CUDA starts)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "opengjk-gpu_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "GJK+EPA pairs/s on 1 GB300 (FP32, <=1e-5 rel err)"
WORKLOADS = {
    "powerlaw": dict(desc="GJK+EPA, 1,000,000 pairs, power-law vertex counts on [4,1024] (exp -1.5), "
                          "ellipsoid point sets, ~50% overlapping", n_pairs=1_000_000),
    "ellipsoid": dict(desc="GJK+EPA, 100,000 pairs, log-uniform vertex counts on [8,256], "
                           "ellipsoid point sets, ~50% overlapping", n_pairs=100_000),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="powerlaw", choices=sorted(WORKLOADS))
    ap.add_argument("--pairs", type=int, default=0, help="override the workload's pair count")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the kernel autotuner")
    ap.add_argument("--tune-reps", type=int, default=3, help="timed runs per candidate in the autotuner (best kept)")
    ap.add_argument("--choice", default="",
                    help='kernel variants instead of autotuning, as printed in "kernel_choice" (JSON)')
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop report")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip timing the reference's own GPU kernels on the same workload")
    ap.add_argument("--chunks", type=int, default=6, help="pieces of the end-to-end streamed call")
    ap.add_argument("--profile-launches", action="store_true",
                    help="one untimed step only (for ncu launch lists)")
    return ap.parse_args()


def make_batch(name: str, n_pairs: int, seed: int):
    from ogx import workloads as W
    if name == "powerlaw":
        return W.powerlaw(seed=seed, n_pairs=n_pairs)
    return W.ellipsoid(seed=seed, n_pairs=n_pairs)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class NvmlClockSampler:
    """SM clock, its maximum, power and clock-event reasons read through NVML every
    `period_s` during the timed region (read-only queries; the timed region of a default
    run lasts ~0.1 s, too short for nvidia-smi's sampling period)."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, gpu: int, period_s: float = 0.002):
        import ctypes
        self.ct = ctypes
        self.period = period_s
        self.samples = []
        self._stop = threading.Event()
        self._t = None
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.nv = nv
        self.dev = ctypes.c_void_p()
        ok = False
        try:  # the NVML device of this CUDA device, by UUID (NVML and CUDA numbering can differ)
            import torch
            uuid = str(torch.cuda.get_device_properties(gpu).uuid)
            ok = nv.nvmlDeviceGetHandleByUUID(("GPU-" + uuid).encode(), ctypes.byref(self.dev)) == 0
        except Exception:
            ok = False
        if not ok and nv.nvmlDeviceGetHandleByIndex_v2(gpu, ctypes.byref(self.dev)) != 0:
            raise RuntimeError("no NVML handle")
        self._reasons = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        nv.nvmlDeviceGetMaxClockInfo(self.dev, 1, ctypes.byref(mx))
        self.max_mhz = float(mx.value)

    def _run(self):
        c = self.ct
        mhz, mw, r = c.c_uint(), c.c_uint(), c.c_ulonglong()
        while not self._stop.is_set():
            if self.nv.nvmlDeviceGetClockInfo(self.dev, 1, c.byref(mhz)) == 0:
                self.nv.nvmlDeviceGetPowerUsage(self.dev, c.byref(mw))
                self._reasons(self.dev, c.byref(r))
                self.samples.append((float(mhz.value), mw.value / 1e3, int(r.value)))
            self._stop.wait(self.period)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=5)
        self.nv.nvmlShutdown()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["unsampled"], "samples": 0}
        sm = [s[0] for s in self.samples]
        reasons = sorted({name for s in self.samples for bit, name in self.REASONS.items() if s[2] & bit})
        return {"sm_mhz": statistics.median(sm), "sm_min_mhz": min(sm), "sm_max_mhz": self.max_mhz,
                "power_w_median": statistics.median(s[1] for s in self.samples), "reasons": reasons,
                "samples": len(self.samples), "source": f"NVML every {self.period * 1e3:.0f} ms"}


def clock_sampler(gpu: int):
    """NVML sampler, or nvidia-smi's where NVML cannot be loaded."""
    try:
        return NvmlClockSampler(gpu)
    except Exception:
        return ClockSampler(gpu)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.samples = []
        self._proc = None
        self._t = None

    def _read(self):
        for line in self._proc.stdout:
            f = [x.strip() for x in line.strip().split(",")]
            if len(f) >= 7:
                self.samples.append(f)

    def __enter__(self):
        try:
            # one nvidia-smi process sampling every 100 ms until stopped
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self._proc = None
        return self

    def __exit__(self, *a):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
            if self._t:
                self._t.join(timeout=5)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if len(s) > 3 + k and s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def bench_config(spec: dict, n: int, batch, world: int) -> dict:
    """The workload, identical in both arms' lines."""
    return {"workload": spec["desc"], "pairs_per_gpu": n, "seed": 1000,
            "mean_vertices_per_body": round(float(batch.counts.mean()), 4),
            "l2": "inputs (pool %.2f GB) larger than L2, no flush" % (batch.coords.nbytes / 1e9),
            "parallelism": f"replicas x{world}"}


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def cpu_single_thread(batch, seconds: float = 3.0) -> dict:
    """The reference's own CPU loop as it ships: one thread, pair after pair, GJK then EPA
    (examples/cpu/example.cpp:13-40), on the first pairs of the workload for ~`seconds`."""
    from oracle import orc
    use_ref = orc.ref_available()
    n0 = min(batch.n_pairs, 500)
    t = time.perf_counter()
    _cpu_run(orc, batch.subset(np.arange(n0)), orc.MODE_GJK_EPA, 1, use_ref)
    per_pair = max((time.perf_counter() - t) / n0, 1e-9)
    n = int(min(batch.n_pairs, max(n0, seconds / per_pair)))
    t = time.perf_counter()
    _cpu_run(orc, batch.subset(np.arange(n)), orc.MODE_GJK_EPA, 1, use_ref)
    dt = time.perf_counter() - t
    return {"value": n / dt, "unit": "pairs/s", "cores": 1, "kind": "reference" if use_ref else "port",
            "sample": f"first {n} pairs of the workload, one thread, FP32 reference tolerances, {dt:.1f} s"}


def cpu_baseline(batch, seconds: float = 12.0, mode="gjk_epa"):
    """Reference CPU GJK+EPA on the host cores (all threads), on a bounded sample of the
    same workload: the reference's own CPU build when present, else the oracle port."""
    from oracle import orc
    threads = os.cpu_count() or 1
    use_ref = orc.ref_available()
    kind = "reference" if use_ref else "port"
    m = orc.MODE_GJK_EPA
    # calibrate the sample size on a small slice
    n0 = min(batch.n_pairs, 4000)
    sub = batch.subset(np.arange(n0))
    t = time.perf_counter()
    _cpu_run(orc, sub, m, threads, use_ref)
    per_pair = max((time.perf_counter() - t) / n0, 1e-9)
    n = int(min(batch.n_pairs, max(n0, seconds / per_pair)))
    sub = batch.subset(np.arange(n))
    # whole passes over the sample until about `wall` seconds have gone by (the whole
    # workload takes well under a second on a many-core host)
    wall = 3.0
    passes, t = 0, time.perf_counter()
    while True:
        _cpu_run(orc, sub, m, threads, use_ref)
        passes += 1
        dt = time.perf_counter() - t
        if dt >= wall or passes >= 50:
            break
    return {"value": passes * n / dt, "unit": "pairs/s", "cores": threads,
            "kind": kind, "sample": f"first {n} pairs of the workload x {passes} passes, FP32 reference "
                                   f"tolerances, {threads} threads, {dt:.1f} s ({dt * threads:.0f} core-s)",
            "cpu_model": cpu_model(), "cores_1": cpu_single_thread(batch)}


def fp64_plain_report(calls: int = 20) -> dict:
    """The FP64 plain-GJK configuration (1,000 pairs of 32-point bodies on spheres, radius
    U[0.5, 2], centres U[-5, 5]^3, double coordinates) through the FP64 drop-in
    (`ogx_compute_minimum_distance_f64`: double descriptors in, 184-byte simplices and
    double distances out, host arrays), median host time of `calls` calls; beside it the
    reference's FP64 CPU GJK (the oracle, which is pinned to it bit for bit) on the same
    inputs, one thread and all host threads."""
    import ctypes
    from ogx import _lib, workloads as W
    from oracle import orc
    b = W.plain(seed=1000, n_pairs=1000, dtype=np.float64)
    c64 = np.ascontiguousarray(b.coords)
    poly = np.dtype([("numpoints", "<i4"), ("s", "<f8", (3,)), ("s_idx", "<i4"), ("coord", "<u8")], align=True)
    smp_t = np.dtype([("nvrtx", "<i4"), ("vrtx", "<f8", (4, 3)), ("vrtx_idx", "<i4", (4, 2)),
                      ("witnesses", "<f8", (2, 3))], align=True)

    def desc(idx):
        d = np.zeros(len(idx), poly)
        d["numpoints"] = b.counts[idx]
        d["coord"] = c64.ctypes.data + 24 * b.offsets[idx].astype(np.uint64)
        return d
    d1, d2 = desc(b.pairs[:, 0]), desc(b.pairs[:, 1])
    n = b.n_pairs
    smp, dist = np.zeros(n, smp_t), np.zeros(n)
    L = _lib.load()
    fn = L.ogx_compute_minimum_distance_f64
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4
    args = (n, d1.ctypes.data, d2.ctypes.data, smp.ctypes.data, dist.ctypes.data)
    for _ in range(3):
        _lib.check(fn(*args))
    ts = []
    for _ in range(calls):
        t = time.perf_counter()
        _lib.check(fn(*args))
        ts.append(time.perf_counter() - t)
    ms = float(np.median(ts)) * 1e3
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK, precision="f64")
    sep = o["dist"] > 1e-5 * np.maximum(1.0, np.abs(c64).max())
    rel = float(np.max(np.abs(dist[sep] - o["dist"][sep]) / o["dist"][sep])) if sep.any() else 0.0
    cpu = {}
    for threads in (1, os.cpu_count() or 1):
        reps, t = 0, time.perf_counter()
        while True:
            orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK, precision="f64", threads=threads)
            reps += 1
            dt = time.perf_counter() - t
            if dt >= 0.5 or reps >= 200:
                break
        cpu[f"threads_{threads}"] = reps * n / dt
    return {"workload": "plain GJK, FP64, 1,000 pairs, 32 points per body on spheres (radius U[0.5, 2], "
                        "centres U[-5, 5]^3), seed 1000",
            "value": n / (ms / 1e3), "unit": "pairs/s", "ms_per_call": ms,
            "path": "ogx_compute_minimum_distance_f64, host arrays in and out, host clock, median of "
                    f"{calls} calls",
            "max_rel_err_vs_fp64_oracle": rel,
            "cpu_fp64_pairs_per_s": cpu, "cpu_kind": "port (the reference's CPU GJK restated, pinned to it)"}


def plain_form_baseline(batch, device: int, steps: int = 3) -> dict:
    """The reference's own GPU kernels (GJK/gpu/openGJK.cu, FP32 as shipped, compiled for
    sm_103a) on the same workload with the points resident: its fused indexed call's
    device part (simplices zeroed, GJK kernel, EPA kernel) per step, CUDA events."""
    import torch
    from oracle import plain_form
    if not plain_form.available():
        return {"unavailable": "the reference's GPU kernels were not compiled (needs the reference sources)"}
    dev = torch.device("cuda", device)
    coords = torch.from_numpy(batch.coords).to(dev)
    pairs = torch.from_numpy(np.ascontiguousarray(batch.pairs)).to(dev)
    pf = plain_form.PlainForm(device).load(coords, batch.offsets, batch.counts)
    st = torch.cuda.Stream(dev)
    with torch.cuda.stream(st):
        out = pf.run(pairs)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(st)
    with torch.cuda.stream(st):
        for _ in range(steps):
            pf.run(pairs, out)
    ev1.record(st)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    # host to host as the reference's fused indexed call moves the data
    # (GJK/gpu/openGJK.cu:3274-3310; its allocations and frees left out): points and body
    # descriptors up from pinned memory, pairs up, kernels, simplices / distances / normals
    # down to pinned memory
    h_coords = torch.from_numpy(batch.coords).pin_memory()
    h_desc = pf.polytopes.cpu().pin_memory()
    h_pairs = torch.from_numpy(np.ascontiguousarray(batch.pairs)).pin_memory()
    h_out = {k: torch.empty(v.shape, dtype=v.dtype).pin_memory() for k, v in out.items()}
    h2d = h_coords.numel() * 4 + h_desc.numel() + h_pairs.numel() * 4
    d2h = sum(t.numel() * t.element_size() for t in h_out.values())

    def host_step():
        with torch.cuda.stream(st):
            coords.copy_(h_coords, non_blocking=True)
            pf.polytopes.copy_(h_desc, non_blocking=True)
            pairs.copy_(h_pairs, non_blocking=True)
            pf.run(pairs, out)
            for k in h_out:
                h_out[k].copy_(out[k], non_blocking=True)
        st.synchronize()
    host_step()
    t0 = time.perf_counter()
    for _ in range(steps):
        host_step()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / steps
    pf.close()
    return {"value": batch.n_pairs / (ms / 1e3), "unit": "pairs/s", "ms_per_step": ms, "steps": steps,
            "e2e": {"value": batch.n_pairs / (e2e_ms / 1e3), "unit": "pairs/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "path": "the reference's indexed call sequence without its allocations: copies up, "
                            "kernels, copies down, in order on one stream, host clock"},
            "kind": "reference GPU kernels",
            "source": "GJK/gpu/openGJK.cu indexed GJK + EPA kernels, FP32 as shipped, compiled for sm_103a, "
                      "shipped launch shapes (GJK: 256-thread blocks, 8 threads per pair; EPA: 4 pairs of "
                      "32 threads per block, 39,264 B shared memory)",
            "sample": "the whole workload, points resident in HBM, 1 warm-up step"}


def dropin_e2e(batch, calls: int = 3) -> dict:
    """End to end through the reference-named drop-in call compute_gjk_epa_indexed
    (GJK/gpu/openGJK.h:497): host gkPolytope descriptors and pairs in, host simplices,
    distances and normals out, in pageable host memory as a reference caller holds them;
    host clock, median of `calls` calls after one warm-up call."""
    from ogx import refapi
    pool = refapi.Polytopes(batch.coords, batch.counts, batch.offsets)
    pairs = np.ascontiguousarray(batch.pairs, np.int32)
    refapi.compute_gjk_epa_indexed(pool, pairs)
    times = []
    for _ in range(calls):
        t = time.perf_counter()
        refapi.compute_gjk_epa_indexed(pool, pairs)
        times.append(time.perf_counter() - t)
    ms = 1e3 * statistics.median(times)
    return {"value": batch.n_pairs / (ms / 1e3), "unit": "pairs/s", "ms_per_call": ms,
            "calls": calls, "call_ms": [round(1e3 * t, 2) for t in times],
            "h2d_bytes_per_step": int(batch.coords.nbytes + pairs.nbytes),
            "d2h_bytes_per_step": int(batch.n_pairs * (108 + 4 + 12)),
            "path": "compute_gjk_epa_indexed (reference-named C++ entry; ogx_compute_gjk_epa_indexed), "
                    "pageable host arrays, host clock"}


def latency_summary(reqs) -> dict:
    """p50 / p99 of the requests' latencies, the median of each phase, and the mean
    phases of the ticks at or above the p99 (what the tail is made of)."""
    lat = np.array([r.latency_ms for r in reqs])
    ph = np.array([r.phases_ms for r in reqs])
    lag = np.array([r.lag_ms for r in reqs])
    p99 = float(np.percentile(lat, 99))
    tail = ph[lat >= min(p99, lat.max())]
    names = ("queued", "staging", "device", "rest")
    sched = lat + lag
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": p99,
            "from_arrival_p50_ms": float(np.percentile(sched, 50)),
            "from_arrival_p99_ms": float(np.percentile(sched, 99)),
            "submit_lag_p50_ms": float(np.percentile(lag, 50)), "submit_lag_max_ms": float(lag.max()),
            "phases_median_ms": dict(zip(names, np.round(np.median(ph, axis=0), 4).tolist())),
            "phases_tail_ms": dict(zip(names, np.round(tail.mean(axis=0), 4).tolist()))}


def serving_report(device: int, seed: int = 77, slots: int = 4, max_in_flight: int = 600_000) -> dict:
    """Serving loop on 20k resident rigid bodies (log-uniform 8-512 vertices): ticks of
    1k-200k candidate pairs (log-uniform) arrive as a Poisson process; each tick uploads
    new poses and submits its pairs; latency = submit -> results in host memory.  Phase 1
    mixes tick sizes at ~50% of the measured capacity, phase 2 sends only 200k-pair ticks
    at ~50% of the capacity for them."""
    import threading as th
    from ogx import serving
    from ogx import workloads as W
    scene = W.serving_scene(seed=seed)
    n_lists = 24
    sizes = W.tick_sizes(seed, n_lists)
    sizes[-6:] = 200_000
    lists = [scene.candidate_pairs(t, int(n)) for t, n in enumerate(sizes)]
    xfs = [scene.transforms(t) for t in range(n_lists)]
    srv = serving.Server(scene.counts, scene.local, device=device, slots=slots, slot_pairs=262144,
                         max_pairs_in_flight=max_in_flight, world_slots=8, warm_start=True)
    try:
        # capacity: back-to-back requests of each list, results waited in order
        def burst(idx):
            t0 = time.perf_counter()
            reqs = []
            for i in idx:
                v = srv.set_transforms(xfs[i])
                reqs.append(srv.submit(v, lists[i]))
            for r in reqs:
                srv.wait(r).release()
            return time.perf_counter() - t0
        burst(range(n_lists))  # warm-up (and warm-start table fill)
        dt = burst(range(n_lists))
        cap_pairs_s = float(sizes.sum()) / dt
        big = [i for i in range(n_lists) if sizes[i] == 200_000]
        dt_big = burst(big)
        cap_big_hz = len(big) / dt_big

        def run(phase_lists, rate_hz, n_ticks, seed2):
            arrivals = W.poisson_arrivals(seed2, n_ticks, rate_hz)
            order = np.random.default_rng(seed2).choice(phase_lists, size=n_ticks)
            out = [None] * n_ticks
            lag = [0.0] * n_ticks
            t0 = time.perf_counter() + 0.05

            def submitter():
                for k in range(n_ticks):
                    while time.perf_counter() < t0 + arrivals[k]:
                        time.sleep(5e-5)
                    i = int(order[k])
                    v = srv.set_transforms(xfs[i])
                    lag[k] = (time.perf_counter() - t0 - arrivals[k]) * 1e3
                    out[k] = srv.submit(v, lists[i])
            thr = th.Thread(target=submitter)
            thr.start()
            done = []
            for k in range(n_ticks):
                while out[k] is None:
                    time.sleep(5e-5)
                done.append(srv.wait(out[k]))
                done[-1].release()
            thr.join()
            span = time.perf_counter() - t0
            pairs = float(sum(sizes[int(i)] for i in order))
            for r, g in zip(done, lag):
                r.lag_ms = g
            return done, pairs / span

        mix_rate = 0.5 * cap_pairs_s / float(sizes.mean())
        lat_mix, thr_mix = run(list(range(n_lists)), mix_rate, 300, seed + 1)
        big_rate = 0.5 * cap_big_hz
        lat_big, thr_big = run(big, big_rate, 100, seed + 2)
        # the same ticks at lighter loads: where the tail comes from sharing the GPU
        load_curve = {}
        for frac, n_ticks in ((0.25, 100), (0.1, 60)):
            lat_l, thr_l = run(big, frac * cap_big_hz, n_ticks, seed + 4)
            load_curve[f"{int(frac * 100)}%"] = {"rate_hz": frac * cap_big_hz, "ticks": len(lat_l),
                                                 "pairs_per_s": thr_l, **latency_summary(lat_l)}

        # phase 3: the pairs come from the device broad phase (boxes grown by one tick of
        # the fastest motion, 50 * dt), GJK + EPA on them, nothing on the host in between
        cell, margin = 5.0, 50.0 * scene.dt

        def broad_burst(n):
            t0 = time.perf_counter()
            reqs = [srv.submit_broadphase(srv.set_transforms(xfs[k % n_lists]), cell, margin) for k in range(n)]
            found = []
            for r in reqs:
                found.append(int(srv.wait(r).count[0]))
                r.release()
            return time.perf_counter() - t0, found
        broad_burst(n_lists)
        dtb, found = broad_burst(n_lists)
        cap_broad_hz = n_lists / dtb
        broad_rate = 0.5 * cap_broad_hz
        arrivals = W.poisson_arrivals(seed + 3, 200, broad_rate)
        outb = [None] * len(arrivals)
        lagb = [0.0] * len(arrivals)
        t0 = time.perf_counter() + 0.05

        def submitter_b():
            for k in range(len(arrivals)):
                while time.perf_counter() < t0 + arrivals[k]:
                    time.sleep(5e-5)
                v = srv.set_transforms(xfs[k % n_lists])
                lagb[k] = (time.perf_counter() - t0 - arrivals[k]) * 1e3
                outb[k] = srv.submit_broadphase(v, cell, margin)
        thr = th.Thread(target=submitter_b)
        thr.start()
        lat_b = []
        for k in range(len(arrivals)):
            while outb[k] is None:
                time.sleep(5e-5)
            lat_b.append(srv.wait(outb[k]))
            lat_b[-1].release()
            lat_b[-1].lag_ms = lagb[k]
        thr.join()

        # world copy against the transform fused into the kernels (the same 200k-pair
        # ticks): one tick at a time, from the pose upload to results in host memory
        def alone(server, reps=30):
            out = []
            for k in range(reps):
                i = big[k % len(big)]
                t1 = time.perf_counter()
                r = server.wait(server.submit(server.set_transforms(xfs[i]), lists[i]))
                out.append((time.perf_counter() - t1) * 1e3)
                r.release()
            return out
        alone(srv, 6)
        alone_copy = alone(srv)
    finally:
        srv.close()
    fsrv = serving.Server(scene.counts, scene.local, device=device, slots=slots, slot_pairs=262144,
                          max_pairs_in_flight=max_in_flight, world_slots=8, warm_start=True, fused_transform=True)
    try:
        srv = fsrv
        burst(range(n_lists))
        dt_fbig = burst(big)
        alone(fsrv, 6)
        alone_fused = alone(fsrv)
        lat_fbig, thr_fbig = run(big, big_rate, 100, seed + 2)
    finally:
        fsrv.close()

    def pct(v):
        return {"p50_ms": float(np.percentile(v, 50)), "p99_ms": float(np.percentile(v, 99))}
    return {
        "bodies": scene.n_bodies, "mean_vertices": float(scene.counts.mean()),
        "tick_pairs": "log-uniform [1k, 200k] (phase 1), 200k (phase 2)",
        "arrivals": "Poisson", "warm_start": True, "slots": slots, "max_pairs_in_flight": max_in_flight,
        "capacity_pairs_per_s": cap_pairs_s, "capacity_200k_ticks_per_s": cap_big_hz,
        "mixed": {"rate_hz": mix_rate, "ticks": len(lat_mix), "pairs_per_s": thr_mix, **latency_summary(lat_mix)},
        "ticks_200k": {"rate_hz": big_rate, "ticks": len(lat_big), "pairs_per_s": thr_big,
                       **latency_summary(lat_big)},
        "ticks_200k_lighter_loads": load_curve,
        "broadphase_ticks": {"rate_hz": broad_rate, "ticks": len(lat_b), "cell": cell, "margin": margin,
                             "mean_pairs_per_tick": float(np.mean(found)),
                             "capacity_ticks_per_s": cap_broad_hz, **latency_summary(lat_b)},
        "transform_fused_vs_world_copy": {
            "what": "200k-pair ticks: world copy per pose version (k_transform) against the pose applied "
                    "by the GJK/EPA kernels as they read the points (fused_transform); alone = one tick at "
                    "a time, pose upload to results in host memory; poisson = the ticks_200k load",
            "world_copy": {"alone": pct(alone_copy), "capacity_200k_ticks_per_s": cap_big_hz},
            "fused": {"alone": pct(alone_fused), "capacity_200k_ticks_per_s": len(big) / dt_fbig,
                      "poisson": {"rate_hz": big_rate, "pairs_per_s": thr_fbig, **latency_summary(lat_fbig)}},
        },
        "latency": "submit -> results in host memory, host clock; phases: queued for a slot, host "
                   "staging, device (events around the request's work), rest (issue and completion "
                   "detection)",
    }


def load_traffic() -> dict:
    """DRAM traffic of each kernel relative to its algorithmic bytes, from the committed
    ncu summary (profiles/dram_traffic.json: dram__bytes_read.sum + dram__bytes_write.sum
    of one captured launch over the algorithmic bytes of the units it processed)."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def _cpu_run(orc, b, mode, threads, use_ref):
    if use_ref:
        # the reference's own per-pair functions, pair ranges over host threads
        import concurrent.futures as cf
        chunks = np.array_split(np.arange(b.n_pairs), threads)
        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda c: orc.run_reference(b.coords, b.offsets, b.counts, b.pairs[c], mode=mode,
                                                    precision="f32"), chunks))
    else:
        orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=mode, precision="f32", threads=threads)


def run_reference_arm(args):
    rank, world, _ = dist_env()
    world = max(world, args.gpus)
    if rank != 0:
        return
    spec = WORKLOADS[args.workload]
    n = args.pairs or spec["n_pairs"]
    batch = make_batch(args.workload, n, seed=1000)
    from oracle import orc
    orc.build()
    threads = os.cpu_count() or 1
    use_ref = orc.ref_available()
    # each step: a bounded sample (~4 s of CPU work) of the same workload
    n0 = min(n, 4000)
    t = time.perf_counter()
    _cpu_run(orc, batch.subset(np.arange(n0)), orc.MODE_GJK_EPA, threads, use_ref)
    per_pair = (time.perf_counter() - t) / n0
    ns = int(min(n, max(n0, 4.0 / max(per_pair, 1e-9))))
    sample = batch.subset(np.arange(ns))
    for _ in range(args.warmup):
        _cpu_run(orc, sample.subset(np.arange(min(ns, 2000))), orc.MODE_GJK_EPA, threads, use_ref)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        _cpu_run(orc, sample, orc.MODE_GJK_EPA, threads, use_ref)
        times.append(time.perf_counter() - t)
    ms = 1e3 * statistics.mean(times)
    value = ns / (ms / 1e3)
    kind = "reference" if use_ref else "port"
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(spec, n, batch, world),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": kind,
                         "sample": f"first {ns} of {n} pairs per step, {threads} host threads",
                         "cpu_model": cpu_model(), "cores_1": cpu_single_thread(batch)},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    from ogx import build, engine, _lib

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    build.build()
    spec = WORKLOADS[args.workload]
    n = args.pairs or spec["n_pairs"]
    batch = make_batch(args.workload, n, seed=1000 + rank)   # weak scaling: own shard per rank
    alg_bytes = batch.algorithmic_bytes(with_epa=True)
    stream = torch.cuda.Stream()
    ctx = engine.Context(local, stream=stream)
    pool = engine.Pool(ctx, batch.counts)
    coords_pinned = torch.from_numpy(batch.coords).pin_memory()
    pairs_pinned = torch.from_numpy(np.ascontiguousarray(batch.pairs)).pin_memory()
    pool.upload(coords_pinned)
    pairs = pairs_pinned.to(f"cuda:{local}", non_blocking=True)
    out = engine.Results(n, pairs.device)
    torch.cuda.synchronize()
    if args.choice:
        for kind, row in json.loads(args.choice).items():
            for b, (L, K) in enumerate(row):
                ctx.set_kernel_choice(kind, b, L, K)
        choice = ctx.kernel_choice()
    else:
        choice = ctx.autotune(pool, pairs, reps=args.tune_reps) if not args.no_tune else ctx.kernel_choice()
    torch.cuda.synchronize()

    # one instrumented step: per-kernel CUDA-event times and work counts
    ctx.set_timing(True)
    with torch.cuda.stream(stream):
        engine.run(ctx, pool, pairs, engine.MODE_GJK_EPA, out=out)
    ktimes = ctx.kernel_times()
    counts = ctx.work_counts()
    ctx.set_timing(False)
    dist_after = out.dist.cpu().numpy()
    if args.profile_launches:
        torch.cuda.synchronize()
        return

    # the step as one CUDA graph launch (the call's launch sequence is fixed)
    graph = engine.Graph(ctx, pool, pairs, engine.MODE_GJK_EPA, out=out)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            graph.launch()
    launches_per_step = graph.kernel_launches
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with clock_sampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        with torch.cuda.stream(stream):
            for _ in range(args.steps):
                graph.launch()
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n / (ms / 1e3)

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        host_out = {k: torch.empty(v.shape, dtype=v.dtype).pin_memory()
                    for k, v in (("simplex", out.simplex), ("dist", out.dist), ("normal", out.normal),
                                 ("status", out.status))}
        d2h = sum(t.numel() * t.element_size() for t in host_out.values())
        h2d = coords_pinned.numel() * 4 + pairs_pinned.numel() * 4
        e2e_steps = max(3, min(args.steps, 20))

        def e2e_step():
            # one public call from pinned host arrays to pinned host arrays
            engine.streamed(ctx, pool, coords_pinned, pairs_pinned, host_out, chunks=args.chunks)

        for _ in range(max(1, args.warmup)):
            e2e_step()
        torch.cuda.synchronize()
        per_call = []
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            t1 = time.perf_counter()
            e2e_step()
            per_call.append((time.perf_counter() - t1) * 1e3)
        ems = (time.perf_counter() - t0) * 1e3 / e2e_steps
        if world > 1:
            t = torch.tensor([ems], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ems = float(t.item())
        # the same transfers and kernels one after another, with an event between phases
        ph = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        with torch.cuda.stream(stream):
            ph[0].record(stream)
            pool.upload(coords_pinned)
            ph[1].record(stream)
            pairs.copy_(pairs_pinned, non_blocking=True)
            ph[2].record(stream)
            graph.launch()
            ph[3].record(stream)
            for k in ("simplex", "dist", "normal", "status"):
                host_out[k].copy_(getattr(out, k), non_blocking=True)
            ph[4].record(stream)
        torch.cuda.synchronize()
        serial = {name: round(ph[i].elapsed_time(ph[i + 1]), 4)
                  for i, name in enumerate(("pool_upload", "pairs_upload", "kernels", "results_download"))}
        e2e = {"value": world * n / (ems / 1e3), "unit": "pairs/s", "ms_per_step": ems,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "path": f"ogx_gjk_epa_streamed (pool points and pairs up, results down, {args.chunks} chunks "
                       "overlapped with the kernels), pinned host buffers, host clock",
               "calls": e2e_steps,
               "call_ms": {"min": round(min(per_call), 3), "median": round(statistics.median(per_call), 3),
                           "max": round(max(per_call), 3), "each": [round(x, 2) for x in per_call]},
               "serial_phases_ms": serial}

    if rank != 0:
        graph.close()
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # roofline of the dominant kernel
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    tot = sum(t for _, t in ktimes)
    # kernel families: the seven bucket launches of k_gjk (and of k_epa) are one kernel
    fam_ms, fam_n = {}, {}
    for name, t in ktimes:
        f = "k_" + name.split("<")[0].split(">")[0]
        fam_ms[f] = fam_ms.get(f, 0.0) + t
        fam_n[f] = fam_n.get(f, 0) + 1
    dom = max(fam_ms, key=fam_ms.get)
    nv = batch.pair_vertex_counts()
    contact = dist_after <= 0.0
    if dom == "k_gjk":
        # every pair: both bodies' points, the pair, distance and simplex
        dom_bytes, units = int(12 * nv.sum() + 120 * n), n
    elif dom == "k_epa":
        # every contact: both bodies' points, the pair, depth, simplex and normal
        dom_bytes, units = int(12 * nv[contact].sum() + 132 * contact.sum()), int(contact.sum())
    else:
        dom_bytes, units = int(alg_bytes), n
    achieved = dom_bytes / (fam_ms[dom] / 1e3) / 1e9
    traffic = None
    tr = load_traffic().get(dom)
    if tr:
        traffic = tr["traffic_over_algorithmic"] * dom_bytes / fam_n[dom]
    pipeline_gbs = alg_bytes / (ms / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": f"{dom} ({fam_n[dom]} bucket launches)", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_src,
            "traffic": traffic, "traffic_source": tr["source"] if tr else None,
            "algorithmic_bytes_per_launch": dom_bytes / fam_n[dom], "units_per_step": units,
            "kernel_share": fam_ms[dom] / tot if tot else None,
            "pipeline_achieved": pipeline_gbs, "pipeline_frac": pipeline_gbs / peak,
            "algorithmic_bytes_per_step": int(alg_bytes)}

    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(spec, n, batch, world),
        "launch": f"one CUDA graph per step ({launches_per_step} kernels)",
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clk.summary(),
        "roofline": roof,
        "kernels_ms": {k: round(v, 4) for k, v in ktimes},
        "work": counts,
        "kernel_choice": choice,
        "autotuned": not args.no_tune and not args.choice,
    }
    if e2e:
        line["e2e"] = e2e
        if world == 1:
            line["dropin_e2e"] = dropin_e2e(batch)
    parity_rep = os.path.join(ROOT, "profiles", "parity_powerlaw_1M.json")
    if args.workload == "powerlaw" and n == 1_000_000 and os.path.exists(parity_rep):
        # the parity report of this workload (seed 1000) from the full-size GPU test
        # (tests/test_gpu_fullsize.py): every pair against the FP64 oracle
        with open(parity_rep) as f:
            rep = json.load(f)["report"]
        line["parity"] = {k: rep[k] for k in (
            "pairs", "in_band", "verdict_mismatch", "sep_rel_max", "sep_rel_violations", "sep_normal_err_max",
            "sep_normal_violations", "contacts", "depth_err_max", "depth_violations", "oracle_suboptimal",
            "normal_err_max", "normal_equivalent", "normal_violations") if k in rep}
        line["parity"]["source"] = "profiles/parity_powerlaw_1M.json (tests/test_gpu_fullsize.py, same batch)"
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(batch)
        if world == 1:
            line["fp64_plain_1k"] = fp64_plain_report()
    if not args.no_plain and world == 1:
        line["plain_form"] = plain_form_baseline(batch, local)
        if "value" in line["plain_form"]:
            line["plain_form"]["engine_speedup"] = value / line["plain_form"]["value"]
            if e2e:
                line["plain_form"]["engine_e2e_speedup"] = e2e["value"] / line["plain_form"]["e2e"]["value"]
    if not args.no_serving:
        # the server brings its own contexts: release this one (its streams included)
        graph.close()
        del out, pairs
        pool.close()
        ctx.close()
        torch.cuda.empty_cache()
        line["serving"] = serving_report(local)
    print(json.dumps(line), flush=True)
    graph.close()
    pool.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
