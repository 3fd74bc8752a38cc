"""Host-side logic of the benchmark's serving report (no GPU): latency percentiles, the
latency from each tick's scheduled arrival, and the phases of the tail."""
import os
import sys
import types

import numpy as np


def _bench():
    # importing the benchmark sets process-wide CUDA settings: put them back afterwards
    saved, env = sys.argv, dict(os.environ)
    sys.argv = ["bench.py"]
    try:
        import bench
    finally:
        sys.argv = saved
        os.environ.clear()
        os.environ.update(env)
    return bench


def test_latency_summary():
    bench = _bench()
    rng = np.random.default_rng(3)
    reqs = []
    for k in range(200):
        q, stg, dev, rest = 0.01, 0.02, 1.0 + rng.random(), 0.05
        if k == 7:  # one tick that waited for a slot
            q = 5.0
        r = types.SimpleNamespace(phases_ms=(q, stg, dev, rest), lag_ms=0.1 + 0.01 * (k % 3))
        r.latency_ms = q + stg + dev + rest
        reqs.append(r)
    out = bench.latency_summary(reqs)
    lat = np.array([r.latency_ms for r in reqs])
    assert out["p50_ms"] == np.percentile(lat, 50)
    assert out["p99_ms"] == np.percentile(lat, 99)
    sched = lat + np.array([r.lag_ms for r in reqs])
    assert out["from_arrival_p99_ms"] == np.percentile(sched, 99)
    assert abs(out["submit_lag_max_ms"] - 0.12) < 1e-12
    # the slowest ticks are at or above the p99, and the one that queued is among them
    assert out["phases_tail_ms"]["queued"] > 1.0
    assert out["phases_median_ms"]["queued"] == 0.01
