"""Serving loop (ogx_server_*): resident bodies, transform versions, continuous batching
of pair requests.  Results are checked against the batch engine on the same world-space
points and against the FP64 oracle; each request's results must be the same alone and in
a mix of concurrent requests."""
import numpy as np
import pytest

import parity
from ogx import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    return W.serving_scene(seed=31, n_bodies=3000)


def _server(scene, **kw):
    from ogx import serving
    return serving.Server(scene.counts, scene.local, **kw)


def _batch(scene, world, pairs):
    return W.Batch(world, scene.offsets, scene.counts, pairs, "serving")


class _DeviceArray:
    """A raw device pointer viewed as a 1-D float32 array (CUDA array interface)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f4", "data": (ptr, False), "version": 3}


def test_world_copy_is_exact(scene):
    """The transform kernel's world points equal the host formula bit for bit."""
    import torch
    from ogx import pool as P
    with _server(scene, warm_start=False) as srv:
        xf = scene.transforms(5)
        v = srv.set_transforms(xf)
        pts, _ = srv.world_layout(v)
        packed, _ = P.pack(scene.world(xf), scene.counts)
        torch.cuda.synchronize()
        got = torch.as_tensor(_DeviceArray(pts, packed.shape[0]), device="cuda").cpu().numpy()
    assert np.array_equal(got, packed)


def test_request_matches_engine(scene, engine):
    """Without warm starts a request gives exactly the batch engine's results on the
    world-space points of its version."""
    xf = scene.transforms(2)
    pairs = scene.candidate_pairs(2, 4000)
    with _server(scene, warm_start=False) as srv:
        v = srv.set_transforms(xf)
        req = srv.wait(srv.submit(v, pairs))
    ref = engine.query(_batch(scene, scene.world(xf), pairs), engine.MODE_GJK_EPA)
    assert np.array_equal(req.dist, ref["dist"])
    assert np.array_equal(req.normal, ref["normal"])
    assert np.array_equal(req.simplex["witnesses"], ref["simplex"]["witnesses"])
    assert req.latency_ms > 0


def test_same_alone_and_in_the_mix(scene):
    """Continuous batching: requests admitted while others run, over more requests than
    slots; each request's results equal its results when run alone."""
    rng = np.random.default_rng(4)
    ticks = [3, 4, 5, 6]
    with _server(scene, warm_start=False, slots=2, slot_pairs=20000, max_pairs_in_flight=30000) as srv:
        vers = {t: srv.set_transforms(scene.transforms(t)) for t in ticks}
        jobs = []
        for t in ticks:
            for n in (500, 7000, 19000):
                pairs = scene.candidate_pairs(t, n)
                jobs.append((vers[t], pairs[rng.permutation(n)]))
        alone = [srv.wait(srv.submit(v, p)) for v, p in jobs]
        mixed = [srv.submit(v, p) for v, p in jobs]
        mixed = [srv.wait(r) for r in mixed]
    for a, m in zip(alone, mixed):
        assert np.array_equal(a.dist, m.dist)
        assert np.array_equal(a.normal, m.normal)
        assert np.array_equal(a.status, m.status)


def test_warm_start_parity(scene, orc):
    """With warm starts (GJK starting from the previous tick's simplex) the results stay
    within the parity tolerances of the FP64 oracle, tick after tick."""
    with _server(scene, warm_start=True) as srv:
        for t in (10, 11, 12):
            xf = scene.transforms(t)
            pairs = scene.candidate_pairs(t, 6000)
            v = srv.set_transforms(xf)
            req = srv.wait(srv.submit(v, pairs))
            b = _batch(scene, scene.world(xf), pairs)
            o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64",
                        threads=16)
            rep = parity.check(b, req.results(), o, label=f"tick{t}")
            parity.assert_parity(rep, max_witness_mismatch_frac=2e-3)


def _agree(b, a, m):
    """Two engine results of one request agree within the parity tolerances: the same
    verdict outside the contact band, separated distances within 2 REL relative, depths
    within 2 ABS4 (each is within one tolerance of the oracle)."""
    s = parity.pair_scale(b)
    da, dm = a["dist"].astype(np.float64), m["dist"].astype(np.float64)
    band = np.minimum(np.abs(da), np.abs(dm)) <= 2 * parity.BAND * s
    ca, cm = (a["status"] & 8) != 0, (m["status"] & 8) != 0
    assert np.all((ca == cm) | band)
    sep = ~ca & ~cm & ~band
    assert np.all(np.abs(da[sep] - dm[sep]) <= 2 * parity.REL * np.abs(da[sep]))
    con = ca & cm & ~band
    assert np.all(np.abs(da[con] - dm[con]) <= 2 * parity.ABS4)


def _copy(req):
    return {k: v.copy() for k, v in req.results().items()}


def test_warm_start_mix_parity(scene, orc):
    """Continuous batching with warm starts on, as the serving benchmark runs: more
    requests than slots, ticks that share most body pairs, so requests read and write the
    shared warm-start table while others run.  A request's starting simplex then depends on
    what ran before it, so alone and mixed results need not be bit-identical; each must
    meet every parity rule against the FP64 oracle, and the two runs of a request must agree
    within the stated tolerances."""
    rng = np.random.default_rng(12)
    ticks = [20, 21, 22, 23]
    kw = dict(warm_start=True, slots=2, slot_pairs=20000, max_pairs_in_flight=30000)
    jobs = []
    for t in ticks:
        for n in (3000, 9000, 16000):
            jobs.append((t, scene.candidate_pairs(t, n)[rng.permutation(n)]))
    with _server(scene, **kw) as srv:
        vers = {t: srv.set_transforms(scene.transforms(t)) for t in ticks}
        alone = [_copy(srv.wait(srv.submit(vers[t], p))) for t, p in jobs]
    with _server(scene, **kw) as srv:
        vers = {t: srv.set_transforms(scene.transforms(t)) for t in ticks}
        reqs = [srv.submit(vers[t], p) for t, p in jobs]
        mixed = [_copy(srv.wait(r)) for r in reqs]
    with _server(scene, **dict(kw, warm_start=False)) as srv:
        vers = {t: srv.set_transforms(scene.transforms(t)) for t in ticks}
        cold = [_copy(srv.wait(srv.submit(vers[t], p))) for t, p in jobs]
    warm_hits = 0
    for (t, pairs), a, m, c in zip(jobs, alone, mixed, cold):
        b = _batch(scene, scene.world(scene.transforms(t)), pairs)
        o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64", threads=16)
        for res, label in ((a, "alone"), (m, "mixed")):
            parity.assert_parity(parity.check(b, res, o, label=f"tick{t}-{len(pairs)}-{label}"),
                                 max_witness_mismatch_frac=2e-3)
        _agree(b, a, m)
        warm_hits += int(np.sum(a["dist"] != c["dist"]))
    # the warm starts did change starting points (results differ in their last bits from
    # the cold run somewhere), so the mix above really shared the warm-start table
    assert warm_hits > 0


def test_wait_timeout_returns_busy(scene):
    """A wait whose host-side time limit runs out before the request is done returns
    OGX_ERR_BUSY and leaves the request registered; a later wait collects its results."""
    from ogx import _lib
    pairs = scene.candidate_pairs(8, 60000)
    with _server(scene, warm_start=False) as srv:
        v = srv.set_transforms(scene.transforms(8))
        req = srv.submit(v, pairs)
        with pytest.raises(_lib.OgxError) as ei:
            srv.wait(req, timeout_s=1e-6)
        assert ei.value.status == _lib.ERR_BUSY
        assert not req.done
        srv.wait(req, timeout_s=60.0)
        assert req.done and np.isfinite(req.dist).all()


def test_admission_limits(scene):
    from ogx import _lib
    with _server(scene, warm_start=False, slots=1, slot_pairs=1000, max_pairs_in_flight=1000,
                 world_slots=2) as srv:
        v = srv.set_transforms(scene.transforms(0))
        with pytest.raises(_lib.OgxError):
            srv.submit(v, scene.candidate_pairs(0, 1001))
        with pytest.raises(_lib.OgxError):
            srv.submit(v + 1, scene.candidate_pairs(0, 10))
        reqs = [srv.submit(v, scene.candidate_pairs(0, 900)) for _ in range(5)]
        for r in reqs:
            srv.wait(r)
        assert all(np.isfinite(r.dist).all() for r in reqs)
        # the ring holds two versions: two more updates retire version v
        srv.set_transforms(scene.transforms(1))
        v2 = srv.set_transforms(scene.transforms(2))
        with pytest.raises(_lib.OgxError):
            srv.submit(v, scene.candidate_pairs(0, 10))
        assert srv.wait(srv.submit(v2, scene.candidate_pairs(2, 10))).dist.shape == (10,)


def test_broadphase_request_matches_engine(scene, engine):
    """A broad-phase request (device grid, then GJK + EPA, all on the device) gives the
    standalone broad phase's pairs and the batch engine's results on them."""
    import torch
    xf = scene.transforms(7)
    with _server(scene, warm_start=False) as srv:
        v = srv.set_transforms(xf)
        req = srv.wait(srv.submit_broadphase(v, cell=4.0, margin=0.5, max_pairs=100_000))
    n = req.n_run
    assert req.count[1] == 0 and n == req.count[0] > 50
    world = scene.world(xf)
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, scene.counts)
    pool.upload(world)
    br = engine.Broad(ctx, scene.n_bodies)
    pairs, count, _ = br.run(pool, 4.0, 0.5, max_pairs=100_000)
    assert count == req.count[0]
    assert np.array_equal(pairs.cpu().numpy(), req.pairs[:n])
    ref = engine.run(ctx, pool, pairs.contiguous(), engine.MODE_GJK_EPA).to_host()
    ctx.synchronize()
    assert np.array_equal(req.dist[:n], ref["dist"])
    assert np.array_equal(req.normal[:n], ref["normal"])


def test_latency_phases(scene):
    """The latency breakdown of a request adds up: queued, staging, device and the rest
    are non-negative (the rest within clock skew) and sum to the latency."""
    pairs = scene.candidate_pairs(4, 20000)
    with _server(scene) as srv:
        for t in range(3):
            v = srv.set_transforms(scene.transforms(4 + t))
            req = srv.wait(srv.submit(v, pairs))
            q, stg, dev, rest = req.phases_ms
            assert q >= 0 and stg >= 0 and dev > 0, req.phases_ms
            assert rest > -0.05, req.phases_ms
            assert abs(q + stg + dev + rest - req.latency_ms) < 1e-6
            assert dev <= req.latency_ms + 0.05


def test_result_sets_recycled(scene, engine):
    """A released request's page-locked arrays serve the next request (no pinned
    allocation per request), and its results are still exact; release() before the
    request was waited for is refused."""
    xf = scene.transforms(9)
    with _server(scene, warm_start=False, slots=2, result_sets=1) as srv:
        v = srv.set_transforms(xf)
        first = srv.submit(v, scene.candidate_pairs(9, 3000))
        with pytest.raises(RuntimeError):
            first.release()
        srv.wait(first)
        addr = first.dist.ctypes.data
        first.release()
        assert first.dist is None
        pairs = scene.candidate_pairs(9, 5000)
        second = srv.wait(srv.submit(v, pairs))
        assert second.dist.ctypes.data == addr
        ref = engine.query(_batch(scene, scene.world(xf), pairs), engine.MODE_GJK_EPA)
        assert np.array_equal(second.dist, ref["dist"])
        assert np.array_equal(second.simplex["witnesses"], ref["simplex"]["witnesses"])
        # while the one set is held by an unreleased request, the next one gets a new set
        third = srv.submit(v, scene.candidate_pairs(9, 3000))
        assert third.dist.ctypes.data != addr
        srv.wait(third)


def test_concurrent_transform_uploads(scene, engine):
    """Pose uploads from several threads at once each get their own version, and each of
    the resident versions holds exactly its own poses."""
    from concurrent.futures import ThreadPoolExecutor
    ticks = [11, 12, 13, 14, 15, 16]
    pairs = scene.candidate_pairs(16, 2000)
    with _server(scene, warm_start=False, world_slots=4) as srv:
        with ThreadPoolExecutor(3) as ex:
            vers = dict(ex.map(lambda t: (t, srv.set_transforms(scene.transforms(t))), ticks))
        assert sorted(vers.values()) == list(range(min(vers.values()), min(vers.values()) + len(ticks)))
        resident = sorted(vers, key=vers.get)[-4:]
        for t in resident:
            req = srv.wait(srv.submit(vers[t], pairs))
            ref = engine.query(_batch(scene, scene.world(scene.transforms(t)), pairs), engine.MODE_GJK_EPA)
            assert np.array_equal(req.dist, ref["dist"]), t


def test_non_finite_pose_refused(scene):
    """A pose update holding a NaN or an infinity is refused (it would put non-finite
    points into the world copy every request of the version reads); the server keeps
    working with the versions it has."""
    from ogx import _lib
    with _server(scene, warm_start=False) as srv:
        v = srv.set_transforms(scene.transforms(1))
        xf = scene.transforms(2)
        xf[17, 4] = np.nan
        with pytest.raises(_lib.OgxError) as ei:
            srv.set_transforms(xf)
        assert ei.value.status == -1 and "body 17" in str(ei.value)
        xf[17, 4] = 0.0
        xf[5, 10] = np.inf
        with pytest.raises(_lib.OgxError):
            srv.set_transforms(xf)
        req = srv.wait(srv.submit(v, scene.candidate_pairs(1, 500)))
        assert np.isfinite(req.dist).all()


def test_fused_transform_matches_host_build(scene, twin):
    """A fused-transform server (no world copy: the kernels apply each body's pose as
    they read its points) gives the host build's posed pipeline results on the same
    request, as the world-frame kernels give the host build's world-frame results."""
    xf = scene.transforms(7)
    pairs = scene.candidate_pairs(7, 12000)
    with _server(scene, warm_start=False, fused_transform=True) as srv:
        req = srv.wait(srv.submit(srv.set_transforms(xf), pairs))
        res = _copy(req)
    h = twin.run(W.Batch(scene.local, scene.offsets, scene.counts, pairs, "serving"), xf=xf)
    same = res["dist"] == h["dist"]
    assert same.mean() > 0.995, same.mean()
    close = np.abs(res["dist"].astype(np.float64) - h["dist"]) <= 1e-6 * np.maximum(1, np.abs(h["dist"]))
    assert close.mean() > 0.999


def test_fused_transform_parity(scene, orc, twin):
    """Fused-transform ticks with warm starts meet every parity rule against the FP64
    oracle on their world points (pose_point of every body point), and agree with a
    world-copy server's results on the same tick.  The two servers' world points differ
    in their last bits (an FP32 multiply-add chain against a product rounded once from
    FP64: about one ulp of coordinates up to 50), so the comparison allows twice that
    difference on top of the parity tolerances."""
    with _server(scene, warm_start=True, fused_transform=True) as fused, _server(scene, warm_start=True) as copy:
        for t in (30, 31, 32):
            xf = scene.transforms(t)
            pairs = scene.candidate_pairs(t, 8000)
            a = _copy(fused.wait(fused.submit(fused.set_transforms(xf), pairs)))
            c = _copy(copy.wait(copy.submit(copy.set_transforms(xf), pairs)))
            posed = twin.pose_points(scene.counts, scene.local, xf)
            b = _batch(scene, posed, pairs)
            o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64",
                        threads=16)
            parity.assert_parity(parity.check(b, a, o, label=f"fused tick{t}"), max_witness_mismatch_frac=2e-3)
            dp = float(np.abs(posed.astype(np.float64) - scene.world(xf)).max())
            assert dp <= 1e-5
            da, dc = a["dist"].astype(np.float64), c["dist"].astype(np.float64)
            band = np.minimum(np.abs(da), np.abs(dc)) <= 2 * parity.BAND * parity.pair_scale(b) + 2 * dp
            ca, cc = (a["status"] & 8) != 0, (c["status"] & 8) != 0
            assert np.all((ca == cc) | band)
            sep = ~ca & ~cc & ~band
            assert np.all(np.abs(da[sep] - dc[sep]) <= 2 * parity.REL * np.abs(da[sep]) + 2 * dp)
            con = ca & cc & ~band
            assert np.all(np.abs(da[con] - dc[con]) <= 2 * parity.ABS4 + 2 * dp)


def test_fused_transform_refuses_world_copy_uses(scene):
    """A fused-transform server keeps no world copy: broad-phase requests and the world
    layout are refused with OGX_ERR_INVALID, pair requests run."""
    from ogx import _lib
    with _server(scene, warm_start=False, fused_transform=True) as srv:
        v = srv.set_transforms(scene.transforms(1))
        with pytest.raises(_lib.OgxError):
            srv.world_layout(v)
        with pytest.raises(_lib.OgxError):
            srv.submit_broadphase(v, cell=5.0, margin=0.5, max_pairs=1000)
        assert srv.wait(srv.submit(v, scene.candidate_pairs(1, 100))).dist.shape == (100,)


def test_admission_by_device_memory(scene):
    """Requests are admitted by device memory: with a byte budget of one and a half
    requests' working memory, requests run one at a time (the peak bytes in flight is one
    request's), and each result equals the same request run alone.  Without a budget the
    server derives one from the free device memory."""
    n = 10000
    with _server(scene, warm_start=False) as srv:
        adm = srv.admission()
        assert adm["bytes_per_pair"] > 200 and adm["max_bytes_in_flight"] > 10 * n * adm["bytes_per_pair"]
        v = srv.set_transforms(scene.transforms(2))
        pairs = [scene.candidate_pairs(2, n)[np.random.default_rng(k).permutation(n)] for k in range(4)]
        alone = [_copy(srv.wait(srv.submit(v, p))) for p in pairs]
    budget = int(1.5 * n * adm["bytes_per_pair"])
    with _server(scene, warm_start=False, max_bytes_in_flight=budget) as srv:
        v = srv.set_transforms(scene.transforms(2))
        reqs = [srv.submit(v, p) for p in pairs]
        got = [_copy(srv.wait(r)) for r in reqs]
        adm2 = srv.admission()
    assert adm2["max_bytes_in_flight"] == budget
    assert adm2["peak_bytes_in_flight"] == n * adm["bytes_per_pair"]
    for a, g in zip(alone, got):
        assert np.array_equal(a["dist"], g["dist"]) and np.array_equal(a["normal"], g["normal"])
