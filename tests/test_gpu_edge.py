"""Edge cases of the GPU engine: empty batches, invalid indices, degenerate bodies,
large bodies (memory-streamed bucket), determinism, mode consistency."""
import ctypes

import numpy as np
import pytest

from ogx import workloads as W

pytestmark = pytest.mark.gpu

# agreement of separated-pair normals between a fused GJK+EPA call and GJK then EPA-only
SEP_NORMAL_AGREE = 1e-5


def test_empty_batch(engine):
    import torch
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, np.array([4, 4], np.int32))
    pool.upload(np.zeros((8, 3), np.float32))
    pairs = torch.zeros((0, 2), dtype=torch.int32, device="cuda")
    res = engine.run(ctx, pool, pairs)
    ctx.synchronize()
    assert res.dist.numel() == 0
    assert ctx.last_launches == 0


def test_bad_indices_flagged(engine):
    import torch
    from ogx import _lib
    ctx = engine.Context(0)
    b = W.plain(seed=3, n_pairs=4)
    pool = engine.Pool(ctx, b.counts)
    pool.upload(b.coords)
    pairs = torch.tensor([[0, 1], [0, 99], [-1, 2], [2, 3]], dtype=torch.int32, device="cuda")
    out = engine.run(ctx, pool, pairs).to_host()
    st = out["status"]
    assert st[1] & _lib.PAIR_BAD_INPUT and st[2] & _lib.PAIR_BAD_INPUT
    assert np.isnan(out["dist"][1]) and np.isnan(out["dist"][2])
    assert not (st[0] & _lib.PAIR_BAD_INPUT) and np.isfinite(out["dist"][[0, 3]]).all()


def test_invalid_arguments_raise(engine):
    from ogx import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.ogx_ctx_create(0, None, None, ctypes.byref(h)) == 0
    try:
        pool = ctypes.c_void_p()
        bad = np.array([3, 0], np.int32)
        rc = lib.ogx_pool_create(h, 2, bad.ctypes.data, ctypes.byref(pool))
        assert rc == -1 and b"points" in lib.ogx_last_error()
        cfg = _lib.default_config()
        cfg.epa_max_iter = 1000
        assert lib.ogx_ctx_set_config(h, ctypes.byref(cfg)) == -1
        assert lib.ogx_gjk(h, None, 1, None, None, None, None) == -1
    finally:
        lib.ogx_ctx_destroy(h)


def test_degenerate_bodies(engine, orc):
    """Single points, segments, identical and touching bodies follow the reference's
    semantics (e.g. identical bodies: GJK starts at v = 0, EPA's simplex growth finds
    no new point and reports depth 0, GJK/cpu/EPA.c:378-419)."""
    rng = np.random.default_rng(5)
    bodies = [
        np.array([[0, 0, 0]], np.float32), np.array([[3, 0, 0]], np.float32),      # point-point
        np.array([[0, 0, 0], [1, 0, 0]], np.float32), np.array([[0.5, 2, 0]], np.float32),  # segment-point
        W.cube(), W.cube(),                                                          # identical cubes
        W.cube(), (W.cube() + np.float32([2.0, 0, 0])),                              # touching faces
        W.cube(), (W.cube() + np.float32([0.5, 0.3, 0.1])),                          # overlapping cubes
        rng.normal(size=(7, 3)).astype(np.float32), np.array([[0.0, 0.0, 0.0]], np.float32),
    ]
    b = W.from_bodies(bodies)
    res = engine.query(b, engine.MODE_GJK_EPA)
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64")
    assert abs(res["dist"][0] - 3.0) < 1e-6
    assert np.all(np.abs(res["dist"] - o["dist"]) < 1e-5), (res["dist"], o["dist"])
    assert abs(res["dist"][4] + 1.5) < 1e-5  # overlapping cubes: depth 1.5 along x
    assert np.all(np.isfinite(res["dist"]))
    assert np.all(np.abs(np.linalg.norm(res["normal"], axis=1) - 1) < 1e-5)


def test_large_bodies_streamed_bucket(engine, orc):
    """Bodies above 512 points run from memory instead of registers."""
    import parity
    b = W.ellipsoid(seed=8, n_pairs=300, lo=600, hi=3000)
    res = engine.query(b, engine.MODE_GJK_EPA)
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64", threads=16)
    parity.assert_parity(parity.check(b, res, o, label="large"), max_witness_mismatch_frac=0.02)


def test_deterministic_and_batch_independent(engine):
    """Each pair's result is the same alone and inside a larger mixed batch."""
    b = W.powerlaw(seed=9, n_pairs=4000)
    full = engine.query(b, engine.MODE_GJK_EPA)
    again = engine.query(b, engine.MODE_GJK_EPA)
    for k in ("dist", "normal", "status"):
        assert np.array_equal(full[k], again[k])
    sub = np.arange(0, 4000, 37)
    part = engine.query(b.subset(sub), engine.MODE_GJK_EPA)
    assert np.array_equal(part["dist"], full["dist"][sub])
    assert np.array_equal(part["normal"], full["normal"][sub])


def test_epa_only_matches_fused(engine):
    import torch
    b = W.ellipsoid(seed=10, n_pairs=2000)
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, b.counts)
    pool.upload(b.coords)
    pairs = torch.from_numpy(b.pairs).cuda()
    fused = engine.run(ctx, pool, pairs, engine.MODE_GJK_EPA).to_host()
    r = engine.Results(b.n_pairs, pairs.device, with_normals=True)
    engine.run(ctx, pool, pairs, engine.MODE_GJK, out=r)
    engine.run(ctx, pool, pairs, engine.MODE_EPA, out=r)
    sep = r.to_host()
    assert np.array_equal(fused["dist"], sep["dist"])
    # contacts run the same EPA; a separated pair's normal comes from the GJK pass's own
    # closest point in the fused call and is re-solved from the stored simplex in the
    # EPA-only call: the two agree to that point's FP32 accuracy (a few 1e-6)
    assert np.allclose(fused["normal"], sep["normal"], atol=SEP_NORMAL_AGREE)


def test_reference_tolerance_mode(engine, orc):
    """With the reference's FP32 constants the engine stays within the reference's own
    CPU-vs-GPU tolerance (1e-3, examples/main.cpp:184-188) of its FP32 CPU result."""
    from ogx import _lib
    b = W.ellipsoid(seed=12, n_pairs=5000)
    res = engine.query(b, engine.MODE_GJK_EPA, config=_lib.reference_config())
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f32")
    diff = np.abs(res["dist"] - o["dist"])
    assert np.mean(diff <= 1e-3) > 0.995, np.mean(diff <= 1e-3)


def test_graph_replay_matches_calls(engine):
    """A captured call replayed as one CUDA graph launch gives the direct call's results,
    also after the pair buffer's contents change."""
    import torch
    b = W.powerlaw(seed=41, n_pairs=4000)
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, b.counts)
    pool.upload(b.coords)
    pairs = torch.from_numpy(np.ascontiguousarray(b.pairs)).cuda()
    ref = engine.run(ctx, pool, pairs, engine.MODE_GJK_EPA).to_host()
    g = engine.Graph(ctx, pool, pairs, engine.MODE_GJK_EPA)
    assert g.kernel_launches == ctx.last_launches
    for _ in range(2):
        got = g.launch().to_host()
        ctx.synchronize()
        assert np.array_equal(got["dist"], ref["dist"]) and np.array_equal(got["normal"], ref["normal"])
    flipped = pairs.flip(0).contiguous()
    pairs.copy_(flipped)
    ref2 = engine.run(ctx, pool, flipped, engine.MODE_GJK_EPA).to_host()
    got2 = g.launch().to_host()
    ctx.synchronize()
    assert np.array_equal(got2["dist"], ref2["dist"])
    g.close()


def test_pinned_upload_reads_host_directly(engine):
    """A page-locked source is packed straight from host memory; the pool equals the one
    staged from a pageable array."""
    import torch
    b = W.powerlaw(seed=43, n_pairs=3000)
    ctx = engine.Context(0)
    pa, pb = engine.Pool(ctx, b.counts), engine.Pool(ctx, b.counts)
    pa.upload(b.coords)
    pinned = torch.from_numpy(b.coords).pin_memory()
    pb.upload(pinned)
    ctx.synchronize()
    pairs = torch.from_numpy(np.ascontiguousarray(b.pairs)).cuda()
    ra = engine.run(ctx, pa, pairs).to_host()
    rb = engine.run(ctx, pb, pairs).to_host()
    ctx.synchronize()
    assert np.array_equal(ra["dist"], rb["dist"]) and np.array_equal(ra["normal"], rb["normal"])


def test_pageable_upload_direct_or_staged_alike(engine, monkeypatch):
    """A pageable source is packed straight from host memory where the device reads
    pageable memory (a Grace system), else staged through pinned memory
    (OGX_UPLOAD_STAGED=1): the same pool either way, and the call returns with the
    source no longer needed (overwriting it afterwards changes nothing)."""
    import torch
    b = W.powerlaw(seed=45, n_pairs=3000)
    ctx = engine.Context(0)
    pairs = torch.from_numpy(np.ascontiguousarray(b.pairs)).cuda()
    res = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("OGX_UPLOAD_STAGED", mode)
        src = b.coords.copy()
        pool = engine.Pool(ctx, b.counts)
        pool.upload(src)
        src[:] = np.nan  # the call returned: the pool no longer reads the source
        res[mode] = engine.run(ctx, pool, pairs).to_host()
        ctx.synchronize()
    for k in ("dist", "normal", "status"):
        assert np.array_equal(res["0"][k], res["1"][k])
    assert np.isfinite(res["0"]["dist"]).all()


@pytest.mark.parametrize("chunks", [1, 3, 8])
def test_streamed_call_matches_batched(engine, chunks):
    """The host-to-host call with overlapped chunks gives the results of the device
    call on the same pool, for pairs that reference bodies in any order."""
    import torch
    b = W.powerlaw(seed=44, n_pairs=5000)
    pairs = np.ascontiguousarray(b.pairs.copy())
    pairs[::7] = pairs[::7][:, ::-1]            # some pairs reversed
    pairs[100:200] = pairs[4800:4900]           # some pairs refer to late bodies early
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, b.counts)
    coords = torch.from_numpy(b.coords).pin_memory()
    out = engine.streamed(ctx, pool, coords, pairs, chunks=chunks)
    ref = engine.run(ctx, pool, torch.from_numpy(pairs).cuda()).to_host()
    ctx.synchronize()
    assert np.array_equal(out["dist"], ref["dist"])
    assert np.array_equal(out["normal"], ref["normal"])
    assert np.array_equal(out["simplex"]["witnesses"], ref["simplex"]["witnesses"])


@pytest.mark.parametrize("lanes", [1, 3, 8])
def test_streamed_ranges_match_batched(engine, lanes):
    """Caller-given pair ranges (uneven, some empty, bad indices inside) and lane counts
    give the results of the device call; bad range bounds are refused."""
    import torch
    from ogx import _lib
    b = W.powerlaw(seed=45, n_pairs=3000)
    pairs = np.ascontiguousarray(b.pairs.copy())
    pairs[50] = (0, 10 ** 7)                     # flagged, needs no body
    pairs[2990] = (3, 1)                         # last range refers to early bodies
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, b.counts)
    coords = torch.from_numpy(b.coords).pin_memory()
    bounds = [0, 10, 10, 700, 701, 2500, 2999, 3000]
    out = engine.streamed(ctx, pool, coords, pairs, bounds=bounds, lanes=lanes)
    ref = engine.run(ctx, pool, torch.from_numpy(pairs).cuda()).to_host()
    ctx.synchronize()
    assert out["status"][50] & _lib.PAIR_BAD_INPUT
    ok = np.ones(len(pairs), bool)
    ok[50] = False
    assert np.array_equal(out["dist"][ok], ref["dist"][ok])
    assert np.array_equal(out["normal"], ref["normal"], equal_nan=True)
    assert np.array_equal(out["simplex"]["witnesses"][ok], ref["simplex"]["witnesses"][ok])
    assert np.array_equal(out["status"], ref["status"])
    for bad in ([0, 5, 3, 3000], [1, 3000], [0, 2999], [0]):
        with pytest.raises(RuntimeError):
            engine.streamed(ctx, pool, coords, pairs, bounds=bad, lanes=lanes)
    with pytest.raises(RuntimeError):
        engine.streamed(ctx, pool, coords, pairs, bounds=[0, 3000], lanes=9)


def test_stage_timeline(engine):
    """The stage timeline of a concurrent call names every bucket's GJK and EPA kernel and
    the passes after them, with times from the call's start that end at the join; results
    are unchanged by recording it."""
    import torch
    b = W.powerlaw(seed=46, n_pairs=20000)
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, b.counts)
    pool.upload(b.coords)
    pairs = torch.from_numpy(np.ascontiguousarray(b.pairs)).cuda()
    ref = engine.run(ctx, pool, pairs).to_host()
    ctx.set_stage_timeline(True)
    got = engine.run(ctx, pool, pairs).to_host()
    tl = dict(ctx.stage_timeline())
    ctx.set_stage_timeline(False)
    ctx.synchronize()
    assert np.array_equal(got["dist"], ref["dist"])
    names = {f"gjk{s}" for s in ("<=16", "<=32", "<=64", "<=128", "<=256", "<=512", ">512")}
    names |= {n.replace("gjk", "epa") for n in names} | {"refine", "epa_late", "epa_spill", "polish", "end"}
    assert set(tl) == names, sorted(tl)
    assert all(0.0 <= v <= tl["end"] + 1e-3 for v in tl.values()), tl
    assert tl["refine"] <= tl["epa_late"] + 1e-3


def test_non_finite_coordinates_flagged(engine):
    """A body with a NaN or an infinite coordinate makes its pairs bad input -- status
    OGX_PAIR_BAD_INPUT, distance NaN, normal (1,0,0), simplex with no vertex -- through the
    engine, the streamed call and the reference-compatible API; every other pair's results
    are those of the same batch with finite points, and an upload of finite points clears
    the mark.  (The reference checks no input; a non-finite point there gives undefined
    results.)"""
    import torch
    from ogx import _lib, refapi
    b = W.ellipsoid(seed=45, n_pairs=600)
    coords = b.coords.copy()
    coords[b.offsets[3] + 1, 0] = np.nan
    coords[b.offsets[10], 2] = np.inf
    coords[b.offsets[401] + b.counts[401] - 1, 1] = -np.inf
    flagged = np.isin(b.pairs, [3, 10, 401]).any(axis=1)
    assert flagged.sum() == 3
    bad = W.Batch(coords, b.offsets, b.counts, b.pairs, "non-finite")
    ref = engine.query(b, engine.MODE_GJK_EPA)

    def check(got, with_status=True):
        if with_status:
            assert np.all(got["status"][flagged] & _lib.PAIR_BAD_INPUT)
            assert not np.any(got["status"][~flagged] & _lib.PAIR_BAD_INPUT)
            assert np.all(got["simplex"]["nvrtx"][flagged] == 0)
        assert np.isnan(got["dist"][flagged]).all()
        assert np.array_equal(got["normal"][flagged], np.tile(np.float32([1, 0, 0]), (3, 1)))
        assert np.array_equal(got["dist"][~flagged], ref["dist"][~flagged])
        assert np.array_equal(got["normal"][~flagged], ref["normal"][~flagged])

    check(engine.query(bad, engine.MODE_GJK_EPA))
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, b.counts)
    check(engine.streamed(ctx, pool, torch.from_numpy(coords).pin_memory(), np.ascontiguousarray(b.pairs)))
    pool.upload(b.coords)  # finite points again: nothing flagged
    again = engine.run(ctx, pool, torch.from_numpy(np.ascontiguousarray(b.pairs)).cuda()).to_host()
    ctx.synchronize()
    assert np.array_equal(again["dist"], ref["dist"]) and not np.any(again["status"] & _lib.PAIR_BAD_INPUT)
    bd1, bd2, _ = refapi.from_batch(bad)
    smp, dist, nrm = refapi.compute_gjk_epa(bd1, bd2)
    check({"dist": dist, "normal": nrm, "simplex": smp}, with_status=False)
    assert np.all(smp["nvrtx"][flagged] == 0)
