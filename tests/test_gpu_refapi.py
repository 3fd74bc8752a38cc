"""The reference-compatible entry points (OpenGJK-GPU's host API names and conventions)
agree with the engine API and with the FP64 oracle."""
import numpy as np
import pytest

import parity
from ogx import refapi, workloads as W

pytestmark = pytest.mark.gpu

# agreement of separated-pair normals between a fused GJK+EPA call and GJK then EPA-only
# (the fused call uses its GJK closest point, EPA-only re-solves it from the simplex)
SEP_NORMAL_AGREE = 1e-5


def _res(smp, dist, nrm, status_contact):
    return {"dist": dist, "simplex": smp, "normal": nrm, "status": status_contact}


def test_compute_gjk_epa_matches_engine(engine, orc):
    b = W.ellipsoid(seed=41, n_pairs=3000)
    bd1, bd2, _ = refapi.from_batch(b)
    smp, dist, nrm = refapi.compute_gjk_epa(bd1, bd2)
    eng = engine.query(b, engine.MODE_GJK_EPA)
    assert np.array_equal(dist, eng["dist"])
    assert np.array_equal(nrm, eng["normal"])
    assert refapi.last_gpu_ms() > 0.0
    o = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f64")
    parity.assert_parity(parity.check(b, _res(smp, dist, nrm, eng["status"]), o, label="refapi"))


def test_distances_then_epa_matches_fused(engine):
    """GJK::GPU::computeDistances followed by GJK::GPU::computeEPA on its outputs equals
    GJK::GPU::computeGJKAndEPA (the reference's API cross-consistency check,
    examples/main.cpp:378-644)."""
    b = W.powerlaw(seed=42, n_pairs=3000)
    bd1, bd2, _ = refapi.from_batch(b)
    smp, dist = refapi.compute_minimum_distance(bd1, bd2)
    nrm = refapi.compute_epa(bd1, bd2, smp, dist)
    smp2, dist2, nrm2 = refapi.compute_gjk_epa(bd1, bd2)
    assert np.array_equal(dist, dist2)
    # separated normals: the fused call's from its GJK closest point, the EPA-only call's
    # re-solved from the simplex (they agree to that point's FP32 accuracy)
    assert np.allclose(nrm, nrm2, atol=SEP_NORMAL_AGREE)
    w1, w2, n3 = refapi.compute_collision_information(bd1, bd2, smp.copy(), dist.copy())
    assert np.allclose(w1, smp2["witnesses"][:, 0], atol=1e-6)
    assert np.allclose(n3, nrm2, atol=SEP_NORMAL_AGREE)


def test_indexed_matches_pairwise(engine):
    b = W.ellipsoid(seed=43, n_pairs=2000)
    bd1, bd2, pool = refapi.from_batch(b)
    rng = np.random.default_rng(0)
    pairs = np.ascontiguousarray(b.pairs[rng.permutation(b.n_pairs)])
    smp, dist, nrm = refapi.compute_gjk_epa_indexed(pool, pairs)
    eng = engine.query(W.Batch(b.coords, b.offsets, b.counts, pairs, "perm"), engine.MODE_GJK_EPA)
    assert np.array_equal(dist, eng["dist"])
    s2, d2 = refapi.compute_minimum_distance_indexed(pool, pairs)
    sep = dist > 0
    assert np.array_equal(d2[sep], dist[sep])


def test_usage_known_answers(engine):
    """The reference's usage examples through the compatible API: userP/userQ distance
    3.653650 (README.md:113) and the rotated-cube EPA depth (FP64 oracle: 1.5)."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "usage_gjk.npz"))
    b = W.Batch(z["coords"], z["offsets"], z["counts"], z["pairs"], "usage")
    bd1, bd2, _ = refapi.from_batch(b)
    smp, dist = refapi.compute_minimum_distance(bd1, bd2)
    assert f"{dist[0]:.6f}" == "3.653650"
    assert [f"{x:.6f}" for x in smp["witnesses"][0, 0]] == ["1.025173", "1.490318", "0.255463"]
    c = W.from_bodies([W.cube(), W.rotated_cube()])
    bd1, bd2, _ = refapi.from_batch(c)
    smp, dist, nrm = refapi.compute_gjk_epa(bd1, bd2)
    z2 = np.load(os.path.join(os.path.dirname(__file__), "golden", "usage_epa.npz"))
    assert abs(dist[0] - z2["f64_dist"][0]) < 1e-4


def test_device_api(engine):
    """Mid-level and indexed *_device entry points: descriptors and coordinates in device
    memory (as a caller that transforms its pool with its own kernels provides them)."""
    import ctypes
    import torch
    from ogx import _lib
    L = refapi.lib()
    b = W.ellipsoid(seed=44, n_pairs=1500)
    coords = torch.from_numpy(b.coords.copy()).cuda()
    desc = np.zeros(b.n_bodies, dtype=_lib.POLYTOPE_DTYPE)
    desc["numpoints"] = b.counts
    desc["coord"] = coords.data_ptr() + 12 * b.offsets.astype(np.uint64)
    d_desc = torch.from_numpy(desc.view(np.uint8).copy()).cuda()
    d_pairs = torch.from_numpy(np.ascontiguousarray(b.pairs)).cuda()
    d_smp = torch.zeros((b.n_pairs, 27), dtype=torch.int32, device="cuda")
    d_dist = torch.zeros(b.n_pairs, dtype=torch.float32, device="cuda")
    d_nrm = torch.zeros((b.n_pairs, 3), dtype=torch.float32, device="cuda")
    P = ctypes.c_void_p
    _lib.check(L.ogx_compute_minimum_distance_indexed_device(b.n_pairs, P(d_desc.data_ptr()), P(d_pairs.data_ptr()),
                                                             P(d_smp.data_ptr()), P(d_dist.data_ptr())))
    _lib.check(L.ogx_compute_epa_indexed_device(b.n_pairs, P(d_desc.data_ptr()), P(d_pairs.data_ptr()),
                                                P(d_smp.data_ptr()), P(d_dist.data_ptr()), P(d_nrm.data_ptr())))
    eng = engine.query(b, engine.MODE_GJK_EPA)
    assert np.array_equal(d_dist.cpu().numpy(), eng["dist"])
    assert np.allclose(d_nrm.cpu().numpy(), eng["normal"], atol=SEP_NORMAL_AGREE)
    # bd1 / bd2 descriptor arrays in device memory
    d1 = torch.from_numpy(desc[b.pairs[:, 0]].view(np.uint8).copy()).cuda()
    d2 = torch.from_numpy(desc[b.pairs[:, 1]].view(np.uint8).copy()).cuda()
    d_dist2 = torch.zeros_like(d_dist)
    _lib.check(L.ogx_compute_minimum_distance_device(b.n_pairs, P(d1.data_ptr()), P(d2.data_ptr()),
                                                     P(d_smp.data_ptr()), P(d_dist2.data_ptr())))
    g = engine.query(b, engine.MODE_GJK)
    assert np.array_equal(d_dist2.cpu().numpy(), g["dist"])


def test_empty_and_invalid(engine):
    import ctypes
    from ogx import _lib
    L = refapi.lib()
    assert L.ogx_compute_gjk_epa(0, None, None, None, None, None) == 0  # n <= 0: no work
    bad = np.zeros(2, dtype=_lib.POLYTOPE_DTYPE)  # numpoints 0
    smp = np.zeros(1, _lib.SIMPLEX_DTYPE)
    dist = np.zeros(1, np.float32)
    rc = L.ogx_compute_minimum_distance(1, bad[:1].ctypes.data, bad[1:].ctypes.data, smp.ctypes.data,
                                        dist.ctypes.data)
    assert rc == -1 and b"numpoints" in L.ogx_last_error()


def test_host_calls_pack_in_place_or_gathered_alike(engine, monkeypatch):
    """Host-buffer calls build the pool either on the device straight from the caller's
    arrays (devices that read pageable host memory) or from a host gather into pinned
    staging (OGX_COMPAT_GATHER=1, and every other device): the same bits, non-finite
    bodies flagged either way."""
    b = W.powerlaw(seed=44, n_pairs=4000)
    coords = b.coords.copy()
    coords[b.offsets[7] + 2, 1] = np.nan  # body 7: pair 3 is bad input
    b = W.Batch(coords, b.offsets, b.counts, b.pairs, b.name)
    bd1, bd2, pool = refapi.from_batch(b)
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("OGX_COMPAT_GATHER", mode)
        smp, dist, nrm = refapi.compute_gjk_epa(bd1, bd2)
        smp_i, dist_i, nrm_i = refapi.compute_gjk_epa_indexed(pool, np.ascontiguousarray(b.pairs))
        out[mode] = (smp.tobytes(), dist.copy(), nrm.copy(), smp_i.tobytes(), dist_i.copy())
    a, g = out["0"], out["1"]
    assert a[0] == g[0] and a[3] == g[3]
    for x, y in ((a[1], g[1]), (a[2], g[2]), (a[4], g[4])):
        assert np.array_equal(x, y, equal_nan=True)
    assert np.isnan(a[1][3]) and np.isfinite(np.delete(a[1], 3)).all()
