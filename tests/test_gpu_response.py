"""Collision response (ogx_contact_response) against a float64 restatement of the same
impulse model on the host, and the sign convention end to end: bodies pushed apart."""
import numpy as np
import pytest

from ogx import workloads as W

pytestmark = pytest.mark.gpu


def _qrot(q, v):
    u, w = q[..., :3], q[..., 3:4]
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def _host_response(state, pairs, dist, nrm, wit, eps, beta, e_rest, e_thr):
    n = state["pos"].shape[0]
    dv = np.zeros((n, 3)); dw = np.zeros((n, 3)); dp = np.zeros((n, 3))
    S = {k: v.astype(np.float64) for k, v in state.items()}
    for p in range(pairs.shape[0]):
        a, b = pairs[p]
        if dist[p] > eps or a == b:
            continue
        nn = nrm[p].astype(np.float64)
        if np.linalg.norm(nn) < 1e-4:
            continue
        nn /= np.linalg.norm(nn)
        ima, imb = S["inv_mass"][a], S["inv_mass"][b]
        ra = wit[p, 0] - S["pos"][a]
        rb = wit[p, 1] - S["pos"][b]
        if dist[p] < 0 and ima + imb > 0:
            corr = beta * (-dist[p]) / (ima + imb)
            dp[a] -= corr * ima * nn
            dp[b] += corr * imb * nn
        rv = (S["vel"][b] + np.cross(S["ang"][b], rb)) - (S["vel"][a] + np.cross(S["ang"][a], ra))
        vn = rv @ nn
        if vn > 0:
            continue
        qa, qb = S["quat"][a], S["quat"][b]
        qai, qbi = qa * [-1, -1, -1, 1], qb * [-1, -1, -1, 1]
        ta, tb = _qrot(qai, np.cross(ra, nn)), _qrot(qbi, np.cross(rb, nn))
        Ita, Itb = S["inv_inertia"][a] * ta, S["inv_inertia"][b] * tb
        den = ima + imb + ta @ Ita + tb @ Itb
        if den <= 0:
            continue
        e = e_rest if -vn > e_thr else 0.0
        j = -(1 + e) * vn / den
        dv[a] -= j * nn * ima
        dv[b] += j * nn * imb
        dw[a] += _qrot(qa, -j * Ita)
        dw[b] += _qrot(qb, j * Itb)
    return S["vel"] + dv, S["ang"] + dw, S["pos"] + dp


def _scene(seed=5, n=600):
    import torch
    sc = W.serving_scene(seed=seed, n_bodies=n, half=6.0)
    xf = sc.transforms(0)
    world = sc.world(xf)
    rng = np.random.default_rng(seed)
    R, pos = sc.poses(0)
    # quaternion (x, y, z, w) of each rotation
    q = np.zeros((n, 4))
    tr = np.trace(R, axis1=1, axis2=2)
    q[:, 3] = np.sqrt(np.maximum(0, 1 + tr)) / 2
    q[:, 0] = np.copysign(np.sqrt(np.maximum(0, 1 + R[:, 0, 0] - R[:, 1, 1] - R[:, 2, 2])) / 2, R[:, 2, 1] - R[:, 1, 2])
    q[:, 1] = np.copysign(np.sqrt(np.maximum(0, 1 - R[:, 0, 0] + R[:, 1, 1] - R[:, 2, 2])) / 2, R[:, 0, 2] - R[:, 2, 0])
    q[:, 2] = np.copysign(np.sqrt(np.maximum(0, 1 - R[:, 0, 0] - R[:, 1, 1] + R[:, 2, 2])) / 2, R[:, 1, 0] - R[:, 0, 1])
    state = {"pos": pos.astype(np.float32), "quat": q.astype(np.float32),
             "vel": rng.uniform(-3, 3, (n, 3)).astype(np.float32), "ang": rng.uniform(-1, 1, (n, 3)).astype(np.float32),
             "inv_mass": rng.uniform(0.2, 2.0, n).astype(np.float32),
             "inv_inertia": rng.uniform(0.2, 2.0, (n, 3)).astype(np.float32)}
    dev = {k: torch.from_numpy(v).cuda() for k, v in state.items()}
    return sc, world, state, dev


def test_response_matches_host_model(engine):
    import torch
    sc, world, state, dev = _scene()
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, sc.counts)
    pool.upload(world)
    br = engine.Broad(ctx, sc.n_bodies)
    pairs, count, _ = br.run(pool, 4.0, 0.0)
    pairs = pairs.contiguous()
    res = engine.run(ctx, pool, pairs, engine.MODE_GJK_EPA)
    out = engine.contact_response(ctx, dev, pairs, res)
    ctx.synchronize()
    h = res.to_host()
    assert (h["dist"] < 0).sum() > 20
    vel, ang, pos = _host_response(state, pairs.cpu().numpy(), h["dist"], h["normal"],
                                   h["simplex"]["witnesses"].astype(np.float64), 1.1920929e-07, 0.2, 0.5, 1.0)
    for name, ref in (("vel", vel), ("ang", ang), ("pos", pos)):
        got = out[name].cpu().numpy()
        assert np.allclose(got, ref, rtol=1e-4, atol=1e-4), name
    # deterministic: the same call twice gives the same bits
    out2 = engine.contact_response(ctx, dev, pairs, res)
    ctx.synchronize()
    assert all(torch.equal(out[k], out2[k]) for k in out)


def test_response_pushes_bodies_apart(engine):
    """Two overlapping cubes approaching along x: after the response they separate
    (normal from body 1 to body 2, impulses of opposite sign)."""
    import torch
    a = W.cube()
    b = W.cube() + np.float32([1.5, 0.0, 0.0])
    batch = W.from_bodies([a, b])
    ctx = engine.Context(0)
    pool = engine.Pool(ctx, batch.counts)
    pool.upload(batch.coords)
    pairs = torch.tensor([[0, 1]], dtype=torch.int32, device="cuda")
    res = engine.run(ctx, pool, pairs, engine.MODE_GJK_EPA)
    f = lambda x: torch.tensor(np.asarray(x, np.float32), device="cuda")
    state = {"pos": f([[0, 0, 0], [1.5, 0, 0]]), "quat": f([[0, 0, 0, 1], [0, 0, 0, 1]]),
             "vel": f([[2, 0, 0], [-2, 0, 0]]), "ang": f([[0, 0, 0], [0, 0, 0]]), "inv_mass": f([1, 1]),
             "inv_inertia": f([[1, 1, 1], [1, 1, 1]])}
    out = engine.contact_response(ctx, state, pairs, res, restitution=0.0)
    ctx.synchronize()
    v = out["vel"].cpu().numpy().astype(np.float64)
    w = out["ang"].cpu().numpy().astype(np.float64)
    p = out["pos"].cpu().numpy()
    h = res.to_host()
    n = h["normal"][0].astype(np.float64)
    wit = h["simplex"]["witnesses"][0].astype(np.float64)
    assert h["dist"][0] < 0 and n[0] > 0.99      # normal from body 1 towards body 2
    ra, rb = wit[0] - [0, 0, 0], wit[1] - [1.5, 0, 0]
    vn = ((v[1] + np.cross(w[1], rb)) - (v[0] + np.cross(w[0], ra))) @ n
    assert vn >= -1e-5                            # no longer approaching at the contact
    assert v[0, 0] < 2 and v[1, 0] > -2          # both slowed along the normal
    assert p[0, 0] < 0 < p[1, 0] - 1.5           # positions corrected apart
