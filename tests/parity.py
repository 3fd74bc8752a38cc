"""Parity rules of the engine against the FP64 oracle (the reference's CPU GJK/EPA run
in double precision on the same FP32 inputs widened exactly to double).

Tolerances (stated once, used by every parity test):
  * contact band: a pair whose oracle distance satisfies |d| <= BAND * s, with
    s = max(1, largest |coordinate| of the pair), is "in the band" -- FP32 inputs cannot
    decide its verdict; there only |d - d_oracle| <= 2 * BAND * s is required.
  * verdict (contact / separated) identical outside the band.
  * separated pairs outside the band: |d - d_oracle| <= REL * d_oracle (REL = 1e-5) --
    or a smaller distance certified exact (witnesses convex combinations of the final
    simplex's points, bodies separated along w1 - w0 by |w1 - w0|): the reference's GJK
    can cycle to its iteration cap on a wrong feature; counted as sep_oracle_suboptimal.
  * contacts outside the band: |depth - depth_oracle| <= ABS4, normal within ABS4 (L2)
    -- or, where the minimum-translation direction is ill-conditioned (dense point
    clouds: many near-optimal faces), a normal along which the bodies' exact support
    depth exceeds the oracle's depth by at most EQUIV * max(1, depth) (EQUIV = 1e-6);
    witnesses satisfy w0 - w1 = depth * n and lie on the support planes of their bodies
    within ABS4; where the oracle's own witnesses are self-consistent and the contact
    features are unique, they agree with the oracle's within ABS4 (ABS4 = 1e-4) -- for
    all but a stated small fraction: dense clouds (hundreds of points per body) make the
    contact point ill-conditioned, and the invariants above are what certify those.
  * separated normals: within ABS4 (L2) of the oracle's normalize(w1 - w0) -- or, where
    near-parallel closest features make that direction ill-conditioned, a normal along
    which the bodies are separated by the oracle's distance within EQUIV * max(1, s, d)
    (s as for the band: the FP32 normal's rounding moves support values by ~1e-7 s);
    counted as sep_normal_equivalent.
  * separated witnesses: |w1 - w0| = d within ABS4 * max(1, d), and both witnesses on
    their bodies' supporting planes normal to the engine's normal within ABS4;
    where the oracle's
    closest features are unique the witnesses agree with the oracle's within ABS4, except
    that a pair meeting the two invariants is accepted (near-parallel closest features:
    the closest pair is not unique to within the distance tolerance).
"""
import numpy as np

BAND = 1e-5
REL = 1e-5
ABS4 = 1e-4
EQUIV = 1e-6


def pair_scale(b):
    m = np.maximum.reduceat(np.abs(b.coords).max(axis=1), b.offsets)
    return np.maximum(1.0, np.maximum(m[b.pairs[:, 0]], m[b.pairs[:, 1]]))


def support_gaps(b, w0, w1, n):
    """n.w0 - max_A n.a  and  min_B n.b - n.w1 per pair (both ~0 for valid witnesses)."""
    ga = np.empty(len(n))
    gb = np.empty(len(n))
    for i in range(len(n)):
        A = b.body(b.pairs[i, 0]).astype(np.float64)
        B = b.body(b.pairs[i, 1]).astype(np.float64)
        ga[i] = n[i] @ w0[i] - (A @ n[i]).max()
        gb[i] = (B @ n[i]).min() - n[i] @ w1[i]
    return ga, gb


def unique_contact(b, n, tol=1e-6):
    """Contact features unique: at most 4 support points within tol of the planes."""
    u = np.zeros(len(n), bool)
    for i in range(len(n)):
        A = b.body(b.pairs[i, 0]).astype(np.float64)
        B = b.body(b.pairs[i, 1]).astype(np.float64)
        pa, pb = A @ n[i], B @ n[i]
        ca = np.sum(pa >= pa.max() - tol)
        cb = np.sum(pb <= pb.min() + tol)
        u[i] = (ca + cb <= 4) and not (ca >= 3 and cb >= 2) and not (cb >= 3 and ca >= 2)
    return u


def _in_hull_of(w, pts, tol):
    """w is a convex combination of the (at most 3) points pts, within tol."""
    P = np.asarray(pts, np.float64)
    if len(P) == 1:
        return np.linalg.norm(w - P[0]) <= tol
    E = (P[1:] - P[0]).T
    lam, *_ = np.linalg.lstsq(E, w - P[0], rcond=None)
    full = np.concatenate([[1.0 - lam.sum()], lam])
    return np.linalg.norm(P[0] + E @ lam - w) <= tol and np.all(full >= -1e-6)


def _sep_certified(b, res, i):
    """The engine's separated result of pair i is the exact distance (see check)."""
    s = res["simplex"][i]
    n = int(s["nvrtx"])
    if not 1 <= n <= 3:
        return False
    A = b.body(b.pairs[i, 0]).astype(np.float64)
    B = b.body(b.pairs[i, 1]).astype(np.float64)
    ia, ib = s["vrtx_idx"][:n, 0], s["vrtx_idx"][:n, 1]
    if ia.min() < 0 or ia.max() >= len(A) or ib.min() < 0 or ib.max() >= len(B):
        return False
    w0, w1 = s["witnesses"][0].astype(np.float64), s["witnesses"][1].astype(np.float64)
    scale = max(1.0, np.abs(A).max(), np.abs(B).max())
    tol = 1e-6 * scale
    if not (_in_hull_of(w0, A[ia], tol) and _in_hull_of(w1, B[ib], tol)):
        return False
    dv = w1 - w0
    dl = np.linalg.norm(dv)
    nrm = dv / dl
    separation = (B @ nrm).min() - (A @ nrm).max()
    return abs(separation - dl) <= REL * dl + tol and abs(dl - float(res["dist"][i])) <= REL * dl + tol


def check(b, res, o, *, label="", witness_sample=2000, contact_status_bit=8):
    """Compare engine results `res` (dict: dist, simplex, normal, status) with oracle
    results `o` (orc.RESULT_DTYPE, FP64, GJK+EPA).  Returns a report; raises nothing."""
    d = res["dist"].astype(np.float64)
    d64 = o["dist"]
    s = pair_scale(b)
    band = np.abs(d64) <= BAND * s
    col64 = o["epa_exit"] > 0
    col = (res["status"] & contact_status_bit) != 0
    rep = {"label": label, "pairs": len(d), "in_band": int(band.sum())}
    rep["verdict_mismatch"] = int(np.sum((col != col64) & ~band))
    rep["band_abs_violations"] = int(np.sum(band & (np.abs(d - d64) > 2 * BAND * s)))
    sep = ~col64 & ~col & ~band
    rel = np.abs(d[sep] - d64[sep]) / d64[sep] if sep.any() else np.zeros(0)
    rep["separated"] = int(sep.sum())
    rep["sep_rel_max"] = float(rel.max()) if rel.size else 0.0
    # A separated distance below the oracle's is a certified improvement when it is the
    # exact distance: the engine's witnesses are convex combinations of its final
    # simplex's points of each body (so the true distance is at most |w1 - w0|) and the
    # bodies' separation along w1 - w0 equals |w1 - w0| (so it is at least that).  The
    # reference's GJK can cycle until its iteration cap on a wrong feature.
    far_sep = np.flatnonzero(sep)[rel > REL]
    better_ids = {int(i) for i in far_sep if d[i] < d64[i] and _sep_certified(b, res, i)}
    rep["sep_oracle_suboptimal"] = len(better_ids)
    rep["sep_rel_violations"] = int(far_sep.size - len(better_ids))
    # the normal of a separated pair is the reference's normalize(w1 - w0), (1,0,0) when
    # the witnesses coincide (GJK/cpu/EPA.c:350-360), the direction of the distance
    # vector; where near-parallel closest features make that direction ill-conditioned,
    # a normal along which the bodies are separated by the oracle's distance within
    # EQUIV * max(1, d) is accepted and counted (as for contact normals)
    if res.get("normal") is not None and sep.any():
        sn = np.linalg.norm(res["normal"][sep].astype(np.float64) - o["normal"][sep], axis=1)
        rep["sep_normal_err_max"] = float(sn.max())
        far_n = np.flatnonzero(sep)[sn > ABS4]
        equiv = 0
        for i in far_n:
            if int(i) in better_ids:
                equiv += 1
                continue
            A = b.body(b.pairs[i, 0]).astype(np.float64)
            B = b.body(b.pairs[i, 1]).astype(np.float64)
            n = res["normal"][i].astype(np.float64)
            n /= np.linalg.norm(n)
            # the FP32 normal's own rounding moves support values by ~1e-7 * |coordinates|
            if (B @ n).min() - (A @ n).max() >= d64[i] - EQUIV * max(1.0, s[i], d64[i]):
                equiv += 1
        rep["sep_normal_equivalent"] = equiv
        rep["sep_normal_violations"] = int(far_n.size - equiv)
    else:
        rep["sep_normal_err_max"] = 0.0
        rep["sep_normal_equivalent"] = 0
        rep["sep_normal_violations"] = 0
    both = col & col64 & ~band
    rep["contacts"] = int(both.sum())
    dd = np.abs(d[both] - d64[both])
    rep["depth_err_max"] = float(dd.max()) if dd.size else 0.0
    # A depth smaller than the oracle's is a certified improvement when the bodies'
    # exact support depth along the engine's normal confirms it: any direction bounds
    # the minimum translation distance from above (the reference EPA can stop on a
    # wrong face when the origin lies almost on the Minkowski boundary).
    bad = np.flatnonzero(both)[dd > ABS4]
    better = 0
    for i in bad:
        if -d[i] < -d64[i]:
            A = b.body(b.pairs[i, 0]).astype(np.float64)
            B = b.body(b.pairs[i, 1]).astype(np.float64)
            n = res["normal"][i].astype(np.float64)
            n /= np.linalg.norm(n)
            if (A @ n).max() - (B @ n).min() <= -d[i] + EQUIV * max(1.0, -d[i]):
                better += 1
    rep["oracle_suboptimal"] = better
    rep["depth_violations"] = int(bad.size - better)
    nn = np.linalg.norm(res["normal"][both].astype(np.float64) - o["normal"][both], axis=1)
    rep["normal_err_max"] = float(nn.max()) if nn.size else 0.0
    far = np.flatnonzero(both)[nn > ABS4]
    equiv = 0
    for i in far:
        A = b.body(b.pairs[i, 0]).astype(np.float64)
        B = b.body(b.pairs[i, 1]).astype(np.float64)
        n = res["normal"][i].astype(np.float64)
        n /= np.linalg.norm(n)
        if (A @ n).max() - (B @ n).min() - (-d64[i]) <= EQUIV * max(1.0, -d64[i]):
            equiv += 1
    rep["normal_equivalent"] = equiv
    rep["normal_violations"] = int(far.size - equiv)
    # witnesses of contacts
    idx = np.flatnonzero(both)[:witness_sample]
    if idx.size:
        w = res["simplex"]["witnesses"][idx].astype(np.float64)
        n = res["normal"][idx].astype(np.float64)
        depth = -d[idx]
        incons = np.linalg.norm((w[:, 0] - w[:, 1]) - depth[:, None] * n, axis=1)
        sb = b.subset(idx)
        ga, gb = support_gaps(sb, w[:, 0], w[:, 1], n)
        rep["witness_inconsistent"] = int(np.sum(incons > ABS4))
        rep["witness_off_support"] = int(np.sum((np.abs(ga) > ABS4) | (np.abs(gb) > ABS4)))
        ow = o["wit"][idx]
        oincons = np.linalg.norm((ow[:, 0] - ow[:, 1]) - (-d64[idx])[:, None] * o["normal"][idx], axis=1)
        ok = (oincons <= ABS4) & unique_contact(sb, o["normal"][idx])
        werr = np.abs(w - ow).reshape(len(idx), -1).max(axis=1)
        rep["witness_compared"] = int(ok.sum())
        rep["witness_mismatch"] = int(np.sum(ok & (werr > ABS4)))
    else:
        rep.update(witness_inconsistent=0, witness_off_support=0, witness_compared=0, witness_mismatch=0)
    # separated witnesses: w1 - w0 has length d; compared with the oracle's where the
    # closest features are unique
    sidx = np.flatnonzero(sep)[:witness_sample]
    if sidx.size:
        ws = res["simplex"]["witnesses"][sidx].astype(np.float64)
        ow = o["wit"][sidx]
        gap = np.abs(np.linalg.norm(ws[:, 1] - ws[:, 0], axis=1) - d64[sidx])
        rep["sep_witness_length_violations"] = int(np.sum(gap > ABS4 * np.maximum(1.0, d64[sidx])))
        if res.get("normal") is not None:  # the engine's normal: the direction of -v
            dirn = res["normal"][sidx].astype(np.float64)
        else:
            dirn = ow[:, 1] - ow[:, 0]
        dirn /= np.maximum(np.linalg.norm(dirn, axis=1, keepdims=True), 1e-300)
        sb = b.subset(sidx)
        ok = unique_contact(sb, -dirn)
        werr = np.abs(ws - ow).reshape(len(sidx), -1).max(axis=1)
        # a closest pair is valid when both witnesses lie on their bodies' supporting
        # planes normal to the distance vector (unique for convex bodies, even where the
        # witnesses are not; the oracle's direction is used, FP32 witnesses of a small
        # distance do not resolve it); near-parallel closest features make the pair
        # ill-conditioned, and a valid pair is accepted there
        ga, gb = support_gaps(sb, ws[:, 0], ws[:, 1], dirn)
        valid = (np.abs(ga) <= ABS4) & (np.abs(gb) <= ABS4)
        rep["sep_witness_off_support"] = int(np.sum(~valid))
        rep["sep_witness_compared"] = int(ok.sum())
        rep["sep_witness_err_max"] = float(werr[ok].max()) if ok.any() else 0.0
        rep["sep_witness_valid_elsewhere"] = int(np.sum(ok & (werr > ABS4) & valid))
        rep["sep_witness_violations"] = int(np.sum(ok & (werr > ABS4) & ~valid))
    return rep


def assert_parity(rep, *, max_witness_mismatch_frac=1e-3, max_sep_witness_frac=1e-3):
    msg = str(rep)
    assert rep["verdict_mismatch"] == 0, msg
    assert rep["band_abs_violations"] == 0, msg
    assert rep["sep_rel_violations"] == 0, msg
    assert rep["sep_normal_violations"] == 0, msg
    assert rep["depth_violations"] == 0, msg
    assert rep["normal_violations"] == 0, msg
    assert rep["witness_inconsistent"] == 0, msg
    assert rep["witness_off_support"] == 0, msg
    assert rep["witness_mismatch"] <= max(1, max_witness_mismatch_frac * rep["witness_compared"]), msg
    if "sep_witness_violations" in rep:
        assert rep["sep_witness_length_violations"] == 0, msg
        assert rep["sep_witness_off_support"] == 0, msg
        assert rep["sep_witness_violations"] <= max(1, max_sep_witness_frac * rep["sep_witness_compared"]), msg
