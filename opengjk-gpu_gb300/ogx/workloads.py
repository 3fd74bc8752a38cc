"""Seeded synthetic workloads for the batched GJK/EPA engine.

Every generator returns a :class:`Batch`: one pool of bodies (points of all bodies
concatenated, xyz float32) and a list of body-index pairs.  The workloads follow the
five benchmark configurations of the engine:

* ``plain``    -- 32-point spheres, radius U[0.5, 2], centres U[-5, 5]^3 (FP64 check set)
* ``ellipsoid``-- log-uniform vertex counts in [8, 256] on random ellipsoids (semi-axes
  U[0.3, 2], uniform random rotation), centres placed so that about half the pairs
  overlap
* ``powerlaw`` -- the ellipsoid shapes with vertex counts from a discrete power law
  p(n) ~ n^-1.5 on [4, 1024]
* ``stress``   -- near-touching ellipsoids (gap log-uniform in [1e-7, 1e-2]), axis-aligned
  boxes face-to-face and edge-to-edge, near-coplanar thin disks
* ``sphere_shell`` -- the reference's own benchmark shape (examples/main.cpp:79-94:
  points on a shell of radius U[1, 1.5] around an offset)

The reference draws its inputs from an unseeded C ``rand()`` (examples/main.cpp:102);
these generators are seeded numpy streams with the shapes and value ranges of the
benchmark configurations instead.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# Placement calibration for the ellipsoid workloads.  The separation of a pair's
# centres along a random unit direction u is  K * (h_A(u) + h_B(-u)) * U[0.6, 1.4],
# where h is the support extent of the sampled points.  h_A(u) + h_B(-u) is the
# separation at which a plane normal to u first separates the bodies, which
# over-estimates the touching separation (the sampled hull is smaller than its
# ellipsoid and other separating axes exist).  K was chosen per workload so that about
# half of the pairs overlap (measured with the FP64 oracle on 20k pairs: 0.89 gives
# 49-50% for the log-uniform [8, 256] workload, 0.82 gives ~50% for the power law).
PLACEMENT_K = 0.89
PLACEMENT_K_POWERLAW = 0.82


@dataclasses.dataclass
class Batch:
    coords: np.ndarray   # (P, 3) float32, all bodies' points
    offsets: np.ndarray  # (B,) int64, first point of each body
    counts: np.ndarray   # (B,) int32, points per body
    pairs: np.ndarray    # (N, 2) int32, body indices of each pair
    name: str = ""
    meta: dict = dataclasses.field(default_factory=dict)

    @property
    def n_pairs(self) -> int:
        return int(self.pairs.shape[0])

    @property
    def n_bodies(self) -> int:
        return int(self.counts.shape[0])

    def pair_vertex_counts(self) -> np.ndarray:
        return self.counts[self.pairs[:, 0]].astype(np.int64) + self.counts[self.pairs[:, 1]]

    def algorithmic_bytes(self, with_epa: bool = True) -> int:
        """Bytes the path must move once per pass: 12 B per point of both bodies,
        8 B of pair indices, 4 B distance, 108 B simplex (incl. witnesses) and 12 B
        normal (EPA) per pair."""
        per_pair = 8 + 4 + 108 + (12 if with_epa else 0)
        return int(12 * self.pair_vertex_counts().sum() + per_pair * self.n_pairs)

    def body(self, b: int) -> np.ndarray:
        o = int(self.offsets[b])
        return self.coords[o:o + int(self.counts[b])]

    def subset(self, idx) -> "Batch":
        return Batch(self.coords, self.offsets, self.counts, self.pairs[idx], self.name, self.meta)


def _offsets(counts: np.ndarray) -> np.ndarray:
    off = np.zeros(counts.shape[0], dtype=np.int64)
    np.cumsum(counts[:-1], out=off[1:])
    return off


def _unit_vectors(rng: np.random.Generator, n: int) -> np.ndarray:
    v = rng.standard_normal((n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def _rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotation matrices from uniform unit quaternions."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack(
        [
            np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
            np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
            np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
        ],
        axis=1,
    )


def _segment_max(values: np.ndarray, offsets: np.ndarray) -> np.ndarray:
    return np.maximum.reduceat(values, offsets)


def _segment_argmax(values: np.ndarray, offsets: np.ndarray, counts: np.ndarray) -> np.ndarray:
    """Index (into `values`) of the first maximum of each segment."""
    m = np.repeat(_segment_max(values, offsets), counts)
    hit = np.flatnonzero(values == m)
    body = np.repeat(np.arange(counts.shape[0]), counts)[hit]
    first = np.full(counts.shape[0], -1, dtype=np.int64)
    # keep the first hit per body
    order = np.unique(body, return_index=True)[1]
    first[body[order]] = hit[order]
    return first


def _ellipsoid_points(rng, counts: np.ndarray, chunk: int = 1 << 22) -> np.ndarray:
    """Points uniform on a unit sphere, mapped by diag(a), a ~ U[0.3, 2]^3, then a random
    rotation -- one ellipsoid per body, centred at the origin (float64)."""
    nb = counts.shape[0]
    axes = rng.uniform(0.3, 2.0, size=(nb, 3))
    rot = _rotations(rng, nb)
    total = int(counts.sum())
    pts = np.empty((total, 3), dtype=np.float64)
    body_of = np.repeat(np.arange(nb, dtype=np.int64), counts)
    for s in range(0, total, chunk):
        e = min(total, s + chunk)
        b = body_of[s:e]
        u = _unit_vectors(rng, e - s) * axes[b]
        pts[s:e] = np.einsum("nij,nj->ni", rot[b], u)
    return pts


def _place_pairs(rng, pts64: np.ndarray, counts: np.ndarray, offsets: np.ndarray,
                 centre_box: float, k: float | None = None):
    """Translate body 2i+1 relative to body 2i so that about half the pairs overlap."""
    if k is None:
        k = PLACEMENT_K
    nb = counts.shape[0]
    npairs = nb // 2
    u = _unit_vectors(rng, npairs)
    body_of = np.repeat(np.arange(nb, dtype=np.int64), counts)
    pair_of = body_of // 2
    sgn = np.where(body_of % 2 == 0, 1.0, -1.0)
    proj = np.einsum("ni,ni->n", pts64, u[pair_of]) * sgn
    h = _segment_max(proj, offsets)
    sep = k * (h[0::2] + h[1::2]) * rng.uniform(0.6, 1.4, size=npairs)
    centres = rng.uniform(-centre_box, centre_box, size=(npairs, 3))
    shift = np.empty((nb, 3))
    shift[0::2] = centres
    shift[1::2] = centres + sep[:, None] * u
    pts64 += shift[body_of]
    return pts64


def plain(seed: int = 1, n_pairs: int = 1000, n_verts: int = 32, dtype=np.float32) -> Batch:
    """32 points uniform on the unit sphere x r ~ U[0.5, 2] + c ~ U[-5, 5]^3 (float32
    coordinates; dtype=np.float64 keeps them in double, the inputs of FP64 callers)."""
    rng = np.random.default_rng(seed)
    nb = 2 * n_pairs
    counts = np.full(nb, n_verts, dtype=np.int32)
    r = rng.uniform(0.5, 2.0, size=nb)
    c = rng.uniform(-5.0, 5.0, size=(nb, 3))
    u = _unit_vectors(rng, nb * n_verts).reshape(nb, n_verts, 3)
    pts = (u * r[:, None, None] + c[:, None, :]).reshape(-1, 3)
    pairs = np.arange(nb, dtype=np.int32).reshape(-1, 2)
    return Batch(pts.astype(dtype), _offsets(counts), counts, pairs, "plain",
                 {"n_verts": n_verts})


def _loguniform_counts(rng, n: int, lo: int, hi: int) -> np.ndarray:
    return np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi + 1), size=n))).astype(np.int32).clip(lo, hi)


def _powerlaw_counts(rng, n: int, lo: int = 4, hi: int = 1024, expo: float = -1.5) -> np.ndarray:
    support = np.arange(lo, hi + 1, dtype=np.float64)
    cdf = np.cumsum(support ** expo)
    cdf /= cdf[-1]
    return (lo + np.searchsorted(cdf, rng.uniform(0.0, 1.0, size=n), side="right")).clip(lo, hi).astype(np.int32)


def ellipsoid(seed: int = 2, n_pairs: int = 100_000, lo: int = 8, hi: int = 256,
              centre_box: float = 5.0) -> Batch:
    """GJK+EPA workload: log-uniform vertex counts on random ellipsoids, ~50% overlap."""
    rng = np.random.default_rng(seed)
    counts = _loguniform_counts(rng, 2 * n_pairs, lo, hi)
    offsets = _offsets(counts)
    pts = _place_pairs(rng, _ellipsoid_points(rng, counts), counts, offsets, centre_box)
    pairs = np.arange(2 * n_pairs, dtype=np.int32).reshape(-1, 2)
    return Batch(pts.astype(np.float32), offsets, counts, pairs, "ellipsoid",
                 {"lo": lo, "hi": hi})


def powerlaw(seed: int = 3, n_pairs: int = 1_000_000, lo: int = 4, hi: int = 1024,
             centre_box: float = 5.0) -> Batch:
    """Uneven batching workload: power-law vertex counts, the ellipsoid shapes."""
    rng = np.random.default_rng(seed)
    counts = _powerlaw_counts(rng, 2 * n_pairs, lo, hi)
    offsets = _offsets(counts)
    pts = _place_pairs(rng, _ellipsoid_points(rng, counts), counts, offsets, centre_box,
                       PLACEMENT_K_POWERLAW)
    pairs = np.arange(2 * n_pairs, dtype=np.int32).reshape(-1, 2)
    return Batch(pts.astype(np.float32), offsets, counts, pairs, "powerlaw",
                 {"lo": lo, "hi": hi, "exponent": -1.5})


def sphere_shell(seed: int = 4, n_pairs: int = 1000, n_verts: int = 500) -> Batch:
    """The reference benchmark's bodies: points at radius U[1, 1.5] around an offset
    in [-5, 5]^3 (examples/main.cpp:79-94), here uniform on the sphere."""
    rng = np.random.default_rng(seed)
    nb = 2 * n_pairs
    counts = np.full(nb, n_verts, dtype=np.int32)
    r = rng.uniform(1.0, 1.5, size=(nb, n_verts, 1))
    c = rng.uniform(-5.0, 5.0, size=(nb, 1, 3))
    u = _unit_vectors(rng, nb * n_verts).reshape(nb, n_verts, 3)
    pts = (u * r + c).reshape(-1, 3)
    pairs = np.arange(nb, dtype=np.int32).reshape(-1, 2)
    return Batch(pts.astype(np.float32), _offsets(counts), counts, pairs, "sphere_shell",
                 {"n_verts": n_verts})


def _box_points(half: np.ndarray) -> np.ndarray:
    signs = np.array([[sx, sy, sz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)], dtype=np.float64)
    return signs[None, :, :] * half[:, None, :]


def stress(seed: int = 5, n_pairs: int = 200_000) -> Batch:
    """Mixed-precision stress set: one third each of (i) near-touching ellipsoids whose
    support points are aligned so that the distance is exactly the drawn gap,
    (ii) 8-point axis-aligned boxes face-to-face / edge-to-edge with a signed gap, and
    (iii) 64-point disks of thickness 1e-4 stacked almost coplanar with a signed gap.
    Gaps are log-uniform in [1e-7, 1e-2] (signed for boxes and disks)."""
    rng = np.random.default_rng(seed)
    n1 = n_pairs // 3
    n2 = n_pairs // 3
    n3 = n_pairs - n1 - n2
    parts_pts, parts_counts, kinds, gaps_all = [], [], [], []

    # (i) near-touching ellipsoids
    counts = _loguniform_counts(rng, 2 * n1, 8, 256)
    offsets = _offsets(counts)
    pts = _ellipsoid_points(rng, counts)
    u = _unit_vectors(rng, n1)
    gap = np.exp(rng.uniform(math.log(1e-7), math.log(1e-2), size=n1))
    body_of = np.repeat(np.arange(2 * n1, dtype=np.int64), counts)
    pair_of = body_of // 2
    sgn = np.where(body_of % 2 == 0, 1.0, -1.0)
    proj = np.einsum("ni,ni->n", pts, u[pair_of]) * sgn
    arg = _segment_argmax(proj, offsets, counts)
    a_star = pts[arg[0::2]]
    b_star = pts[arg[1::2]]
    centres = rng.uniform(-5.0, 5.0, size=(n1, 3))
    shift = np.empty((2 * n1, 3))
    shift[0::2] = centres
    shift[1::2] = centres + a_star + gap[:, None] * u - b_star
    pts += shift[body_of]
    parts_pts.append(pts)
    parts_counts.append(counts)
    kinds.append(np.zeros(n1, dtype=np.int8))
    gaps_all.append(gap)

    # (ii) boxes: face-to-face along x, or edge-to-edge along x and y
    half_a = rng.uniform(0.3, 2.0, size=(n2, 3))
    half_b = rng.uniform(0.3, 2.0, size=(n2, 3))
    g = np.exp(rng.uniform(math.log(1e-7), math.log(1e-2), size=n2)) * rng.choice([-1.0, 1.0], size=n2)
    edge = rng.uniform(size=n2) < 0.5
    centres = rng.uniform(-5.0, 5.0, size=(n2, 3))
    off = np.zeros((n2, 3))
    off[:, 0] = half_a[:, 0] + half_b[:, 0] + g
    lat = rng.uniform(-0.5, 0.5, size=(n2, 2)) * np.minimum(half_a[:, 1:], half_b[:, 1:])
    off[:, 1:] = lat
    off[edge, 1] = half_a[edge, 1] + half_b[edge, 1] + g[edge]
    pa = _box_points(half_a) + centres[:, None, :]
    pb = _box_points(half_b) + (centres + off)[:, None, :]
    bx = np.stack([pa, pb], axis=1).reshape(-1, 3)
    parts_pts.append(bx)
    parts_counts.append(np.full(2 * n2, 8, dtype=np.int32))
    kinds.append(np.where(edge, 2, 1).astype(np.int8))
    gaps_all.append(g)

    # (iii) near-coplanar thin disks (two rings of 32 points, 1e-4 apart)
    thick = 1e-4
    r_a = rng.uniform(0.5, 2.0, size=n3)
    r_b = rng.uniform(0.5, 2.0, size=n3)
    ang = np.linspace(0.0, 2 * math.pi, 32, endpoint=False)
    ring = np.stack([np.cos(ang), np.sin(ang), np.zeros_like(ang)], -1)
    disk = np.concatenate([ring, ring + [0.0, 0.0, thick]], axis=0)  # (64, 3)
    rot = _rotations(rng, n3)
    tilt = rng.uniform(-1e-3, 1e-3, size=(n3, 2))
    g3 = np.exp(rng.uniform(math.log(1e-7), math.log(1e-2), size=n3)) * rng.choice([-1.0, 1.0], size=n3)
    lat3 = rng.uniform(0.2, 0.9, size=n3) * (r_a + r_b)
    phi = rng.uniform(0.0, 2 * math.pi, size=n3)
    da = disk[None] * np.stack([r_a, r_a, np.ones(n3)], -1)[:, None, :]
    db = disk[None] * np.stack([r_b, r_b, np.ones(n3)], -1)[:, None, :]
    # tiny tilt of disk B about x and y, then put it on top of A with the signed gap
    cx, sx = np.cos(tilt[:, 0]), np.sin(tilt[:, 0])
    cy, sy = np.cos(tilt[:, 1]), np.sin(tilt[:, 1])
    y1 = db[..., 1] * cx[:, None] - db[..., 2] * sx[:, None]
    z1 = db[..., 1] * sx[:, None] + db[..., 2] * cx[:, None]
    x2 = db[..., 0] * cy[:, None] + z1 * sy[:, None]
    z2 = -db[..., 0] * sy[:, None] + z1 * cy[:, None]
    db = np.stack([x2, y1, z2], -1)
    db += np.stack([lat3 * np.cos(phi), lat3 * np.sin(phi), thick + g3], -1)[:, None, :]
    centres = rng.uniform(-5.0, 5.0, size=(n3, 3))
    da = np.einsum("nij,nkj->nki", rot, da) + centres[:, None, :]
    db = np.einsum("nij,nkj->nki", rot, db) + centres[:, None, :]
    dk = np.stack([da, db], axis=1).reshape(-1, 3)
    parts_pts.append(dk)
    parts_counts.append(np.full(2 * n3, 64, dtype=np.int32))
    kinds.append(np.full(n3, 3, dtype=np.int8))
    gaps_all.append(g3)

    counts = np.concatenate(parts_counts)
    pts = np.concatenate(parts_pts).astype(np.float32)
    pairs = np.arange(counts.shape[0], dtype=np.int32).reshape(-1, 2)
    return Batch(pts, _offsets(counts), counts, pairs, "stress",
                 {"kind": np.concatenate(kinds), "gap": np.concatenate(gaps_all)})


def cube(half: float = 1.0) -> np.ndarray:
    """8 corners of an axis-aligned cube of half-size `half`, x slowest, z fastest."""
    return _box_points(np.array([[half] * 3]))[0].astype(np.float32)


def rotated_cube(angle_deg: float = 45.0, shift=(1.0, 0.0, 0.0)) -> np.ndarray:
    """The cube rotated by `angle_deg` about x, then y, then z, then translated --
    the body of the reference's EPA usage example (examples/usage/EPAUsage.cpp)."""
    a = math.radians(angle_deg)
    c, s = math.cos(a), math.sin(a)
    rx = np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
    ry = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
    rz = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])
    p = cube().astype(np.float64) @ (rz @ ry @ rx).T
    return (p + np.asarray(shift)).astype(np.float32)


def from_bodies(bodies, pairs=None, name: str = "custom") -> Batch:
    """Batch from a list of (n, 3) point arrays; default pairs (0,1), (2,3), ..."""
    counts = np.array([len(b) for b in bodies], dtype=np.int32)
    coords = np.concatenate([np.asarray(b, dtype=np.float32).reshape(-1, 3) for b in bodies])
    if pairs is None:
        pairs = np.arange(len(bodies) - len(bodies) % 2, dtype=np.int32).reshape(-1, 2)
    return Batch(coords, _offsets(counts), counts, np.asarray(pairs, dtype=np.int32).reshape(-1, 2), name)


REGISTRY = {
    "plain": plain,
    "ellipsoid": ellipsoid,
    "powerlaw": powerlaw,
    "sphere_shell": sphere_shell,
    "stress": stress,
}


# ---------------------------------------------------------------------------------
# serving scene: resident rigid bodies moving in a box, candidate pairs per tick

@dataclasses.dataclass
class Scene:
    """Bodies in their own frame plus their motion.  Body b has counts[b] points
    (local, float32, concatenated in `local`), starts at pos0[b] with orientation rot0[b]
    and moves with velocity vel[b] (reflected at the walls of the box [-half, half]^3)
    and angular velocity omg[b]."""
    local: np.ndarray
    counts: np.ndarray
    offsets: np.ndarray
    pos0: np.ndarray
    vel: np.ndarray
    rot0: np.ndarray
    omg: np.ndarray
    half: float
    dt: float

    @property
    def n_bodies(self) -> int:
        return int(self.counts.shape[0])

    def poses(self, tick: int):
        """Rotation matrices (B, 3, 3) and positions (B, 3) at `tick`, float64."""
        t = tick * self.dt
        span = 2.0 * self.half
        p = self.pos0 + self.vel * t + self.half  # in [0, 2 half) before folding
        p = np.mod(p, 2.0 * span)
        p = np.where(p > span, 2.0 * span - p, p) - self.half
        ang = np.linalg.norm(self.omg, axis=1) * t
        axis = self.omg / np.maximum(np.linalg.norm(self.omg, axis=1, keepdims=True), 1e-300)
        c, s = np.cos(ang)[:, None, None], np.sin(ang)[:, None, None]
        x, y, z = axis[:, 0], axis[:, 1], axis[:, 2]
        K = np.zeros((self.n_bodies, 3, 3))
        K[:, 0, 1], K[:, 0, 2], K[:, 1, 0] = -z, y, z
        K[:, 1, 2], K[:, 2, 0], K[:, 2, 1] = -x, -y, x
        R = np.eye(3)[None] + s * K + (1.0 - c) * (K @ K)
        return R @ self.rot0, p

    def transforms(self, tick: int) -> np.ndarray:
        """(B, 12) float32: row-major rotation then translation (the server's layout)."""
        R, p = self.poses(tick)
        return np.concatenate([R.reshape(-1, 9), p], axis=1).astype(np.float32)

    def world(self, xf: np.ndarray) -> np.ndarray:
        """World points of all bodies for the float32 transforms `xf`, computed exactly as
        the server does: ((R0 x + R1 y) + R2 z) + t in float64, rounded once."""
        body = np.repeat(np.arange(self.n_bodies), self.counts)
        m = xf.astype(np.float64)[body]
        p = self.local.astype(np.float64)
        out = np.empty_like(p)
        for r in range(3):
            out[:, r] = ((m[:, 3 * r] * p[:, 0] + m[:, 3 * r + 1] * p[:, 1]) + m[:, 3 * r + 2] * p[:, 2]) + m[:, 9 + r]
        return out.astype(np.float32)

    def candidate_pairs(self, tick: int, n_pairs: int) -> np.ndarray:
        """A broad-phase stand-in: the n_pairs closest body pairs by centre distance
        (k-nearest neighbours of every body, i < j), int32 (n, 2)."""
        from scipy.spatial import cKDTree
        _, p = self.poses(tick)
        k = min(self.n_bodies - 1, max(2, int(math.ceil(2.5 * n_pairs / self.n_bodies)) + 1))
        d, j = cKDTree(p).query(p, k=k + 1)
        i = np.repeat(np.arange(self.n_bodies), k)
        j = j[:, 1:].reshape(-1)
        d = d[:, 1:].reshape(-1)
        keep = i < j
        i, j, d = i[keep], j[keep], d[keep]
        order = np.argsort(d, kind="stable")[:n_pairs]
        return np.stack([i[order], j[order]], axis=1).astype(np.int32)


def serving_scene(seed: int = 6, n_bodies: int = 20_000, lo: int = 8, hi: int = 512,
                  half: float = 50.0, speed: float = 50.0, dt: float = 1.0 / 60.0) -> Scene:
    """20k rigid bodies, log-uniform vertex counts in [8, 512] on random ellipsoids,
    positions uniform in [-half, half]^3, velocities uniform in [-speed, speed]^3,
    angular velocities up to 2 rad/s."""
    rng = np.random.default_rng(seed)
    counts = _loguniform_counts(rng, n_bodies, lo, hi)
    local = _ellipsoid_points(rng, counts).astype(np.float32)
    pos0 = rng.uniform(-half, half, size=(n_bodies, 3))
    vel = rng.uniform(-speed, speed, size=(n_bodies, 3))
    rot0 = _rotations(rng, n_bodies)
    omg = _unit_vectors(rng, n_bodies) * rng.uniform(0.0, 2.0, size=(n_bodies, 1))
    return Scene(local, counts, _offsets(counts), pos0, vel, rot0, omg, half, dt)


def tick_sizes(seed: int, n_ticks: int, lo: int = 1_000, hi: int = 200_000) -> np.ndarray:
    """Pairs per tick, log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), size=n_ticks))).astype(np.int64)


def poisson_arrivals(seed: int, n: int, rate_hz: float) -> np.ndarray:
    """Arrival times (s) of a Poisson process of the given rate."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_hz, size=n))
