// ogx_epa.cuh -- EPA penetration depth for one colliding pair, run by a team of L lanes.
//
// Semantics follow the reference's computeCollisionInformation (GJK/cpu/EPA.c:362-863,
// GJK/gpu/openGJK.cu:1836-2726): a separated pair only gets its contact normal
// (normalised w1 - w0); a contact whose GJK simplex has fewer than four points is grown
// by supports along fixed directions (point, edge-perpendicular, triangle normal and its
// opposite) and reported with depth 0 when no new point appears; otherwise the simplex
// seeds a polytope that is expanded towards its closest face until the support point
// along that face's normal does not improve on it.  The result is depth = -distance of
// the closest face, its normal, and witnesses from the origin's barycentric position on
// that face (clamped to the triangle as in EPA.c:238-304).
//
// Design (not the reference's):
//  * The polytope keeps face adjacency.  The faces visible from the new point are found
//    in parallel (faces are split over the lanes), the horizon is every edge of a visible
//    face whose neighbour is not visible, and new faces are linked to each other through
//    two per-vertex tables -- O(F) per step instead of the reference's O(F^2) edge
//    de-duplication.  Winding is inherited from the horizon edge, so no centroid test.
//  * Face normals are computed once when the face is created (the reference recomputes
//    all of them every step) in FP32, in FP64 from the exact points for sliver faces.
//  * Polytope capacity is 68 vertices / 132 faces, enough for the 64-step cap (the
//    reference's 128-face list can overflow in its last steps).
//  * Duplicate detection compares the support pair's vertex indices.
//  * The chosen face can be re-solved in FP64 afterwards (same pass as the GJK polish).
#pragma once

#include "ogx_common.cuh"
#include "ogx_gjk.cuh"

namespace ogx {

// Shared-memory working set of one pair, for at most VMAX polytope vertices and FMAX
// faces (5728 bytes at 68 / 132, the capacity of 64 expansions; 2288 bytes at 28 / 52).
template <int VMAX, int FMAX>
struct EpaMemT {
  static constexpr int kV = VMAX;
  static constexpr int kF = FMAX;
  float4 fn[FMAX];          // unit outward normal, w = plane distance from origin
  float4 vp[VMAX];          // polytope vertices (Minkowski points)
  int2 vid[VMAX];           // (index in body 1, index in body 2)
  uint8_t fv[FMAX][4];      // face vertices a, b, c; [3] = 1 when the face is alive
  uint8_t fa[FMAX][4];      // fa[f][e]: face across edge e = (v_e, v_{e+1 mod 3})
  uint8_t vis[FMAX];        // visible from the new point (this step)
  uint8_t vlist[FMAX];      // visible faces in increasing order (this step)
  uint8_t hz[FMAX][4];      // horizon edges (this step): a, b, face beyond
  uint8_t hstart[VMAX];     // new face whose horizon edge starts at vertex
  uint8_t hend[VMAX];       // new face whose horizon edge ends at vertex
};
// full capacity: every pair within the 64-expansion cap
typedef EpaMemT<kEpaVmax, kEpaFmax> EpaMem;
// small capacity: 24 expansions; a pair that needs more is handed to a full-capacity pass
constexpr int kEpaSmallIters = 24;
typedef EpaMemT<4 + kEpaSmallIters, 4 + 2 * kEpaSmallIters> EpaMemSmall;
// full capacity for the certified re-run: every face's plane is also kept in FP64
struct EpaMemCert : EpaMem {
  double4 fn64[kEpaFmax];  // unit outward normal and plane distance, FP64 from exact points
};
OGX_HD double4* plane64_slot(EpaMemCert& M, int f) { return &M.fn64[f]; }

// A small-capacity expansion that ran out of room, kept for the full-capacity pass to
// continue from instead of starting again: the polytope and the loop state at the top of
// the iteration that overflowed.  The full pass makes the same decisions up to there (the
// face slots do not depend on the capacity), so the result is the same as a restart.
struct EpaResume {
  int pair, nv, fend, it, st, status;
  float scale2;
  float4 fn[EpaMemSmall::kF];
  float4 vp[EpaMemSmall::kV];
  int2 vid[EpaMemSmall::kV];
  uint8_t fv[EpaMemSmall::kF][4];
  uint8_t fa[EpaMemSmall::kF][4];
};
// where a spilling expansion saves itself: cap records in buf, *count the next free one
// (buf null or full: the full pass restarts the contact)
struct EpaResumeSink {
  EpaResume* buf;
  int* count;
  int cap;
};
template <class Mem>
OGX_HD double4* plane64_slot(Mem&, int) { return nullptr; }

// The certified re-run.  An FP32 expansion that stops with the support still above the
// closest face by more than rounding (kEpaCertGain * scale; the FP32 test accepts up to
// epa_rel * scale), or whose support repeats a vertex before converging, is run again at
// full capacity with every face plane in FP64 from the exact points, visibility decided
// on those planes, exact (FP64) supports, and convergence when the support improves on
// the closest face by at most kEpaCertTol * max(1, scale).
constexpr float kEpaCertGain = 2.5e-7f;
constexpr double kEpaCertTol = 1e-10;
// Thin contacts: the closest face within kEpaThin * scale of the origin (thin bodies such
// as 1e-4-thick disks, or barely overlapping ones).  Their long, flat faces carry FP32
// normals whose rounding (~1e-6) can hide a support that improves on the face by more
// than the FP32 convergence tolerance; at FP32 convergence such a contact is checked with
// exact supports along its face's FP64 plane and run again certified if they improve on
// the face by more than that tolerance.
constexpr float kEpaThin = 1e-3f;
// Largest squared sine of the angle between the closest face and a neighbour the
// origin's projection moves to, for the FP32 pass to accept the neighbour's result.
constexpr float kEpaHopSin2 = 1e-10f;
constexpr double kEpaCertVis = 1e-12;

struct EpaOut {
  float dist;   // -depth for contacts, the GJK distance otherwise
  fv3 w0, w1;   // witnesses
  fv3 nrm;      // contact normal, body 1 -> body 2
  int status;
  int iters;
  int face[3][2];  // vertex index pairs of the final face (FP64 re-solve)
  bool polish;
  bool spill;      // ran out of (small) capacity: nothing written, run again at full capacity
  bool spill64;    // ... because the FP32 expansion met an inconsistent horizon: the re-run
                   // solves every face plane in FP64
  int resume;      // a capacity spill saved to this EpaResume record (-1: none)
};

OGX_HD fv3 unit_or_x(fv3 d) {
  const float n = sqrtf(dot(d, d));
  if (n > FLT_EPSILON) return d * (1.0f / n) ;
  return v3<float>(1.0f, 0.0f, 0.0f);
}

// Normal of a separated pair: the reference's normalize(w1 - w0) with (1,0,0) when the
// witnesses coincide (GJK/cpu/EPA.c:350-360).  In exact arithmetic w1 - w0 = -v, v the
// closest point of the Minkowski difference to the origin, and the normal is computed
// from -v: v carries the accuracy of the distance (each component rounded relative to
// itself), while the difference of two FP32 witnesses keeps their absolute rounding, a
// few 1e-7 of the coordinates, which is more than 1e-4 of a distance below ~1e-3.
OGX_HD fv3 sep_normal(const GjkState& g) { return unit_or_x(-g.v); }

// The same normal from a GJK simplex given by a caller (EPA-only calls): v is re-solved
// from the simplex's points of the two bodies (exact Minkowski differences, closest point
// in double-float, as the certified re-solve of the GJK pass does); where the simplex's
// vertex indices do not address the bodies, the reference's rule on the given witnesses.
OGX_HD fv3 simplex_sep_normal(const MemBodies& B, const gkSimplex& s) {
  const int n = s.nvrtx;
  bool ok = n >= 1 && n <= 3;
  xv3 P[3];
  for (int j = 0; j < 3; ++j) {
    if (!ok || j >= n) break;
    const int ia = s.vrtx_idx[j][0], ib = s.vrtx_idx[j][1];
    ok = ia >= 0 && ia < B.n[0] && ib >= 0 && ib < B.n[1];
    if (ok) P[j] = xdiff(B.point(0, ia), B.point(1, ib));
  }
  if (ok) {
    df lam[4];
    xv3 v;
    closest_on_simplex_t<df>(n, P, lam, v);
    return unit_or_x(v3<float>(-to_float(v.x), -to_float(v.y), -to_float(v.z)));
  }
  const fv3 w0 = v3<float>(s.witnesses[0][0], s.witnesses[0][1], s.witnesses[0][2]);
  const fv3 w1 = v3<float>(s.witnesses[1][0], s.witnesses[1][1], s.witnesses[1][2]);
  return unit_or_x(w1 - w0);
}

// support of the Minkowski difference along d (first maximum wins, EPA.c:307-344)
template <class Team, class Bodies>
OGX_HD fv3 msupport(const Team& t, const Bodies& B, fv3 d, int& ia, int& ib) {
  float ba, bb;
  B.scan(t, 0, d, ba, ia);
  B.scan(t, 1, -d, bb, ib);
  t.argmax(ba, ia);
  t.argmax(bb, ib);
  return B.point(0, ia) - B.point(1, ib);
}

// FP64 plane (unit normal, offset) of live face f from its exact points; w = INFINITY
// for a degenerate face
template <class Mem, class Bodies>
OGX_HD double4 face_plane64(const Mem& M, const Bodies& B, int f) {
  const int a = M.fv[f][0], b = M.fv[f][1], c = M.fv[f][2];
  const dv3 q0 = B.dpoint(0, M.vid[a].x) - B.dpoint(1, M.vid[a].y);
  const dv3 q1 = B.dpoint(0, M.vid[b].x) - B.dpoint(1, M.vid[b].y);
  const dv3 q2 = B.dpoint(0, M.vid[c].x) - B.dpoint(1, M.vid[c].y);
  const dv3 m = cross(q1 - q0, q2 - q0);
  const double mm = dot(m, m);
  if (!(mm > 0.0)) return make_double4_(0.0, 0.0, 0.0, (double)INFINITY);
  const double inv = 1.0 / sqrt(mm);
  return make_double4_(m.x * inv, m.y * inv, m.z * inv, dot(m, q0) * inv);
}

// Thin-contact check at FP32 convergence: true when exact supports along face f's FP64
// plane improve on the face by more than tol.
template <class Team, class Bodies, class Mem>
OGX_HD bool thin_gain_exceeds(const Team& t, const Bodies& B, const Mem& M, int f, float tol) {
  const double4 p = face_plane64(M, B, f);
  if (!(p.w < (double)INFINITY)) return false;
  const dv3 n64 = v3<double>(p.x, p.y, p.z);
  double ha, hb;
  exact_support(t, B, 0, n64, ha);
  exact_support(t, B, 1, -n64, hb);
  return ha + hb - p.w > (double)tol;
}

// plane of face (a, b, c): FP32, FP64 from exact points for slivers
template <class Mem, class Bodies>
OGX_HD float4 face_plane(const Mem& M, const Bodies& B, int a, int b, int c, bool escalate, bool all64,
                         int& status, double4* p64 = nullptr) {
  const float4 P0 = M.vp[a], P1 = M.vp[b], P2 = M.vp[c];
  const fv3 p0 = v3<float>(P0.x, P0.y, P0.z);
  const fv3 e0 = v3<float>(P1.x, P1.y, P1.z) - p0;
  const fv3 e1 = v3<float>(P2.x, P2.y, P2.z) - p0;
  const fv3 n = cross(e0, e1);
  const float nn = dot(n, n);
  const float s = l1(e0) * l1(e1);
  float4 r;
  if (all64 || (escalate && nn < 1e-6f * s * s)) {
    // sine of the face angle below ~1e-3: FP32 normal unreliable
    const dv3 q0 = B.dpoint(0, M.vid[a].x) - B.dpoint(1, M.vid[a].y);
    const dv3 q1 = B.dpoint(0, M.vid[b].x) - B.dpoint(1, M.vid[b].y);
    const dv3 q2 = B.dpoint(0, M.vid[c].x) - B.dpoint(1, M.vid[c].y);
    const dv3 m = cross(q1 - q0, q2 - q0);
    const double mm = dot(m, m);
    status |= OGX_S_EPA_ESCALATED;
    if (mm > 0.0) {
      const double inv = 1.0 / sqrt(mm);
      r.x = (float)(m.x * inv);
      r.y = (float)(m.y * inv);
      r.z = (float)(m.z * inv);
      r.w = (float)(dot(m, q0) * inv);
      if (p64) *p64 = make_double4_(m.x * inv, m.y * inv, m.z * inv, dot(m, q0) * inv);
    } else {
      r.x = r.y = r.z = 0.0f;
      r.w = INFINITY;  // degenerate: never the closest face, never visible
      if (p64) *p64 = make_double4_(0.0, 0.0, 0.0, (double)INFINITY);
    }
    return r;
  }
  if (nn > 0.0f) {
    const float inv = 1.0f / sqrtf(nn);
    r.x = n.x * inv;
    r.y = n.y * inv;
    r.z = n.z * inv;
    r.w = r.x * p0.x + r.y * p0.y + r.z * p0.z;
  } else {
    r.x = r.y = r.z = 0.0f;
    r.w = INFINITY;
  }
  return r;
}

// barycentric weights of the origin's projection on triangle (p0, p1, p2), clamped to
// the triangle's edges as EPA.c:238-304 does
OGX_HD int tri_weights(fv3 p0, fv3 p1, fv3 p2, float* l) {
  const fv3 e0 = p1 - p0, e1 = p2 - p0;
  const float d00 = dot(e0, e0), d01 = dot(e0, e1), d11 = dot(e1, e1);
  const float d20 = -dot(p0, e0), d21 = -dot(p0, e1);
  const float den = d00 * d11 - d01 * d01;
  if (fabsf(den) < FLT_EPSILON) {
    l[0] = l[1] = l[2] = 1.0f / 3.0f;
    return -1;
  }
  const float inv = 1.0f / den;
  const float u = (d11 * d20 - d01 * d21) * inv;
  const float v = (d00 * d21 - d01 * d20) * inv;
  const float w = 1.0f - u - v;
  if (w < 0.0f) {
    const fv3 e12 = p2 - p1;
    float tt = -dot(p1, e12) / dot(e12, e12);
    tt = fmaxf(0.0f, fminf(1.0f, tt));
    l[0] = 0.0f;
    l[1] = 1.0f - tt;
    l[2] = tt;
    return 1;  // beyond edge p1-p2 (edge 1 of the face)
  } else if (u < 0.0f) {
    float tt = -dot(p0, e1) / dot(e1, e1);
    tt = fmaxf(0.0f, fminf(1.0f, tt));
    l[0] = 1.0f - tt;
    l[1] = 0.0f;
    l[2] = tt;
    return 2;  // beyond edge p2-p0
  } else if (v < 0.0f) {
    float tt = -dot(p0, e0) / dot(e0, e0);
    tt = fmaxf(0.0f, fminf(1.0f, tt));
    l[0] = 1.0f - tt;
    l[1] = tt;
    l[2] = 0.0f;
    return 0;  // beyond edge p0-p1
  }
  l[0] = w;
  l[1] = u;
  l[2] = v;
  return -1;
}

// Result from face f.  When the origin's projection falls outside f and the face across
// that edge lies in the same plane (the Minkowski face of an edge-edge or face-face
// contact is split into coplanar triangles), the neighbour that holds the projection is
// used, so that w0 - w1 = depth * normal holds.
template <class Mem, class Bodies>
// With rerun_ok, returns true when the origin's projection leaves the closest face
// towards a neighbour more than 1e-5 rad off its plane (sine from the cross product of the
// two FP32 normals, kEpaHopSin2): nothing is emitted then and the caller runs the contact
// again with FP64 planes.  Without (the FP64-plane pass
// itself, whose closest face is picked on the planes rounded to float, so two faces a
// rounding apart can swap), the result comes from that near-coplanar neighbour, which
// holds the projection.
OGX_HD bool epa_emit(const Mem& M, const Bodies& B, int f, float tie, EpaOut& o, bool rerun_ok) {
  int a = M.fv[f][0], b = M.fv[f][1], c = M.fv[f][2];
  float l[3];
  for (int hop = 0; hop < 4; ++hop) {
    a = M.fv[f][0];
    b = M.fv[f][1];
    c = M.fv[f][2];
    const float4 P0 = M.vp[a], P1 = M.vp[b], P2 = M.vp[c];
    const int out = tri_weights(v3<float>(P0.x, P0.y, P0.z), v3<float>(P1.x, P1.y, P1.z),
                                v3<float>(P2.x, P2.y, P2.z), l);
    if (out < 0) break;
    const int g2 = M.fa[f][out];
    const float4 nf = M.fn[f], ng = M.fn[g2];
    const bool near = M.fv[g2][3] && fabsf(ng.w - nf.w) <= tie &&
                      (nf.x * ng.x + nf.y * ng.y + nf.z * ng.z) > 1.0f - 1e-5f;
    if (!near) break;
    // In exact arithmetic the origin projects into the closest face of the convex
    // polytope, so a neighbour it leaves through is coplanar with it (a flat patch split
    // into triangles -- two points of one body against two of the other make an exact
    // parallelogram: the witnesses come from the neighbour).  A neighbour more than 1e-5
    // rad off -- FP32 planes made the polytope a little non-convex or ranked the faces
    // wrongly, on dense flat patches -- would give a normal up to a few 1e-4 off and
    // witnesses off the normal: the FP32 pass runs the contact again on FP64 planes.
    const float sx = nf.y * ng.z - nf.z * ng.y, sy = nf.z * ng.x - nf.x * ng.z, sz = nf.x * ng.y - nf.y * ng.x;
    if (sx * sx + sy * sy + sz * sz > kEpaHopSin2 && rerun_ok) return true;
    f = g2;
  }
  const int2 ia = M.vid[a], ib = M.vid[b], ic = M.vid[c];
  o.w0 = B.point(0, ia.x) * l[0] + B.point(0, ib.x) * l[1] + B.point(0, ic.x) * l[2];
  o.w1 = B.point(1, ia.y) * l[0] + B.point(1, ib.y) * l[1] + B.point(1, ic.y) * l[2];
  const float4 n = M.fn[f];
  o.nrm = v3<float>(n.x, n.y, n.z);
  o.dist = -n.w;
  o.face[0][0] = ia.x;
  o.face[0][1] = ia.y;
  o.face[1][0] = ib.x;
  o.face[1][1] = ib.y;
  o.face[2][0] = ic.x;
  o.face[2][1] = ic.y;
  return false;
}

OGX_HD void epa_touch(fv3 a, fv3 b, EpaOut& o) {
  o.dist = 0.0f;
  o.w0 = a;
  o.w1 = b;
  o.nrm = unit_or_x(b - a);
  o.status |= OGX_S_EPA_TOUCH;
}

// exact FP64 re-solve of the final face (plane, depth, witnesses)
template <class Bodies>
OGX_HD void epa_polish(const Bodies& B, EpaOut& o) {
  // double-float arithmetic (about 48 bits) on the FP32 pipes: FP64 issues at 1/64 of
  // the FP32 rate on this part, and the results are rounded to float
  fv3 A[3], Bq[3];
  xv3 Q[3];
  for (int k = 0; k < 3; ++k) {
    A[k] = B.point(0, o.face[k][0]);
    Bq[k] = B.point(1, o.face[k][1]);
    Q[k] = xdiff(A[k], Bq[k]);
  }
  const df zero = sc<df>(0.0f), one = sc<df>(1.0f);
  const xv3 m = cross(Q[1] - Q[0], Q[2] - Q[0]);
  const df mm = dot(m, m);
  if (!(mm > zero)) return;
  const df inv = one / df_sqrt(mm);
  xv3 n = m * inv;
  df d = dot(n, Q[0]);
  // keep the orientation chosen during the expansion
  if (n.x * sc<df>(o.nrm.x) + n.y * sc<df>(o.nrm.y) + n.z * sc<df>(o.nrm.z) < zero) {
    n = -n;
    d = -d;
  }
  // barycentric weights of the projection of the origin, clamped like tri_weights
  const xv3 e0 = Q[1] - Q[0], e1 = Q[2] - Q[0];
  const df d00 = dot(e0, e0), d01 = dot(e0, e1), d11 = dot(e1, e1);
  const df d20 = -dot(Q[0], e0), d21 = -dot(Q[0], e1);
  const df den = d00 * d11 - d01 * d01;
  const df third = one / sc<df>(3.0f);
  df l[3] = {third, third, third};
  if (den.hi != 0.0f) {
    const df u = (d11 * d20 - d01 * d21) / den;
    const df v = (d00 * d21 - d01 * d20) / den;
    const df w = one - u - v;
    if (w < zero) {
      const xv3 e12 = Q[2] - Q[1];
      df tt = -dot(Q[1], e12) / dot(e12, e12);
      tt = tt < zero ? zero : (tt > one ? one : tt);
      l[0] = zero; l[1] = one - tt; l[2] = tt;
    } else if (u < zero) {
      df tt = -dot(Q[0], e1) / dot(e1, e1);
      tt = tt < zero ? zero : (tt > one ? one : tt);
      l[0] = one - tt; l[1] = zero; l[2] = tt;
    } else if (v < zero) {
      df tt = -dot(Q[0], e0) / dot(e0, e0);
      tt = tt < zero ? zero : (tt > one ? one : tt);
      l[0] = one - tt; l[1] = tt; l[2] = zero;
    } else {
      l[0] = w; l[1] = u; l[2] = v;
    }
  }
  auto lift = [](fv3 p) { return v3<df>(sc<df>(p.x), sc<df>(p.y), sc<df>(p.z)); };
  const xv3 w0 = lift(A[0]) * l[0] + lift(A[1]) * l[1] + lift(A[2]) * l[2];
  const xv3 w1 = lift(Bq[0]) * l[0] + lift(Bq[1]) * l[1] + lift(Bq[2]) * l[2];
  o.w0 = v3<float>(to_float(w0.x), to_float(w0.y), to_float(w0.z));
  o.w1 = v3<float>(to_float(w1.x), to_float(w1.y), to_float(w1.z));
  o.nrm = v3<float>(to_float(n.x), to_float(n.y), to_float(n.z));
  o.dist = to_float(-d);
  o.status |= OGX_S_POLISHED;
}

template <class Team, class Mem>
OGX_HD void epa_save(const Team& t, const Mem& M, const EpaResumeSink& sink, EpaOut& o, int nv, int fend,
                     int it, int st, float scale2) {
  if (!sink.buf) return;
  int slot = -1;
  if (t.lane() == 0) {
#if defined(__CUDA_ARCH__)
    slot = atomicAdd(sink.count, 1);
#else
    slot = (*sink.count)++;
#endif
  }
  slot = t.imax(slot);
  if (slot >= sink.cap) return;
  EpaResume& R = sink.buf[slot];
  for (int j = t.lane(); j < nv; j += Team::L) {
    R.vp[j] = M.vp[j];
    R.vid[j] = M.vid[j];
  }
  for (int f = t.lane(); f < fend; f += Team::L) {
    R.fn[f] = M.fn[f];
    for (int k = 0; k < 4; ++k) {
      R.fv[f][k] = M.fv[f][k];
      R.fa[f][k] = M.fa[f][k];
    }
  }
  if (t.lane() == 0) {
    R.nv = nv;
    R.fend = fend;
    R.it = it;
    R.st = st;
    R.status = o.status;
    R.scale2 = scale2;
  }
  o.resume = slot;
}

// Run EPA for one pair whose GJK result is g.  `M` is this pair's shared working set.
//
// One expansion step, with the faces of the polytope split over the team's lanes
// (face f on lane f mod L):
//   1. every lane tests its live faces for visibility from the new point q and keeps the
//      closest face that stays (not visible);
//   2. visible faces are ranked in increasing slot order and horizon edges in increasing
//      (face, edge) order with ballots, so slot assignment does not depend on L; new face
//      k takes the k-th visible slot, then fresh slots at the end of the used range;
//   3. faces beyond the horizon are relinked to the new faces, the visible faces retired;
//   4. new faces are linked to each other through the per-vertex tables and their planes
//      computed; the closest new face joins the lane's candidate.
// The next step's closest face is the team's minimum over the candidates.
// kCert (the full-capacity re-run only): with FP64 face planes on, run the certified
// expansion described at kEpaCertGain.
// sink: where a capacity spill saves itself (small pass); rs: a saved expansion to
// continue instead of starting from the GJK simplex (full pass).
template <bool kCert = false, class Team, class Bodies, class Mem>
OGX_HD void epa_pair(const Team& t, const Bodies& B, const Config& cfg, const GjkState& g,
                     Mem& M, EpaOut& o, bool can_spill, EpaResumeSink sink = EpaResumeSink{nullptr, nullptr, 0},
                     const EpaResume* rs = nullptr) {
  const int L = Team::L;
  const int lane = t.lane();
  const bool escalate = (cfg.flags & OGX_F_FP64_ESCALATE) != 0;
  const bool all64 = (cfg.flags & OGX_F_EPA_FP64_PLANES) != 0;
  const bool cert = kCert && all64;
  o.status = 0;
  o.iters = 0;
  o.polish = false;
  o.spill = false;
  o.spill64 = false;
  o.resume = -1;
  o.dist = g.dist;
  o.w0 = g.w0;
  o.w1 = g.w1;
  o.nrm = unit_or_x(g.w1 - g.w0);
  if (g.n != 4 && g.dist > FLT_EPSILON) return;  // separated (EPA.c:369-373)
  o.status |= OGX_S_EPA_RUN;
  float scale2 = 0.0f;
  int st = 0;
  // per-lane closest candidate (slot, plane distance); -1 = none
  float cbd = INFINITY;
  int cbest = -1;
  int nv = 4, fend = 4;
  int it = 0;
  if (rs) {
    nv = rs->nv;
    fend = rs->fend;
    it = rs->it;
    st = rs->st;
    scale2 = rs->scale2;
    o.status = rs->status;
    for (int j = lane; j < nv; j += L) {
      M.vp[j] = rs->vp[j];
      M.vid[j] = rs->vid[j];
    }
    for (int f = lane; f < fend; f += L) {
      M.fn[f] = rs->fn[f];
      for (int k = 0; k < 4; ++k) {
        M.fv[f][k] = rs->fv[f][k];
        M.fa[f][k] = rs->fa[f][k];
      }
    }
    t.sync();
    for (int f = lane; f < fend; f += L)
      if (M.fv[f][3] && M.fn[f].w < cbd) {
        cbd = M.fn[f].w;
        cbest = f;
      }
  } else {

  // ---- grow the simplex to a tetrahedron (EPA.c:375-583)
  // simplex in registers: every index below is a constant after unrolling
  fv3 P[4];
  int IA[4], IB[4];
  int n = g.n;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    P[j] = g.P[j];
    IA[j] = g.ia[j];
    IB[j] = g.ib[j];
  }
  const float e2 = FLT_EPSILON * FLT_EPSILON;
  auto is_new = [&](fv3 q, int qa, int qb) {
    bool fresh = true;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const fv3 d = q - P[j];
      if (j < n && (dot(d, d) < e2 || (IA[j] == qa && IB[j] == qb))) fresh = false;
    }
    return fresh;
  };
  auto append = [&](fv3 q, int qa, int qb) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (j == n) {
        P[j] = q;
        IA[j] = qa;
        IB[j] = qb;
      }
    ++n;
  };
  if (n == 1) {
    int qa, qb;
    const fv3 q = msupport(t, B, P[0], qa, qb);
    if (!is_new(q, qa, qb)) {
      epa_touch(B.point(0, qa), B.point(1, qb), o);
      return;
    }
    append(q, qa, qb);
  }
  if (n == 2) {
    const fv3 e = P[1] - P[0];
    fv3 axis = v3<float>(1.0f, 0.0f, 0.0f);
    const float el = sqrtf(dot(e, e));
    if (el > FLT_EPSILON && fabsf(e.x) > 0.9f * el) axis = v3<float>(0.0f, 1.0f, 0.0f);
    fv3 d = cross(e, axis);
    if (dot(d, d) < FLT_EPSILON) d = cross(e, v3<float>(0.0f, 0.0f, 1.0f));
    int qa, qb;
    const fv3 q = msupport(t, B, d, qa, qb);
    if (!is_new(q, qa, qb)) {
      epa_touch(B.point(0, qa), B.point(1, qb), o);
      return;
    }
    append(q, qa, qb);
  }
  if (n == 3) {
    fv3 d = cross(P[1] - P[0], P[2] - P[0]);
    int qa, qb;
    fv3 q = msupport(t, B, d, qa, qb);
    if (!is_new(q, qa, qb)) {
      q = msupport(t, B, -d, qa, qb);
      if (!is_new(q, qa, qb)) {
        epa_touch(B.point(0, qa), B.point(1, qb), o);
        return;
      }
    }
    append(q, qa, qb);
  }

  // ---- tetrahedron
  const float vol = dot(P[1] - P[0], cross(P[2] - P[0], P[3] - P[0]));
  // outward faces of a positively oriented tetrahedron (0,1,2,3); swap 1 and 2 otherwise:
  // (0, i2, i1), (0, i1, 3), (i1, i2, 3), (i2, 0, 3).  Face across edge k of face f
  // (edge k = vertices k, k+1 mod 3) is the same for both orientations.
  const int i1 = vol >= 0.0f ? 1 : 2, i2 = vol >= 0.0f ? 2 : 1;
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      M.vp[j] = make_float4_(P[j].x, P[j].y, P[j].z, 0.0f);
      M.vid[j] = make_int2_(IA[j], IB[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) scale2 = fmaxf(scale2, dot(P[j], P[j]));
  t.sync();
  for (int f = lane; f < 4; f += L) {
    const int va = f == 2 ? i1 : (f == 3 ? i2 : 0);
    const int vb = f == 0 ? i2 : (f == 1 ? i1 : (f == 2 ? i2 : 0));
    const int vc = f == 0 ? i1 : 3;
    M.fv[f][0] = (uint8_t)va;
    M.fv[f][1] = (uint8_t)vb;
    M.fv[f][2] = (uint8_t)vc;
    M.fv[f][3] = 1;
    // {3,2,1}, {0,2,3}, {0,3,1}, {0,1,2}
    M.fa[f][0] = (uint8_t)(f == 0 ? 3 : 0);
    M.fa[f][1] = (uint8_t)(f == 0 || f == 1 ? 2 : (f == 2 ? 3 : 1));
    M.fa[f][2] = (uint8_t)(f == 0 ? 1 : (f == 1 ? 3 : (f == 2 ? 1 : 2)));
    const float4 pl = face_plane(M, B, va, vb, vc, escalate, all64, st, plane64_slot(M, f));
    M.fn[f] = pl;
    if (pl.w < cbd) {
      cbd = pl.w;
      cbest = f;
    }
  }
  t.sync();
  }

  const float tol_floor = cfg.epa_tol;
  int best = -1;
  bool done = false;
  bool thin = false;
  float thin_tol = 0.0f;
  while (it < cfg.epa_max_iter) {
    ++it;
    // closest live face
    float bd = cbd;
    best = cbest;
    t.argmin(bd, best);
    if (best < 0 || !(bd < INFINITY)) {
      o.status |= OGX_S_EPA_TOPOLOGY;
      best = -1;
      done = true;
      break;
    }
    const float4 nf = M.fn[best];
    const fv3 n = v3<float>(nf.x, nf.y, nf.z);
    int qa, qb;
    fv3 q;
    dv3 q64 = v3<double>(0.0, 0.0, 0.0);
    float scale;
    bool conv;
    float gain = 0.0f;
    if (cert) {
      // exact supports along the closest face's FP64 normal
      const double4 pl = *plane64_slot(M, best);
      const dv3 n64 = v3<double>(pl.x, pl.y, pl.z);
      double ha, hb;
      qa = exact_support(t, B, 0, n64, ha);
      qb = exact_support(t, B, 1, -n64, hb);
      q = B.point(0, qa) - B.point(1, qb);
      q64 = B.dpoint(0, qa) - B.dpoint(1, qb);
      scale = sqrtf(fmaxf(scale2, dot(q, q)));
      conv = !(ha + hb - pl.w > kEpaCertTol * fmax(1.0, (double)scale));
    } else {
      q = msupport(t, B, n, qa, qb);
      scale = sqrtf(fmaxf(scale2, dot(q, q)));
      const float tol = fmaxf(tol_floor, cfg.epa_rel * scale);
      gain = dot(n, q) - bd;
      conv = gain < tol;
      // a thin contact: the FP32 test may have been fooled by the face normal's rounding;
      // checked after the loop (its FP64 scans would weigh on the loop's registers)
      thin = conv && !all64 && escalate && can_spill && !(gain > kEpaCertGain * scale) && bd < kEpaThin * scale;
      thin_tol = tol;
    }
    if (conv) {
      if (!cert && escalate && can_spill && !all64 && gain > kEpaCertGain * scale) {
        o.spill = true;
        o.spill64 = true;
        return;
      }
      o.status |= OGX_S_EPA_CONVERGED;
      done = true;
      break;
    }
    bool dup = false;
    for (int j = lane; j < nv; j += L) {
      const int2 id = M.vid[j];
      dup |= (id.x == qa && id.y == qb);
    }
    if (t.any(dup)) {
      // the support is already a vertex although the closest face is not converged:
      // FP32 planes put a vertex in front of a face; re-run certified
      if (!cert && escalate && can_spill && !all64) {
        o.spill = true;
        o.spill64 = true;
        return;
      }
      o.status |= OGX_S_EPA_DUPLICATE;
      done = true;
      break;
    }
    if (nv >= Mem::kV) {
      if (can_spill) {
        epa_save(t, M, sink, o, nv, fend, it - 1, st, scale2);
        o.spill = true;
        return;
      }
      o.status |= OGX_S_EPA_CAPACITY;
      done = true;
      break;
    }
    const int p = nv;
    if (lane == 0) {
      M.vp[p] = make_float4_(q.x, q.y, q.z, 0.0f);
      M.vid[p] = make_int2_(qa, qb);
    }
    ++nv;
    scale2 = fmaxf(scale2, dot(q, q));
    const float vis_eps = cfg.epa_vis * scale;

    // 1. faces seen from q; the closest face that stays
    cbd = INFINITY;
    cbest = -1;
    int nvis = 0;
    for (int f0 = 0; f0 < fend; f0 += L) {
      const int f = f0 + lane;
      bool s = false;
      if (f < fend && M.fv[f][3]) {
        const float4 fp = M.fn[f];
        if (cert) {
          const double4 pl = *plane64_slot(M, f);
          s = (pl.x * q64.x + pl.y * q64.y + pl.z * q64.z) - pl.w > kEpaCertVis * (double)scale;
        } else {
          s = (fp.x * q.x + fp.y * q.y + fp.z * q.z) - fp.w > vis_eps;
        }
        if (!s && fp.w < cbd) {
          cbd = fp.w;
          cbest = f;
        }
      }
      if (f < fend) M.vis[f] = s;
      const uint32_t m = t.ballot(s);
      if (s) M.vlist[nvis + popc32(m & t.below())] = (uint8_t)f;
      nvis += popc32(m);
    }
    t.sync();
    // the closest face must be seen (gain >= tol > vis threshold); otherwise stop (or,
    // from the small pass, start again with FP64 planes in the full pass)
    if (!M.vis[best]) {
      if (can_spill && escalate) {
        o.spill = true;
        o.spill64 = true;
        return;
      }
      o.status |= OGX_S_EPA_TOPOLOGY;
      done = true;
      break;
    }
    // 2. horizon edges: edge e of a visible face whose neighbour is not visible
    int htot = 0;
    for (int k0 = 0; k0 < nvis; k0 += L) {
      const int k = k0 + lane;
      bool h[3] = {false, false, false};
      int f = 0;
      if (k < nvis) {
        f = M.vlist[k];
        for (int e = 0; e < 3; ++e) h[e] = !M.vis[M.fa[f][e]];
      }
      const uint32_t m0 = t.ballot(h[0]), m1 = t.ballot(h[1]), m2 = t.ballot(h[2]);
      const uint32_t lo = t.below();
      int r = htot + popc32(m0 & lo) + popc32(m1 & lo) + popc32(m2 & lo);
      for (int e = 0; e < 3; ++e) {
        if (!h[e]) continue;
        if (r < Mem::kF) {
          M.hz[r][0] = M.fv[f][e];
          M.hz[r][1] = M.fv[f][(e + 1) % 3];
          M.hz[r][2] = M.fa[f][e];
        }
        ++r;
      }
      htot += popc32(m0) + popc32(m1) + popc32(m2);
    }
    // new face k goes to vlist[k] (k < nvis), else to fresh slot fend + k - nvis
    if (htot < 3) {
      if (can_spill && escalate) {
        o.spill = true;
        o.spill64 = true;
        return;
      }
      o.status |= OGX_S_EPA_TOPOLOGY;
      done = true;
      break;
    }
    if (fend + (htot > nvis ? htot - nvis : 0) > Mem::kF) {
      if (can_spill) {
        epa_save(t, M, sink, o, nv - 1, fend, it - 1, st, scale2);  // before q was added
        o.spill = true;
        return;
      }
      o.status |= OGX_S_EPA_CAPACITY;
      done = true;
      break;
    }
    t.sync();
    // 3. relink the faces outside the horizon, index the horizon by its vertices, retire
    // the visible faces
    for (int k = lane; k < htot; k += L) {
      const int s = k < nvis ? M.vlist[k] : fend + k - nvis;
      const int a = M.hz[k][0], b = M.hz[k][1], g2 = M.hz[k][2];
      for (int m = 0; m < 3; ++m)
        if (M.fv[g2][m] == b && M.fv[g2][(m + 1) % 3] == a) M.fa[g2][m] = (uint8_t)s;
      M.hstart[a] = (uint8_t)s;
      M.hend[b] = (uint8_t)s;
    }
    for (int k = lane; k < nvis; k += L) M.fv[M.vlist[k]][3] = 0;
    t.sync();
    // a vertex that starts (or ends) two horizon edges means the horizon is not one
    // simple loop; keep the closest face found this step and stop
    bool bad = false;
    for (int k = lane; k < htot; k += L) {
      const int s = k < nvis ? M.vlist[k] : fend + k - nvis;
      bad |= (M.hstart[M.hz[k][0]] != s) || (M.hend[M.hz[k][1]] != s);
    }
    if (t.any(bad)) {
      if (can_spill && escalate) {
        o.spill = true;
        o.spill64 = true;
        return;
      }
      o.status |= OGX_S_EPA_TOPOLOGY;
      done = true;
      break;
    }
    // 4. new face (a, b, p) across each horizon edge a->b
    for (int k = lane; k < htot; k += L) {
      const int s = k < nvis ? M.vlist[k] : fend + k - nvis;
      const int a = M.hz[k][0], b = M.hz[k][1];
      M.fv[s][0] = (uint8_t)a;
      M.fv[s][1] = (uint8_t)b;
      M.fv[s][2] = (uint8_t)p;
      M.fa[s][0] = M.hz[k][2];
      M.fa[s][1] = M.hstart[b];
      M.fa[s][2] = M.hend[a];
      const float4 pl = face_plane(M, B, a, b, p, escalate, all64, st, plane64_slot(M, s));
      M.fn[s] = pl;
      M.fv[s][3] = 1;
      if (pl.w < cbd || (pl.w == cbd && s < cbest)) {
        cbd = pl.w;
        cbest = s;
      }
    }
    if (htot > nvis) fend += htot - nvis;
    t.sync();
  }
  o.iters = it;
  o.status |= st ? OGX_S_EPA_ESCALATED : 0;
  o.status |= cert ? OGX_S_EPA_CERTIFIED : 0;
  if (!done) {
    // iteration cap: closest current face
    float bd = cbd;
    best = cbest;
    t.argmin(bd, best);
    o.status |= OGX_S_EPA_CAP;
  }
  if (thin && best >= 0 && thin_gain_exceeds(t, B, M, best, thin_tol)) {
    o.spill = true;
    o.spill64 = true;
    return;
  }
  if (best >= 0) {
    const bool rerun = !cert && escalate && can_spill && !all64;
    if (epa_emit(M, B, best, fmaxf(cfg.epa_tol, cfg.epa_rel * sqrtf(scale2)), o, rerun)) {
      o.spill = true;
      o.spill64 = true;
      return;
    }
    o.polish = (cfg.flags & OGX_F_FP64_POLISH) != 0;
  }
}

}  // namespace ogx
