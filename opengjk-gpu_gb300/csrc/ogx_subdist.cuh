// ogx_subdist.cuh -- FP32 sub-distance step of GJK with all sign decisions computed up
// front, branch-free, from shared dot products.
//
// The decisions are those of the signed-volume sub-distance algorithm of
// GJK/cpu/openGJK.c:219-613 (S1D/S2D/S3D with the hff1/hff2/hff3 tests).  With q1 the
// newest simplex point and e_k = P_k - q1 for the older points P_k:
//   hff1(q1, P_k)      "the origin projects beyond q1 towards P_k" <=>  a_k = q1.e_k < 0
//   hff2(q1, P_j, P_k)  <=>  q1.(e_j x (e_j x e_k)) < 0  <=>  a_j (e_j.e_k) - a_k (e_j.e_j) < 0
//   hff3(q1, P_j, P_k)  <=>  q1.(P_j x P_k) <= 0       <=>  q1.(e_j x e_k) <= 0
// (the last two use a x (b x c) = b (a.c) - c (a.b) and q1.(q1 x .) = 0).  So a
// tetrahedron step needs 3 dots a_k, 6 dots e_j.e_k and 3 cross products, about 160 FP32
// operations, instead of one inlined cross-product chain per test.  Every value carries a
// forward error bound; a decision inside its bound sets its bit in `unc`.
//
// The decision tree itself (which vertices stay, in which order, and what kind of
// projection gives the new direction) runs on the predicate bits only: a few integer
// branches, the only divergent part.  Projections reuse the same dot products.
#pragma once

#include "ogx_common.cuh"

namespace ogx {

// predicate bits of a tetrahedron step (older slots 0, 1, 2; q1 = slot 3)
enum : uint32_t {
  PB_K0 = 1u << 0,  // hff1(q1, P0)   (K(s) = bit s)
  PB_NEG = 1u << 3, // det(e1, e0, e2) <= 0   (the reference's det134 <= 0)
  PB_F2 = 1u << 4,  // hff3(q1, P1, P0)
  PB_F3 = 1u << 5,  // hff3(q1, P0, P2)
  PB_F4 = 1u << 6,  // hff3(q1, P2, P1)
  PB_D = 7,         // hff2(q1, Pj, Pk) at bit PB_D + dpair(j, k)
};

OGX_HD int dpair(int j, int k) {  // (0,1) (1,0) (0,2) (2,0) (1,2) (2,1)
  const int lo = j < k ? j : k, hi = j < k ? k : j;
  const int base = (lo == 0 && hi == 1) ? 0 : (lo == 0 ? 2 : 4);
  return base + (j > k ? 1 : 0);
}

// outcome of a step: new simplex = slots s[0..n) (3 = q1), and how v is obtained
enum { SO_VERTEX = 0, SO_LINE = 1, SO_PLANE = 2, SO_ZERO = 3, SO_KEEP = 4 };
struct SubOut {
  int n;
  int s[3];
  int kind;       // SO_*
  int a, b;       // older slots spanning the line (a) or the plane (a, b) with q1
  uint32_t used;  // predicate bits the decision consulted
};

struct Bits {
  uint32_t v, used;
  OGX_HD bool operator()(uint32_t m) {
    used |= m;
    return (v & m) != 0u;
  }
  OGX_HD bool D(int j, int k) { return (*this)(1u << (PB_D + dpair(j, k))); }
  OGX_HD bool K(int s) { return (*this)(1u << s); }
};

OGX_HD SubOut so_vertex(int s) {
  SubOut o;
  o.n = 1; o.s[0] = s; o.s[1] = o.s[2] = 0; o.kind = SO_VERTEX; o.a = o.b = 0; o.used = 0;
  return o;
}
OGX_HD SubOut so_line(int first, int second, int a) {
  SubOut o;
  o.n = 2; o.s[0] = first; o.s[1] = second; o.s[2] = 0; o.kind = SO_LINE; o.a = a; o.b = 0; o.used = 0;
  return o;
}
OGX_HD SubOut so_plane(int s0, int s1, int s2, int a, int b) {
  SubOut o;
  o.n = 3; o.s[0] = s0; o.s[1] = s1; o.s[2] = s2; o.kind = SO_PLANE; o.a = a; o.b = b; o.used = 0;
  return o;
}

// triangle (older slots t0 = "q3", t1 = "q2", newest slot q) -- openGJK.c:270-313
OGX_HD SubOut tri_tree(Bits& B, int t0, int t1, int q) {
  const bool k12 = B.K(t1), k13 = B.K(t0);
  if (k12) {
    if (!B.D(t1, t0)) {
      if (k13 && B.D(t0, t1)) return so_line(t0, q, t0);
      return so_plane(t0, t1, q, t0, t1);
    }
    return so_line(q, t1, t1);
  }
  if (k13) {
    if (B.D(t0, t1)) return so_line(t0, q, t0);
    return so_plane(t0, t1, q, t0, t1);
  }
  return so_vertex(q);
}

// tetrahedron, older slots 0 (q4), 1 (q3), 2 (q2), newest 3 -- openGJK.c:315-613
OGX_HD SubOut tetra_tree(Bits& B) {
  const bool l2 = B.K(2), l3 = B.K(1), l4 = B.K(0);
  const int nkeep = (int)l2 + (int)l3 + (int)l4;
  if (nkeep == 0) return so_vertex(3);
  const int neg = B(PB_NEG) ? 1 : 0;
  const int f2 = ((B(PB_F2) ? 1 : 0) - neg) != 0;
  const int f3 = ((B(PB_F3) ? 1 : 0) - neg) != 0;
  const int f4 = ((B(PB_F4) ? 1 : 0) - neg) != 0;
  SubOut o;
  switch (f2 + f3 + f4) {
    case 3:
      o = so_vertex(3);
      o.n = 4;
      o.kind = SO_ZERO;
      return o;
    case 2:
      if (!f2) return tri_tree(B, 0, 1, 3);  // [q4, q3, q1]
      if (!f3) return tri_tree(B, 0, 2, 3);  // [q4, q2, q1]
      return tri_tree(B, 1, 2, 3);           // [q3, q2, q1]
    case 1: {
      int k, i, j;
      if (f2) { k = 2; i = 1; j = 0; } else if (f3) { k = 1; i = 0; j = 2; } else { k = 0; i = 2; j = 1; }
      const bool lk = B.K(k), li = B.K(i), lj = B.K(j);
      if (nkeep == 1) {
        if (lk) {
          if (!B.D(k, i)) return so_plane(k, i, 3, i, k);
          if (!B.D(k, j)) return so_plane(k, j, 3, j, k);
          return so_line(k, 3, k);
        }
        if (li) {
          if (!B.D(i, k)) return so_plane(k, i, 3, i, k);
          return so_line(i, 3, i);
        }
        if (!B.D(j, k)) return so_plane(k, j, 3, j, k);
        return so_line(j, 3, j);
      }
      if (nkeep == 2) {
        if (li) {
          if (!B.D(k, i)) {
            if (!B.D(i, k)) return so_plane(k, i, 3, i, k);
            return so_line(k, 3, k);
          }
          if (!B.D(k, j)) return so_plane(k, j, 3, j, k);
          return so_line(k, 3, k);
        }
        if (lj) {
          if (!B.D(k, j)) {
            if (!B.D(j, k)) return so_plane(k, j, 3, j, k);
            return so_line(j, 3, j);
          }
          if (!B.D(k, i)) return so_plane(k, i, 3, i, k);
          return so_line(k, 3, k);
        }
        // neither edge test holds: the reference keeps slots 0..2 and v (openGJK.c:494)
        o = so_plane(0, 1, 2, 0, 1);
        o.kind = SO_KEEP;
        return o;
      }
      const bool d_ik = B.D(i, k), d_jk = B.D(j, k), d_ki = B.D(k, i), d_kj = B.D(k, j);
      if (d_ki && d_kj) return so_line(k, 3, k);
      if (d_ki) return d_jk ? so_line(j, 3, j) : so_plane(k, j, 3, k, j);
      return d_ik ? so_line(i, 3, i) : so_plane(k, i, 3, k, i);
    }
    default: {  // case 0
      if (nkeep == 1) {
        int k, i, j;
        if (l3) { k = 2; i = 1; j = 0; } else if (l4) { k = 1; i = 0; j = 2; } else { k = 0; i = 2; j = 1; }
        if (!B.D(i, j)) return so_plane(j, i, 3, i, j);
        if (!B.D(i, k)) return so_plane(k, i, 3, i, k);
        return so_line(i, 3, i);
      }
      if (nkeep == 2) {
        int k, i, j;
        if (!l3) { k = 2; i = 1; j = 0; } else if (!l4) { k = 1; i = 0; j = 2; } else { k = 0; i = 2; j = 1; }
        if (!B.D(j, k)) {
          if (!B.D(k, j)) return so_plane(k, j, 3, j, k);
          if (!B.D(k, i)) return so_plane(k, i, 3, k, i);
          return so_line(k, 3, k);
        }
        if (!B.D(j, i)) return so_plane(j, i, 3, i, j);
        return so_line(j, 3, j);
      }
      // all three edge tests hold but no face looks at the origin: unchanged
      o = so_plane(0, 1, 2, 0, 1);
      o.n = 4;
      o.kind = SO_KEEP;
      return o;
    }
  }
}

// ------------------------------------------------------------------------------
// The decision as a table: every outcome of step_decide packed in 32 bits, indexed by
// the predicate bits the decision can read (13 for a tetrahedron step, 4 for a triangle,
// 1 for a segment).  One load replaces the branches of the tree, which the lanes of a
// warp (different pairs, different bits) would otherwise take one path after another.
constexpr int kSubTab3 = 1 << 13;           // first triangle entry
constexpr int kSubTab2 = kSubTab3 + 16;     // first segment entry
constexpr int kSubTabSize = kSubTab2 + 2;

OGX_HD int subtab_index(int n, uint32_t bits) {
  if (n == 4) return (int)(bits & 0x1fffu);
  if (n == 3)
    return kSubTab3 + (int)((bits & 3u) | (((bits >> (PB_D + 0)) & 1u) << 2) | (((bits >> (PB_D + 1)) & 1u) << 3));
  return kSubTab2 + (int)(bits & 1u);
}

// n-1 (2 bits) | s0, s1, s2 (2 bits each) | kind (3) | a, b (2 each) | used (13)
OGX_HD uint32_t pack_subout(const SubOut& o) {
  return (uint32_t)(o.n - 1) | ((uint32_t)o.s[0] << 2) | ((uint32_t)o.s[1] << 4) | ((uint32_t)o.s[2] << 6) |
         ((uint32_t)o.kind << 8) | ((uint32_t)o.a << 11) | ((uint32_t)o.b << 13) | ((o.used & 0x1fffu) << 15);
}
OGX_HD SubOut unpack_subout(uint32_t c) {
  SubOut o;
  o.n = (int)(c & 3u) + 1;
  o.s[0] = (int)((c >> 2) & 3u);
  o.s[1] = (int)((c >> 4) & 3u);
  o.s[2] = (int)((c >> 6) & 3u);
  o.kind = (int)((c >> 8) & 7u);
  o.a = (int)((c >> 11) & 3u);
  o.b = (int)((c >> 13) & 3u);
  o.used = (c >> 15) & 0x1fffu;
  return o;
}

// ------------------------------------------------------------------------------
// FP32 predicate values and bounds

struct StepIn {
  fv3 q1;      // newest point
  fv3 e[3];    // older points minus q1
  float a[3];  // q1 . e_k
  float g[3][3];
  fv3 c01, c02, c12;  // e0 x e1, e0 x e2, e1 x e2
  float qc01, qc02, qc12;  // q1 . c
};

OGX_HD fv3 sel3(int s, fv3 a, fv3 b, fv3 c, fv3 d) {
  return s == 0 ? a : (s == 1 ? b : (s == 2 ? c : d));
}
OGX_HD int seli(int s, int a, int b, int c, int d) { return s == 0 ? a : (s == 1 ? b : (s == 2 ? c : d)); }

// predicate bits of the n-point step (n = 2, 3, 4; newest point P[n-1]) and the bits of
// the decisions that fall inside their rounding bound
OGX_HD void step_predicates(int n, const fv3* P, StepIn& S, uint32_t& bits, uint32_t& unc) {
  const float E = FLT_EPSILON;
  const fv3 q1 = n == 4 ? P[3] : (n == 3 ? P[2] : P[1]);
  S.q1 = q1;
  const float lq = l1(q1);
  bits = 0u;
  unc = 0u;
  float le[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    S.e[k] = P[k] - q1;
    le[k] = l1(S.e[k]);
    S.a[k] = dot(q1, S.e[k]);
    // hff1: q1.(q1 - P_k) > 0  <=>  a_k < 0; bound covers the rounding of e_k too
    const float ba = 8.0f * E * lq * (le[k] + lq);
    bits |= (S.a[k] < 0.0f ? 1u : 0u) << k;
    unc |= (fabsf(S.a[k]) <= ba ? 1u : 0u) << k;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int k = j; k < 3; ++k) S.g[j][k] = S.g[k][j] = dot(S.e[j], S.e[k]);
  // hff2 values d(j,k) = a_j g_jk - a_k g_jj  (< 0: the origin is beyond edge q1-P_j)
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (j == k) continue;
      const float t1 = S.a[j] * S.g[j][k], t2 = S.a[k] * S.g[j][j];
      const float dv = t1 - t2;
      const float bd = 16.0f * E * lq * (le[j] + lq) * le[j] * (le[j] + le[k]);
      const int bit = PB_D + dpair(j, k);
      bits |= (dv < 0.0f ? 1u : 0u) << bit;
      unc |= (fabsf(dv) <= bd ? 1u : 0u) << bit;
    }
  S.c01 = cross(S.e[0], S.e[1]);
  S.c02 = cross(S.e[0], S.e[2]);
  S.c12 = cross(S.e[1], S.e[2]);
  S.qc01 = dot(q1, S.c01);
  S.qc02 = dot(q1, S.c02);
  S.qc12 = dot(q1, S.c12);
  if (n == 4) {
    const float det = dot(S.e[1], S.c02);  // e1 . (e0 x e2) = the reference's det134
    const float bdet = 16.0f * E * le[0] * le[1] * le[2];
    bits |= det <= 0.0f ? PB_NEG : 0u;
    unc |= fabsf(det) <= bdet ? PB_NEG : 0u;
    // hff3 (<= 0 drops): q1.(e1 x e0) = -qc01, q1.(e0 x e2) = qc02, q1.(e2 x e1) = -qc12
    const float bf01 = 16.0f * E * lq * (le[0] + lq) * (le[1] + lq);
    const float bf02 = 16.0f * E * lq * (le[0] + lq) * (le[2] + lq);
    const float bf12 = 16.0f * E * lq * (le[1] + lq) * (le[2] + lq);
    bits |= (-S.qc01 <= 0.0f) ? PB_F2 : 0u;
    bits |= (S.qc02 <= 0.0f) ? PB_F3 : 0u;
    bits |= (-S.qc12 <= 0.0f) ? PB_F4 : 0u;
    unc |= fabsf(S.qc01) <= bf01 ? PB_F2 : 0u;
    unc |= fabsf(S.qc02) <= bf02 ? PB_F3 : 0u;
    unc |= fabsf(S.qc12) <= bf12 ? PB_F4 : 0u;
  }
}

// decision of the n-point step from its predicate bits
OGX_HD SubOut step_decide(int n, uint32_t bits) {
  Bits B{bits, 0u};
  SubOut o;
  if (n == 4) {
    o = tetra_tree(B);
  } else if (n == 3) {
    o = tri_tree(B, 0, 1, 2);
  } else {
    // segment: openGJK.c:257-268
    o = B.K(0) ? so_line(0, 1, 0) : so_vertex(1);
  }
  o.used = B.used;
  return o;
}

// the whole table (host): entry i is step_decide of the bits that index i
inline void fill_subtab(uint32_t* tab) {
  for (uint32_t bits = 0; bits < (1u << 13); ++bits) tab[bits] = pack_subout(step_decide(4, bits));
  for (uint32_t k = 0; k < 16; ++k) {
    const uint32_t bits = (k & 3u) | (((k >> 2) & 1u) << (PB_D + 0)) | (((k >> 3) & 1u) << (PB_D + 1));
    tab[kSubTab3 + k] = pack_subout(step_decide(3, bits));
  }
  for (uint32_t k = 0; k < 2; ++k) tab[kSubTab2 + k] = pack_subout(step_decide(2, k));
}

// new direction v from the outcome (all candidates computed, then selected)
OGX_HD fv3 step_direction(int n, const StepIn& S, const SubOut& o, fv3 vold) {
  // line through q1 and P_a: v = q1 - e_a (a_a / g_aa)
  const int a = o.a, b = o.b;
  const fv3 ea = a == 0 ? S.e[0] : (a == 1 ? S.e[1] : S.e[2]);
  const float aa = a == 0 ? S.a[0] : (a == 1 ? S.a[1] : S.a[2]);
  const float gaa = a == 0 ? S.g[0][0] : (a == 1 ? S.g[1][1] : S.g[2][2]);
  const fv3 vline = S.q1 - ea * (aa / gaa);
  // plane through q1, P_a, P_b: normal c = e_a x e_b (sign irrelevant), v = c (q1.c)/(c.c)
  const int pab = (a < b ? a : b) * 3 + (a < b ? b : a);  // 1 -> 01, 2 -> 02, 5 -> 12
  const fv3 c = pab == 1 ? S.c01 : (pab == 2 ? S.c02 : S.c12);
  const float qc = pab == 1 ? S.qc01 : (pab == 2 ? S.qc02 : S.qc12);
  const fv3 vplane = c * (qc / dot(c, c));
  switch (o.kind) {
    case SO_VERTEX: return S.q1;
    case SO_LINE: return vline;
    case SO_PLANE: return vplane;
    case SO_ZERO: return v3<float>(0.f, 0.f, 0.f);
    default: return vold;
  }
}

}  // namespace ogx
