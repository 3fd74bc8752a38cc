// ogx_gjk.cuh -- GJK distance for one pair, run by a team of L lanes.
//
// Algorithm (the reference's GJK, GJK/cpu/openGJK.c:952-1056 and
// GJK/gpu/openGJK.cu:1253-1425): start from v = A[0] - B[0]; each iteration takes the
// support points s_A(-v), s_B(v), stops when the new point cannot reduce |v| (relative
// gap test), otherwise appends w = s_A - s_B to the simplex and runs the signed-volume
// sub-distance algorithm (Montanari's hff tests, openGJK.c:219-613), which returns the
// point of the simplex closest to the origin and drops the vertices it does not need.
//
// What differs from the reference, and why:
//  * The support scans are split over the team's lanes and combined with a shuffle
//    argmax; the tie rule (keep the previous support unless strictly beaten, then the
//    lowest index) is the reference CPU's rule (openGJK.c:615-639).
//  * Every lane runs the sub-distance redundantly, so nothing is broadcast.
//  * The sub-distance runs in FP32.  Each sign decision carries a forward error bound;
//    if any decision of a step falls inside its bound, the whole step is re-run in FP64
//    on the exact Minkowski points re-read from the pool (OGX_F_FP64_ESCALATE).
//  * Termination also stops when the support pair is already in the simplex (no
//    progress is possible) and when the gap is below FP32 rounding of |v| |w|.
//  * The final simplex of a separated pair is re-solved in FP64 (exact closest point of
//    the final feature, certified by an exact support check, else GJK continues in FP64;
//    OGX_F_FP64_POLISH); on the device that runs as a separate pass.
#pragma once

#include "ogx_common.cuh"
#include "ogx_subdist.cuh"

namespace ogx {

template <class T>
struct Eps {
  static constexpr double v = 0.0;
};
template <>
struct Eps<float> {
  static constexpr double v = FLT_EPSILON;
};

// flag set when a decision falls inside its rounding bound
struct Unc {
  bool hit;
};

template <class T>
struct Vx {
  vec3<T> p;
  int k;  // slot of this vertex in the caller's simplex
};

template <class T>
struct Sx {
  int n;
  Vx<T> v[4];
};

template <class T>
OGX_HD T tabs(T x) {
  return x < T(0) ? -x : x;
}

// (p - q) . p > 0 : the origin projects beyond p towards q (openGJK.c:219-230)
template <class T>
OGX_HD bool edge_keeps(vec3<T> p, vec3<T> q, Unc& u) {
  T acc = T(0);
  acc += (p.x * p.x - p.x * q.x);
  acc += (p.y * p.y - p.y * q.y);
  acc += (p.z * p.z - p.z * q.z);
  if (Eps<T>::v != 0.0) {
    const T perm = p.x * p.x + tabs(p.x * q.x) + p.y * p.y + tabs(p.y * q.y) + p.z * p.z +
                   tabs(p.z * q.z);
    if (tabs(acc) <= T(16.0 * Eps<T>::v) * perm) u.hit = true;
  }
  return acc > T(0);
}

// origin beyond edge pq, away from r, in the plane pqr (openGJK.c:232-248)
template <class T>
OGX_HD bool edge_drops(vec3<T> p, vec3<T> q, vec3<T> r, Unc& u) {
  const vec3<T> e1 = q - p, e2 = r - p;
  const vec3<T> nrm = cross(e1, cross(e1, e2));
  const T val = dot(p, nrm);
  if (Eps<T>::v != 0.0) {
    const T b = l1(e1);
    if (tabs(val) <= T(64.0 * Eps<T>::v) * l1(p) * b * b * l1(e2)) u.hit = true;
  }
  return val < T(0);
}

// origin on the far side of triangle (p, q, r) seen from ... (openGJK.c:250-255)
template <class T>
OGX_HD bool face_drops(vec3<T> p, vec3<T> q, vec3<T> r, Unc& u) {
  const T val = dot(p, cross(q, r));
  if (Eps<T>::v != 0.0) {
    if (tabs(val) <= T(32.0 * Eps<T>::v) * l1(p) * l1(q) * l1(r)) u.hit = true;
  }
  return val <= T(0);
}

template <class T>
OGX_HD void onto_line(vec3<T> p, vec3<T> q, vec3<T>& out) {
  const vec3<T> d = p - q;
  const T t = dot(p, d) / dot(d, d);
  out = p - d * t;
}

template <class T>
OGX_HD void onto_plane(vec3<T> p, vec3<T> q, vec3<T> r, vec3<T>& out, Unc& u) {
  const vec3<T> nrm = cross(p - q, p - r);
  const T nn = dot(nrm, nrm);
  if (Eps<T>::v != 0.0) {
    const T b = T(32.0 * Eps<T>::v) * l1(p - q) * l1(p - r);
    if (nn <= b * b) u.hit = true;
  }
  out = nrm * (dot(nrm, p) / nn);
}

template <class T>
OGX_HD void keep1(Sx<T>& s, const Vx<T>& a) {
  s.n = 1;
  s.v[0] = a;
}
template <class T>
OGX_HD void keep2(Sx<T>& s, const Vx<T>& a, const Vx<T>& b) {
  s.n = 2;
  s.v[0] = a;
  s.v[1] = b;
}
template <class T>
OGX_HD void keep3(Sx<T>& s, const Vx<T>& a, const Vx<T>& b, const Vx<T>& c) {
  s.n = 3;
  s.v[0] = a;
  s.v[1] = b;
  s.v[2] = c;
}

// segment: newest vertex v[1]
template <class T>
OGX_HD void sub_segment(Sx<T>& s, vec3<T>& dir, Unc& u) {
  const Vx<T> q1 = s.v[1], q2 = s.v[0];
  if (edge_keeps(q1.p, q2.p, u)) {
    onto_line(q1.p, q2.p, dir);
  } else {
    dir = q1.p;
    keep1(s, q1);
  }
}

// triangle: newest vertex v[2]
template <class T>
OGX_HD void sub_triangle(Sx<T>& s, vec3<T>& dir, Unc& u) {
  const Vx<T> q1 = s.v[2], q2 = s.v[1], q3 = s.v[0];
  const bool k12 = edge_keeps(q1.p, q2.p, u);
  const bool k13 = edge_keeps(q1.p, q3.p, u);
  int pick = 0;  // 0 plane, 1 segment q1-q3, 2 segment q1-q2, 3 vertex q1
  if (k12) {
    if (!edge_drops(q1.p, q2.p, q3.p, u)) {
      if (k13 && edge_drops(q1.p, q3.p, q2.p, u)) pick = 1;
    } else {
      pick = 2;
    }
  } else if (k13) {
    if (edge_drops(q1.p, q3.p, q2.p, u)) pick = 1;
  } else {
    pick = 3;
  }
  if (pick == 0) {
    onto_plane(q1.p, q2.p, q3.p, dir, u);
  } else if (pick == 1) {
    onto_line(q1.p, q3.p, dir);
    keep2(s, q3, q1);
  } else if (pick == 2) {
    onto_line(q1.p, q2.p, dir);
    keep2(s, q1, q2);
  } else {
    dir = q1.p;
    keep1(s, q1);
  }
}

// (k, i, j) naming of the three older tetrahedron vertices (openGJK.c:405-417)
template <class T>
OGX_HD void name_kij(int which, const Vx<T>& q2, const Vx<T>& q3, const Vx<T>& q4, Vx<T>& sk,
                     Vx<T>& si, Vx<T>& sj) {
  if (which == 0) {
    sk = q2; si = q3; sj = q4;
  } else if (which == 1) {
    sk = q3; si = q4; sj = q2;
  } else {
    sk = q4; si = q2; sj = q3;
  }
}

template <class T>
OGX_HD void pick_plane(Sx<T>& s, const Vx<T>& a, const Vx<T>& b, const Vx<T>& q1,
                       const vec3<T>& pp, const vec3<T>& pq, vec3<T>& dir, Unc& u) {
  keep3(s, a, b, q1);
  onto_plane(q1.p, pp, pq, dir, u);
}
template <class T>
OGX_HD void pick_line(Sx<T>& s, const Vx<T>& a, const Vx<T>& q1, vec3<T>& dir) {
  keep2(s, a, q1);
  onto_line(q1.p, a.p, dir);
}

// tetrahedron: newest vertex v[3] (decision tree of openGJK.c:315-613)
template <class T>
OGX_HD void sub_tetra(Sx<T>& s, vec3<T>& dir, Unc& u) {
  const Vx<T> q1 = s.v[3], q2 = s.v[2], q3 = s.v[1], q4 = s.v[0];
  const bool l2 = edge_keeps(q1.p, q2.p, u);
  const bool l3 = edge_keeps(q1.p, q3.p, u);
  const bool l4 = edge_keeps(q1.p, q4.p, u);
  const int nkeep = (int)l2 + (int)l3 + (int)l4;
  if (nkeep == 0) {
    dir = q1.p;
    keep1(s, q1);
    return;
  }
  const vec3<T> e2 = q2.p - q1.p, e3 = q3.p - q1.p, e4 = q4.p - q1.p;
  const T vol = dot(e3, cross(e4, e2));
  if (Eps<T>::v != 0.0) {
    if (tabs(vol) <= T(32.0 * Eps<T>::v) * l1(e2) * l1(e3) * l1(e4)) u.hit = true;
  }
  const int neg = vol <= T(0);
  int f2 = (int)face_drops(q1.p, q3.p, q4.p, u) - neg;
  int f3 = (int)face_drops(q1.p, q4.p, q2.p, u) - neg;
  int f4 = (int)face_drops(q1.p, q2.p, q3.p, u) - neg;
  f2 *= f2;
  f3 *= f3;
  f4 *= f4;
  Vx<T> sk, si, sj;
  switch (f2 + f3 + f4) {
    case 3:
      dir = v3<T>(T(0), T(0), T(0));
      return;
    case 2:
      if (!f2)
        keep3(s, q4, q3, q1);
      else if (!f3)
        keep3(s, q4, q2, q1);
      else
        keep3(s, q3, q2, q1);
      sub_triangle(s, dir, u);
      return;
    case 1: {
      s.n = 3;
      name_kij(f2 ? 0 : (f3 ? 1 : 2), q2, q3, q4, sk, si, sj);
      const bool lk = edge_keeps(q1.p, sk.p, u);
      const bool li = edge_keeps(q1.p, si.p, u);
      const bool lj = edge_keeps(q1.p, sj.p, u);
      if (nkeep == 1) {
        if (lk) {
          if (!edge_drops(q1.p, sk.p, si.p, u))
            pick_plane(s, sk, si, q1, si.p, sk.p, dir, u);
          else if (!edge_drops(q1.p, sk.p, sj.p, u))
            pick_plane(s, sk, sj, q1, sj.p, sk.p, dir, u);
          else
            pick_line(s, sk, q1, dir);
        } else if (li) {
          if (!edge_drops(q1.p, si.p, sk.p, u))
            pick_plane(s, sk, si, q1, si.p, sk.p, dir, u);
          else
            pick_line(s, si, q1, dir);
        } else {
          if (!edge_drops(q1.p, sj.p, sk.p, u))
            pick_plane(s, sk, sj, q1, sj.p, sk.p, dir, u);
          else
            pick_line(s, sj, q1, dir);
        }
      } else if (nkeep == 2) {
        if (li) {
          if (!edge_drops(q1.p, sk.p, si.p, u)) {
            if (!edge_drops(q1.p, si.p, sk.p, u))
              pick_plane(s, sk, si, q1, si.p, sk.p, dir, u);
            else
              pick_line(s, sk, q1, dir);
          } else if (!edge_drops(q1.p, sk.p, sj.p, u)) {
            pick_plane(s, sk, sj, q1, sj.p, sk.p, dir, u);
          } else {
            pick_line(s, sk, q1, dir);
          }
        } else if (lj) {
          if (!edge_drops(q1.p, sk.p, sj.p, u)) {
            if (!edge_drops(q1.p, sj.p, sk.p, u))
              pick_plane(s, sk, sj, q1, sj.p, sk.p, dir, u);
            else
              pick_line(s, sj, q1, dir);
          } else if (!edge_drops(q1.p, sk.p, si.p, u)) {
            pick_plane(s, sk, si, q1, si.p, sk.p, dir, u);
          } else {
            pick_line(s, sk, q1, dir);
          }
        } else {
          u.hit = true;  // inconsistent tests: only possible through rounding
        }
      } else {
        const bool d_ik = edge_drops(q1.p, si.p, sk.p, u);
        const bool d_jk = edge_drops(q1.p, sj.p, sk.p, u);
        const bool d_ki = edge_drops(q1.p, sk.p, si.p, u);
        const bool d_kj = edge_drops(q1.p, sk.p, sj.p, u);
        if (d_ki && d_kj)
          pick_line(s, sk, q1, dir);
        else if (d_ki) {
          if (d_jk)
            pick_line(s, sj, q1, dir);
          else
            pick_plane(s, sk, sj, q1, sk.p, sj.p, dir, u);
        } else {
          if (d_ik)
            pick_line(s, si, q1, dir);
          else
            pick_plane(s, sk, si, q1, sk.p, si.p, dir, u);
        }
      }
      return;
    }
    case 0:
      if (nkeep == 1) {
        name_kij(l3 ? 0 : (l4 ? 1 : 2), q2, q3, q4, sk, si, sj);
        if (!edge_drops(q1.p, si.p, sj.p, u))
          pick_plane(s, sj, si, q1, si.p, sj.p, dir, u);
        else if (!edge_drops(q1.p, si.p, sk.p, u))
          pick_plane(s, sk, si, q1, si.p, sk.p, dir, u);
        else
          pick_line(s, si, q1, dir);
      } else if (nkeep == 2) {
        s.n = 3;
        name_kij(!l3 ? 0 : (!l4 ? 1 : 2), q2, q3, q4, sk, si, sj);
        if (!edge_drops(q1.p, sj.p, sk.p, u)) {
          if (!edge_drops(q1.p, sk.p, sj.p, u))
            pick_plane(s, sk, sj, q1, sj.p, sk.p, dir, u);
          else if (!edge_drops(q1.p, sk.p, si.p, u))
            pick_plane(s, sk, si, q1, sk.p, si.p, dir, u);
          else
            pick_line(s, sk, q1, dir);
        } else if (!edge_drops(q1.p, sj.p, si.p, u)) {
          pick_plane(s, sj, si, q1, si.p, sj.p, dir, u);
        } else {
          pick_line(s, sj, q1, dir);
        }
      } else {
        u.hit = true;  // all three edges keep but no face looks at the origin
      }
      return;
    default:
      return;
  }
}

template <class T>
OGX_HD void subdistance(Sx<T>& s, vec3<T>& dir, Unc& u) {
  if (s.n == 4)
    sub_tetra(s, dir, u);
  else if (s.n == 3)
    sub_triangle(s, dir, u);
  else if (s.n == 2)
    sub_segment(s, dir, u);
}

// --------------------------------------------------------------------------------
// exact closest point of a simplex with <= 3 vertices to the origin, FP64
// (region tests of Ericson, Real-Time Collision Detection, sec. 5.1.5, restated)

template <class T>
OGX_HD void closest_on_simplex_t(int n, const vec3<T>* P, T* lam, vec3<T>& v) {
  const T zero = sc<T>(0.0f), one = sc<T>(1.0f);
  lam[0] = one;
  lam[1] = lam[2] = lam[3] = zero;
  if (n == 1) {
    v = P[0];
    return;
  }
  if (n == 2) {
    const vec3<T> e = P[1] - P[0];
    const T ee = dot(e, e);
    T t = ee > zero ? -dot(P[0], e) / ee : zero;
    t = t < zero ? zero : (t > one ? one : t);
    lam[0] = one - t;
    lam[1] = t;
    v = P[0] + e * t;
    return;
  }
  const vec3<T> a = P[0], b = P[1], c = P[2];
  const vec3<T> ab = b - a, ac = c - a;
  const T d1 = -dot(ab, a), d2 = -dot(ac, a);
  if (d1 <= zero && d2 <= zero) {
    v = a;
    return;
  }
  const T d3 = -dot(ab, b), d4 = -dot(ac, b);
  if (d3 >= zero && d4 <= d3) {
    lam[0] = zero;
    lam[1] = one;
    v = b;
    return;
  }
  const T vc = d1 * d4 - d3 * d2;
  if (vc <= zero && d1 >= zero && d3 <= zero) {
    const T t = d1 / (d1 - d3);
    lam[0] = one - t;
    lam[1] = t;
    v = a + ab * t;
    return;
  }
  const T d5 = -dot(ab, c), d6 = -dot(ac, c);
  if (d6 >= zero && d5 <= d6) {
    lam[0] = zero;
    lam[2] = one;
    v = c;
    return;
  }
  const T vb = d5 * d2 - d1 * d6;
  if (vb <= zero && d2 >= zero && d6 <= zero) {
    const T t = d2 / (d2 - d6);
    lam[0] = one - t;
    lam[2] = t;
    v = a + ac * t;
    return;
  }
  const T va = d3 * d6 - d5 * d4;
  if (va <= zero && (d4 - d3) >= zero && (d5 - d6) >= zero) {
    const T t = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    lam[0] = zero;
    lam[1] = one - t;
    lam[2] = t;
    v = b + (c - b) * t;
    return;
  }
  const T den = one / (va + vb + vc);
  const T s1 = vb * den, s2 = vc * den;
  lam[0] = one - s1 - s2;
  lam[1] = s1;
  lam[2] = s2;
  v = a + ab * s1 + ac * s2;
}
OGX_HD void closest_on_simplex(int n, const dv3* P, double* lam, dv3& v) { closest_on_simplex_t<double>(n, P, lam, v); }

// --------------------------------------------------------------------------------
// per-pair GJK

struct GjkState {
  int n;        // simplex size (4 = origin enclosed)
  fv3 P[4];     // simplex Minkowski points, newest last
  int ia[4], ib[4];
  fv3 v;        // closest point of the simplex to the origin
  float dist;
  float wmax2;  // max |P|^2 seen (scale of the problem)
  fv3 w0, w1;   // witnesses on body 1 and body 2
  int iters;
  int status;
  int exit;     // why the loop ended (GJK_EXIT_*)
  bool polish;  // separated: certify and re-solve (or continue) in FP64
  int wa, wb;   // support pair along the final direction
  bool certain; // that support is the exact (FP64) support along the exact direction
};

// loop exit reasons (reported in status bits 16..18)
enum {
  GJK_EXIT_GAP_REL = 1,   // |v|^2 - v.w <= eps_rel |v|^2
  GJK_EXIT_GAP_NOISE = 2, // gap below the FP32 rounding floor (or eps_tot)
  GJK_EXIT_NULL_V = 3,    // |v| < eps_rel
  GJK_EXIT_DUPLICATE = 4, // support pair already in the simplex
  GJK_EXIT_CONTACT = 5,   // |v| negligible against the simplex scale
  GJK_EXIT_ENCLOSED = 6,  // origin inside the tetrahedron
  GJK_EXIT_CAP = 7,       // iteration cap
};

// The pair is in contact (EPA runs) when GJK enclosed the origin or the distance is
// below FLT_EPSILON -- the reference's FP32 test (GJK/cpu/EPA.c:370).
OGX_HD bool gjk_contact(const GjkState& g) { return g.n == 4 || !(g.dist > FLT_EPSILON); }

// barycentric weights of the closest point v of the final simplex, FP32
OGX_HD void simplex_weights(const GjkState& g, float* lam) {
  lam[0] = 1.0f;
  lam[1] = lam[2] = lam[3] = 0.0f;
  if (g.n == 2) {
    const fv3 e = g.P[1] - g.P[0];
    const float ee = dot(e, e);
    float t = ee > 0.0f ? -dot(g.P[0], e) / ee : 0.0f;
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    lam[0] = 1.0f - t;
    lam[1] = t;
  } else if (g.n == 3) {
    const fv3 e1 = g.P[1] - g.P[0], e2 = g.P[2] - g.P[0];
    const float g11 = dot(e1, e1), g12 = dot(e1, e2), g22 = dot(e2, e2);
    const float r1 = -dot(g.P[0], e1), r2 = -dot(g.P[0], e2);
    const float det = g11 * g22 - g12 * g12;
    if (det != 0.0f) {
      const float a1 = (g22 * r1 - g12 * r2) / det;
      const float a2 = (g11 * r2 - g12 * r1) / det;
      lam[0] = 1.0f - a1 - a2;
      lam[1] = a1;
      lam[2] = a2;
    }
  } else if (g.n == 4) {
    const fv3 e1 = g.P[1] - g.P[0], e2 = g.P[2] - g.P[0], e3 = g.P[3] - g.P[0];
    const fv3 c23 = cross(e2, e3), c31 = cross(e3, e1), c12 = cross(e1, e2);
    const float det = dot(e1, c23);
    if (det != 0.0f) {
      const fv3 o = -g.P[0];
      const float a1 = dot(o, c23) / det, a2 = dot(o, c31) / det, a3 = dot(o, c12) / det;
      lam[0] = 1.0f - a1 - a2 - a3;
      lam[1] = a1;
      lam[2] = a2;
      lam[3] = a3;
    }
  }
}

// FP64 re-run of one sub-distance step on the exact Minkowski points (cold path: taken
// when an FP32 decision of the step falls inside its rounding bound).  Returns the new
// slot order in `order` and the new direction.
template <class Mem>
#if defined(__CUDACC__)
__noinline__
#endif
OGX_HD int escalate_step(const Mem B, int n, const int* ia, const int* ib, fv3 vold, int* order, fv3* vout) {
  Sx<double> sd;
  sd.n = n;
  for (int j = 0; j < n; ++j) {
    sd.v[j].p = B.dpoint(0, ia[j]) - B.dpoint(1, ib[j]);
    sd.v[j].k = j;
  }
  dv3 vd = cvt<double>(vold);
  Unc ud{false};
  subdistance(sd, vd, ud);
  for (int j = 0; j < sd.n; ++j) order[j] = sd.v[j].k;
  *vout = cvt<float>(vd);
  return sd.n;
}

// GJK as a resumable loop: gjk_start sets the state up, each gjk_iterate runs one
// iteration (support, termination tests, sub-distance step) until r.done, gjk_end
// finishes (witnesses, certification).  gjk_pair chains them.
struct GjkRun {
  fv3 v;
  fv3 P[4];  // simplex in registers: slots 0..3, newest last; every index is unrolled
  int IA[4], IB[4];
  int n;
  float wmax2;
  fv3 sa, sb;
  int ia, ib;
  int k;
  int status, exit;
  bool done;
};

template <class Bodies>
OGX_HD void gjk_start(const Bodies& B, GjkRun& r, int start_a = 0, int start_b = 0) {
  // first point of the Minkowski difference: point 0 of each body (the reference's
  // start), or a warm-start pair of vertex indices (e.g. the previous frame's simplex)
  const fv3 a0 = B.point(0, start_a), b0 = B.point(1, start_b);
  r.v = a0 - b0;
  r.P[0] = r.v;
  r.P[1] = r.P[2] = r.P[3] = r.v;
  r.IA[0] = start_a;
  r.IB[0] = start_b;
  r.IA[1] = r.IA[2] = r.IA[3] = r.IB[1] = r.IB[2] = r.IB[3] = -1;
  r.n = 1;
  r.wmax2 = 0.0f;
  r.sa = a0;
  r.sb = b0;
  r.ia = start_a;
  r.ib = start_b;
  r.k = 0;
  r.status = 0;
  r.exit = 0;
  r.done = false;
}

template <class Team, class Bodies>
OGX_HD void gjk_iterate(const Team& t, const Bodies& B, const Config& cfg, GjkRun& r,
                        const uint32_t* subtab = nullptr) {
  const bool reftol = (cfg.flags & OGX_F_REFERENCE_TOL) != 0;
  const bool escalate = (cfg.flags & OGX_F_FP64_ESCALATE) != 0;
  const float eps_rel2 = cfg.gjk_eps_rel * cfg.gjk_eps_rel;
  // |v| this small against the simplex points is below FP32 resolution: stop
  const float contact = reftol ? cfg.gjk_eps_tot : 0.5f * FLT_EPSILON;
  fv3& v = r.v;
  fv3* P = r.P;
  int* IA = r.IA;
  int* IB = r.IB;
  int& n = r.n;
  float& wmax2 = r.wmax2;
  fv3& sa = r.sa;
  fv3& sb = r.sb;
  int& ia = r.ia;
  int& ib = r.ib;
  int& k = r.k;
  ++k;
    const fv3 mv = -v;
    float ba, bb;
    int xa, xb;
    B.scan(t, 0, mv, ba, xa);
    B.scan(t, 1, v, bb, xb);
    t.argmax(ba, xa);
    t.argmax(bb, xb);
    if (ba > sdot(sa, mv)) {
      ia = xa;
      sa = B.point(0, xa);
    }
    if (bb > sdot(sb, v)) {
      ib = xb;
      sb = B.point(1, xb);
    }
    const fv3 w = sa - sb;
    const float vv = dot(v, v);
    const float gap = vv - dot(v, w);
    float floor_ = cfg.gjk_eps_tot;
    if (!reftol) {
      const float nv = sqrtf(vv);
      floor_ = fmaxf(floor_, cfg.gjk_noise * FLT_EPSILON * nv * (nv + sqrtf(dot(w, w))));
    }
    if (gap <= cfg.gjk_eps_rel * vv) {
      r.exit = GJK_EXIT_GAP_REL;
      r.done = true;
      return;
    }
    if (gap < floor_) {
      r.exit = GJK_EXIT_GAP_NOISE;
      r.done = true;
      return;
    }
    if (vv < eps_rel2) {
      r.exit = GJK_EXIT_NULL_V;
      r.done = true;
      return;
    }
    if (!reftol) {
      bool dup = false;
#pragma unroll
      for (int j = 0; j < 4; ++j) dup |= (j < n) && IA[j] == ia && IB[j] == ib;
      if (dup) {
        r.exit = GJK_EXIT_DUPLICATE;
        r.done = true;
        return;
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (j == n) {
        P[j] = w;
        IA[j] = ia;
        IB[j] = ib;
      }
    ++n;

    StepIn S;
    uint32_t bits, unc;
    step_predicates(n, P, S, bits, unc);
    // the decision: one load from the table on the device, the tree on the host
    SubOut o;
#if defined(__CUDA_ARCH__)
    if (subtab)
      o = unpack_subout(__ldg(subtab + subtab_index(n, bits)));
    else
#endif
      o = step_decide(n, bits);
    // degenerate spans make the projection itself unreliable
    if (o.kind == SO_LINE) {
      const float ge = o.a == 0 ? S.g[0][0] : (o.a == 1 ? S.g[1][1] : S.g[2][2]);
      const float lq = l1(S.q1);
      if (!(ge > 64.0f * FLT_EPSILON * FLT_EPSILON * lq * lq)) unc |= o.used | 1u;
    } else if (o.kind == SO_PLANE) {
      const fv3 ea = o.a == 0 ? S.e[0] : (o.a == 1 ? S.e[1] : S.e[2]);
      const fv3 eb = o.b == 0 ? S.e[0] : (o.b == 1 ? S.e[1] : S.e[2]);
      const int pab = (o.a < o.b ? o.a : o.b) * 3 + (o.a < o.b ? o.b : o.a);
      const fv3 c = pab == 1 ? S.c01 : (pab == 2 ? S.c02 : S.c12);
      const float bc = 32.0f * FLT_EPSILON * l1(ea) * l1(eb);
      if (!(dot(c, c) > bc * bc)) unc |= o.used | 1u;
    }
    int nn;
    fv3 P2[3];
    int A2[3], B2[3];
    if ((unc & o.used) != 0u && escalate) {
      int order[4] = {0, 1, 2, 3};
      int ias[4], ibs[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        ias[j] = IA[j];
        ibs[j] = IB[j];
      }
      fv3 vd;
      nn = escalate_step(B.mem_view(), n, ias, ibs, v, order, &vd);
      v = vd;
      r.status |= OGX_S_GJK_ESCALATED;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int sj = order[j];
        P2[j] = sel3(sj, P[0], P[1], P[2], P[3]);
        A2[j] = seli(sj, IA[0], IA[1], IA[2], IA[3]);
        B2[j] = seli(sj, IB[0], IB[1], IB[2], IB[3]);
      }
    } else {
      v = step_direction(n, S, o, v);
      // slots are numbered for the tetrahedron (newest = 3); map for smaller steps
      nn = o.n;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int sj = (o.s[j] == 3) ? (n - 1) : o.s[j];
        P2[j] = sel3(sj, P[0], P[1], P[2], P[3]);
        A2[j] = seli(sj, IA[0], IA[1], IA[2], IA[3]);
        B2[j] = seli(sj, IB[0], IB[1], IB[2], IB[3]);
      }
    }
    if (nn < 4) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        P[j] = P2[j];
        IA[j] = A2[j];
        IB[j] = B2[j];
      }
    }
    n = nn;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (j < n) wmax2 = fmaxf(wmax2, dot(P[j], P[j]));
    if (dot(v, v) <= contact * contact * wmax2) {
      r.exit = GJK_EXIT_CONTACT;
      r.done = true;
      return;
    }
    if (n == 4) {
      r.exit = GJK_EXIT_ENCLOSED;
      r.done = true;
      return;
    }
    if (k == cfg.gjk_max_iter) {
      r.exit = GJK_EXIT_CAP;
      r.done = true;
      return;
    }
}

template <class Team, class Bodies>
OGX_HD void gjk_end(const Team& t, const Bodies& B, const Config& cfg, const GjkRun& r, GjkState& g) {
  const fv3 v = r.v;
  const fv3* P = r.P;
  const int* IA = r.IA;
  const int* IB = r.IB;
  const int n = r.n;
  const float wmax2 = r.wmax2;
  const int ia = r.ia, ib = r.ib;
  const int k = r.k;
  g.status = r.status;
  g.exit = r.exit;
  g.n = n;
  g.wmax2 = wmax2;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    g.P[j] = P[j];
    g.ia[j] = IA[j];
    g.ib[j] = IB[j];
  }
  if (k == cfg.gjk_max_iter && g.n != 4) g.status |= OGX_S_GJK_CAP;
  g.status |= g.exit << 16;
  g.iters = k;
  g.v = v;
  g.dist = sqrtf(dot(v, v));

  float lam[4];
  simplex_weights(g, lam);
  fv3 w0 = v3<float>(0.f, 0.f, 0.f), w1 = w0;
#pragma unroll
  for (int j = 0; j < 4; ++j)
    if (j < n) {
      w0 = w0 + B.point(0, IA[j]) * lam[j];
      w1 = w1 + B.point(1, IB[j]) * lam[j];
    }
  g.w0 = w0;
  g.w1 = w1;

  // FP32 error of |v| is a few ulp of the simplex scale; ask for an FP64 re-solve when
  // that is not small against the distance.
  g.polish = false;
  g.certain = false;
  g.wa = ia;
  g.wb = ib;
  if ((cfg.flags & OGX_F_FP64_POLISH) && g.n >= 1 && g.n <= 3 && !gjk_contact(g)) {
    // Every separated pair is certified or continued in FP64: a stop on the FP32 gap
    // bounds the distance (about 1e-7 relative) but not its direction, which on flat
    // closest features can stay ~1e-4 off until the exact feature is found; a pair that
    // ran into the iteration cap has not converged at all (the region decisions can cycle).
    g.polish = true;
  }
  if (g.polish) {
    // Is the exact support along the exact closest point v64 one of the final simplex's
    // own points?  Then GJK's stop is exact and the FP64 closest point of the simplex is
    // the answer.  Each body's points outside the simplex must trail its best point by
    // more than twice the error of an FP32 support value against the exact value along
    // v64: FP32 dot rounding (4 eps amax |v|_1) plus the FP32 projection error of v
    // (16 eps |W| per component).
    int exa[3], exb[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      exa[j] = j < n ? IA[j] : -1;
      exb[j] = j < n ? IB[j] : -1;
    }
    float a1, ao, am, b1, bo, bm;
    B.scan_excl(t, 0, -v, exa, a1, ao, am);
    B.scan_excl(t, 1, v, exb, b1, bo, bm);
    a1 = t.fmax_(a1);
    ao = t.fmax_(ao);
    am = t.fmax_(am);
    b1 = t.fmax_(b1);
    bo = t.fmax_(bo);
    bm = t.fmax_(bm);
    const float dv = 16.0f * FLT_EPSILON * sqrtf(g.wmax2) * 3.0f;
    const float l1v = fabsf(v.x) + fabsf(v.y) + fabsf(v.z);
    const float ea = 4.0f * FLT_EPSILON * am * l1v + am * dv;
    const float eb = 4.0f * FLT_EPSILON * bm * l1v + bm * dv;
    g.certain = (a1 - ao > 2.0f * ea) && (b1 - bo > 2.0f * eb);
  }
}

template <class Team, class Bodies>
OGX_HD void gjk_pair(const Team& t, const Bodies& B, const Config& cfg, GjkState& g, int start_a = 0,
                     int start_b = 0, const uint32_t* subtab = nullptr) {
  GjkRun r;
  gjk_start(B, r, start_a, start_b);
  while (!r.done) gjk_iterate(t, B, cfg, r, subtab);
  gjk_end(t, B, cfg, r, g);
}

// Exact (FP64) support index of body w along d.  An FP32 scan finds the maximum m of
// fl(x . d32); every point whose exact value could exceed the true maximum satisfies
// fl(x . d32) >= m - 2e with e >= |fl(x . d32) - x . d| <= 2 FLT_EPSILON |x|_max |d|_1
// (rounding of d to FP32 plus the FP32 dot product), so only those few candidates are
// evaluated in FP64.  Ties go to the lowest index.
template <class Team, class Bodies, class T>
OGX_HD int exact_support(const Team& t, const Bodies& B, int w, vec3<T> d, T& val) {
  const auto& M = B.mem_view();  // points by index (posed where the bodies are)
  const fv3 fd = v3<float>(to_float(d.x), to_float(d.y), to_float(d.z));
  const int n = M.n[w];
  float m = -INFINITY, amax = 0.0f;
  for (int i = t.lane(); i < n; i += Team::L) {
    const fv3 p = M.point(w, i);
    m = fmaxf(m, sdot(p, fd));
    amax = fmaxf(amax, fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))));
  }
  m = t.fmax_(m);
  amax = t.fmax_(amax);
  // bodies given in double: the float points are the inputs rounded (half an ulp each),
  // one more FLT_EPSILON * amax * |d|_1 of difference to cover
  const float ef = Bodies::kExact64 ? 5.0f : 4.0f;
  const float e = ef * FLT_EPSILON * amax * (fabsf(fd.x) + fabsf(fd.y) + fabsf(fd.z)) + FLT_MIN;
  const float lo = m - 2.0f * e;
  T best = sc<T>(-INFINITY);
  int bi = 0x7fffffff;
  for (int i = t.lane(); i < n; i += Team::L) {
    const fv3 pf = M.point(w, i);
    if (sdot(pf, fd) < lo) continue;
    T x;
    if constexpr (Bodies::kExact64) {
      const dv3 p = B.dpoint(w, i);
      x = p.x * d.x + p.y * d.y + p.z * d.z;
    } else {
      x = sc<T>(pf.x) * d.x + sc<T>(pf.y) * d.y + sc<T>(pf.z) * d.z;
    }
    if (x > best || (x == best && i < bi)) {
      best = x;
      bi = i;
    }
  }
  t.argmax_t(best, bi);
  val = best;
  return bi;
}

// the Minkowski point a_i - b_j exactly (double), or as double-float components
template <class T>
struct Tag {};
template <class Bodies>
OGX_HD dv3 mpoint(Tag<double>, const Bodies& B, int i, int j) { return B.dpoint(0, i) - B.dpoint(1, j); }
template <class Bodies>
OGX_HD xv3 mpoint(Tag<df>, const Bodies& B, int i, int j) { return xdiff(B.point(0, i), B.point(1, j)); }

// FP64 continuation of GJK from the FP32 result: exact supports, FP64 sub-distance,
// stop when the FP64 gap |v|^2 - v.w <= 1e-12 |v|^2 or the support repeats.  Certifies
// (or corrects) the FP32 answer; sets g.n = 4 if the origin turns out to be enclosed.
// Split in three so that a warp can run the supports of 32 pairs cooperatively while
// each lane keeps its own pair's state (refine_begin, then refine_step with the exact
// supports along -v / v until done, then refine_end).
// written for double and double-float; the continuation runs in FP64: its progress
// and gap tests need |v|^2 to about 1e-12 relative, and near-coplanar thin bodies put the
// origin 1e-5 of the coordinates' scale from the simplex, where the 48 bits of
// double-float leave |v|^2 with ~1e-10 relative noise (it stopped a step early on some
// 1e-4-thick disks).  The one-shot re-solves (refine_certain, epa_polish) have no such
// decision and run in double-float.
template <class T>
struct RefineStateT {
  Sx<T> s;
  int ia[4], ib[4];
  vec3<T> v;
  T lam[4];   // barycentric weights of v on s (valid while no step changed s)
  bool lam_valid;
  T wmax2;
  int it, max_iter;
  bool done, enclosed;
};
typedef RefineStateT<double> RefineState;

template <class Bodies, class T>
OGX_HD void refine_begin(const Bodies& B, const GjkState& g, int max_iter, RefineStateT<T>& r) {
  Sx<T>& s = r.s;
  const T zero = sc<T>(0.0f);
  s.n = g.n > 3 ? 3 : g.n;
  for (int j = 0; j < s.n; ++j) {
    r.ia[j] = g.ia[j];
    r.ib[j] = g.ib[j];
    s.v[j].p = mpoint(Tag<T>(), B, r.ia[j], r.ib[j]);
    s.v[j].k = j;
  }
  // exact closest point of the FP32 result's simplex; keep only the vertices it uses
  vec3<T> P[3];
  for (int j = 0; j < s.n; ++j) P[j] = s.v[j].p;
  T lam[4];
  closest_on_simplex_t<T>(s.n, P, lam, r.v);
  {
    Sx<T> q;
    q.n = 0;
    int qa[4], qb[4];
    for (int j = 0; j < s.n; ++j)
      if (lam[j] > zero || (s.n == 1)) {
        q.v[q.n] = s.v[j];
        qa[q.n] = r.ia[j];
        qb[q.n] = r.ib[j];
        q.n++;
      }
    T ql[4] = {sc<T>(1.0f), zero, zero, zero};
    int m = 0;
    for (int j = 0; j < s.n; ++j)
      if (lam[j] > zero || (s.n == 1)) ql[m++] = lam[j];
    r.lam_valid = q.n > 0;
    if (q.n == 0) {
      q.v[0] = s.v[0];
      qa[0] = r.ia[0];
      qb[0] = r.ib[0];
      q.n = 1;
    }
    s = q;
    for (int j = 0; j < s.n; ++j) {
      r.ia[j] = qa[j];
      r.ib[j] = qb[j];
      s.v[j].k = j;
      r.lam[j] = ql[j];
    }
  }
  r.wmax2 = zero;
  for (int j = 0; j < s.n; ++j) r.wmax2 = tmax(r.wmax2, dot(s.v[j].p, s.v[j].p));
  r.max_iter = max_iter;
  r.enclosed = false;
  r.it = g.certain ? max_iter + 1 : 0;  // the FP32 pass proved the simplex final
  r.done = r.it >= max_iter;
}

// Closest point of a simplex to the origin by exhaustive search (Johnson's method without
// the region tests): every sub-simplex that holds the newest vertex s.v[s.n-1] is solved
// on its affine hull (Gram system), those whose barycentric weights are all >= 0 are
// feasible, and the feasible one nearest the origin wins (fewer vertices on ties).  In
// exact arithmetic the closest point after a GJK step lies on such a sub-simplex.  Cold
// path: taken when the signed-volume region decisions made no progress -- on some
// configurations the hff tests of the reference's sub-distance (GJK/cpu/openGJK.c:315-613)
// pick a region whose point is farther than the last one, and GJK then cycles until its
// iteration cap (the reference's own FP64 code does so on a pair of the 1M-pair power-law
// batch and returns a distance 1.3% too large).  Returns the reduced simplex in s (slots
// keep their .k) and its closest point in v; s.n == 4 means the origin is enclosed.
template <class T>
OGX_COLD void closest_exhaustive(Sx<T>& s, vec3<T>& v) {
  const int n = s.n;
  const int nw = n - 1;
  const T zero = T(0);
  T best = T(INFINITY);
  int best_mask = 1 << nw, best_k = 5;
  vec3<T> best_v = s.v[nw].p;
  for (int mask = 1; mask < (1 << n); ++mask) {
    if (!(mask & (1 << nw))) continue;
    int idx[4], k = 0;
    idx[k++] = nw;  // the newest vertex first
    for (int j = 0; j < n; ++j)
      if (j != nw && (mask & (1 << j))) idx[k++] = j;
    const vec3<T> p0 = s.v[idx[0]].p;
    T lam[4] = {T(1), zero, zero, zero};
    bool ok = true;
    if (k >= 2) {
      vec3<T> e[3];
      for (int a = 1; a < k; ++a) e[a - 1] = s.v[idx[a]].p - p0;
      const int m = k - 1;
      T G[3][3], r[3];
      for (int a = 0; a < m; ++a) {
        r[a] = -dot(p0, e[a]);
        for (int c = 0; c < m; ++c) G[a][c] = dot(e[a], e[c]);
      }
      T x[3] = {zero, zero, zero};
      if (m == 1) {
        ok = G[0][0] > zero;
        if (ok) x[0] = r[0] / G[0][0];
      } else if (m == 2) {
        const T det = G[0][0] * G[1][1] - G[0][1] * G[1][0];
        ok = det > zero;
        if (ok) {
          x[0] = (r[0] * G[1][1] - G[0][1] * r[1]) / det;
          x[1] = (G[0][0] * r[1] - r[0] * G[1][0]) / det;
        }
      } else {
        // x = adj(G) r / det(G), adj(G)[i][j] = C[j][i] with C the cofactor matrix
        T C[3][3];
        C[0][0] = G[1][1] * G[2][2] - G[1][2] * G[2][1];
        C[0][1] = G[1][2] * G[2][0] - G[1][0] * G[2][2];
        C[0][2] = G[1][0] * G[2][1] - G[1][1] * G[2][0];
        C[1][0] = G[0][2] * G[2][1] - G[0][1] * G[2][2];
        C[1][1] = G[0][0] * G[2][2] - G[0][2] * G[2][0];
        C[1][2] = G[0][1] * G[2][0] - G[0][0] * G[2][1];
        C[2][0] = G[0][1] * G[1][2] - G[0][2] * G[1][1];
        C[2][1] = G[0][2] * G[1][0] - G[0][0] * G[1][2];
        C[2][2] = G[0][0] * G[1][1] - G[0][1] * G[1][0];
        const T det = G[0][0] * C[0][0] + G[0][1] * C[0][1] + G[0][2] * C[0][2];
        ok = det > zero;
        if (ok)
          for (int a = 0; a < 3; ++a) x[a] = (C[0][a] * r[0] + C[1][a] * r[1] + C[2][a] * r[2]) / det;
      }
      T sum = zero;
      for (int a = 0; a < m; ++a) {
        lam[a + 1] = x[a];
        sum = sum + x[a];
      }
      lam[0] = T(1) - sum;
    }
    if (!ok) continue;
    bool feasible = true;
    for (int a = 0; a < k; ++a) feasible = feasible && !(lam[a] < zero);
    if (!feasible) continue;
    vec3<T> p = p0 * lam[0];
    for (int a = 1; a < k; ++a) p = p + s.v[idx[a]].p * lam[a];
    const T d2 = k == 4 ? zero : dot(p, p);  // a feasible tetrahedron holds the origin
    if (d2 < best || (d2 == best && k < best_k)) {
      best = d2;
      best_mask = mask;
      best_k = k;
      best_v = k == 4 ? vec3<T>{zero, zero, zero} : p;
    }
  }
  Sx<T> q;
  q.n = 0;
  for (int j = 0; j < n; ++j)
    if (best_mask & (1 << j)) q.v[q.n++] = s.v[j];
  s = q;
  v = best_v;
}

// one iteration with the exact supports xa (body 1 along -v) and xb (body 2 along v)
template <class Bodies, class T>
OGX_HD void refine_step(const Bodies& B, RefineStateT<T>& r, int xa, int xb) {
  Sx<T>& s = r.s;
  const vec3<T> w = mpoint(Tag<T>(), B, xa, xb);
  const T vv = dot(r.v, r.v);
  // FP64 gap test.  In exact arithmetic v.p_j = |v|^2 for every vertex p_j of the
  // current feature, so the gap |v|^2 - v.w equals v.(p_j - w); that form rounds in
  // proportion to |p_j - w| (small near convergence) instead of |w|^2.  Relative
  // tolerance of the FP64 oracle (eps * 1e4) and a rounding floor.
  T gap = sc<T>(INFINITY), dmax = sc<T>(0.0f);
  for (int j = 0; j < s.n; ++j) {
    const vec3<T> e = s.v[j].p - w;
    gap = tmin(gap, dot(r.v, e));
    dmax = tmax(dmax, dot(e, e));
  }
  const T floor64 = T(4.0 * prec_eps<T>()) * tsqrt(r.wmax2) * tsqrt(dmax);
  if (gap <= T(1e-12) * vv || gap <= floor64) {
    r.done = true;
    return;
  }
  bool dup = false;
  for (int j = 0; j < s.n; ++j) dup |= (r.ia[j] == xa && r.ib[j] == xb);
  if (dup) {
    r.done = true;
    return;
  }
  const Sx<T> prev = s;
  int pa[4], pb[4];
  for (int j = 0; j < s.n; ++j) {
    pa[j] = r.ia[j];
    pb[j] = r.ib[j];
  }
  const vec3<T> vprev = r.v;
  s.v[s.n].p = w;
  s.v[s.n].k = s.n;
  r.ia[s.n] = xa;
  r.ib[s.n] = xb;
  s.n++;
  Unc u{false};
  subdistance(s, r.v, u);
  r.lam_valid = false;
  if (s.n != 4 && !(dot(r.v, r.v) < vv * T(1.0 - 1e-12))) {
    // the region decisions made no progress although the gap says progress is possible:
    // solve the step again by exhaustive search on the grown simplex
    Sx<T> t = prev;
    t.v[t.n].p = w;
    t.v[t.n].k = t.n;
    t.n++;
    vec3<T> vt;
    closest_exhaustive(t, vt);
    if (t.n == 4 || dot(vt, vt) < vv * T(1.0 - 1e-12)) {
      s = t;
      r.v = vt;
    }
  }
  if (s.n != 4 && !(dot(r.v, r.v) < vv * T(1.0 - 1e-12))) {
    // still none: a tie support spanning a degenerate simplex -- keep the last answer
    s = prev;
    r.v = vprev;
    for (int j = 0; j < s.n; ++j) {
      r.ia[j] = pa[j];
      r.ib[j] = pb[j];
    }
    r.done = true;
    return;
  }
  int na[4], nb[4];
  for (int j = 0; j < s.n; ++j) {
    na[j] = r.ia[s.v[j].k];
    nb[j] = r.ib[s.v[j].k];
  }
  for (int j = 0; j < s.n; ++j) {
    r.ia[j] = na[j];
    r.ib[j] = nb[j];
    s.v[j].k = j;
    r.wmax2 = tmax(r.wmax2, dot(s.v[j].p, s.v[j].p));
  }
  if (s.n == 4) {
    r.enclosed = true;
    r.done = true;
    return;
  }
  ++r.it;
  if (r.it >= r.max_iter) r.done = true;
}

template <class Bodies, class T>
OGX_HD void refine_end(const Bodies& B, const RefineStateT<T>& r, GjkState& g) {
  const Sx<T>& s = r.s;
  g.n = s.n;
  for (int j = 0; j < s.n; ++j) {
    g.ia[j] = r.ia[j];
    g.ib[j] = r.ib[j];
    g.P[j] = v3<float>(to_float(s.v[j].p.x), to_float(s.v[j].p.y), to_float(s.v[j].p.z));
  }
  g.status |= (r.it == r.max_iter + 1) ? OGX_S_POLISHED : (OGX_S_POLISHED | OGX_S_GJK_ESCALATED);
  if (r.it == r.max_iter) g.status |= OGX_S_GJK_CAP;
  if (r.enclosed) {
    g.v = v3<float>(0.f, 0.f, 0.f);
    g.dist = 0.0f;
    return;
  }
  T lam[4];
  vec3<T> v;
  if (r.lam_valid) {
    // the simplex is the one refine_begin solved: reuse its closest point
    v = r.v;
    for (int j = 0; j < 4; ++j) lam[j] = r.lam[j];
  } else {
    vec3<T> P[3];
    for (int j = 0; j < s.n; ++j) P[j] = s.v[j].p;
    closest_on_simplex_t<T>(s.n, P, lam, v);
  }
  // The distance needs the FP64 closest point; its square root and the witnesses do
  // not: FP32 from here on (|v|^2 rounded once, then a correctly rounded sqrtf: 1 ulp;
  // witnesses to a few ulp of the coordinates, the 1e-4 witness tolerance being far
  // above).  FP64 issues at 1/64 of the FP32 rate here.
  fv3 w0 = v3<float>(0.f, 0.f, 0.f), w1 = w0;
  for (int j = 0; j < s.n; ++j) {
    const float l = to_float(lam[j]);
    w0 = w0 + B.point(0, r.ia[j]) * l;
    w1 = w1 + B.point(1, r.ib[j]) * l;
  }
  g.v = v3<float>(to_float(v.x), to_float(v.y), to_float(v.z));
  g.dist = sqrtf(to_float(dot(v, v)));
  g.w0 = w0;
  g.w1 = w1;
}

// The re-solve of a pair whose final simplex the FP32 pass proved final (its support is
// certified), in double-float arithmetic on the FP32 pipes instead of FP64: the exact
// Minkowski points a - b, the closest point of their simplex to about 48 bits, the
// vertices it uses; then, as refine_end, FP32 witnesses and a correctly rounded distance.
template <class Bodies>
OGX_HD void refine_certain(const Bodies& B, GjkState& g) {
  const int n0 = g.n > 3 ? 3 : g.n;
  xv3 P[3];
  int ia[3], ib[3];
  for (int j = 0; j < n0; ++j) {
    ia[j] = g.ia[j];
    ib[j] = g.ib[j];
    P[j] = xdiff(B.point(0, ia[j]), B.point(1, ib[j]));
  }
  df lam[4];
  xv3 v;
  closest_on_simplex_t<df>(n0, P, lam, v);
  // keep the vertices the closest point uses (the single vertex of a point simplex)
  int m = 0;
  float ql[3] = {1.0f, 0.0f, 0.0f};
  int qa[3] = {ia[0], 0, 0}, qb[3] = {ib[0], 0, 0};
  xv3 Q[3];
  Q[0] = P[0];
  for (int j = 0; j < n0; ++j)
    if (lam[j] > sc<df>(0.0f) || n0 == 1) {
      Q[m] = P[j];
      qa[m] = ia[j];
      qb[m] = ib[j];
      ql[m] = to_float(lam[j]);
      ++m;
    }
  if (m == 0) {  // as the FP64 path: the first vertex alone
    m = 1;
    ql[0] = 1.0f;
    v = P[0];
  }
  g.n = m;
  for (int j = 0; j < m; ++j) {
    g.ia[j] = qa[j];
    g.ib[j] = qb[j];
    g.P[j] = v3<float>(Q[j].x.hi, Q[j].y.hi, Q[j].z.hi);
  }
  g.status |= OGX_S_POLISHED;
  fv3 w0 = v3<float>(0.f, 0.f, 0.f), w1 = w0;
  for (int j = 0; j < m; ++j) {
    w0 = w0 + B.point(0, qa[j]) * ql[j];
    w1 = w1 + B.point(1, qb[j]) * ql[j];
  }
  g.v = v3<float>(to_float(v.x), to_float(v.y), to_float(v.z));
  g.dist = sqrtf(to_float(dot(v, v)));
  g.w0 = w0;
  g.w1 = w1;
}

template <class Team, class Bodies>
OGX_HD void gjk_refine(const Team& t, const Bodies& B, GjkState& g, int max_iter) {
  if (g.certain) {
    refine_certain(B, g);
    return;
  }
  RefineState r;
  refine_begin(B, g, max_iter, r);
  while (!r.done) {
    double va, vb;
    const int xa = exact_support(t, B, 0, -r.v, va);
    const int xb = exact_support(t, B, 1, r.v, vb);
    refine_step(B, r, xa, xb);
  }
  refine_end(B, r, g);
}

// FP64 re-solve of the final simplex: exact Minkowski points, exact closest point.
template <class Bodies>
OGX_HD void gjk_polish(const Bodies& B, GjkState& g) {
  dv3 P[3];
  for (int j = 0; j < g.n && j < 3; ++j) P[j] = B.dpoint(0, g.ia[j]) - B.dpoint(1, g.ib[j]);
  double lam[4];
  dv3 v;
  closest_on_simplex(g.n, P, lam, v);
  dv3 w0 = v3<double>(0.0, 0.0, 0.0), w1 = w0;
  for (int j = 0; j < g.n; ++j) {
    w0 = w0 + B.dpoint(0, g.ia[j]) * lam[j];
    w1 = w1 + B.dpoint(1, g.ib[j]) * lam[j];
  }
  g.v = cvt<float>(v);
  g.dist = (float)sqrt(dot(v, v));
  g.w0 = cvt<float>(w0);
  g.w1 = cvt<float>(w1);
  g.status |= OGX_S_POLISHED;
}

}  // namespace ogx
