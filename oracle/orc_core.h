/*
 * orc_core.h -- CPU restatement of the reference GJK distance and EPA penetration
 * algorithms.  TEST INFRASTRUCTURE ONLY: this file is the parity oracle for the GPU
 * engine and the timed CPU baseline.  Nothing in the product library links it.
 *
 * The file is a "template": orc.c includes it twice, once with ORC_REAL = float and
 * once with ORC_REAL = double, and ORC_FN(name) appends the matching suffix.  Every
 * arithmetic expression keeps the operation order of the reference so that the FP32
 * and FP64 instantiations reproduce the reference's own CPU build bit for bit (the
 * tests check this against the reference sources compiled unmodified).
 *
 * Reference files (paths inside the OpenGJK-GPU project):
 *   GJK/cpu/openGJK.c  -- GJK with the signed-volume sub-distance algorithm
 *   GJK/cpu/EPA.c      -- simplex growth + expanding polytope algorithm
 *   GJK/common.h       -- gkFloat / gkEpsilon precision switch, data types
 */

#define ORC_CAT_(a, b) a##b
#define ORC_CAT(a, b) ORC_CAT_(a, b)
#define ORC_FN(name) ORC_CAT(name, ORC_SFX)

typedef ORC_REAL ORC_FN(real);
#define R ORC_FN(real)

/* One simplex vertex: Minkowski point p = A[a] - B[b]. */
typedef struct {
  R p[3];
  int a, b;
} ORC_FN(vtx);

/* GJK simplex; the most recently added vertex is always v[n-1]
 * (GJK/common.h:84-89, gkSimplex). */
typedef struct {
  int n;
  ORC_FN(vtx) v[4];
  R wit[2][3];
} ORC_FN(smx);

/* A body: n points, xyz interleaved (GJK/common.h:68-78, gkPolytope.coord). */
typedef struct {
  int n;
  const R* xyz;
} ORC_FN(body);

/* ------------------------------------------------------------------------- */
/* small vector helpers; operation order as GJK/cpu/openGJK.c:44-45,167-181  */

static inline R ORC_FN(dot)(const R* a, const R* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

static inline void ORC_FN(cross)(const R* a, const R* b, R* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

/* triple product p . (q x r) written out as GJK/cpu/openGJK.c:167-173 */
static inline R ORC_FN(det3)(const R* p, const R* q, const R* r) {
  return p[0] * ((q[1] * r[2]) - (r[1] * q[2])) - p[1] * (q[0] * r[2] - r[0] * q[2]) +
         p[2] * (q[0] * r[1] - r[0] * q[1]);
}

static inline void ORC_FN(copy3)(R* d, const R* s) {
  d[0] = s[0];
  d[1] = s[1];
  d[2] = s[2];
}

/* closest point to the origin on the line through p, q (GJK/cpu/openGJK.c:183-196) */
static void ORC_FN(onto_line)(const R* p, const R* q, R* out) {
  R d[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
  const R t = ORC_FN(dot)(p, d) / ORC_FN(dot)(d, d);
  for (int c = 0; c < 3; ++c) out[c] = p[c] - d[c] * t;
}

/* closest point to the origin on the plane through p, q, r (GJK/cpu/openGJK.c:198-217) */
static void ORC_FN(onto_plane)(const R* p, const R* q, const R* r, R* out) {
  R d1[3], d2[3], nrm[3];
  for (int c = 0; c < 3; ++c) d1[c] = p[c] - q[c];
  for (int c = 0; c < 3; ++c) d2[c] = p[c] - r[c];
  ORC_FN(cross)(d1, d2, nrm);
  const R t = ORC_FN(dot)(nrm, p) / ORC_FN(dot)(nrm, nrm);
  for (int c = 0; c < 3; ++c) out[c] = nrm[c] * t;
}

/* edge test: is the origin's projection beyond p in the direction of q?
 * (GJK/cpu/openGJK.c:219-230) */
static int ORC_FN(edge_keeps)(const R* p, const R* q) {
  R acc = 0;
  for (int c = 0; c < 3; ++c) acc += (p[c] * p[c] - p[c] * q[c]);
  return acc > 0;
}

/* in-plane test for edge pq of triangle pqr (GJK/cpu/openGJK.c:232-248):
 * returns 1 when the origin lies on the far side of pq from r. */
static int ORC_FN(edge_drops)(const R* p, const R* q, const R* r) {
  R e1[3], e2[3], t[3], nrm[3];
  for (int c = 0; c < 3; ++c) e1[c] = q[c] - p[c];
  for (int c = 0; c < 3; ++c) e2[c] = r[c] - p[c];
  ORC_FN(cross)(e1, e2, t);
  ORC_FN(cross)(e1, t, nrm);
  return ORC_FN(dot)(p, nrm) < 0;
}

/* face orientation test (GJK/cpu/openGJK.c:250-255) */
static int ORC_FN(face_drops)(const R* p, const R* q, const R* r) {
  R nrm[3];
  ORC_FN(cross)(q, r, nrm);
  return ORC_FN(dot)(p, nrm) <= 0;
}

static inline void ORC_FN(set1)(ORC_FN(smx) * s, ORC_FN(vtx) a) {
  s->n = 1;
  s->v[0] = a;
}
static inline void ORC_FN(set2)(ORC_FN(smx) * s, ORC_FN(vtx) a, ORC_FN(vtx) b) {
  s->n = 2;
  s->v[0] = a;
  s->v[1] = b;
}
static inline void ORC_FN(set3)(ORC_FN(smx) * s, ORC_FN(vtx) a, ORC_FN(vtx) b, ORC_FN(vtx) c) {
  s->n = 3;
  s->v[0] = a;
  s->v[1] = b;
  s->v[2] = c;
}

/* ------------------------------------------------------------------------- */
/* signed-volume sub-distance algorithm                                       */

/* segment (GJK/cpu/openGJK.c:257-268) */
static void ORC_FN(sub1)(ORC_FN(smx) * s, R* dir) {
  const ORC_FN(vtx) q1 = s->v[1], q2 = s->v[0];
  if (ORC_FN(edge_keeps)(q1.p, q2.p)) {
    ORC_FN(onto_line)(q1.p, q2.p, dir);
  } else {
    ORC_FN(copy3)(dir, q1.p);
    ORC_FN(set1)(s, q1);
  }
}

/* triangle (GJK/cpu/openGJK.c:270-313) */
static void ORC_FN(sub2)(ORC_FN(smx) * s, R* dir) {
  const ORC_FN(vtx) q1 = s->v[2], q2 = s->v[1], q3 = s->v[0];
  const int k12 = ORC_FN(edge_keeps)(q1.p, q2.p);
  const int k13 = ORC_FN(edge_keeps)(q1.p, q3.p);
  int use13 = 0; /* 1: answer is segment q1-q3; 2: segment q1-q2; 0: the plane */
  if (k12) {
    if (!ORC_FN(edge_drops)(q1.p, q2.p, q3.p)) {
      if (k13 && ORC_FN(edge_drops)(q1.p, q3.p, q2.p)) use13 = 1;
    } else {
      use13 = 2;
    }
  } else if (k13) {
    if (ORC_FN(edge_drops)(q1.p, q3.p, q2.p)) use13 = 1;
  } else {
    ORC_FN(copy3)(dir, q1.p);
    ORC_FN(set1)(s, q1);
    return;
  }
  if (use13 == 0) {
    ORC_FN(onto_plane)(q1.p, q2.p, q3.p, dir);
  } else if (use13 == 1) {
    ORC_FN(onto_line)(q1.p, q3.p, dir);
    ORC_FN(set2)(s, q3, q1);
  } else {
    ORC_FN(onto_line)(q1.p, q2.p, dir);
    ORC_FN(set2)(s, q1, q2);
  }
}

/* The three ways the reference names the non-newest tetrahedron vertices
 * (k, i, j) as slots of the simplex array: (2,1,0), (1,0,2), (0,2,1)
 * (GJK/cpu/openGJK.c:405-417, 542-553, 572-583).  With q2=v[2], q3=v[1], q4=v[0]
 * those are (q2,q3,q4), (q3,q4,q2), (q4,q2,q3). */
static void ORC_FN(pick_kij)(int which, const ORC_FN(vtx) * q2, const ORC_FN(vtx) * q3,
                             const ORC_FN(vtx) * q4, ORC_FN(vtx) * sk, ORC_FN(vtx) * si,
                             ORC_FN(vtx) * sj) {
  if (which == 0) {
    *sk = *q2; *si = *q3; *sj = *q4;
  } else if (which == 1) {
    *sk = *q3; *si = *q4; *sj = *q2;
  } else {
    *sk = *q4; *si = *q2; *sj = *q3;
  }
}

/* tetrahedron (GJK/cpu/openGJK.c:315-613) */
static void ORC_FN(sub3)(ORC_FN(smx) * s, R* dir) {
  const ORC_FN(vtx) q1 = s->v[3], q2 = s->v[2], q3 = s->v[1], q4 = s->v[0];
  R e2[3], e3[3], e4[3];
  for (int c = 0; c < 3; ++c) {
    e2[c] = q2.p[c] - q1.p[c];
    e3[c] = q3.p[c] - q1.p[c];
    e4[c] = q4.p[c] - q1.p[c];
  }
  const int l2 = ORC_FN(edge_keeps)(q1.p, q2.p);
  const int l3 = ORC_FN(edge_keeps)(q1.p, q3.p);
  const int l4 = ORC_FN(edge_keeps)(q1.p, q4.p);
  const int nkeep = l2 + l3 + l4;
  if (nkeep == 0) {
    ORC_FN(copy3)(dir, q1.p);
    ORC_FN(set1)(s, q1);
    return;
  }
  const int neg = (ORC_FN(det3)(e3, e4, e2) <= 0);
  int f2 = ORC_FN(face_drops)(q1.p, q3.p, q4.p) - neg;
  int f3 = ORC_FN(face_drops)(q1.p, q4.p, q2.p) - neg;
  int f4 = ORC_FN(face_drops)(q1.p, q2.p, q3.p) - neg;
  f2 *= f2;
  f3 *= f3;
  f4 *= f4;
  ORC_FN(vtx) sk, si, sj;

  switch (f2 + f3 + f4) {
    case 3: /* origin enclosed */
      dir[0] = 0;
      dir[1] = 0;
      dir[2] = 0;
      s->n = 4;
      return;

    case 2: /* one face looks at the origin: drop the opposite vertex, solve the triangle */
      if (!f2)
        ORC_FN(set3)(s, q4, q3, q1);
      else if (!f3)
        ORC_FN(set3)(s, q4, q2, q1);
      else
        ORC_FN(set3)(s, q3, q2, q1);
      ORC_FN(sub2)(s, dir);
      return;

    case 1: { /* two faces look at the origin */
      s->n = 3;
      ORC_FN(pick_kij)(f2 ? 0 : (f3 ? 1 : 2), &q2, &q3, &q4, &sk, &si, &sj);
      const int lk = ORC_FN(edge_keeps)(q1.p, sk.p);
      const int li = ORC_FN(edge_keeps)(q1.p, si.p);
      const int lj = ORC_FN(edge_keeps)(q1.p, sj.p);
      if (nkeep == 1) {
        if (lk) {
          if (!ORC_FN(edge_drops)(q1.p, sk.p, si.p)) {
            ORC_FN(set3)(s, sk, si, q1);
            ORC_FN(onto_plane)(q1.p, si.p, sk.p, dir);
          } else if (!ORC_FN(edge_drops)(q1.p, sk.p, sj.p)) {
            ORC_FN(set3)(s, sk, sj, q1);
            ORC_FN(onto_plane)(q1.p, sj.p, sk.p, dir);
          } else {
            ORC_FN(set2)(s, sk, q1);
            ORC_FN(onto_line)(q1.p, sk.p, dir);
          }
        } else if (li) {
          if (!ORC_FN(edge_drops)(q1.p, si.p, sk.p)) {
            ORC_FN(set3)(s, sk, si, q1);
            ORC_FN(onto_plane)(q1.p, si.p, sk.p, dir);
          } else {
            ORC_FN(set2)(s, si, q1);
            ORC_FN(onto_line)(q1.p, si.p, dir);
          }
        } else {
          if (!ORC_FN(edge_drops)(q1.p, sj.p, sk.p)) {
            ORC_FN(set3)(s, sk, sj, q1);
            ORC_FN(onto_plane)(q1.p, sj.p, sk.p, dir);
          } else {
            ORC_FN(set2)(s, sj, q1);
            ORC_FN(onto_line)(q1.p, sj.p, dir);
          }
        }
      } else if (nkeep == 2) {
        /* the first two vertices of the simplex array are kept below when neither
         * edge test holds (GJK/cpu/openGJK.c:494-496 leaves the simplex as is) */
        if (li) {
          if (!ORC_FN(edge_drops)(q1.p, sk.p, si.p)) {
            if (!ORC_FN(edge_drops)(q1.p, si.p, sk.p)) {
              ORC_FN(set3)(s, sk, si, q1);
              ORC_FN(onto_plane)(q1.p, si.p, sk.p, dir);
            } else {
              ORC_FN(set2)(s, sk, q1);
              ORC_FN(onto_line)(q1.p, sk.p, dir);
            }
          } else if (!ORC_FN(edge_drops)(q1.p, sk.p, sj.p)) {
            ORC_FN(set3)(s, sk, sj, q1);
            ORC_FN(onto_plane)(q1.p, sj.p, sk.p, dir);
          } else {
            ORC_FN(set2)(s, sk, q1);
            ORC_FN(onto_line)(q1.p, sk.p, dir);
          }
        } else if (lj) {
          if (!ORC_FN(edge_drops)(q1.p, sk.p, sj.p)) {
            if (!ORC_FN(edge_drops)(q1.p, sj.p, sk.p)) {
              ORC_FN(set3)(s, sk, sj, q1);
              ORC_FN(onto_plane)(q1.p, sj.p, sk.p, dir);
            } else {
              ORC_FN(set2)(s, sj, q1);
              ORC_FN(onto_line)(q1.p, sj.p, dir);
            }
          } else if (!ORC_FN(edge_drops)(q1.p, sk.p, si.p)) {
            ORC_FN(set3)(s, sk, si, q1);
            ORC_FN(onto_plane)(q1.p, si.p, sk.p, dir);
          } else {
            ORC_FN(set2)(s, sk, q1);
            ORC_FN(onto_line)(q1.p, sk.p, dir);
          }
        }
      } else if (nkeep == 3) {
        const int d_ik = ORC_FN(edge_drops)(q1.p, si.p, sk.p);
        const int d_jk = ORC_FN(edge_drops)(q1.p, sj.p, sk.p);
        const int d_ki = ORC_FN(edge_drops)(q1.p, sk.p, si.p);
        const int d_kj = ORC_FN(edge_drops)(q1.p, sk.p, sj.p);
        if (d_ki && d_kj) {
          ORC_FN(set2)(s, sk, q1);
          ORC_FN(onto_line)(q1.p, sk.p, dir);
        } else if (d_ki) {
          if (d_jk) {
            ORC_FN(set2)(s, sj, q1);
            ORC_FN(onto_line)(q1.p, sj.p, dir);
          } else {
            ORC_FN(set3)(s, sk, sj, q1);
            ORC_FN(onto_plane)(q1.p, sk.p, sj.p, dir);
          }
        } else {
          if (d_ik) {
            ORC_FN(set2)(s, si, q1);
            ORC_FN(onto_line)(q1.p, si.p, dir);
          } else {
            ORC_FN(set3)(s, sk, si, q1);
            ORC_FN(onto_plane)(q1.p, sk.p, si.p, dir);
          }
        }
      }
      return;
    }

    case 0: /* no face looks at the origin */
      if (nkeep == 1) {
        ORC_FN(pick_kij)(l3 ? 0 : (l4 ? 1 : 2), &q2, &q3, &q4, &sk, &si, &sj);
        if (!ORC_FN(edge_drops)(q1.p, si.p, sj.p)) {
          ORC_FN(set3)(s, sj, si, q1);
          ORC_FN(onto_plane)(q1.p, si.p, sj.p, dir);
        } else if (!ORC_FN(edge_drops)(q1.p, si.p, sk.p)) {
          ORC_FN(set3)(s, sk, si, q1);
          ORC_FN(onto_plane)(q1.p, si.p, sk.p, dir);
        } else {
          ORC_FN(set2)(s, si, q1);
          ORC_FN(onto_line)(q1.p, si.p, dir);
        }
      } else if (nkeep == 2) {
        s->n = 3;
        ORC_FN(pick_kij)(!l3 ? 0 : (!l4 ? 1 : 2), &q2, &q3, &q4, &sk, &si, &sj);
        if (!ORC_FN(edge_drops)(q1.p, sj.p, sk.p)) {
          if (!ORC_FN(edge_drops)(q1.p, sk.p, sj.p)) {
            ORC_FN(set3)(s, sk, sj, q1);
            ORC_FN(onto_plane)(q1.p, sj.p, sk.p, dir);
          } else if (!ORC_FN(edge_drops)(q1.p, sk.p, si.p)) {
            ORC_FN(set3)(s, sk, si, q1);
            ORC_FN(onto_plane)(q1.p, sk.p, si.p, dir);
          } else {
            ORC_FN(set2)(s, sk, q1);
            ORC_FN(onto_line)(q1.p, sk.p, dir);
          }
        } else if (!ORC_FN(edge_drops)(q1.p, sj.p, si.p)) {
          ORC_FN(set3)(s, sj, si, q1);
          ORC_FN(onto_plane)(q1.p, si.p, sj.p, dir);
        } else {
          ORC_FN(set2)(s, sj, q1);
          ORC_FN(onto_line)(q1.p, sj.p, dir);
        }
      }
      /* nkeep == 3 leaves simplex and direction unchanged (openGJK.c:538-608) */
      return;
    default:
      return;
  }
}

/* support point of one body: keeps the previous support unless a vertex is strictly
 * better; the first strictly better vertex in index order wins (openGJK.c:615-639) */
static void ORC_FN(support)(const ORC_FN(body) * bd, const R* d, R* sp, int* sid) {
  R best = ORC_FN(dot)(sp, d);
  int win = -1;
  for (int i = 0; i < bd->n; ++i) {
    const R s = ORC_FN(dot)(&bd->xyz[3 * i], d);
    if (s > best) {
      best = s;
      win = i;
    }
  }
  if (win != -1) {
    ORC_FN(copy3)(sp, &bd->xyz[3 * win]);
    *sid = win;
  }
}

/* ------------------------------------------------------------------------- */
/* witness points (openGJK.c:658-950)                                          */

static inline const R* ORC_FN(pt)(const ORC_FN(body) * bd, int i) { return &bd->xyz[3 * i]; }

static void ORC_FN(wit0)(const ORC_FN(body) * A, const ORC_FN(body) * B, ORC_FN(smx) * s) {
  const R* a = ORC_FN(pt)(A, s->v[0].a);
  const R* b = ORC_FN(pt)(B, s->v[0].b);
  for (int c = 0; c < 3; ++c) {
    s->wit[0][c] = a[c];
    s->wit[1][c] = b[c];
  }
}

static void ORC_FN(wit1)(const ORC_FN(body) * A, const ORC_FN(body) * B, ORC_FN(smx) * s) {
  R e[3], o[3];
  for (int c = 0; c < 3; ++c) {
    e[c] = s->v[1].p[c] - s->v[0].p[c];
    o[c] = -s->v[0].p[c];
  }
  const R g = ORC_FN(dot)(e, e);
  if (g == 0.0) ORC_FN(wit0)(A, B, s); /* the reference falls through afterwards */
  const R l1 = ORC_FN(dot)(e, o) / g;
  const R l0 = 1.0 - l1;
  const R *a0 = ORC_FN(pt)(A, s->v[0].a), *b0 = ORC_FN(pt)(B, s->v[0].b);
  const R *a1 = ORC_FN(pt)(A, s->v[1].a), *b1 = ORC_FN(pt)(B, s->v[1].b);
  for (int c = 0; c < 3; ++c) {
    s->wit[0][c] = a0[c] * l0 + a1[c] * l1;
    s->wit[1][c] = b0[c] * l0 + b1[c] * l1;
  }
}

static void ORC_FN(wit2)(const ORC_FN(body) * A, const ORC_FN(body) * B, ORC_FN(smx) * s) {
  R e1[3], e2[3], o[3];
  for (int c = 0; c < 3; ++c) {
    e1[c] = s->v[1].p[c] - s->v[0].p[c];
    e2[c] = s->v[2].p[c] - s->v[0].p[c];
    o[c] = -s->v[0].p[c];
  }
  const R g11 = ORC_FN(dot)(e1, e1);
  const R g12 = ORC_FN(dot)(e1, e2);
  const R g22 = ORC_FN(dot)(e2, e2);
  const R det = g11 * g22 - g12 * g12;
  if (det == 0.0) ORC_FN(wit1)(A, B, s);
  const R r1 = ORC_FN(dot)(e1, o);
  const R r2 = ORC_FN(dot)(e2, o);
  const R m11 = g22 / det;
  const R m12 = -g12 / det;
  const R m22 = g11 / det;
  const R l1 = m11 * r1 + m12 * r2;
  const R l2 = m12 * r1 + m22 * r2;
  const R l0 = 1.0 - l1 - l2; /* evaluated in double as in the reference */
  if (l0 < ORC_EPS) {
    s->n = 2;
    s->v[0] = s->v[2];
    ORC_FN(wit1)(A, B, s);
  } else if (l1 < ORC_EPS) {
    s->n = 2;
    s->v[1] = s->v[2];
    ORC_FN(wit1)(A, B, s);
  } else if (l2 < ORC_EPS) {
    s->n = 2;
    ORC_FN(wit1)(A, B, s);
  }
  /* the 3-point blend below always runs, over the (possibly re-ordered) indices */
  const R *a0 = ORC_FN(pt)(A, s->v[0].a), *b0 = ORC_FN(pt)(B, s->v[0].b);
  const R *a1 = ORC_FN(pt)(A, s->v[1].a), *b1 = ORC_FN(pt)(B, s->v[1].b);
  const R *a2 = ORC_FN(pt)(A, s->v[2].a), *b2 = ORC_FN(pt)(B, s->v[2].b);
  for (int c = 0; c < 3; ++c) {
    s->wit[0][c] = a0[c] * l0 + a1[c] * l1 + a2[c] * l2;
    s->wit[1][c] = b0[c] * l0 + b1[c] * l1 + b2[c] * l2;
  }
}

static void ORC_FN(wit3)(const ORC_FN(body) * A, const ORC_FN(body) * B, ORC_FN(smx) * s) {
  R e1[3], e2[3], e3[3], o[3];
  for (int c = 0; c < 3; ++c) {
    e1[c] = s->v[1].p[c] - s->v[0].p[c];
    e2[c] = s->v[2].p[c] - s->v[0].p[c];
    e3[c] = s->v[3].p[c] - s->v[0].p[c];
    o[c] = -s->v[0].p[c];
  }
  const R g11 = ORC_FN(dot)(e1, e1);
  const R g12 = ORC_FN(dot)(e1, e2);
  const R g13 = ORC_FN(dot)(e1, e3);
  const R g22 = ORC_FN(dot)(e2, e2);
  const R g23 = ORC_FN(dot)(e2, e3);
  const R g33 = ORC_FN(dot)(e3, e3);
  const R c11 = g22 * g33 - g23 * g23;
  const R c12 = g12 * g33 - g13 * g23;
  const R c13 = g12 * g23 - g13 * g22;
  const R det = g11 * c11 - g12 * c12 + g13 * c13;
  if (det == 0.0) ORC_FN(wit2)(A, B, s);
  const R r1 = ORC_FN(dot)(e1, o);
  const R r2 = ORC_FN(dot)(e2, o);
  const R r3 = ORC_FN(dot)(e3, o);
  const R c22 = g11 * g33 - g13 * g13;
  const R c23 = g11 * g23 - g12 * g13;
  const R c33 = g11 * g22 - g12 * g12;
  const R m11 = c11 / det;
  const R m12 = -c12 / det;
  const R m13 = c13 / det;
  const R m22 = c22 / det;
  const R m23 = -c23 / det;
  const R m33 = c33 / det;
  const R l1 = m11 * r1 + m12 * r2 + m13 * r3;
  const R l2 = m12 * r1 + m22 * r2 + m23 * r3;
  const R l3 = m13 * r1 + m23 * r2 + m33 * r3;
  const R l0 = 1.0 - l1 - l2 - l3; /* double arithmetic as in the reference */
  if (l0 < ORC_EPS) {
    s->n = 3;
    s->v[0] = s->v[3];
    ORC_FN(wit2)(A, B, s);
  } else if (l1 < ORC_EPS) {
    s->n = 3;
    s->v[1] = s->v[3];
    ORC_FN(wit2)(A, B, s);
  } else if (l2 < ORC_EPS) {
    s->n = 3;
    s->v[2] = s->v[3];
    ORC_FN(wit2)(A, B, s);
  } else if (l3 < ORC_EPS) {
    s->n = 3;
    ORC_FN(wit2)(A, B, s);
  }
  const R *a0 = ORC_FN(pt)(A, s->v[0].a), *b0 = ORC_FN(pt)(B, s->v[0].b);
  const R *a1 = ORC_FN(pt)(A, s->v[1].a), *b1 = ORC_FN(pt)(B, s->v[1].b);
  const R *a2 = ORC_FN(pt)(A, s->v[2].a), *b2 = ORC_FN(pt)(B, s->v[2].b);
  const R *a3 = ORC_FN(pt)(A, s->v[3].a), *b3 = ORC_FN(pt)(B, s->v[3].b);
  for (int c = 0; c < 3; ++c) {
    s->wit[0][c] = a0[c] * l0 + a1[c] * l1 + a2[c] * l2 + a3[c] * l3;
    s->wit[1][c] = b0[c] * l0 + b1[c] * l1 + b2[c] * l2 + b3[c] * l3;
  }
}

/* ------------------------------------------------------------------------- */
/* GJK distance (openGJK.c:952-1056).  eps_rel / eps_tot / max_iter are the    */
/* reference constants unless the caller overrides them.                       */

typedef struct {
  R eps_rel;
  R eps_tot;
  int max_iter;
} ORC_FN(gjk_cfg);

static R ORC_FN(gjk)(const ORC_FN(body) * A, const ORC_FN(body) * B, const ORC_FN(gjk_cfg) * cfg,
                      ORC_FN(smx) * s, int* iters) {
  const R eps_rel = cfg->eps_rel, eps_tot = cfg->eps_tot;
  const R eps_rel2 = eps_rel * eps_rel;
  R v[3], mv[3], w[3], sa[3], sb[3];
  int ia = 0, ib = 0;
  R wmax2 = 0;
  unsigned k = 0;

  for (int c = 0; c < 3; ++c) v[c] = A->xyz[c] - B->xyz[c];
  s->n = 1;
  ORC_FN(copy3)(s->v[0].p, v);
  s->v[0].a = 0;
  s->v[0].b = 0;
  ORC_FN(copy3)(sa, A->xyz);
  ORC_FN(copy3)(sb, B->xyz);

  do {
    k++;
    for (int c = 0; c < 3; ++c) mv[c] = -v[c];
    ORC_FN(support)(A, mv, sa, &ia);
    ORC_FN(support)(B, v, sb, &ib);
    for (int c = 0; c < 3; ++c) w[c] = sa[c] - sb[c];

    const R gap = ORC_FN(dot)(v, v) - ORC_FN(dot)(v, w);
    if (gap <= (eps_rel * ORC_FN(dot)(v, v)) || gap < eps_tot) break;
    if (ORC_FN(dot)(v, v) < eps_rel2) break;

    ORC_FN(vtx) nw;
    ORC_FN(copy3)(nw.p, w);
    nw.a = ia;
    nw.b = ib;
    s->v[s->n++] = nw;
    if (s->n == 4)
      ORC_FN(sub3)(s, v);
    else if (s->n == 3)
      ORC_FN(sub2)(s, v);
    else if (s->n == 2)
      ORC_FN(sub1)(s, v);

    for (int j = 0; j < s->n; ++j) {
      const R t = ORC_FN(dot)(s->v[j].p, s->v[j].p);
      if (t > wmax2) wmax2 = t;
    }
    if (ORC_FN(dot)(v, v) <= (eps_tot * eps_tot * wmax2)) break;
  } while (s->n != 4 && (int)k != cfg->max_iter);

  switch (s->n) {
    case 4: ORC_FN(wit3)(A, B, s); break;
    case 3: ORC_FN(wit2)(A, B, s); break;
    case 2: ORC_FN(wit1)(A, B, s); break;
    case 1: ORC_FN(wit0)(A, B, s); break;
    default: break;
  }
  if (iters) *iters = (int)k;
  return ORC_SQRT(ORC_FN(dot)(v, v));
}

/* ------------------------------------------------------------------------- */
/* EPA (GJK/cpu/EPA.c)                                                          */

#define ORC_EPA_FACES 128
#define ORC_EPA_VERTS (ORC_EPA_FACES + 4)

typedef struct {
  int v[3];
  int id[3][2];
  R nrm[3];
  R dist;
  int live;
} ORC_FN(face);

typedef struct {
  R p[ORC_EPA_VERTS][3];
  int id[ORC_EPA_VERTS][2];
  int nv;
  ORC_FN(face) f[ORC_EPA_FACES];
  int fend; /* one past the highest slot in use */
} ORC_FN(poly);

typedef struct {
  int a, b; /* polytope vertex ids */
  int ia[2], ib[2];
  int live;
} ORC_FN(edge);

/* EPA.c:92-129 */
static void ORC_FN(face_plane)(ORC_FN(poly) * P, int fi) {
  ORC_FN(face)* F = &P->f[fi];
  const R *p0 = P->p[F->v[0]], *p1 = P->p[F->v[1]], *p2 = P->p[F->v[2]];
  R e0[3], e1[3];
  for (int c = 0; c < 3; ++c) {
    e0[c] = p1[c] - p0[c];
    e1[c] = p2[c] - p0[c];
  }
  ORC_FN(cross)(e0, e1, F->nrm);
  const R n2 = ORC_FN(dot)(F->nrm, F->nrm);
  if (n2 > ORC_EPS * ORC_EPS) {
    const R len = ORC_SQRT(n2);
    for (int c = 0; c < 3; ++c) F->nrm[c] /= len;
    F->dist = ORC_FN(dot)(F->nrm, p0);
    if (F->dist < 0) {
      for (int c = 0; c < 3; ++c) F->nrm[c] = -F->nrm[c];
      F->dist = -F->dist;
    }
  } else {
    F->live = 0;
    F->dist = (R)1e10;
  }
}

/* EPA.c:132-140 */
static int ORC_FN(face_sees)(const ORC_FN(poly) * P, int fi, const R* q) {
  const ORC_FN(face)* F = &P->f[fi];
  if (!F->live) return 0;
  const R* p0 = P->p[F->v[0]];
  R d[3];
  for (int c = 0; c < 3; ++c) d[c] = q[c] - p0[c];
  return ORC_FN(dot)(F->nrm, d) > ORC_EPS;
}

/* orient face fi so that its normal points away from `ctr` (EPA.c:204-232, 791-819) */
static void ORC_FN(face_orient)(ORC_FN(poly) * P, int fi, const R* ctr) {
  ORC_FN(face)* F = &P->f[fi];
  const R *p0 = P->p[F->v[0]], *p1 = P->p[F->v[1]], *p2 = P->p[F->v[2]];
  R e0[3], e1[3], n[3], tc[3];
  for (int c = 0; c < 3; ++c) {
    e0[c] = p1[c] - p0[c];
    e1[c] = p2[c] - p0[c];
  }
  ORC_FN(cross)(e0, e1, n);
  for (int c = 0; c < 3; ++c) tc[c] = ctr[c] - p0[c];
  if (ORC_FN(dot)(n, tc) > 0) {
    int t = F->v[1];
    F->v[1] = F->v[2];
    F->v[2] = t;
    int t0 = F->id[1][0], t1 = F->id[1][1];
    F->id[1][0] = F->id[2][0];
    F->id[1][1] = F->id[2][1];
    F->id[2][0] = t0;
    F->id[2][1] = t1;
  }
}

/* tetrahedron from the GJK simplex (EPA.c:144-235) */
static void ORC_FN(poly_init)(ORC_FN(poly) * P, const ORC_FN(smx) * s, R* ctr) {
  static const int tri[4][3] = {{0, 1, 2}, {0, 3, 1}, {0, 2, 3}, {1, 3, 2}};
  memset(P->f, 0, sizeof(P->f));
  P->nv = 4;
  for (int i = 0; i < 4; ++i) {
    ORC_FN(copy3)(P->p[i], s->v[i].p);
    P->id[i][0] = s->v[i].a;
    P->id[i][1] = s->v[i].b;
  }
  ctr[0] = ctr[1] = ctr[2] = 0;
  for (int i = 0; i < 4; ++i)
    for (int c = 0; c < 3; ++c) ctr[c] += P->p[i][c] * (R)0.25;
  for (int f = 0; f < 4; ++f) {
    for (int k = 0; k < 3; ++k) {
      P->f[f].v[k] = tri[f][k];
      P->f[f].id[k][0] = s->v[tri[f][k]].a;
      P->f[f].id[k][1] = s->v[tri[f][k]].b;
    }
    P->f[f].live = 1;
  }
  for (int f = 0; f < 4; ++f) ORC_FN(face_orient)(P, f, ctr);
  P->fend = 4;
}

/* barycentric coordinates of the origin's projection on a triangle, clamped to
 * the triangle's edges (EPA.c:238-304) */
static void ORC_FN(bary)(const R* p0, const R* p1, const R* p2, R* l) {
  R e0[3], e1[3];
  for (int c = 0; c < 3; ++c) {
    e0[c] = p1[c] - p0[c];
    e1[c] = p2[c] - p0[c];
  }
  const R d00 = ORC_FN(dot)(e0, e0);
  const R d01 = ORC_FN(dot)(e0, e1);
  const R d11 = ORC_FN(dot)(e1, e1);
  const R d20 = -ORC_FN(dot)(p0, e0);
  const R d21 = -ORC_FN(dot)(p0, e1);
  const R den = d00 * d11 - d01 * d01;
  if (ORC_FABS(den) < ORC_EPS) {
    l[0] = l[1] = l[2] = (R)1.0 / (R)3.0;
    return;
  }
  const R inv = (R)1.0 / den;
  const R u = (d11 * d20 - d01 * d21) * inv;
  const R v = (d00 * d21 - d01 * d20) * inv;
  const R w = (R)1.0 - u - v;
  if (w < 0) {
    R e12[3];
    for (int c = 0; c < 3; ++c) e12[c] = p2[c] - p1[c];
    R t = -ORC_FN(dot)(p1, e12) / ORC_FN(dot)(e12, e12);
    t = ORC_FMAX((R)0.0, ORC_FMIN((R)1.0, t));
    l[0] = 0;
    l[1] = (R)1.0 - t;
    l[2] = t;
  } else if (u < 0) {
    R t = -ORC_FN(dot)(p0, e1) / ORC_FN(dot)(e1, e1);
    t = ORC_FMAX((R)0.0, ORC_FMIN((R)1.0, t));
    l[0] = (R)1.0 - t;
    l[1] = 0;
    l[2] = t;
  } else if (v < 0) {
    R t = -ORC_FN(dot)(p0, e0) / ORC_FN(dot)(e0, e0);
    t = ORC_FMAX((R)0.0, ORC_FMIN((R)1.0, t));
    l[0] = (R)1.0 - t;
    l[1] = t;
    l[2] = 0;
  } else {
    l[0] = w;
    l[1] = u;
    l[2] = v;
  }
}

/* Minkowski support s_A(d) - s_B(-d); the first maximum in index order wins
 * (EPA.c:307-344) */
static void ORC_FN(msupport)(const ORC_FN(body) * A, const ORC_FN(body) * B, const R* d, R* out,
                             int* oid) {
  R m1 = (R)-1e10f, m2 = (R)-1e10f;
  int w1 = -1, w2 = -1;
  for (int i = 0; i < A->n; ++i) {
    const R* x = &A->xyz[3 * i];
    const R t = x[0] * d[0] + x[1] * d[1] + x[2] * d[2];
    if (t > m1) {
      m1 = t;
      w1 = i;
    }
  }
  for (int i = 0; i < B->n; ++i) {
    const R* x = &B->xyz[3 * i];
    const R t = x[0] * d[0] + x[1] * d[1] + x[2] * d[2];
    if (-t > m2) {
      m2 = -t;
      w2 = i;
    }
  }
  if (w1 >= 0 && w2 >= 0) {
    for (int c = 0; c < 3; ++c) out[c] = A->xyz[3 * w1 + c] - B->xyz[3 * w2 + c];
    oid[0] = w1;
    oid[1] = w2;
  }
}

/* unit vector from w0 to w1, (1,0,0) when they coincide (EPA.c:350-360) */
static void ORC_FN(normal_from)(const R* w0, const R* w1, R* n) {
  R d[3] = {w1[0] - w0[0], w1[1] - w0[1], w1[2] - w0[2]};
  const R len = ORC_SQRT(ORC_FN(dot)(d, d));
  if (len > ORC_EPS) {
    n[0] = d[0] / len;
    n[1] = d[1] / len;
    n[2] = d[2] / len;
  } else {
    n[0] = 1.0f;
    n[1] = 0.0f;
    n[2] = 0.0f;
  }
}

/* witnesses, normal and depth from face fi (EPA.c:637-650) */
static void ORC_FN(epa_emit)(const ORC_FN(body) * A, const ORC_FN(body) * B, const ORC_FN(poly) * P,
                             int fi, ORC_FN(smx) * s, R* dist, R* nrm) {
  const ORC_FN(face)* F = &P->f[fi];
  R l[3];
  ORC_FN(bary)(P->p[F->v[0]], P->p[F->v[1]], P->p[F->v[2]], l);
  for (int c = 0; c < 3; ++c) {
    s->wit[0][c] = A->xyz[3 * F->id[0][0] + c] * l[0] + A->xyz[3 * F->id[1][0] + c] * l[1] +
                   A->xyz[3 * F->id[2][0] + c] * l[2];
    s->wit[1][c] = B->xyz[3 * F->id[0][1] + c] * l[0] + B->xyz[3 * F->id[1][1] + c] * l[1] +
                   B->xyz[3 * F->id[2][1] + c] * l[2];
    nrm[c] = F->nrm[c];
  }
  *dist = -F->dist;
}

/* contact result when the simplex cannot be grown: depth 0 at the support pair */
static void ORC_FN(epa_touch)(const ORC_FN(body) * A, const ORC_FN(body) * B, int ia, int ib,
                              ORC_FN(smx) * s, R* dist, R* nrm) {
  *dist = 0.0f;
  for (int c = 0; c < 3; ++c) {
    s->wit[0][c] = A->xyz[3 * ia + c];
    s->wit[1][c] = B->xyz[3 * ib + c];
  }
  ORC_FN(normal_from)(s->wit[0], s->wit[1], nrm);
}

/* is q at least eps away from the first m simplex points? (EPA.c:452-463) */
static int ORC_FN(is_new)(const ORC_FN(smx) * s, int m, const R* q) {
  const R e2 = ORC_EPS * ORC_EPS;
  for (int k = 0; k < m; ++k) {
    const R dx = q[0] - s->v[k].p[0];
    const R dy = q[1] - s->v[k].p[1];
    const R dz = q[2] - s->v[k].p[2];
    if (dx * dx + dy * dy + dz * dz < e2) return 0;
  }
  return 1;
}

static void ORC_FN(push)(ORC_FN(smx) * s, const R* q, const int* qid) {
  ORC_FN(copy3)(s->v[s->n].p, q);
  s->v[s->n].a = qid[0];
  s->v[s->n].b = qid[1];
  s->n++;
}

/* exit codes reported beside each EPA result (the reference has none) */
#ifndef ORC_EPA_CODES_
#define ORC_EPA_CODES_
enum { ORC_EPA_SKIPPED = 0, ORC_EPA_CONVERGED = 1, ORC_EPA_DUPLICATE = 2, ORC_EPA_ITER_CAP = 3,
       ORC_EPA_TOUCH = 4, ORC_EPA_STALLED = 5 };
#endif

typedef struct {
  R tol;
  int max_iter;
} ORC_FN(epa_cfg);

/* computeCollisionInformation (EPA.c:362-863).  Returns one of the exit codes. */
static int ORC_FN(epa)(const ORC_FN(body) * A, const ORC_FN(body) * B, const ORC_FN(epa_cfg) * cfg,
                       ORC_FN(smx) * s, R* dist, R* nrm, int* iters) {
  if (iters) *iters = 0;
  if (*dist > ORC_EPS) {
    ORC_FN(normal_from)(s->wit[0], s->wit[1], nrm);
    return ORC_EPA_SKIPPED;
  }

  if (s->n != 4) {
    R q[3], d[3];
    int qid[2] = {0, 0};
    if (s->n == 1) { /* EPA.c:378-419 */
      ORC_FN(msupport)(A, B, s->v[0].p, q, qid);
      if (ORC_FN(is_new)(s, 1, q)) {
        ORC_FN(push)(s, q, qid);
      } else {
        ORC_FN(epa_touch)(A, B, qid[0], qid[1], s, dist, nrm);
        return ORC_EPA_TOUCH;
      }
    }
    if (s->n == 2) { /* EPA.c:420-484 */
      R edge[3], axis[3] = {1.0f, 0.0f, 0.0f};
      for (int c = 0; c < 3; ++c) edge[c] = s->v[1].p[c] - s->v[0].p[c];
      const R elen = ORC_SQRT(ORC_FN(dot)(edge, edge));
      if (elen > ORC_EPS && ORC_FABS(edge[0]) > 0.9f * elen) {
        axis[0] = 0.0f;
        axis[1] = 1.0f;
        axis[2] = 0.0f;
      }
      ORC_FN(cross)(edge, axis, d);
      if (ORC_FN(dot)(d, d) < ORC_EPS) {
        axis[0] = 0.0f;
        axis[1] = 0.0f;
        axis[2] = 1.0f;
        ORC_FN(cross)(edge, axis, d);
      }
      ORC_FN(msupport)(A, B, d, q, qid);
      if (ORC_FN(is_new)(s, 2, q)) {
        ORC_FN(push)(s, q, qid);
      } else {
        ORC_FN(epa_touch)(A, B, qid[0], qid[1], s, dist, nrm);
        return ORC_EPA_TOUCH;
      }
    }
    if (s->n == 3) { /* EPA.c:485-569: triangle normal, then its opposite */
      R e0[3], e1[3];
      for (int c = 0; c < 3; ++c) {
        e0[c] = s->v[1].p[c] - s->v[0].p[c];
        e1[c] = s->v[2].p[c] - s->v[0].p[c];
      }
      ORC_FN(cross)(e0, e1, d);
      ORC_FN(msupport)(A, B, d, q, qid);
      if (ORC_FN(is_new)(s, 3, q)) {
        ORC_FN(push)(s, q, qid);
      } else {
        for (int c = 0; c < 3; ++c) d[c] = -d[c];
      }
      if (s->n == 3) {
        ORC_FN(msupport)(A, B, d, q, qid);
        if (ORC_FN(is_new)(s, 3, q)) {
          ORC_FN(push)(s, q, qid);
        } else {
          ORC_FN(epa_touch)(A, B, qid[0], qid[1], s, dist, nrm);
          return ORC_EPA_TOUCH;
        }
      }
    }
    if (s->n != 4) { /* EPA.c:572-582 */
      const int best = s->n > 0 ? s->n - 1 : 0;
      ORC_FN(epa_touch)(A, B, s->v[best].a, s->v[best].b, s, dist, nrm);
      return ORC_EPA_TOUCH;
    }
  }

  static _Thread_local ORC_FN(poly) P;
  static _Thread_local ORC_FN(edge) E[ORC_EPA_FACES * 3];
  R ctr[3];
  ORC_FN(poly_init)(&P, s, ctr);

  int it = 0;
  int code = ORC_EPA_STALLED;
  while (it < cfg->max_iter && P.nv < ORC_EPA_VERTS - 1) {
    it++;
    for (int f = 0; f < P.fend; ++f)
      if (P.f[f].live) ORC_FN(face_plane)(&P, f);

    int best = -1;
    R bestd = 1e10f;
    for (int f = 0; f < P.fend; ++f) {
      if (!P.f[f].live) continue;
      if (P.f[f].dist >= 0.0f && P.f[f].dist < bestd) {
        bestd = P.f[f].dist;
        best = f;
      }
    }
    if (best < 0) break;

    R q[3];
    int qid[2];
    ORC_FN(msupport)(A, B, P.f[best].nrm, q, qid);
    const R gain = ORC_FN(dot)(P.f[best].nrm, q) - bestd;
    if (gain < cfg->tol) {
      ORC_FN(epa_emit)(A, B, &P, best, s, dist, nrm);
      code = ORC_EPA_CONVERGED;
      break;
    }

    int dup = 0;
    {
      const R e2 = ORC_EPS * ORC_EPS;
      for (int i = 0; i < P.nv; ++i) {
        const R dx = q[0] - P.p[i][0];
        const R dy = q[1] - P.p[i][1];
        const R dz = q[2] - P.p[i][2];
        if (dx * dx + dy * dy + dz * dz < e2) {
          dup = 1;
          break;
        }
      }
    }
    if (dup) {
      ORC_FN(epa_emit)(A, B, &P, best, s, dist, nrm);
      code = ORC_EPA_DUPLICATE;
      break;
    }

    const int nid = P.nv;
    ORC_FN(copy3)(P.p[nid], q);
    P.id[nid][0] = qid[0];
    P.id[nid][1] = qid[1];
    P.nv++;
    const R inv = (R)1.0 / (R)P.nv;
    for (int c = 0; c < 3; ++c) ctr[c] += (q[c] - ctr[c]) * inv;

    /* faces seen from q: collect their edges, then retire them (EPA.c:703-743) */
    int ne = 0;
    for (int f = 0; f < P.fend; ++f) {
      if (!P.f[f].live) continue;
      if (!ORC_FN(face_sees)(&P, f, q)) continue;
      for (int k = 0; k < 3; ++k) {
        if (ne < ORC_EPA_FACES * 3) {
          const int k2 = (k + 1) % 3;
          E[ne].a = P.f[f].v[k];
          E[ne].b = P.f[f].v[k2];
          E[ne].ia[0] = P.f[f].id[k][0];
          E[ne].ia[1] = P.f[f].id[k][1];
          E[ne].ib[0] = P.f[f].id[k2][0];
          E[ne].ib[1] = P.f[f].id[k2][1];
          E[ne].live = 1;
          ne++;
        }
      }
      P.f[f].live = 0;
    }
    /* an edge listed twice lies between two retired faces (EPA.c:746-759) */
    for (int i = 0; i < ne; ++i) {
      if (!E[i].live) continue;
      for (int j = i + 1; j < ne; ++j) {
        if (!E[j].live) continue;
        if ((E[i].a == E[j].a && E[i].b == E[j].b) || (E[i].a == E[j].b && E[i].b == E[j].a)) {
          E[i].live = 0;
          E[j].live = 0;
        }
      }
    }
    /* one new face per horizon edge, in the first free slot (EPA.c:762-825) */
    for (int i = 0; i < ne; ++i) {
      if (!E[i].live) continue;
      int slot = -1;
      for (int j = 0; j < ORC_EPA_FACES; ++j) {
        if (!P.f[j].live) {
          slot = j;
          break;
        }
      }
      if (slot < 0 || slot >= ORC_EPA_FACES) break;
      ORC_FN(face)* F = &P.f[slot];
      F->v[0] = E[i].a;
      F->v[1] = E[i].b;
      F->v[2] = nid;
      F->id[0][0] = E[i].ia[0];
      F->id[0][1] = E[i].ia[1];
      F->id[1][0] = E[i].ib[0];
      F->id[1][1] = E[i].ib[1];
      F->id[2][0] = qid[0];
      F->id[2][1] = qid[1];
      F->live = 1;
      ORC_FN(face_orient)(&P, slot, ctr);
      if (slot >= P.fend) P.fend = slot + 1;
    }
  }

  if (it >= cfg->max_iter) { /* EPA.c:829-863 */
    for (int f = 0; f < P.fend; ++f)
      if (P.f[f].live) ORC_FN(face_plane)(&P, f);
    int best = -1;
    R bestd = 1e10f;
    for (int f = 0; f < P.fend; ++f) {
      if (!P.f[f].live) continue;
      if (P.f[f].dist >= 0.0f && P.f[f].dist < bestd) {
        bestd = P.f[f].dist;
        best = f;
      }
    }
    if (best >= 0) ORC_FN(epa_emit)(A, B, &P, best, s, dist, nrm);
    if (code == ORC_EPA_STALLED) code = ORC_EPA_ITER_CAP;
  }
  if (iters) *iters = it;
  return code;
}

#undef R
