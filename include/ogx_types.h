/*
 * ogx_types.h -- the reference's data types, FP32 layout.
 *
 * These keep the field order and sizes of OpenGJK-GPU's types so that arrays built
 * for the reference can be passed unchanged:
 *   gkPolytope      GJK/common.h:68-78         (32 bytes on LP64)
 *   gkSimplex       GJK/common.h:84-89         (108 bytes)
 *   gkCollisionPair GJK/gpu/openGJK.h:309-312  (8 bytes)
 * The reference compiles with USE_32BITS (GJK/common.h:44), i.e. gkFloat = float;
 * this engine's arithmetic type is float with FP64 only where noted.
 */
#ifndef OGX_TYPES_H_
#define OGX_TYPES_H_

/* FP64 layouts of the same types: the reference built with USE_32BITS off
 * (GJK/common.h:44-60, gkFloat = double): 48 and 184 bytes on LP64.  The *_f64 entry
 * points take these; defining OGX_GKFLOAT_DOUBLE before including this header makes
 * gkFloat, gkPolytope and gkSimplex these types, as the reference's switch does. */
typedef struct ogx_polytope_f64 {
  int numpoints;
  double s[3];
  int s_idx;
  double* coord;
} ogx_polytope_f64;

typedef struct ogx_simplex_f64 {
  int nvrtx;
  double vrtx[4][3];
  int vrtx_idx[4][2];
  double witnesses[2][3];
} ogx_simplex_f64;

#ifndef COMMON_H__ /* the reference's own common.h defines the same types */
#include <float.h>
#ifdef OGX_GKFLOAT_DOUBLE
typedef double gkFloat;
typedef ogx_polytope_f64 gkPolytope;
typedef ogx_simplex_f64 gkSimplex;
/* the FP32 layouts, by their own names (the engine API takes these) */
typedef struct ogx_polytope_f32 {
  int numpoints;
  float s[3];
  int s_idx;
  float* coord;
} ogx_polytope_f32;
typedef struct ogx_simplex_f32 {
  int nvrtx;
  float vrtx[4][3];
  int vrtx_idx[4][2];
  float witnesses[2][3];
} ogx_simplex_f32;
#else
typedef float gkFloat;
typedef struct gkPolytope {
  int numpoints;   /* number of points */
  gkFloat s[3];    /* scratch: last support point (overwritten) */
  int s_idx;       /* scratch: index of the last support point */
  gkFloat* coord;  /* xyz interleaved, owned by the caller */
} gkPolytope;

typedef struct gkSimplex {
  int nvrtx;               /* number of simplex points (4 = origin enclosed) */
  gkFloat vrtx[4][3];      /* simplex points in the Minkowski difference */
  int vrtx_idx[4][2];      /* point indices in body 1 and body 2 */
  gkFloat witnesses[2][3]; /* closest points on body 1 and body 2 */
} gkSimplex;
typedef gkPolytope ogx_polytope_f32;
typedef gkSimplex ogx_simplex_f32;
#endif /* OGX_GKFLOAT_DOUBLE */
/* The reference's common.h (include guard COMMON_H__) declares these same types: a
 * caller that also uses the reference's CPU code includes both headers, and whichever
 * comes first defines the one set of types. */
#define COMMON_H__
#endif /* COMMON_H__ */

#ifndef OGX_NO_COLLISION_PAIR
typedef struct gkCollisionPair {
  int idx1; /* index of the first polytope in the pool */
  int idx2; /* index of the second polytope */
} gkCollisionPair;
#endif

#endif /* OGX_TYPES_H_ */
