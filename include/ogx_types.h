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

#ifndef COMMON_H__ /* the reference's own common.h defines the same types */
#include <float.h>
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
#endif

#ifndef OGX_NO_COLLISION_PAIR
typedef struct gkCollisionPair {
  int idx1; /* index of the first polytope in the pool */
  int idx2; /* index of the second polytope */
} gkCollisionPair;
#endif

#endif /* OGX_TYPES_H_ */
