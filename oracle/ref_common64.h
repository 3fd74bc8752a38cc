/*
 * ref_common64.h -- forced-include header used only when the reference's own CPU
 * sources are compiled in FP64 for validation of the oracle (see Makefile target
 * `ref`).  It pre-empts GJK/common.h (whose include guard is COMMON_H__) with the
 * same type definitions in double precision, which is what the reference's
 * precision switch (GJK/common.h:44, USE_32BITS) selects when it is turned off.
 */
#ifndef COMMON_H__
#define COMMON_H__
#include <float.h>
#define gkFloat double
#define gkEpsilon DBL_EPSILON
#define gkSqrt sqrt
#define gkFmax fmax
#define gkFmin fmin
#define gkFabs fabs
typedef struct gkPolytope {
  int numpoints;
  gkFloat s[3];
  int s_idx;
  gkFloat* coord;
} gkPolytope;
typedef struct gkSimplex {
  int nvrtx;
  gkFloat vrtx[4][3];
  int vrtx_idx[4][2];
  gkFloat witnesses[2][3];
} gkSimplex;
#endif
