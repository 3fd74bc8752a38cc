/*
 * GJK/common.h for callers written against OpenGJK-GPU (GJK/common.h:44-89): with
 * include/compat ahead of the reference's own include path, this header gives the
 * engine's drop-in types instead.  As in the reference, USE_32BITS selects gkFloat =
 * float (the default here, as there); a build that defines OGX_GKFLOAT_DOUBLE gets
 * gkFloat = double with the reference's FP64 layouts and the *_f64 entry points.
 */
#ifndef OGX_COMPAT_GJK_COMMON_H_
#define OGX_COMPAT_GJK_COMMON_H_

#include <float.h>
#include <math.h>

#include "ogx_types.h"

#ifdef OGX_GKFLOAT_DOUBLE
#define gkEpsilon DBL_EPSILON
#define gkSqrt sqrt
#define gkFmax fmax
#define gkFmin fmin
#define gkFabs fabs
#else
#define USE_32BITS
#define gkEpsilon FLT_EPSILON
#define gkSqrt sqrtf
#define gkFmax fmaxf
#define gkFmin fminf
#define gkFabs fabsf
#endif

#endif /* OGX_COMPAT_GJK_COMMON_H_ */
