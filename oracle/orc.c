/*
 * orc.c -- FP32 and FP64 instantiations of the CPU oracle plus a threaded batch
 * driver.  TEST INFRASTRUCTURE ONLY (parity checker and CPU baseline).
 *
 * The batch driver mirrors the reference's CPU facade loops
 * (examples/cpu/example.cpp:13-40): GJK per pair, then
 * computeCollisionInformation per pair, partitioned over threads in contiguous
 * pair ranges.
 */
#include "orc.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---- FP32 ---- */
#define ORC_REAL float
#define ORC_SFX _f32
#define ORC_EPS FLT_EPSILON
#define ORC_SQRT sqrtf
#define ORC_FABS fabsf
#define ORC_FMAX fmaxf
#define ORC_FMIN fminf
#include "orc_core.h"
#undef ORC_REAL
#undef ORC_SFX
#undef ORC_EPS
#undef ORC_SQRT
#undef ORC_FABS
#undef ORC_FMAX
#undef ORC_FMIN

/* ---- FP64 ---- */
#define ORC_REAL double
#define ORC_SFX _f64
#define ORC_EPS DBL_EPSILON
#define ORC_SQRT sqrt
#define ORC_FABS fabs
#define ORC_FMAX fmax
#define ORC_FMIN fmin
#include "orc_core.h"
#undef ORC_REAL
#undef ORC_SFX
#undef ORC_EPS
#undef ORC_SQRT
#undef ORC_FABS
#undef ORC_FMAX
#undef ORC_FMIN

/* The batch driver is written once per precision with the same macro trick. */
#define ORC_BATCH(SFX, REAL, EPS)                                                               \
  typedef struct {                                                                              \
    int lo, hi, mode;                                                                           \
    const REAL* coords;                                                                         \
    const int64_t* offsets;                                                                     \
    const int32_t* counts;                                                                      \
    const int32_t* pairs;                                                                       \
    gjk_cfg##SFX gc;                                                                            \
    epa_cfg##SFX ec;                                                                            \
    orc_result* out;                                                                            \
  } job##SFX;                                                                                   \
                                                                                                \
  static void one##SFX(const job##SFX* J, int i) {                                              \
    const int32_t b1 = J->pairs[2 * i], b2 = J->pairs[2 * i + 1];                               \
    body##SFX A = {J->counts[b1], J->coords + 3 * J->offsets[b1]};                              \
    body##SFX B = {J->counts[b2], J->coords + 3 * J->offsets[b2]};                              \
    orc_result* o = &J->out[i];                                                                 \
    smx##SFX s;                                                                                 \
    memset(&s, 0, sizeof(s));                                                                   \
    REAL dist = 0, nrm[3] = {NAN, NAN, NAN};                                                    \
    int gi = 0, ei = 0, code = 0;                                                               \
    if (J->mode == ORC_MODE_EPA) {                                                              \
      s.n = o->nvrtx;                                                                           \
      for (int k = 0; k < 4; ++k) {                                                             \
        for (int c = 0; c < 3; ++c) s.v[k].p[c] = (REAL)o->vrtx[k][c];                          \
        s.v[k].a = o->idx[k][0];                                                                \
        s.v[k].b = o->idx[k][1];                                                                \
      }                                                                                         \
      for (int w = 0; w < 2; ++w)                                                               \
        for (int c = 0; c < 3; ++c) s.wit[w][c] = (REAL)o->wit[w][c];                           \
      dist = (REAL)o->dist;                                                                     \
      gi = o->gjk_iters;                                                                        \
    } else {                                                                                    \
      dist = gjk##SFX(&A, &B, &J->gc, &s, &gi);                                                 \
    }                                                                                           \
    if (J->mode != ORC_MODE_GJK) code = epa##SFX(&A, &B, &J->ec, &s, &dist, nrm, &ei);          \
    o->dist = dist;                                                                             \
    for (int w = 0; w < 2; ++w)                                                                 \
      for (int c = 0; c < 3; ++c) o->wit[w][c] = s.wit[w][c];                                   \
    for (int c = 0; c < 3; ++c) o->normal[c] = nrm[c];                                          \
    for (int k = 0; k < 4; ++k) {                                                               \
      for (int c = 0; c < 3; ++c) o->vrtx[k][c] = s.v[k].p[c];                                  \
      o->idx[k][0] = s.v[k].a;                                                                  \
      o->idx[k][1] = s.v[k].b;                                                                  \
    }                                                                                           \
    o->nvrtx = s.n;                                                                             \
    o->gjk_iters = gi;                                                                          \
    o->epa_iters = ei;                                                                          \
    o->epa_exit = code;                                                                         \
  }                                                                                             \
                                                                                                \
  static void* worker##SFX(void* arg) {                                                         \
    const job##SFX* J = (const job##SFX*)arg;                                                   \
    for (int i = J->lo; i < J->hi; ++i) one##SFX(J, i);                                         \
    return NULL;                                                                                \
  }                                                                                             \
                                                                                                \
  int orc_run##SFX(int npairs, const REAL* coords, const int64_t* offsets, const int32_t* counts, \
                   const int32_t* pairs, int mode, const orc_config* cfg, orc_result* out,      \
                   int nthreads) {                                                              \
    if (npairs < 0 || mode < ORC_MODE_GJK || mode > ORC_MODE_EPA) return -1;                    \
    if (npairs == 0) return 0;                                                                  \
    if (!coords || !offsets || !counts || !pairs || !out) return -1;                            \
    job##SFX base;                                                                              \
    memset(&base, 0, sizeof(base));                                                             \
    base.mode = mode;                                                                           \
    base.coords = coords;                                                                       \
    base.offsets = offsets;                                                                     \
    base.counts = counts;                                                                       \
    base.pairs = pairs;                                                                         \
    base.out = out;                                                                             \
    base.gc.eps_rel = (REAL)EPS * 1e4f;                                                         \
    base.gc.eps_tot = (REAL)EPS * 1e2f;                                                         \
    base.gc.max_iter = 25;                                                                      \
    base.ec.tol = ((REAL)(EPS) * (REAL)1e2);                                                    \
    base.ec.max_iter = 64;                                                                      \
    if (cfg) {                                                                                  \
      if (cfg->eps_rel > 0) base.gc.eps_rel = (REAL)cfg->eps_rel;                               \
      if (cfg->eps_tot > 0) base.gc.eps_tot = (REAL)cfg->eps_tot;                               \
      if (cfg->gjk_max_iter > 0) base.gc.max_iter = cfg->gjk_max_iter;                          \
      if (cfg->epa_tol > 0) base.ec.tol = (REAL)cfg->epa_tol;                                   \
      if (cfg->epa_max_iter > 0) base.ec.max_iter = cfg->epa_max_iter;                          \
    }                                                                                           \
    if (nthreads <= 1 || npairs < 2 * nthreads) {                                               \
      base.lo = 0;                                                                              \
      base.hi = npairs;                                                                         \
      worker##SFX(&base);                                                                       \
      return 0;                                                                                 \
    }                                                                                           \
    if (nthreads > 256) nthreads = 256;                                                         \
    pthread_t th[256];                                                                          \
    job##SFX jobs[256];                                                                         \
    for (int t = 0; t < nthreads; ++t) {                                                        \
      jobs[t] = base;                                                                           \
      jobs[t].lo = (int)((int64_t)npairs * t / nthreads);                                       \
      jobs[t].hi = (int)((int64_t)npairs * (t + 1) / nthreads);                                 \
      pthread_create(&th[t], NULL, worker##SFX, &jobs[t]);                                      \
    }                                                                                           \
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);                               \
    return 0;                                                                                   \
  }

ORC_BATCH(_f32, float, FLT_EPSILON)
ORC_BATCH(_f64, double, DBL_EPSILON)
