/*
 * orc.h -- C interface of the CPU oracle (test infrastructure only).
 *
 * The oracle restates the reference CPU GJK (GJK/cpu/openGJK.c) and EPA
 * (GJK/cpu/EPA.c) in FP32 and FP64.  Tests use it to check the GPU engine;
 * the benchmark uses it as the timed CPU baseline.  The product library never
 * links it.
 */
#ifndef ORC_H_
#define ORC_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One result per pair.  FP32 results are widened exactly to double. */
typedef struct {
  double dist;         /* GJK distance, or -depth after EPA */
  double wit[2][3];    /* witness on body 1, witness on body 2 */
  double normal[3];    /* EPA contact normal (NaN when EPA left it untouched) */
  double vrtx[4][3];   /* final simplex points */
  int32_t idx[4][2];   /* final simplex vertex indices (body 1, body 2) */
  int32_t nvrtx;       /* final simplex size */
  int32_t gjk_iters;   /* GJK iterations */
  int32_t epa_iters;   /* EPA expansion iterations */
  int32_t epa_exit;    /* 0 skipped, 1 converged, 2 duplicate, 3 iteration cap,
                          4 simplex could not grow (depth 0), 5 stalled */
} orc_result;

/* Work modes. */
enum { ORC_MODE_GJK = 1, ORC_MODE_GJK_EPA = 2, ORC_MODE_EPA = 3 };

/* Tolerances; a field <= 0 selects the reference constant for that precision. */
typedef struct {
  double eps_rel;  /* GJK relative tolerance (reference: eps * 1e4) */
  double eps_tot;  /* GJK absolute tolerance (reference: eps * 1e2) */
  int32_t gjk_max_iter; /* reference: 25 */
  double epa_tol;  /* EPA convergence tolerance (reference: eps * 1e2) */
  int32_t epa_max_iter; /* reference: 64 */
} orc_config;

/*
 * Run `npairs` pairs.  Bodies live in one pool: body b has counts[b] points
 * starting at point offsets[b] of `coords` (xyz interleaved).  pairs holds
 * (idx1, idx2) per pair.  In ORC_MODE_EPA the results array is also the input
 * (dist, simplex and witnesses from a previous GJK run).  nthreads <= 0 uses one
 * thread.  Returns 0, or -1 on invalid arguments.
 */
int orc_run_f32(int npairs, const float* coords, const int64_t* offsets, const int32_t* counts,
                const int32_t* pairs, int mode, const orc_config* cfg, orc_result* out,
                int nthreads);
int orc_run_f64(int npairs, const double* coords, const int64_t* offsets, const int32_t* counts,
                const int32_t* pairs, int mode, const orc_config* cfg, orc_result* out,
                int nthreads);

#ifdef __cplusplus
}
#endif
#endif
