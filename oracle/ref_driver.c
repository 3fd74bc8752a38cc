/*
 * ref_driver.c -- batch driver over the reference's OWN CPU functions, compiled
 * together with the unmodified GJK/cpu/openGJK.c and GJK/cpu/EPA.c (see the
 * Makefile target `ref`).  It only exists to check the oracle restatement bit for
 * bit; it is never part of the product.  The loops follow the reference's CPU
 * facade (examples/cpu/example.cpp:13-40).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "GJK/cpu/EPA.h"
#include "GJK/cpu/openGJK.h"
#include "orc.h"

int ref_run(int npairs, const gkFloat* coords, const int64_t* offsets, const int32_t* counts,
            const int32_t* pairs, int mode, orc_result* out) {
  for (int i = 0; i < npairs; ++i) {
    const int32_t b1 = pairs[2 * i], b2 = pairs[2 * i + 1];
    gkPolytope A, B;
    memset(&A, 0, sizeof(A));
    memset(&B, 0, sizeof(B));
    A.numpoints = counts[b1];
    A.coord = (gkFloat*)(coords + 3 * offsets[b1]);
    B.numpoints = counts[b2];
    B.coord = (gkFloat*)(coords + 3 * offsets[b2]);
    gkSimplex s;
    memset(&s, 0, sizeof(s));
    gkFloat dist = 0, nrm[3] = {NAN, NAN, NAN};
    orc_result* o = &out[i];
    if (mode == ORC_MODE_EPA) {
      s.nvrtx = o->nvrtx;
      for (int k = 0; k < 4; ++k) {
        for (int c = 0; c < 3; ++c) s.vrtx[k][c] = (gkFloat)o->vrtx[k][c];
        s.vrtx_idx[k][0] = o->idx[k][0];
        s.vrtx_idx[k][1] = o->idx[k][1];
      }
      for (int w = 0; w < 2; ++w)
        for (int c = 0; c < 3; ++c) s.witnesses[w][c] = (gkFloat)o->wit[w][c];
      dist = (gkFloat)o->dist;
    } else {
      dist = compute_minimum_distance(A, B, &s);
    }
    if (mode != ORC_MODE_GJK) computeCollisionInformation(&A, &B, &s, &dist, nrm);
    o->dist = dist;
    for (int w = 0; w < 2; ++w)
      for (int c = 0; c < 3; ++c) o->wit[w][c] = s.witnesses[w][c];
    for (int c = 0; c < 3; ++c) o->normal[c] = nrm[c];
    for (int k = 0; k < 4; ++k) {
      for (int c = 0; c < 3; ++c) o->vrtx[k][c] = s.vrtx[k][c];
      o->idx[k][0] = s.vrtx_idx[k][0];
      o->idx[k][1] = s.vrtx_idx[k][1];
    }
    o->nvrtx = s.nvrtx;
    o->gjk_iters = -1;
    o->epa_iters = -1;
    o->epa_exit = -1;
  }
  return 0;
}
