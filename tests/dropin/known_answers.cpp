// A caller of the reference's API, built against the drop-in headers exactly as it would
// be against OpenGJK-GPU (include "examples/gpu/example.h" and "GJK/common.h"; with
// include/compat first on the include path): the usage examples' two known answers
// (README.md:111-137) and the facade's EPA checks.  Body files hold "n" then n lines
// "x y z".  Test program: built and run by tests/test_gpu_dropin.py.
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "GJK/common.h"
#include "examples/gpu/example.h"

static std::vector<gkFloat> read_body(const char* path) {
  std::vector<gkFloat> p;
  FILE* f = fopen(path, "r");
  if (!f) {
    fprintf(stderr, "cannot open %s\n", path);
    exit(2);
  }
  int n = 0;
  if (fscanf(f, "%d", &n) != 1) exit(2);
  for (int i = 0; i < 3 * n; ++i) {
    double v;
    if (fscanf(f, "%lf", &v) != 1) exit(2);
    p.push_back((gkFloat)v);
  }
  fclose(f);
  return p;
}

static gkPolytope as_polytope(std::vector<gkFloat>& p) {
  gkPolytope b;
  b.numpoints = (int)(p.size() / 3);
  b.s[0] = b.s[1] = b.s[2] = 0;
  b.s_idx = 0;
  b.coord = p.data();
  return b;
}

int main(int argc, char** argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: %s P Q cube rotated_cube\n", argv[0]);
    return 2;
  }
  // GJK between the two bodies of the GJK usage example
  std::vector<gkFloat> P = read_body(argv[1]), Q = read_body(argv[2]);
  gkPolytope bd1 = as_polytope(P), bd2 = as_polytope(Q);
  gkSimplex s[1];
  gkFloat d[1];
  GJK::GPU::computeDistances(1, &bd1, &bd2, s, d);
  printf("Distance between bodies %f\n", (double)d[0]);
  printf("Witnesses: (%f, %f, %f) and (%f, %f, %f)\n", (double)s[0].witnesses[0][0], (double)s[0].witnesses[0][1],
         (double)s[0].witnesses[0][2], (double)s[0].witnesses[1][0], (double)s[0].witnesses[1][1],
         (double)s[0].witnesses[1][2]);
  if (!(GJK::GPU::timer().getGpuElapsedTimeForPreviousOperation() > 0.0f)) {
    printf("FAIL timer\n");
    return 1;
  }
  // GJK then EPA between a unit cube and the cube rotated 45 degrees about x, y and z
  std::vector<gkFloat> C = read_body(argv[3]), R = read_body(argv[4]);
  gkPolytope c1 = as_polytope(C), c2 = as_polytope(R);
  gkSimplex e[1];
  gkFloat de[1], nrm[3];
  GJK::GPU::computeDistances(1, &c1, &c2, e, de);
  GJK::GPU::computeEPA(1, &c1, &c2, e, de, nrm);
  printf("Penetration depth: %f\n", -(double)de[0]);
  printf("Witness point on cube 1: (%f, %f, %f)\n", (double)e[0].witnesses[0][0], (double)e[0].witnesses[0][1],
         (double)e[0].witnesses[0][2]);
  printf("Witness point on cube 2: (%f, %f, %f)\n", (double)e[0].witnesses[1][0], (double)e[0].witnesses[1][1],
         (double)e[0].witnesses[1][2]);
  printf("Contact normal (from cube 1 to cube 2): (%f, %f, %f)\n", (double)nrm[0], (double)nrm[1], (double)nrm[2]);
  GJK::GPU::EPATesting();
  return 0;
}
