// examples/gpu/example.h for callers written against OpenGJK-GPU: the GJK::GPU facade
// (examples/gpu/example.h:9-96) from the engine's drop-in header, plus the facade's two
// driver functions, testing() and EPATesting(), written on the drop-in calls.
#pragma once

#include <math.h>
#include <stdio.h>

#include <random>
#include <vector>

#include "GJK/gpu/openGJK.h"

namespace GJK {
namespace GPU {
namespace detail {

// points on a sphere shell of radius U[1, 1.5] around an offset in [-5, 5]^3: the shape
// of the reference's benchmark sweep
inline void shell_points(std::mt19937& g, int n, std::vector<gkFloat>& out) {
  std::uniform_real_distribution<double> u(-1.0, 1.0), r(1.0, 1.5), c(-5.0, 5.0);
  const double cx = c(g), cy = c(g), cz = c(g);
  out.resize(3 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    double x, y, z, l;
    do {
      x = u(g);
      y = u(g);
      z = u(g);
      l = sqrt(x * x + y * y + z * z);
    } while (l < 1e-3 || l > 1.0);
    const double s = r(g) / l;
    out[3 * i] = (gkFloat)(cx + s * x);
    out[3 * i + 1] = (gkFloat)(cy + s * y);
    out[3 * i + 2] = (gkFloat)(cz + s * z);
  }
}

inline std::vector<gkFloat> cube(double half, double dx) {
  std::vector<gkFloat> p;
  for (int k = 0; k < 8; ++k) {
    p.push_back((gkFloat)((k & 1 ? half : -half) + dx));
    p.push_back((gkFloat)(k & 2 ? half : -half));
    p.push_back((gkFloat)(k & 4 ? half : -half));
  }
  return p;
}

inline gkPolytope polytope(std::vector<gkFloat>& pts) {
  gkPolytope p;
  p.numpoints = (int)(pts.size() / 3);
  p.s[0] = p.s[1] = p.s[2] = 0;
  p.s_idx = 0;
  p.coord = pts.data();
  return p;
}

}  // namespace detail

// GPU time of computeDistances over random sphere-shell polytope pairs for every
// (pair count, vertex count) combination, the mean of 10 runs, as CSV rows
// "NumPolytopes,NumVertices,CPU_Time_ms,GPU_Time_ms" (examples/gpu/example.h:70-85).  The
// drop-in has no CPU path of its own, so the CPU column is written as nan.
inline void testing(const int* numPolytopesArray, const int numPolytopesArraySize, const int* numVerticesArray,
                    const int numVerticesArraySize, const char* outputFile) {
  if (!numPolytopesArray || !numVerticesArray || !outputFile) {
    fprintf(stderr, "ERROR: Invalid parameters to testing function\n");
    return;
  }
  FILE* fp = fopen(outputFile, "w");
  if (!fp) {
    fprintf(stderr, "ERROR: Could not open output file %s for writing\n", outputFile);
    return;
  }
  fprintf(fp, "NumPolytopes,NumVertices,CPU_Time_ms,GPU_Time_ms\n");
  std::mt19937 g(12345);
  for (int a = 0; a < numPolytopesArraySize; ++a)
    for (int b = 0; b < numVerticesArraySize; ++b) {
      const int np = numPolytopesArray[a], nv = numVerticesArray[b];
      std::vector<std::vector<gkFloat>> pts(2 * (size_t)np);
      std::vector<gkPolytope> p1(np), p2(np);
      for (int i = 0; i < np; ++i) {
        detail::shell_points(g, nv, pts[2 * i]);
        detail::shell_points(g, nv, pts[2 * i + 1]);
        p1[i] = detail::polytope(pts[2 * i]);
        p2[i] = detail::polytope(pts[2 * i + 1]);
      }
      std::vector<gkSimplex> smp(np);
      std::vector<gkFloat> dist(np);
      float sum = 0.0f;
      for (int run = 0; run < 10; ++run) {
        computeDistances(np, p1.data(), p2.data(), smp.data(), dist.data());
        sum += timer().getGpuElapsedTimeForPreviousOperation();
      }
      fprintf(fp, "%d,%d,nan,%.6f\n", np, nv, sum / 10.0f);
    }
  fclose(fp);
}

// Known-answer checks of GJK + EPA, printed PASS/FAIL (examples/gpu/example.h:87-92):
// unit cubes overlapping by 1 (depth 1 along x), touching cubes (depth 0), cubes 3 apart
// (distance 3, no EPA), and 1000-point spheres of radius 2 centred 1 apart (depth 3).
inline void EPATesting() {
  struct Case {
    const char* name;
    std::vector<gkFloat> a, b;
    double lo, hi;  // expected range of the returned distance (-depth for contacts)
  };
  std::vector<Case> cases;
  cases.push_back({"overlapping unit cubes, offset 1", detail::cube(1.0, 0.0), detail::cube(1.0, 1.0), -1.2, -0.8});
  cases.push_back({"touching cubes", detail::cube(1.0, 0.0), detail::cube(1.0, 2.0), -0.01, 0.01});
  cases.push_back({"cubes 3 apart", detail::cube(1.0, 0.0), detail::cube(1.0, 5.0), 2.9, 3.1});
  {
    std::mt19937 g(7);
    std::normal_distribution<double> n(0.0, 1.0);
    Case c{"spheres of 1000 points, radius 2, centres 1 apart", {}, {}, -3.1, -2.9};
    for (int k = 0; k < 2; ++k) {
      std::vector<gkFloat>& p = k ? c.b : c.a;
      for (int i = 0; i < 1000; ++i) {
        double x = n(g), y = n(g), z = n(g);
        const double l = sqrt(x * x + y * y + z * z);
        p.push_back((gkFloat)(2.0 * x / l + k));
        p.push_back((gkFloat)(2.0 * y / l));
        p.push_back((gkFloat)(2.0 * z / l));
      }
    }
    cases.push_back(c);
  }
  int failed = 0;
  for (Case& c : cases) {
    gkPolytope p1 = detail::polytope(c.a), p2 = detail::polytope(c.b);
    gkSimplex s;
    gkFloat d, nrm[3];
    computeGJKAndEPA(1, &p1, &p2, &s, &d, nrm);
    const bool ok = d > c.lo && d < c.hi;
    failed += !ok;
    printf("%-52s distance %10.6f  normal (%.4f, %.4f, %.4f)  %s\n", c.name, (double)d, (double)nrm[0],
           (double)nrm[1], (double)nrm[2], ok ? "PASSED" : "FAILED");
  }
  printf("EPA tests: %d of %d passed\n", (int)cases.size() - failed, (int)cases.size());
}

}  // namespace GPU
}  // namespace GJK
