// API cross-consistency through the drop-in headers, in the manner of the reference's
// own driver checks (examples/main.cpp:378-644): the high-level, indexed, indexed-device
// and fused calls must agree on the same random pairs, and calls made from several host
// threads at once must give the single-thread results.  Prints one PASS / FAIL line per
// check and returns the number of failures.  Test program: built and run by
// tests/test_gpu_dropin.py.
#include <math.h>
#include <stdio.h>

#include <random>
#include <thread>
#include <vector>

#include "GJK/common.h"
#include "examples/gpu/example.h"

namespace {

int failures = 0;

void report(const char* name, bool ok, double err) {
  printf("%-44s %s  (max difference %.3g, GPU %.4f ms)\n", name, ok ? "PASS" : "FAIL", err,
         (double)GJK::GPU::timer().getGpuElapsedTimeForPreviousOperation());
  failures += !ok;
}

double max_abs(const std::vector<gkFloat>& a, const std::vector<gkFloat>& b) {
  double m = 0.0;
  for (size_t i = 0; i < a.size(); ++i) m = fmax(m, fabs((double)a[i] - (double)b[i]));
  return m;
}

double max_witness(const std::vector<gkSimplex>& a, const std::vector<gkSimplex>& b) {
  double m = 0.0;
  for (size_t i = 0; i < a.size(); ++i)
    for (int w = 0; w < 2; ++w)
      for (int c = 0; c < 3; ++c) m = fmax(m, fabs((double)a[i].witnesses[w][c] - (double)b[i].witnesses[w][c]));
  return m;
}

}  // namespace

int main() {
  const int n = 3000, nv = 60;
  // 2n random sphere-shell bodies; pair i is (2i, 2i+1), centres close enough that about
  // half the pairs overlap
  std::mt19937 g(2024);
  std::uniform_real_distribution<double> u(-1.0, 1.0), r(0.6, 1.2), c(-1.5, 1.5);
  std::vector<std::vector<gkFloat>> pts(2 * n);
  std::vector<gkPolytope> pool(2 * n);
  for (int b = 0; b < 2 * n; ++b) {
    const double cx = c(g), cy = c(g), cz = c(g);
    for (int i = 0; i < nv; ++i) {
      double x, y, z, l;
      do {
        x = u(g);
        y = u(g);
        z = u(g);
        l = sqrt(x * x + y * y + z * z);
      } while (l < 1e-3 || l > 1.0);
      const double s = r(g) / l;
      pts[b].push_back((gkFloat)(cx + s * x));
      pts[b].push_back((gkFloat)(cy + s * y));
      pts[b].push_back((gkFloat)(cz + s * z));
    }
    pool[b].numpoints = nv;
    pool[b].s[0] = pool[b].s[1] = pool[b].s[2] = 0;
    pool[b].s_idx = 0;
    pool[b].coord = pts[b].data();
  }
  std::vector<gkPolytope> bd1(n), bd2(n);
  std::vector<gkCollisionPair> pairs(n);
  for (int i = 0; i < n; ++i) {
    bd1[i] = pool[2 * i];
    bd2[i] = pool[2 * i + 1];
    pairs[i].idx1 = 2 * i;
    pairs[i].idx2 = 2 * i + 1;
  }
  const double tol = 1e-5;

  // reference results: GJK, and GJK + EPA fused
  std::vector<gkSimplex> s0(n), sf(n);
  std::vector<gkFloat> d0(n), df(n), nf(3 * n);
  GJK::GPU::computeDistances(n, bd1.data(), bd2.data(), s0.data(), d0.data());
  report("computeDistances", true, 0.0);
  GJK::GPU::computeGJKAndEPA(n, bd1.data(), bd2.data(), sf.data(), df.data(), nf.data());
  {
    double e = 0.0;
    int contacts = 0;
    for (int i = 0; i < n; ++i)
      if (d0[i] > 0) e = fmax(e, fabs((double)d0[i] - (double)df[i]));
      else ++contacts;
    printf("  (%d of %d pairs in contact)\n", contacts, n);
    report("computeGJKAndEPA: distances of separated pairs", e <= tol && contacts > n / 10 && contacts < n, e);
  }
  {
    std::vector<gkSimplex> s(n);
    std::vector<gkFloat> d(n);
    compute_minimum_distance_indexed(2 * n, n, pool.data(), pairs.data(), s.data(), d.data());
    const double e = max_abs(d, d0);
    report("compute_minimum_distance_indexed", e <= tol, e);
  }
#ifndef OGX_GKFLOAT_DOUBLE
  {
    // the indexed API with device buffers, as the reference's per-frame caller uses it
    gkPolytope* d_polytopes = nullptr;
    gkFloat *d_coords = nullptr, *d_distances = nullptr, *d_normals = nullptr;
    gkCollisionPair* d_pairs = nullptr;
    gkSimplex* d_simplices = nullptr;
    allocate_indexed_device(2 * n, n, pool.data(), &d_polytopes, &d_coords, &d_pairs, &d_simplices, &d_distances,
                            &d_normals);
    upload_pairs_device(n, pairs.data(), d_pairs);
    compute_minimum_distance_indexed_device(n, d_polytopes, d_pairs, d_simplices, d_distances);
    std::vector<gkSimplex> s(n);
    std::vector<gkFloat> d(n);
    copy_results_from_device(n, d_simplices, d_distances, s.data(), d.data());
    const double e = max_abs(d, d0);
    report("compute_minimum_distance_indexed_device", e <= tol, e);
    free_indexed_device(d_polytopes, d_coords, d_pairs, d_simplices, d_distances, d_normals);
  }
#endif
  {
    // GJK, then EPA on its simplices: the fused call's witnesses and normals
    std::vector<gkSimplex> s(n);
    std::vector<gkFloat> d(n), nrm(3 * n), w1(3 * n), w2(3 * n);
    GJK::GPU::computeDistances(n, bd1.data(), bd2.data(), s.data(), d.data());
    std::vector<gkSimplex> s2 = s;
    std::vector<gkFloat> d2 = d;
    GJK::GPU::computeEPA(n, bd1.data(), bd2.data(), s.data(), d.data(), nrm.data());
    double e = fmax(max_abs(d, df), max_witness(s, sf));
    report("computeDistances + computeEPA", e <= tol && max_abs(nrm, nf) <= tol, fmax(e, max_abs(nrm, nf)));
    GJK::GPU::computeCollisionInformation(n, bd1.data(), bd2.data(), s2.data(), d2.data(), w1.data(), w2.data());
    e = 0.0;
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k)
        e = fmax(e, fmax(fabs((double)w1[3 * i + k] - (double)sf[i].witnesses[0][k]),
                         fabs((double)w2[3 * i + k] - (double)sf[i].witnesses[1][k])));
    report("computeCollisionInformation (witnesses)", e <= tol, e);
  }
  {
    std::vector<gkSimplex> s(n);
    std::vector<gkFloat> d(n), nrm(3 * n);
    GJK::GPU::timer().startGpuTimer();
    compute_gjk_epa_indexed(2 * n, n, pool.data(), pairs.data(), s.data(), d.data(), nrm.data());
    GJK::GPU::timer().endGpuTimer();
    const double e = fmax(fmax(max_abs(d, df), max_witness(s, sf)), max_abs(nrm, nf));
    report("compute_gjk_epa_indexed", e <= tol && GJK::GPU::timer().getGpuElapsedTimeForPreviousOperation() > 0, e);
  }
  {
    std::vector<gkSimplex> s(n);
    std::vector<gkFloat> d(n), nrm(3 * n);
    compute_minimum_distance_indexed(2 * n, n, pool.data(), pairs.data(), s.data(), d.data());
    compute_epa_indexed(2 * n, n, pool.data(), pairs.data(), s.data(), d.data(), nrm.data());
    const double e = fmax(fmax(max_abs(d, df), max_witness(s, sf)), max_abs(nrm, nf));
    report("compute_epa_indexed", e <= tol, e);
  }
  {
    // four host threads calling at once: each call runs on an engine context of its own
    const int nt = 4;
    std::vector<std::vector<gkSimplex>> s(nt, std::vector<gkSimplex>(n));
    std::vector<std::vector<gkFloat>> d(nt, std::vector<gkFloat>(n)), nrm(nt, std::vector<gkFloat>(3 * n));
    std::vector<std::thread> th;
    for (int k = 0; k < nt; ++k)
      th.emplace_back([&, k] {
        for (int rep = 0; rep < 3; ++rep)
          GJK::GPU::computeGJKAndEPA(n, bd1.data(), bd2.data(), s[k].data(), d[k].data(), nrm[k].data());
      });
    for (auto& t : th) t.join();
    bool same = true;
    for (int k = 0; k < nt; ++k)
      for (int i = 0; i < n; ++i) {
        same = same && d[k][i] == df[i];
        for (int c = 0; c < 3; ++c) same = same && nrm[k][3 * i + c] == nf[3 * i + c];
      }
    report("computeGJKAndEPA from 4 threads at once", same, 0.0);
  }
  printf("%d failure(s)\n", failures);
  return failures;
}
