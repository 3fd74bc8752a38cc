// ogx_bodies.cuh -- where the two bodies of a pair are read from during the scans.
//
// Two sources implement the same interface:
//   MemBodies   -- every scan re-reads the body from memory (host test build, and the
//                  device path for bodies too large to keep in registers)
//   RegBodies   -- device only: each lane of the team keeps K float4 blocks of x, y and
//                  z of both bodies in registers for the whole GJK/EPA run, so the pool
//                  is read from HBM exactly once per pair.
// scan() returns the lane-local best (value, index) of <point, d>; the caller combines
// lanes with team.argmax (max value, ties to the smaller index).
#pragma once

#include "ogx_common.cuh"

namespace ogx {

// The support values of a block of 4 points (x, y, z planes) along d: sdot() of each
// point.  On the device two points at a time with the packed FP32 instructions of this
// architecture: a multiply and two fused multiply-adds round exactly as sdot()'s, in half
// the instructions.
OGX_HD void sdot4(const float4& x, const float4& y, const float4& z, fv3 d, float* v) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
  const float2 dx = make_float2(d.x, d.x), dy = make_float2(d.y, d.y), dz = make_float2(d.z, d.z);
  const float2 a = __ffma2_rn(make_float2(z.x, z.y), dz,
                              __ffma2_rn(make_float2(y.x, y.y), dy, __fmul2_rn(make_float2(x.x, x.y), dx)));
  const float2 b = __ffma2_rn(make_float2(z.z, z.w), dz,
                              __ffma2_rn(make_float2(y.z, y.w), dy, __fmul2_rn(make_float2(x.z, x.w), dx)));
  v[0] = a.x;
  v[1] = a.y;
  v[2] = b.x;
  v[3] = b.y;
#else
  v[0] = sdot(x.x, y.x, z.x, d);
  v[1] = sdot(x.y, y.y, z.y, d);
  v[2] = sdot(x.z, y.z, z.z, d);
  v[3] = sdot(x.w, y.w, z.w, d);
#endif
}

// Fold a block of 4 support values (indices i0..i0+3) into the running (best, bi), point
// by point in index order: a strictly greater value wins, so ties keep the lower index
// and NaN values never win.  Written as selects (no branch for lanes to diverge on).
OGX_HD void block_best(const float* v, int i0, float& best, int& bi) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const bool win = v[c] > best;
    best = win ? v[c] : best;
    bi = win ? i0 + c : bi;
  }
}

struct MemBodies {
  static constexpr bool kExact64 = false;  // dpoint() is the float point widened
  const float* base[2];  // x[0] of each body
  int n[2];
  int n4[2];

  OGX_HD void bind(const float* pool, BodyRef a, BodyRef b) {
    base[0] = pool + 4 * (size_t)a.quad;
    base[1] = pool + 4 * (size_t)b.quad;
    n[0] = a.n;
    n[1] = b.n;
    n4[0] = round4(a.n);
    n4[1] = round4(b.n);
  }
  OGX_HD fv3 point(int w, int i) const {
    const float* p = base[w];
    return v3<float>(p[i], p[n4[w] + i], p[2 * n4[w] + i]);
  }
  OGX_HD dv3 dpoint(int w, int i) const { return cvt<double>(point(w, i)); }
  OGX_HD const MemBodies& mem_view() const { return *this; }

  // lane-local best value over all points, best value over the points whose index is
  // not in ex[0..3) (the final simplex's points of this body), and max |coordinate|
  template <class Team>
  OGX_HD void scan_excl(const Team& t, int w, fv3 d, const int* ex, float& b1, float& bo,
                        float& amax) const {
    b1 = bo = -INFINITY;
    amax = 0.0f;
    const int nb = n4[w] >> 2;
    const float* X = base[w];
    const float* Y = X + n4[w];
    const float* Z = X + 2 * n4[w];
    for (int q = t.lane(); q < nb; q += Team::L) {
      for (int c = 0; c < 4; ++c) {
        const int i = 4 * q + c;
        if (i >= n[w]) break;
        const float v = sdot(X[i], Y[i], Z[i], d);
        b1 = fmaxf(b1, v);
        if (i != ex[0] && i != ex[1] && i != ex[2]) bo = fmaxf(bo, v);
        amax = fmaxf(amax, fmaxf(fabsf(X[i]), fmaxf(fabsf(Y[i]), fabsf(Z[i]))));
      }
    }
  }

  template <class Team>
  OGX_HD void scan(const Team& t, int w, fv3 d, float& best, int& bi) const {
    best = -INFINITY;
    bi = 0x7fffffff;
    const int nb = n4[w] >> 2;
    const float* X = base[w];
    const float* Y = X + n4[w];
    const float* Z = X + 2 * n4[w];
    int q = t.lane();
#if defined(__CUDA_ARCH__)
    // two blocks per step, both blocks' loads issued before either is compared (twice the
    // loads in flight); blocks are still compared in increasing index order
    const float4* X4 = reinterpret_cast<const float4*>(X);
    const float4* Y4 = reinterpret_cast<const float4*>(Y);
    const float4* Z4 = reinterpret_cast<const float4*>(Z);
    for (; q + Team::L < nb; q += 2 * Team::L) {
      const int q2 = q + Team::L;
      const float4 x = __ldg(X4 + q), y = __ldg(Y4 + q), z = __ldg(Z4 + q);
      const float4 x2 = __ldg(X4 + q2), y2 = __ldg(Y4 + q2), z2 = __ldg(Z4 + q2);
      float v[4], v2[4];
      sdot4(x, y, z, d, v);
      sdot4(x2, y2, z2, d, v2);
      block_best(v, 4 * q, best, bi);
      block_best(v2, 4 * q2, best, bi);
    }
#endif
    for (; q < nb; q += Team::L) {
#if defined(__CUDA_ARCH__)
      const float4 x = __ldg(reinterpret_cast<const float4*>(X) + q);
      const float4 y = __ldg(reinterpret_cast<const float4*>(Y) + q);
      const float4 z = __ldg(reinterpret_cast<const float4*>(Z) + q);
#else
      const float4 x = make_float4_(X[4 * q], X[4 * q + 1], X[4 * q + 2], X[4 * q + 3]);
      const float4 y = make_float4_(Y[4 * q], Y[4 * q + 1], Y[4 * q + 2], Y[4 * q + 3]);
      const float4 z = make_float4_(Z[4 * q], Z[4 * q + 1], Z[4 * q + 2], Z[4 * q + 3]);
#endif
      float v[4];
      sdot4(x, y, z, d, v);
      block_best(v, 4 * q, best, bi);
    }
  }
};

// Bodies given in double by the caller (the FP64 drop-in): the pool holds their points
// rounded to float, which the FP32 scans read; dpoint() reads the caller's double
// coordinates (xyz interleaved, point i of body w at aos[w] + 3 i), so the FP64 steps run
// on the exact inputs.
struct D64Bodies : MemBodies {
  static constexpr bool kExact64 = true;
  const double* aos[2];
  OGX_HD void bind64(const float* pool, BodyRef a, BodyRef b, const double* a64, const double* b64) {
    bind(pool, a, b);
    aos[0] = a64;
    aos[1] = b64;
  }
  OGX_HD dv3 dpoint(int w, int i) const { return v3<double>(aos[w][3 * i], aos[w][3 * i + 1], aos[w][3 * i + 2]); }
};

#if defined(__CUDACC__)
template <int L, int K>
struct RegBodies {
  static constexpr bool kExact64 = false;
  float4 x[2][K], y[2][K], z[2][K];
  MemBodies mem;  // for point() lookups by index

  __device__ void bind(const float* pool, BodyRef a, BodyRef b, int lane) {
    mem.bind(pool, a, b);
#pragma unroll
    for (int w = 0; w < 2; ++w) {
      const int nb = mem.n4[w] >> 2;
      const float4* X = reinterpret_cast<const float4*>(mem.base[w]);
#pragma unroll
      for (int j = 0; j < K; ++j) {
        const int q = lane + j * L;
        const int qq = q < nb ? q : 0;  // beyond the body: repeat block 0 (never wins)
        x[w][j] = __ldg(X + qq);
        y[w][j] = __ldg(X + nb + qq);
        z[w][j] = __ldg(X + 2 * nb + qq);
      }
    }
  }
  __device__ fv3 point(int w, int i) const { return mem.point(w, i); }
  __device__ dv3 dpoint(int w, int i) const { return mem.dpoint(w, i); }
  __device__ const MemBodies& mem_view() const { return mem; }

  template <class Team>
  __device__ void scan_excl(const Team& t, int w, fv3 d, const int* ex, float& b1, float& bo,
                            float& amax) const {
    b1 = bo = -INFINITY;
    amax = 0.0f;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const int q4 = 4 * (t.lane() + j * L);
      const float4 X = x[w][j], Y = y[w][j], Z = z[w][j];
      const float xs[4] = {X.x, X.y, X.z, X.w}, ys[4] = {Y.x, Y.y, Y.z, Y.w}, zs[4] = {Z.x, Z.y, Z.z, Z.w};
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int i = q4 + c;
        const bool live = i < mem.n[w];  // padding repeats point 0: skip it here
        const float v = live ? sdot(xs[c], ys[c], zs[c], d) : -INFINITY;
        b1 = fmaxf(b1, v);
        if (i != ex[0] && i != ex[1] && i != ex[2]) bo = fmaxf(bo, v);
        if (live) amax = fmaxf(amax, fmaxf(fabsf(xs[c]), fmaxf(fabsf(ys[c]), fabsf(zs[c]))));
      }
    }
  }

  template <class Team>
  __device__ void scan(const Team& t, int w, fv3 d, float& best, int& bi) const {
    best = -INFINITY;
    bi = 0x7fffffff;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      float v[4];
      sdot4(x[w][j], y[w][j], z[w][j], d, v);
      block_best(v, 4 * (t.lane() + j * L), best, bi);
    }
  }
};
#endif

}  // namespace ogx
