// ogx_bodies.cuh -- where the two bodies of a pair are read from during the scans.
//
// Sources that implement the same interface (and give the same bits):
//   MemBodies     -- every scan re-reads the body from memory (host test build, and the
//                    device path for bodies too large to keep in registers)
//   WideMemBodies -- device only: MemBodies with more loads in flight per lane (GJK)
//   StagedBodies  -- device only: MemBodies with the blocks staged through shared
//                    memory by cp.async, D blocks per lane ahead of the scan
//   RegBodies     -- device only: each lane of the team keeps K float4 blocks of x, y
//                    and z of both bodies in registers for the whole GJK/EPA run, so the
//                    pool is read from HBM exactly once per pair.
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

#if defined(__CUDACC__)
// MemBodies whose scan keeps four blocks per lane in flight (12 float4 loads issued before
// any is compared), then two, then one; the blocks are compared in the same order, so the
// result is MemBodies::scan's.  The GJK kernels use it: their scans over bodies re-read
// from L1/L2 are bound by load latency (13% less time on bodies above 512 points), while
// the register-capped EPA kernels lose more to the registers it takes than they gain.
struct WideMemBodies : MemBodies {
  template <class Team>
  __device__ void scan(const Team& t, int w, fv3 d, float& best, int& bi) const {
    best = -INFINITY;
    bi = 0x7fffffff;
    const int nb = n4[w] >> 2;
    const float* X = base[w];
    const float* Y = X + n4[w];
    const float* Z = X + 2 * n4[w];
    int q = t.lane();
    // four, then two blocks per step, all their loads issued before any is compared
    // (more loads in flight); blocks are still compared in increasing index order
    const float4* X4 = reinterpret_cast<const float4*>(X);
    const float4* Y4 = reinterpret_cast<const float4*>(Y);
    const float4* Z4 = reinterpret_cast<const float4*>(Z);
    for (; q + 3 * Team::L < nb; q += 4 * Team::L) {
      float4 x[4], y[4], z[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        x[u] = __ldg(X4 + q + u * Team::L);
        y[u] = __ldg(Y4 + q + u * Team::L);
        z[u] = __ldg(Z4 + q + u * Team::L);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        float v[4];
        sdot4(x[u], y[u], z[u], d, v);
        block_best(v, 4 * (q + u * Team::L), best, bi);
      }
    }
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
    for (; q < nb; q += Team::L) {
      const float4 x = __ldg(X4 + q), y = __ldg(Y4 + q), z = __ldg(Z4 + q);
      float v[4];
      sdot4(x, y, z, d, v);
      block_best(v, 4 * q, best, bi);
    }
  }
};
#endif

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

// Rigid pose of a body: m[0..9) the rotation R row-major, m[9..12) the translation t.
// A posed point is R p + t in FP32, one fused multiply-add chain per coordinate: the
// serving loop's world copies and the fused-pose sources below evaluate exactly this, so
// both give the same world points bit for bit.
OGX_HD fv3 pose_point(const float* m, fv3 p) {
  return v3<float>(fmaf(m[2], p.z, fmaf(m[1], p.y, fmaf(m[0], p.x, m[9]))),
                   fmaf(m[5], p.z, fmaf(m[4], p.y, fmaf(m[3], p.x, m[10]))),
                   fmaf(m[8], p.z, fmaf(m[7], p.y, fmaf(m[6], p.x, m[11]))));
}
// R^T d: a world direction in the body's frame
OGX_HD fv3 pose_dir(const float* m, fv3 d) {
  return v3<float>(fmaf(m[6], d.z, fmaf(m[3], d.y, m[0] * d.x)),
                   fmaf(m[7], d.z, fmaf(m[4], d.y, m[1] * d.x)),
                   fmaf(m[8], d.z, fmaf(m[5], d.y, m[2] * d.x)));
}

// Bodies kept in their own frame with a pose each (the transform fused into the reads
// instead of a world copy of the pool).  point() is the posed point (pose_point), so every
// step that reads points by index -- simplex and polytope vertices, exact supports, the
// certification scans, the FP64 steps -- sees the world points of a world copy exactly.
// The support scans rotate the direction into the body frame once (pose_dir) and scan
// the body-frame points: the same argmax in exact arithmetic, with the FP32 ranking of
// near-ties free to differ from a scan of the world points; the best value is returned
// in world terms (plus <t, d>) for the callers' comparisons with world points.
template <class Base>
struct Posed : Base {
  const float* xf[2];
  OGX_HD void bind_posed(const float* pool, BodyRef a, BodyRef b, const float* xa, const float* xb) {
    Base::bind(pool, a, b);
    xf[0] = xa;
    xf[1] = xb;
  }
  OGX_HD fv3 point(int w, int i) const { return pose_point(xf[w], Base::point(w, i)); }
  OGX_HD dv3 dpoint(int w, int i) const { return cvt<double>(point(w, i)); }
  OGX_HD const Posed& mem_view() const { return *this; }

  template <class Team>
  OGX_HD void scan(const Team& t, int w, fv3 d, float& best, int& bi) const {
    Base::scan(t, w, pose_dir(xf[w], d), best, bi);
    const float* m = xf[w];
    best += fmaf(m[11], d.z, fmaf(m[10], d.y, m[9] * d.x));
  }
  // as MemBodies::scan_excl, on the posed points
  template <class Team>
  OGX_HD void scan_excl(const Team& t, int w, fv3 d, const int* ex, float& b1, float& bo,
                        float& amax) const {
    b1 = bo = -INFINITY;
    amax = 0.0f;
    for (int i = t.lane(); i < this->n[w]; i += Team::L) {
      const fv3 p = point(w, i);
      const float v = sdot(p.x, p.y, p.z, d);
      b1 = fmaxf(b1, v);
      if (i != ex[0] && i != ex[1] && i != ex[2]) bo = fmaxf(bo, v);
      amax = fmaxf(amax, fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))));
    }
  }
};

#if defined(__CUDACC__)
// 16-byte asynchronous copy from global to shared memory (cp.async, cached in L1), the
// commit of the copies issued since the last commit as one group, and the wait until at
// most N of this thread's groups are still in flight.  A thread waits only for its own
// copies, so these waits always end.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Threads per block of the bucket kernels; the stride between a thread's staging slots.
constexpr int kStageStride = 128;

// Bodies read from memory with the blocks staged through shared memory.  Each lane owns
// D + 1 slots of 3 float4 (the x, y, z planes of one 4-point block) in shared memory and
// keeps D of its blocks in flight with cp.async; a copy is issued into the slot read one
// block earlier, never into the one just read.  A lane scans blocks lane, lane + L, ...
// of body 0, then of body 1, then of body 0 again: the GJK and EPA loops scan the two
// bodies alternately, so the blocks a lane reads next are known whatever the direction,
// and the copies run ahead across scans (the first blocks of the next scan land while
// this one, and the step between the two, run).  The scan reads each block from shared
// memory and the copies keep no registers while in flight (the register-loaded scan has
// at most two blocks in flight per lane).  Results are those of MemBodies::scan: the
// same float4 blocks, the same instructions, the same fold.  A scan out of that order
// (never issued by the loops) drains the copies and restarts the stream at its body.
template <int L, int D>
struct StagedBodies : MemBodies {
  static constexpr int S = D + 1;  // slots
  float4* ring;        // this thread's slots: plane c of slot s at ring[(3 s + c) * kStageStride]
  int lane;
  int nk[2];           // blocks of body w this lane scans
  mutable int cw;      // body of the next scan the stream expects
  mutable int iw, ik;  // next block to issue: k-th block of body iw
  mutable int is, cs;  // slots of the next block to issue / to consume

  __device__ void bind(const float* pool, BodyRef a, BodyRef b, int ln, float4* slots) {
    cp_async_wait<0>();  // the previous pair's copies into these slots have landed
    MemBodies::bind(pool, a, b);
    ring = slots;
    lane = ln;
#pragma unroll
    for (int w = 0; w < 2; ++w) {
      const int nb = n4[w] >> 2;
      nk[w] = nb > lane ? (nb - lane + L - 1) / L : 0;
    }
    restart(0);
  }
  // issue the next block of the stream into slot `is` (an empty group when the lane has
  // no block at all), so that exactly D groups are in flight after each commit
  __device__ void issue() const {
    if (nk[0] + nk[1] > 0) {
      while (ik >= nk[iw]) {  // at most two turns: one body has a block
        iw ^= 1;
        ik = 0;
      }
      const float* X = base[iw] + 4 * (lane + ik * L);
      float4* s = ring + 3 * is * kStageStride;
      cp_async16(s, X);
      cp_async16(s + kStageStride, X + n4[iw]);
      cp_async16(s + 2 * kStageStride, X + 2 * n4[iw]);
      ++ik;
    }
    cp_async_commit();
    is = is + 1 == S ? 0 : is + 1;
  }
  __device__ void restart(int w) const {
    cp_async_wait<0>();
    cw = iw = w;
    ik = 0;
    is = cs = 0;
#pragma unroll
    for (int s = 0; s < D; ++s) issue();
  }

  template <class Team>
  __device__ void scan(const Team& t, int w, fv3 d, float& best, int& bi) const {
    best = -INFINITY;
    bi = 0x7fffffff;
    if (w != cw) restart(w);
    for (int k = 0; k < nk[w]; ++k) {
      cp_async_wait<D - 1>();  // the oldest of the D groups in flight: this block
      const float4* s = ring + 3 * cs * kStageStride;
      const float4 x = s[0], y = s[kStageStride], z = s[2 * kStageStride];
      float v[4];
      sdot4(x, y, z, d, v);
      block_best(v, 4 * (lane + k * L), best, bi);
      cs = cs + 1 == S ? 0 : cs + 1;
      issue();  // into the slot read one block earlier
    }
    cw = w ^ 1;
  }
};

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
