// ogx_common.cuh -- shared definitions of the batched GJK/EPA engine.
//
// Everything in the per-pair algorithm is written once as __host__ __device__ code over
// a "team" of L lanes (SPMD: every lane of the team runs the same code and holds the
// same per-pair state; lanes only split the vertex scans and the EPA face loops).
// On the GPU a team is L lanes of one warp (L = 4, 8, 16 or 32).  The host build
// (SerialTeam, L = 1) exists so that the algorithm can be checked on a CPU-only
// machine; it is compiled into a separate test library, never into the product.
//
// Arithmetic is compiled without contraction on both sides (nvcc --fmad=false,
// g++ -ffp-contract=off); where a fused multiply-add is wanted it is written as
// fmaf() explicitly, so the host build and the device build round identically.
#pragma once

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "ogx.h"

#if defined(__CUDACC__)
#define OGX_HD __host__ __device__ __forceinline__
#define OGX_D __device__ __forceinline__
// a rarely taken path kept out of line, so that its registers do not weigh on the loop
// that calls it
#define OGX_COLD __host__ __device__ __noinline__
#else
#define OGX_HD inline
#define OGX_COLD inline
#endif

#if !defined(__CUDACC__)
// the CUDA vector types the algorithm uses, for the host build
struct float4 {
  float x, y, z, w;
};
struct double4 {
  double x, y, z, w;
};
struct int2 {
  int x, y;
};
#endif

namespace ogx {

OGX_HD float4 make_float4_(float x, float y, float z, float w) {
  float4 r;
  r.x = x;
  r.y = y;
  r.z = z;
  r.w = w;
  return r;
}
OGX_HD double4 make_double4_(double x, double y, double z, double w) {
  double4 r;
  r.x = x;
  r.y = y;
  r.z = z;
  r.w = w;
  return r;
}
OGX_HD int2 make_int2_(int x, int y) {
  int2 r;
  r.x = x;
  r.y = y;
  return r;
}

// ----------------------------------------------------------------------------------
// small vectors

struct f3 {
  float x, y, z;
};
struct d3 {
  double x, y, z;
};

template <class T>
struct vec3 {
  T x, y, z;
};

template <class T>
OGX_HD vec3<T> v3(T x, T y, T z) {
  vec3<T> r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
template <class T>
OGX_HD vec3<T> operator-(vec3<T> a, vec3<T> b) {
  return v3<T>(a.x - b.x, a.y - b.y, a.z - b.z);
}
template <class T>
OGX_HD vec3<T> operator+(vec3<T> a, vec3<T> b) {
  return v3<T>(a.x + b.x, a.y + b.y, a.z + b.z);
}
template <class T>
OGX_HD vec3<T> operator-(vec3<T> a) {
  return v3<T>(-a.x, -a.y, -a.z);
}
template <class T>
OGX_HD vec3<T> operator*(vec3<T> a, T s) {
  return v3<T>(a.x * s, a.y * s, a.z * s);
}
template <class T>
OGX_HD T dot(vec3<T> a, vec3<T> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class T>
OGX_HD vec3<T> cross(vec3<T> a, vec3<T> b) {
  return v3<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T>
OGX_HD T l1(vec3<T> a) {
  return fabs(a.x) + fabs(a.y) + fabs(a.z);
}
OGX_HD float l1(vec3<float> a) { return fabsf(a.x) + fabsf(a.y) + fabsf(a.z); }

template <class T, class U>
OGX_HD vec3<T> cvt(vec3<U> a) {
  return v3<T>((T)a.x, (T)a.y, (T)a.z);
}

typedef vec3<float> fv3;
typedef vec3<double> dv3;

// ----------------------------------------------------------------------------------
// Double-float arithmetic: a value is the unevaluated sum hi + lo of two floats with
// |lo| <= ulp(hi) / 2, about 48 significant bits.  It runs on the FP32 pipes, which issue
// 64 times faster than FP64 on this part.  Error-free transformations: TwoSum (Knuth,
// TAOCP vol. 2, 4.2.2), Fast2Sum and TwoProduct (Dekker, 1971, here with a fused
// multiply-add); addition, multiplication and division as in the double-double
// arithmetic of Hida, Li and Bailey (2001) with float parts.  Every step is an IEEE float
// operation (no contraction), so host and device give the same bits.
struct df {
  float hi, lo;
  df() = default;
  OGX_HD explicit df(int i) : hi((float)i), lo(0.0f) {}
  OGX_HD explicit df(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};
OGX_HD df mk_df(float h, float l) {
  df r;
  r.hi = h;
  r.lo = l;
  return r;
}
OGX_HD df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return mk_df(s, (a - (s - bb)) + (b - bb));
}
OGX_HD df fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = a + b;
  return mk_df(s, b - (s - a));
}
OGX_HD df two_prod(float a, float b) {
  const float p = a * b;
  return mk_df(p, fmaf(a, b, -p));
}
OGX_HD df operator+(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  const df t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}
OGX_HD df operator-(df a) { return mk_df(-a.hi, -a.lo); }
OGX_HD df fabs(df a) { return a.hi < 0.0f ? mk_df(-a.hi, -a.lo) : a; }
OGX_HD df operator-(df a, df b) { return a + (-b); }
OGX_HD df operator*(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return fast_two_sum(p.hi, p.lo);
}
OGX_HD df operator/(df a, df b) {
  const float q1 = a.hi / b.hi;
  df r = a - b * mk_df(q1, 0.0f);
  const float q2 = r.hi / b.hi;
  r = r - b * mk_df(q2, 0.0f);
  const float q3 = r.hi / b.hi;
  return fast_two_sum(q1, q2) + mk_df(q3, 0.0f);
}
// square root: one Newton step from the float root (Karp and Markstein's form)
OGX_HD df df_sqrt(df a) {
  if (!(a.hi > 0.0f)) return mk_df(0.0f, 0.0f);
  const float x = sqrtf(a.hi);
  const df r = a - two_prod(x, x);
  return fast_two_sum(x, r.hi / (2.0f * x));
}
OGX_HD bool operator<(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
OGX_HD bool operator>(df a, df b) { return b < a; }
OGX_HD bool operator<=(df a, df b) { return !(b < a); }
OGX_HD bool operator>=(df a, df b) { return !(a < b); }
OGX_HD bool operator==(df a, df b) { return a.hi == b.hi && a.lo == b.lo; }
OGX_HD df& operator+=(df& a, df b) { return a = a + b; }
template <class T>
OGX_HD T tmin(T a, T b) { return b < a ? b : a; }
template <class T>
OGX_HD T tmax(T a, T b) { return a < b ? b : a; }
OGX_HD double tsqrt(double a) { return sqrt(a); }
OGX_HD df tsqrt(df a) { return df_sqrt(a); }
// unit roundoff-based floor factor of the arithmetic (2^-52 for double, 2^-47 for df)
template <class T>
OGX_HD double prec_eps();
template <>
OGX_HD double prec_eps<double>() { return DBL_EPSILON; }
template <>
OGX_HD double prec_eps<df>() { return 7.105427357601002e-15; }
OGX_HD float to_float(df a) { return a.hi + a.lo; }
OGX_HD float to_float(double a) { return (float)a; }
// scalar constants and conversions for code written once for double and df
template <class T>
OGX_HD T sc(float x);
template <>
OGX_HD double sc<double>(float x) { return (double)x; }
template <>
OGX_HD df sc<df>(float x) { return mk_df(x, 0.0f); }
typedef vec3<df> xv3;
// exact difference of two float points as double-float components
OGX_HD xv3 xdiff(fv3 a, fv3 b) { return v3<df>(two_sum(a.x, -b.x), two_sum(a.y, -b.y), two_sum(a.z, -b.z)); }

// Support-scan dot product.  Written with explicit fused multiply-adds so that the
// value of a vertex is the same wherever it is evaluated (scan, previous support).
OGX_HD float sdot(float x, float y, float z, fv3 d) { return fmaf(z, d.z, fmaf(y, d.y, x * d.x)); }
OGX_HD float sdot(fv3 p, fv3 d) { return sdot(p.x, p.y, p.z, d); }

// ----------------------------------------------------------------------------------
// run-time configuration and per-pair status

// Tolerances of one engine instance: the public ogx_config (include/ogx.h).
typedef ::ogx_config Config;

enum {
  OGX_F_FP64_ESCALATE = OGX_FLAG_FP64_ESCALATE,  // near-degenerate steps re-run in FP64
  OGX_F_FP64_POLISH = OGX_FLAG_FP64_POLISH,      // final simplex / face re-solved in FP64
  OGX_F_REFERENCE_TOL = OGX_FLAG_REFERENCE_TOL,  // reference termination rules
  OGX_F_EPA_FP64_PLANES = OGX_FLAG_EPA_FP64_PLANES,  // every EPA face plane from FP64
};

// Per-pair status bits written beside the results.
enum {
  OGX_S_GJK_CAP = OGX_PAIR_GJK_CAP,
  OGX_S_GJK_ESCALATED = OGX_PAIR_GJK_ESCALATED,
  OGX_S_POLISHED = OGX_PAIR_POLISHED,
  OGX_S_EPA_RUN = OGX_PAIR_EPA_RUN,
  OGX_S_EPA_CONVERGED = OGX_PAIR_EPA_CONVERGED,
  OGX_S_EPA_DUPLICATE = OGX_PAIR_EPA_DUPLICATE,
  OGX_S_EPA_CAP = OGX_PAIR_EPA_CAP,
  OGX_S_EPA_TOUCH = OGX_PAIR_EPA_TOUCH,
  OGX_S_EPA_TOPOLOGY = OGX_PAIR_EPA_TOPOLOGY,
  OGX_S_EPA_CAPACITY = OGX_PAIR_EPA_CAPACITY,
  OGX_S_EPA_ESCALATED = OGX_PAIR_EPA_ESCALATED,
  OGX_S_EPA_CERTIFIED = OGX_PAIR_EPA_CERTIFIED,
  OGX_S_BAD_INPUT = OGX_PAIR_BAD_INPUT,
};

OGX_HD Config default_config() {
  Config c;
  c.gjk_eps_rel = 1e-6f;
  c.gjk_eps_tot = 1e-24f;
  c.gjk_noise = 8.0f;
  c.gjk_max_iter = 32;
  c.epa_tol = 1e-6f;
  c.epa_rel = 2e-6f;
  c.epa_vis = 1e-6f;
  c.epa_max_iter = 64;
  c.flags = OGX_F_FP64_ESCALATE | OGX_F_FP64_POLISH;
  c.polish_rel = 2e-6f;
  return c;
}

// The reference's FP32 constants (GJK/cpu/openGJK.c:41-42,955; GJK/cpu/EPA.c:46,592).
OGX_HD Config reference_config() {
  Config c = default_config();
  c.gjk_eps_rel = FLT_EPSILON * 1e4f;
  c.gjk_eps_tot = FLT_EPSILON * 1e2f;
  c.gjk_noise = 0.0f;
  c.gjk_max_iter = 25;
  c.epa_tol = FLT_EPSILON * 1e2f;
  c.epa_rel = 0.0f;
  c.epa_vis = 0.0f;
  c.epa_max_iter = 64;
  c.flags = OGX_F_REFERENCE_TOL;
  c.polish_rel = 0.0f;
  return c;
}

OGX_HD int popc32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __popc(x);
#else
  return __builtin_popcount(x);
#endif
}

// EPA capacities.  With at most 64 expansions the polytope has at most 68 vertices and
// (Euler, closed triangulated surface) 2*68-4 = 132 faces.
constexpr int kEpaVmax = 68;
constexpr int kEpaFmax = 132;

// ----------------------------------------------------------------------------------
// teams

// Host team of one lane (test build).
struct SerialTeam {
  static constexpr int L = 1;
  OGX_HD int lane() const { return 0; }
  OGX_HD void argmax(float&, int&) const {}
  OGX_HD void argmin(float&, int&) const {}
  OGX_HD void argmax2(float&, int&, float&) const {}
  OGX_HD void argmax_d(double&, int&) const {}
  template <class T>
  OGX_HD void argmax_t(T&, int&) const {}
  OGX_HD bool any(bool p) const { return p; }
  OGX_HD uint32_t ballot(bool p) const { return p ? 1u : 0u; }
  OGX_HD uint32_t below() const { return 0u; }
  OGX_HD int excl_scan(int x, int& total) const {
    total = x;
    return 0;
  }
  OGX_HD int imax(int x) const { return x; }
  OGX_HD float fmax_(float x) const { return x; }
  OGX_HD void sync() const {}
};

#if defined(__CUDACC__)
// L consecutive lanes of a warp (L a power of two <= 32).
template <int L_>
struct WarpTeam {
  static constexpr int L = L_;
  unsigned mask;
  int ln;
  __device__ WarpTeam() {
    const int wl = threadIdx.x & 31;
    ln = wl & (L - 1);
    mask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << (wl & ~(L - 1)));
  }
  __device__ int lane() const { return ln; }
  // max value, ties to the smaller index
  __device__ void argmax(float& v, int& i) const {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
      const float v2 = __shfl_xor_sync(mask, v, o);
      const int i2 = __shfl_xor_sync(mask, i, o);
      if (v2 > v || (v2 == v && i2 < i)) {
        v = v2;
        i = i2;
      }
    }
  }
  // FP64 max value, ties to the smaller index
  __device__ void argmax_d(double& v, int& i) const {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
      const double v2 = __shfl_xor_sync(mask, v, o);
      const int i2 = __shfl_xor_sync(mask, i, o);
      if (v2 > v || (v2 == v && i2 < i)) {
        v = v2;
        i = i2;
      }
    }
  }
  __device__ void argmax_t(double& v, int& i) const { argmax_d(v, i); }
  __device__ void argmax_t(df& v, int& i) const {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
      const df v2 = mk_df(__shfl_xor_sync(mask, v.hi, o), __shfl_xor_sync(mask, v.lo, o));
      const int i2 = __shfl_xor_sync(mask, i, o);
      if (v2 > v || (v2 == v && i2 < i)) {
        v = v2;
        i = i2;
      }
    }
  }
  // best value / index (ties to the smaller index) and the runner-up value over lanes
  __device__ void argmax2(float& b1, int& i1, float& b2) const {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
      const float c1 = __shfl_xor_sync(mask, b1, o);
      const int j1 = __shfl_xor_sync(mask, i1, o);
      const float c2 = __shfl_xor_sync(mask, b2, o);
      const float lo = fminf(b1, c1);
      if (c1 > b1 || (c1 == b1 && j1 < i1)) {
        b1 = c1;
        i1 = j1;
      }
      b2 = fmaxf(fmaxf(b2, c2), lo);
    }
  }
  // min value, ties to the smaller index (index -1 means "none" and loses)
  __device__ void argmin(float& v, int& i) const {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
      const float v2 = __shfl_xor_sync(mask, v, o);
      const int i2 = __shfl_xor_sync(mask, i, o);
      const bool take = (i < 0) ? (i2 >= 0) : (i2 >= 0 && (v2 < v || (v2 == v && i2 < i)));
      if (take) {
        v = v2;
        i = i2;
      }
    }
  }
  __device__ bool any(bool p) const { return (__ballot_sync(mask, p) & mask) != 0u; }
  // bit l = predicate of team lane l
  __device__ uint32_t ballot(bool p) const {
    const uint32_t b = __ballot_sync(mask, p);
    return L == 32 ? b : (b >> ((threadIdx.x & 31) & ~(L - 1))) & ((1u << L) - 1u);
  }
  // team lanes below this one
  __device__ uint32_t below() const { return (1u << ln) - 1u; }
  __device__ int excl_scan(int x, int& total) const {
    int inc = x;
#pragma unroll
    for (int o = 1; o < L; o <<= 1) {
      const int y = __shfl_up_sync(mask, inc, o, L);
      if (ln >= o) inc += y;
    }
    total = __shfl_sync(mask, inc, L - 1, L);
    return inc - x;
  }
  __device__ int imax(int x) const {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(mask, x, o));
    return x;
  }
  __device__ float fmax_(float x) const {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(mask, x, o));
    return x;
  }
  __device__ void sync() const { __syncwarp(mask); }
};
#endif

// ----------------------------------------------------------------------------------
// pool layout
//
// Body b occupies 3 * n4 floats starting at float offset 4 * quad[b] of the pool:
// x[0..n4), y[0..n4), z[0..n4), n4 = n rounded up to a multiple of 4.  The padding
// points repeat point 0, so they never win a support scan (ties go to the lower index).
struct BodyRef {
  uint32_t quad;  // offset of x[0] in float4 units
  int32_t n;      // number of points
};

OGX_HD int round4(int n) { return (n + 3) & ~3; }

// A body whose points hold a NaN or an infinity is marked in the device body table by a
// negated point count (set by the packing kernels); its layout is still that of |n|
// points.  Kernels that lay out or copy a body use body_points(); the binning sees n < 1
// and reports the body's pairs as bad input, so no query kernel ever reads it.
OGX_HD int body_points(BodyRef r) { return r.n < 0 ? -r.n : r.n; }

OGX_HD bool is_finite(float x) {
  uint32_t u;
  memcpy(&u, &x, sizeof u);
  return (u & 0x7f800000u) != 0x7f800000u;
}

}  // namespace ogx
