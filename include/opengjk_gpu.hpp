// opengjk_gpu.hpp -- drop-in C++ names of OpenGJK-GPU's host API over the engine's C ABI.
//
// Code written against the reference includes "GJK/gpu/openGJK.h" and
// "examples/gpu/example.h"; including this header instead (and linking libogx.so)
// gives the same functions with the same arguments:
//   GJK::GPU::computeDistances / computeEPA / computeGJKAndEPA /
//   computeCollisionInformation (README form) / timer()
//   compute_minimum_distance(n, ...), computeCollisionInformation(n, ...),
//   compute_gjk_epa, the mid-level *_device_arrays / *_device functions and the
//   indexed API.
// Like the reference, these functions return void; a failure throws ogx::Error (the
// reference has no error reporting at all; silent failure is not reproduced).
//
// Precision: as the reference's USE_32BITS switch (GJK/common.h:44), gkFloat is float
// unless OGX_GKFLOAT_DOUBLE is defined before this header (include/compat/GJK/common.h
// defines it when USE_32BITS is not); then gkFloat is double, the types have the FP64
// layouts, and the host-buffer and indexed calls go to the *_f64 entry points.  The
// device-buffer (*_device) calls exist in the FP32 build only.
//
// A caller written against the reference keeps its includes: with include/compat and
// include on the include path, "GJK/common.h", "GJK/gpu/openGJK.h" and
// "examples/gpu/example.h" resolve to this header.
#pragma once

#include <chrono>
#include <stdexcept>
#include <string>

#include "ogx.h"

namespace ogx {
struct Error : std::runtime_error {
  ogx_status status;
  Error(ogx_status s, const char* what) : std::runtime_error(std::string(ogx_status_string(s)) + ": " + what), status(s) {}
};
inline void check(ogx_status s) {
  if (s != OGX_OK) throw Error(s, ogx_last_error());
}
}  // namespace ogx

// the C entry point of each call in the build's precision
#ifdef OGX_GKFLOAT_DOUBLE
#define OGX_PREC(name) name##_f64
#else
#define OGX_PREC(name) name
#endif

// ----- GJK/gpu/openGJK.h ---------------------------------------------------------------
inline void compute_minimum_distance(const int n, const gkPolytope* bd1, const gkPolytope* bd2,
                                     gkSimplex* simplices, gkFloat* distances) {
  ogx::check(OGX_PREC(ogx_compute_minimum_distance)(n, bd1, bd2, simplices, distances));
}
inline void computeCollisionInformation(const int n, const gkPolytope* bd1, const gkPolytope* bd2,
                                        gkSimplex* simplices, gkFloat* distances, gkFloat* contact_normals) {
  ogx::check(OGX_PREC(ogx_compute_collision_information)(n, bd1, bd2, simplices, distances, contact_normals));
}
inline void compute_gjk_epa(const int n, const gkPolytope* bd1, const gkPolytope* bd2, gkSimplex* simplices,
                            gkFloat* distances, gkFloat* contact_normals) {
  ogx::check(OGX_PREC(ogx_compute_gjk_epa)(n, bd1, bd2, simplices, distances, contact_normals));
}
#ifndef OGX_GKFLOAT_DOUBLE
inline void allocate_epa_device_arrays(const int n, gkFloat** d_witness1, gkFloat** d_witness2,
                                       gkFloat** d_contact_normals) {
  ogx::check(ogx_allocate_epa_device_arrays(n, d_witness1, d_witness2, d_contact_normals));
}
inline void copy_epa_results_from_device(const int n, const gkFloat* d_witness1, const gkFloat* d_witness2,
                                         const gkFloat* d_contact_normals, gkFloat* witness1, gkFloat* witness2,
                                         gkFloat* contact_normals) {
  ogx::check(ogx_copy_epa_results_from_device(n, d_witness1, d_witness2, d_contact_normals, witness1, witness2,
                                              contact_normals));
}
inline void free_epa_device_arrays(gkFloat* d_witness1, gkFloat* d_witness2, gkFloat* d_contact_normals) {
  ogx::check(ogx_free_epa_device_arrays(d_witness1, d_witness2, d_contact_normals));
}
inline void allocate_and_copy_device_arrays(const int n, const gkPolytope* bd1, const gkPolytope* bd2,
                                            gkPolytope** d_bd1, gkPolytope** d_bd2, gkFloat** d_coord1,
                                            gkFloat** d_coord2, gkSimplex** d_simplices, gkFloat** d_distances) {
  ogx::check(ogx_allocate_and_copy_device_arrays(n, bd1, bd2, d_bd1, d_bd2, d_coord1, d_coord2, d_simplices,
                                                 d_distances));
}
inline void compute_minimum_distance_device(const int n, const gkPolytope* d_bd1, const gkPolytope* d_bd2,
                                            gkSimplex* d_simplices, gkFloat* d_distances) {
  ogx::check(ogx_compute_minimum_distance_device(n, d_bd1, d_bd2, d_simplices, d_distances));
}
inline void compute_epa_device(const int n, const gkPolytope* d_bd1, const gkPolytope* d_bd2,
                               gkSimplex* d_simplices, gkFloat* d_distances, gkFloat* d_contact_normals) {
  ogx::check(ogx_compute_epa_device(n, d_bd1, d_bd2, d_simplices, d_distances, d_contact_normals));
}
inline void copy_results_from_device(const int n, const gkSimplex* d_simplices, const gkFloat* d_distances,
                                     gkSimplex* simplices, gkFloat* distances) {
  ogx::check(ogx_copy_results_from_device(n, d_simplices, d_distances, simplices, distances));
}
inline void free_device_arrays(gkPolytope* d_bd1, gkPolytope* d_bd2, gkFloat* d_coord1, gkFloat* d_coord2,
                               gkSimplex* d_simplices, gkFloat* d_distances) {
  ogx::check(ogx_free_device_arrays(d_bd1, d_bd2, d_coord1, d_coord2, d_simplices, d_distances));
}
inline void allocate_indexed_device(const int num_polytopes, const int max_pairs, const gkPolytope* polytopes,
                                    gkPolytope** d_polytopes, gkFloat** d_coords, gkCollisionPair** d_pairs,
                                    gkSimplex** d_simplices, gkFloat** d_distances, gkFloat** d_contact_normals) {
  ogx::check(ogx_allocate_indexed_device(num_polytopes, max_pairs, polytopes, d_polytopes, d_coords, d_pairs,
                                         d_simplices, d_distances, d_contact_normals));
}
inline void free_indexed_device(gkPolytope* d_polytopes, gkFloat* d_coords, gkCollisionPair* d_pairs,
                                gkSimplex* d_simplices, gkFloat* d_distances, gkFloat* d_contact_normals) {
  ogx::check(ogx_free_indexed_device(d_polytopes, d_coords, d_pairs, d_simplices, d_distances, d_contact_normals));
}
inline void upload_pairs_device(const int num_pairs, const gkCollisionPair* pairs, gkCollisionPair* d_pairs) {
  ogx::check(ogx_upload_pairs_device(num_pairs, pairs, d_pairs));
}
inline void compute_minimum_distance_indexed_device(const int num_pairs, const gkPolytope* d_polytopes,
                                                    const gkCollisionPair* d_pairs, gkSimplex* d_simplices,
                                                    gkFloat* d_distances) {
  ogx::check(ogx_compute_minimum_distance_indexed_device(num_pairs, d_polytopes, d_pairs, d_simplices, d_distances));
}
inline void compute_epa_indexed_device(const int num_pairs, const gkPolytope* d_polytopes,
                                       const gkCollisionPair* d_pairs, gkSimplex* d_simplices, gkFloat* d_distances,
                                       gkFloat* d_contact_normals) {
  ogx::check(ogx_compute_epa_indexed_device(num_pairs, d_polytopes, d_pairs, d_simplices, d_distances,
                                            d_contact_normals));
}
#endif  // !OGX_GKFLOAT_DOUBLE: device-buffer calls
inline void compute_minimum_distance_indexed(const int num_polytopes, const int num_pairs,
                                             const gkPolytope* polytopes, const gkCollisionPair* pairs,
                                             gkSimplex* simplices, gkFloat* distances) {
  ogx::check(OGX_PREC(ogx_compute_minimum_distance_indexed)(num_polytopes, num_pairs, polytopes, pairs, simplices,
                                                            distances));
}
inline void compute_epa_indexed(const int num_polytopes, const int num_pairs, const gkPolytope* polytopes,
                                const gkCollisionPair* pairs, gkSimplex* simplices, gkFloat* distances,
                                gkFloat* contact_normals) {
  ogx::check(OGX_PREC(ogx_compute_epa_indexed)(num_polytopes, num_pairs, polytopes, pairs, simplices, distances,
                                               contact_normals));
}
inline void compute_gjk_epa_indexed(const int num_polytopes, const int num_pairs, const gkPolytope* polytopes,
                                    const gkCollisionPair* pairs, gkSimplex* simplices, gkFloat* distances,
                                    gkFloat* contact_normals) {
  ogx::check(OGX_PREC(ogx_compute_gjk_epa_indexed)(num_polytopes, num_pairs, polytopes, pairs, simplices, distances,
                                                   contact_normals));
}

// ----- examples/gpu/example.h: GJK::GPU ------------------------------------------------
namespace GJK {
namespace GPU {
// The PerformanceTimer of examples/common/timer.h, as GJK::GPU::timer() returns it:
// after a GJK::GPU call, getGpuElapsedTimeForPreviousOperation() is the GPU time of
// that call's engine pipeline (CUDA events, as the reference times its kernels); a
// caller's own startGpuTimer() / endGpuTimer() pair around other calls (the reference's
// driver times its indexed calls so, examples/main.cpp:417-422) measures the host time
// between them, which covers the GPU work because every call returns complete; the CPU
// timer pair is the host clock.  One timer per process, like the reference's function-
// static singleton.
class PerformanceTimer {
 public:
  void startCpuTimer() { t_cpu_ = std::chrono::steady_clock::now(); }
  void endCpuTimer() { cpu_ms_ = ms_since(t_cpu_); }
  void startGpuTimer() { t_gpu_ = std::chrono::steady_clock::now(); }
  void endGpuTimer() { gpu_ms_ = ms_since(t_gpu_); }
  float getCpuElapsedTimeForPreviousOperation() const { return cpu_ms_; }
  float getGpuElapsedTimeForPreviousOperation() const { return gpu_ms_; }
  void record_last_call() { gpu_ms_ = ogx_compat_last_gpu_ms(); }

 private:
  static float ms_since(std::chrono::steady_clock::time_point t) {
    return std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t).count();
  }
  std::chrono::steady_clock::time_point t_cpu_{}, t_gpu_{};
  float cpu_ms_ = 0.0f, gpu_ms_ = 0.0f;
};
inline PerformanceTimer& timer() {
  static PerformanceTimer t;
  return t;
}
inline void computeDistances(const int n, const gkPolytope* bd1, const gkPolytope* bd2, gkSimplex* simplices,
                             gkFloat* distances) {
  ogx::check(OGX_PREC(ogx_compute_minimum_distance)(n, bd1, bd2, simplices, distances));
  timer().record_last_call();
}
inline void computeEPA(const int n, const gkPolytope* bd1, const gkPolytope* bd2, gkSimplex* simplices,
                       gkFloat* distances, gkFloat* contact_normals) {
  ogx::check(OGX_PREC(ogx_compute_collision_information)(n, bd1, bd2, simplices, distances, contact_normals));
  timer().record_last_call();
}
inline void computeGJKAndEPA(const int n, const gkPolytope* bd1, const gkPolytope* bd2, gkSimplex* simplices,
                             gkFloat* distances, gkFloat* contact_normals) {
  ogx::check(OGX_PREC(ogx_compute_gjk_epa)(n, bd1, bd2, simplices, distances, contact_normals));
  timer().record_last_call();
}
inline void computeCollisionInformation(const int n, const gkPolytope* bd1, const gkPolytope* bd2,
                                        gkSimplex* simplices, gkFloat* distances, gkFloat* witness1,
                                        gkFloat* witness2, gkFloat* contact_normals = nullptr) {
  ogx::check(OGX_PREC(ogx_compute_collision_information_witnesses)(n, bd1, bd2, simplices, distances, witness1,
                                                                   witness2, contact_normals));
  timer().record_last_call();
}
}  // namespace GPU
}  // namespace GJK
