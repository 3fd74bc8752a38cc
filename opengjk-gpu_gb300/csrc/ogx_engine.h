// ogx_engine.h -- internal declarations shared by the engine's .cu files.
#pragma once

#include <cuda_runtime.h>
#include <stdarg.h>

#include <vector>

#include "ogx.h"
#include "ogx_kernels.cuh"

struct ogx_ctx {
  int device = 0;
  int sm_count = 0;
  ogx_config cfg;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // per-call work lists (grown on demand)
  int* d_lists = nullptr;
  int* d_elists = nullptr;
  int* d_counts = nullptr;
  ogx::PolishRec* d_polish = nullptr;
  ogx::RefineRec* d_refine = nullptr;
  int* d_refine_full = nullptr;
  int* d_spill = nullptr;
  ogx::EpaResume* d_resume = nullptr;  // kResumeCap saved expansions of capacity spills
  static constexpr int kResumeCap = 4096;
  size_t cap_pairs = 0;
  // staging for host uploads
  void* h_stage = nullptr;
  size_t h_stage_bytes = 0;
  void* d_stage = nullptr;
  size_t d_stage_bytes = 0;
  int last_launches = 0;
  int choice[2][ogx::kBuckets] = {};  // kernel variant per bucket: [0] GJK, [1] EPA
  // optional per-launch timing (CUDA events recorded between the launches of a call)
  bool timing = false;
  static constexpr int kMaxTimed = 32;
  cudaEvent_t ev[kMaxTimed + 1] = {};
  const char* ev_name[kMaxTimed] = {};
  int ev_count = 0;

  void mark(const char* name);  // record an event before the next launch
  // concurrent bucket launches: one stream per size bucket, fork / join events
  bool fork_ok = true;
  int fork_width = ogx::kBuckets;  // bucket streams when forked (2..kBuckets; fixed once created)
  cudaStream_t aux[ogx::kBuckets] = {};
  cudaEvent_t fork_ev = nullptr;
  cudaEvent_t join_ev[ogx::kBuckets] = {};
  cudaStream_t aux_r = nullptr;  // the FP64 refinement's second kernel, beside the EPA buckets
  cudaEvent_t route_ev = nullptr, rjoin_ev = nullptr;
  ogx_status ensure_aux();
  // streamed host-to-host calls: copy streams, events, device input/output buffers
  cudaStream_t up = nullptr, down = nullptr;
  std::vector<cudaEvent_t> sev;
  gkCollisionPair* d_io_pairs = nullptr;
  gkSimplex* d_io_smp = nullptr;
  float* d_io_dist = nullptr;
  float* d_io_nrm = nullptr;
  int32_t* d_io_status = nullptr;
  size_t io_cap = 0;
  std::vector<float> stream_timeline;  // last streamed call with timing on (see ogx.h)
  // stage timeline of forked calls (ogx_ctx_set_stage_timeline): events on the streams
  bool stages = false;
  static constexpr int kMaxStages = 40;
  cudaEvent_t stage_ev[kMaxStages + 1] = {};  // [0] the call's start
  const char* stage_name[kMaxStages] = {};
  int stage_count = 0;
  std::vector<ogx_ctx*> sub;           // streamed calls: contexts running chunks side by side

  ogx_status ensure_scratch(int npairs);
  ogx_status ensure_stage(size_t host_bytes, size_t dev_bytes);
  void free_scratch();
};

struct ogx_pool {
  ogx_ctx* ctx = nullptr;
  int nbodies = 0;
  int64_t npoints = 0;
  size_t nfloats = 0;
  float* d_points = nullptr;
  ogx::BodyRef* d_bodies = nullptr;
  int64_t* d_voff = nullptr;  // first point of each body in the AoS source
  std::vector<int64_t> h_voff;  // the same on the host (chunked uploads)
};

ogx_status ogx_fail(ogx_status s, const char* fmt, ...);
ogx_status ogx_cuda_fail(cudaError_t e, const char* what);
ogx_status pool_pack(ogx_ctx* ctx, const ogx_pool* p, const float* d_aos);
// bytes of a context's work lists per pair of capacity (ogx_ctx::ensure_scratch)
size_t ogx_scratch_bytes_per_pair();
// Does device dev read pageable host memory directly, through the host's page tables
// (cudaDevAttrPageableMemoryAccess and ...UsesHostPageTables: the GPU of a Grace system
// over NVLink-C2C)?  Queried once per device.
bool ogx_pageable_reads(int dev);
ogx_status ogx_run(ogx_ctx* ctx, const float* d_pool, const ogx::BodyRef* d_bodies, int nbodies,
                   int npairs, const gkCollisionPair* d_pairs, gkSimplex* d_smp, float* d_dist,
                   float* d_nrm, int32_t* d_status, int mode, const int2* d_warm = nullptr,
                   const float* d_xf = nullptr);
