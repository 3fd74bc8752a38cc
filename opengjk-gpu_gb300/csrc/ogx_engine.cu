// ogx_engine.cu -- engine half of the C ABI (include/ogx.h): contexts, the device-
// resident polytope pool, and the batched GJK / GJK+EPA / EPA pipelines.
//
// Pipeline of one batched call (all on the context's stream, no host synchronisation):
//   memset counters -> k_bin -> k_gjk x 7 buckets (largest first) -> k_epa x 7 ->
//   k_polish
// Grids are fixed per kernel (occupancy x SM count) and the kernels stride over
// device-side work lists, so a call is a fixed sequence of launches that can be
// captured in a CUDA graph by the caller.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cstdlib>
#include <atomic>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ogx_engine.h"

using namespace ogx;

// ---------------------------------------------------------------------------------
// errors

static thread_local std::string g_err;

ogx_status ogx_fail(ogx_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return s;
}

ogx_status ogx_cuda_fail(cudaError_t e, const char* what) {
  cudaGetLastError();  // clear a non-sticky error
  const ogx_status s = (e == cudaErrorMemoryAllocation) ? OGX_ERR_NOMEM : OGX_ERR_CUDA;
  return ogx_fail(s, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

extern "C" const char* ogx_last_error(void) { return g_err.c_str(); }

extern "C" const char* ogx_status_string(ogx_status s) {
  switch (s) {
    case OGX_OK: return "ok";
    case OGX_ERR_INVALID: return "invalid argument";
    case OGX_ERR_CUDA: return "CUDA error";
    case OGX_ERR_NOMEM: return "out of memory";
    case OGX_ERR_NO_DEVICE: return "no usable GPU";
    case OGX_ERR_CAPACITY: return "capacity exceeded";
    default: return "unknown status";
  }
}

extern "C" const char* ogx_version(void) { return "ogx 0.1 (sm_103a)"; }

extern "C" ogx_status ogx_config_default(ogx_config* cfg) {
  if (!cfg) return ogx_fail(OGX_ERR_INVALID, "cfg is NULL");
  *cfg = default_config();
  return OGX_OK;
}

extern "C" ogx_status ogx_config_reference(ogx_config* cfg) {
  if (!cfg) return ogx_fail(OGX_ERR_INVALID, "cfg is NULL");
  *cfg = reference_config();
  return OGX_OK;
}

static ogx_status check_config(const ogx_config& c) {
  if (!(c.gjk_max_iter >= 1 && c.gjk_max_iter <= 1000))
    return ogx_fail(OGX_ERR_INVALID, "gjk_max_iter must be in [1, 1000]");
  if (!(c.epa_max_iter >= 1 && c.epa_max_iter <= kEpaVmax - 4))
    return ogx_fail(OGX_ERR_INVALID, "epa_max_iter must be in [1, %d]", kEpaVmax - 4);
  if (!(c.gjk_eps_rel >= 0.f) || !(c.gjk_eps_tot >= 0.f) || !(c.epa_tol >= 0.f) ||
      !(c.epa_rel >= 0.f) || !(c.epa_vis >= 0.f) || !(c.gjk_noise >= 0.f) || !(c.polish_rel >= 0.f))
    return ogx_fail(OGX_ERR_INVALID, "tolerances must be >= 0");
  return OGX_OK;
}

// ---------------------------------------------------------------------------------
// kernel table

namespace {

struct Launch {
  BucketKernel fn;
  int L;
  int K;
  size_t smem;
  int grid;  // resident blocks x SMs on the current device
};

std::vector<Launch> g_gjkv, g_epav;  // all compiled variants
std::vector<Launch> g_gjkp, g_epap;  // the posed kernels, one per bucket

constexpr int kBlock = 128;
constexpr int kBucketCap[kBuckets] = {16, 32, 64, 128, 256, 512, 0};

std::mutex g_init_mu;
int g_init_device = -1;
int g_grid_bin = 0, g_grid_polish = 0, g_grid_pack = 0, g_grid_refine = 0, g_grid_spill = 0;
uint32_t* g_subtab = nullptr;  // sub-distance decision table on the initialised device
// per-device autotuned choices (variant index per bucket), -1 = not tuned
int g_tuned[16][2][kBuckets];
bool g_tuned_valid[16];

// Persistent grid of a launch over at most `units` work items of `lanes` lanes each: the
// full resident grid, or fewer blocks when the batch cannot fill it (small batches then
// schedule a few blocks instead of the whole GPU for every one of the call's kernels).
int fit_grid(int full, int units, int lanes) {
  const long long need = ((long long)units * lanes + kBlock - 1) / kBlock;
  return (int)std::max(1LL, std::min((long long)full, need));
}

// can variant v serve bucket b?
bool serves(const Launch& v, int b) {
  const int K = variant_blocks(v.K);
  if (K == 0) return v.L == 32 || b < kBuckets - 1 || v.L >= 8;  // memory-streamed: any size
  if (b == kBuckets - 1) return false;
  const int cap = 4 * v.L * K;
  return cap >= kBucketCap[b] && cap <= 8 * kBucketCap[b];
}

// Default choice before tuning: the variants the autotuner picks on this GPU for the
// 1M-pair power-law batch (the same per bucket across runs): (lanes, K code) per bucket,
// K code = register blocks + (resident blocks per SM << kOccShift).
constexpr int kDefaultGjk[kBuckets][2] = {{1, 4}, {1, 5 << kOccShift}, {2, 4 << kOccShift}, {2, 4 << kOccShift},
                                          {4, 4 << kOccShift}, {8, 4 << kOccShift}, {8, 4 << kOccShift}};
constexpr int kDefaultEpa[kBuckets][2] = {{8, 1 + (5 << kOccShift)}, {8, 1 + (5 << kOccShift)},
                                          {8, 2 + (5 << kOccShift)}, {8, 5 << kOccShift},
                                          {8, 5 << kOccShift},     {8, 5 << kOccShift},
                                          {16, 5 << kOccShift}};

// otherwise one pair per warp, fewest registers that fit
int default_choice(const std::vector<Launch>& vs, int b, bool epa) {
  const int* want = epa ? kDefaultEpa[b] : kDefaultGjk[b];
  for (int i = 0; i < (int)vs.size(); ++i)
    if (vs[i].L == want[0] && vs[i].K == want[1] && serves(vs[i], b)) return i;
  int best = -1;
  for (int i = 0; i < (int)vs.size(); ++i) {
    if (!serves(vs[i], b) || vs[i].L != 32) continue;
    if (b == kBuckets - 1) {
      if (vs[i].K == 0) return i;
      continue;
    }
    if (vs[i].K == 0) continue;
    if (best < 0 || vs[i].K < vs[best].K) best = i;
  }
  return best;
}

ogx_status init_variant(Launch* k, bool epa, int sms) {
  const size_t staging = staging_bytes(variant_stages(k->K));
  k->smem = epa ? (size_t)(kBlock / k->L) * epa_team_stride(k->L) + staging : staging;
  cudaError_t e;
  if (k->smem > 48 * 1024) {
    e = cudaFuncSetAttribute(reinterpret_cast<const void*>(k->fn), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)k->smem);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaFuncSetAttribute");
  }
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k->fn, kBlock, k->smem);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
  if (per_sm < 1) return ogx_fail(OGX_ERR_CUDA, "kernel variant (%d,%d) cannot be resident", k->L, k->K);
  k->grid = per_sm * sms;
  return OGX_OK;
}

ogx_status init_kernels(int device) {
  std::lock_guard<std::mutex> lk(g_init_mu);
  if (g_init_device == device) return OGX_OK;
  int sms = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaDeviceGetAttribute");
  g_gjkv.clear();
  g_epav.clear();
  const KernelInfo* t;
  int n = gjk_variants_a(&t);
  for (int i = 0; i < n; ++i) g_gjkv.push_back(Launch{t[i].fn, t[i].L, t[i].K, 0, 0});
  n = gjk_variants_b(&t);
  for (int i = 0; i < n; ++i) g_gjkv.push_back(Launch{t[i].fn, t[i].L, t[i].K, 0, 0});
  n = gjk_variants_c(&t);
  for (int i = 0; i < n; ++i) g_gjkv.push_back(Launch{t[i].fn, t[i].L, t[i].K, 0, 0});
  n = gjk_variants_d(&t);
  for (int i = 0; i < n; ++i) g_gjkv.push_back(Launch{t[i].fn, t[i].L, t[i].K, 0, 0});
  n = epa_variants_a(&t);
  for (int i = 0; i < n; ++i) g_epav.push_back(Launch{t[i].fn, t[i].L, t[i].K, 0, 0});
  n = epa_variants_b(&t);
  for (int i = 0; i < n; ++i) g_epav.push_back(Launch{t[i].fn, t[i].L, t[i].K, 0, 0});
  n = epa_variants_c(&t);
  for (int i = 0; i < n; ++i) g_epav.push_back(Launch{t[i].fn, t[i].L, t[i].K, 0, 0});
  n = gjk_variants_e(&t);
  for (int i = 0; i < n; ++i) g_gjkv.push_back(Launch{t[i].fn, t[i].L, t[i].K, 0, 0});
  n = epa_variants_d(&t);
  for (int i = 0; i < n; ++i) g_epav.push_back(Launch{t[i].fn, t[i].L, t[i].K, 0, 0});
  for (auto& k : g_gjkv) {
    ogx_status s = init_variant(&k, false, sms);
    if (s) return s;
  }
  for (auto& k : g_epav) {
    ogx_status s = init_variant(&k, true, sms);
    if (s) return s;
  }
  {
    const KernelInfo *pg, *pe;
    posed_variants(&pg, &pe);
    g_gjkp.clear();
    g_epap.clear();
    for (int b = 0; b < kBuckets; ++b) {
      g_gjkp.push_back(Launch{pg[b].fn, pg[b].L, pg[b].K, 0, 0});
      g_epap.push_back(Launch{pe[b].fn, pe[b].L, pe[b].K, 0, 0});
    }
    for (auto& k : g_gjkp) {
      ogx_status s = init_variant(&k, false, sms);
      if (s) return s;
    }
    for (auto& k : g_epap) {
      ogx_status s = init_variant(&k, true, sms);
      if (s) return s;
    }
  }
  g_grid_bin = 4 * sms;
  g_grid_pack = 8 * sms;
  int per_sm = 0;
  e = polish_occupancy(kBlock, &per_sm);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "occupancy(k_polish)");
  g_grid_polish = std::max(1, per_sm) * sms;
  e = epa_spill_occupancy(kBlock, &per_sm);
  if (e != cudaSuccess) return e;
  g_grid_spill = std::max(1, per_sm) * sms;
  e = refine_occupancy(kBlock, &per_sm);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "occupancy(k_refine)");
  g_grid_refine = std::max(1, per_sm) * sms;
  {
    std::vector<uint32_t> tab(kSubTabSize);
    fill_subtab(tab.data());
    if (g_subtab) cudaFree(g_subtab);
    g_subtab = nullptr;
    if ((e = cudaMalloc(&g_subtab, kSubTabSize * sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMemcpy(g_subtab, tab.data(), kSubTabSize * sizeof(uint32_t), cudaMemcpyHostToDevice)) != cudaSuccess)
      return ogx_cuda_fail(e, "decision table");
  }
  g_init_device = device;
  return OGX_OK;
}

void set_defaults(ogx_ctx* ctx) {
  const bool tuned = ctx->device < 16 && g_tuned_valid[ctx->device];
  for (int b = 0; b < kBuckets; ++b) {
    ctx->choice[0][b] = tuned ? g_tuned[ctx->device][0][b] : default_choice(g_gjkv, b, false);
    ctx->choice[1][b] = tuned ? g_tuned[ctx->device][1][b] : default_choice(g_epav, b, true);
  }
}

}  // namespace

// ---------------------------------------------------------------------------------
// context

extern "C" ogx_status ogx_ctx_create(int device, const ogx_config* cfg, void* stream,
                                     ogx_ctx** out) {
  if (!out) return ogx_fail(OGX_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return ogx_fail(OGX_ERR_NO_DEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
  }
  if (device < 0) {
    e = cudaGetDevice(&device);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaGetDevice");
  }
  if (device >= ndev) return ogx_fail(OGX_ERR_INVALID, "device %d of %d", device, ndev);
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
  if (major * 10 + minor != 103)
    return ogx_fail(OGX_ERR_NO_DEVICE, "device %d is sm_%d%d; the library is compiled for sm_103a only", device,
                    major, minor);
  ogx_config c = cfg ? *cfg : default_config();
  ogx_status s = check_config(c);
  if (s) return s;
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaSetDevice");
  s = init_kernels(device);
  if (s) return s;
  ogx_ctx* ctx = new ogx_ctx();
  ctx->device = device;
  ctx->cfg = c;
  set_defaults(ctx);
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (stream) {
    ctx->stream = static_cast<cudaStream_t>(stream);
    ctx->own_stream = false;
  } else {
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete ctx;
      return ogx_cuda_fail(e, "cudaStreamCreate");
    }
    ctx->own_stream = true;
  }
  *out = ctx;
  return OGX_OK;
}

void ogx_ctx::free_scratch() {
  cudaFree(d_lists);
  cudaFree(d_elists);
  cudaFree(d_polish);
  cudaFree(d_counts);
  cudaFree(d_refine);
  cudaFree(d_refine_full);
  cudaFree(d_spill);
  d_spill = nullptr;
  cudaFree(d_resume);
  d_resume = nullptr;
  d_refine = nullptr;
  d_refine_full = nullptr;
  d_lists = d_elists = d_counts = nullptr;
  d_polish = nullptr;
  cap_pairs = 0;
}

extern "C" ogx_status ogx_ctx_destroy(ogx_ctx* ctx) {
  if (!ctx) return OGX_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->free_scratch();
  for (int i = 0; i <= ogx_ctx::kMaxTimed; ++i)
    if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
  for (int i = 0; i <= ogx_ctx::kMaxStages; ++i)
    if (ctx->stage_ev[i]) cudaEventDestroy(ctx->stage_ev[i]);
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  if (ctx->d_stage) cudaFree(ctx->d_stage);
  if (ctx->up) {
    cudaStreamSynchronize(ctx->up);
    cudaStreamDestroy(ctx->up);
  }
  if (ctx->down) {
    cudaStreamSynchronize(ctx->down);
    cudaStreamDestroy(ctx->down);
  }
  for (cudaEvent_t e : ctx->sev) cudaEventDestroy(e);
  for (ogx_ctx* c : ctx->sub) ogx_ctx_destroy(c);
  for (int b = 0; b < kBuckets; ++b) {
    if (ctx->aux[b]) {
      cudaStreamSynchronize(ctx->aux[b]);
      cudaStreamDestroy(ctx->aux[b]);
    }
    if (ctx->join_ev[b]) cudaEventDestroy(ctx->join_ev[b]);
  }
  if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
  if (ctx->aux_r) {
    cudaStreamSynchronize(ctx->aux_r);
    cudaStreamDestroy(ctx->aux_r);
  }

  if (ctx->route_ev) cudaEventDestroy(ctx->route_ev);
  if (ctx->rjoin_ev) cudaEventDestroy(ctx->rjoin_ev);
  cudaFree(ctx->d_io_pairs);
  cudaFree(ctx->d_io_smp);
  cudaFree(ctx->d_io_dist);
  cudaFree(ctx->d_io_nrm);
  cudaFree(ctx->d_io_status);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return OGX_OK;
}

extern "C" ogx_status ogx_ctx_set_config(ogx_ctx* ctx, const ogx_config* cfg) {
  if (!ctx || !cfg) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  ogx_status s = check_config(*cfg);
  if (s) return s;
  ctx->cfg = *cfg;
  return OGX_OK;
}

extern "C" ogx_status ogx_ctx_get_config(const ogx_ctx* ctx, ogx_config* cfg) {
  if (!ctx || !cfg) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  *cfg = ctx->cfg;
  return OGX_OK;
}

extern "C" ogx_status ogx_ctx_set_stream(ogx_ctx* ctx, void* stream) {
  if (!ctx) return ogx_fail(OGX_ERR_INVALID, "ctx is NULL");
  if (ctx->own_stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    ctx->own_stream = false;
  }
  ctx->stream = static_cast<cudaStream_t>(stream);
  return OGX_OK;
}

extern "C" void* ogx_ctx_stream(const ogx_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

extern "C" ogx_status ogx_ctx_synchronize(ogx_ctx* ctx) {
  if (!ctx) return ogx_fail(OGX_ERR_INVALID, "ctx is NULL");
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaStreamSynchronize");
  return OGX_OK;
}

extern "C" int ogx_ctx_last_launches(const ogx_ctx* ctx) { return ctx ? ctx->last_launches : 0; }

void ogx_ctx::mark(const char* name) {
  if (!timing || ev_count >= kMaxTimed) return;
  cudaEventRecord(ev[ev_count], stream);
  ev_name[ev_count] = name;
  ++ev_count;
}

extern "C" ogx_status ogx_ctx_set_timing(ogx_ctx* ctx, int on) {
  if (!ctx) return ogx_fail(OGX_ERR_INVALID, "ctx is NULL");
  cudaSetDevice(ctx->device);
  if (on && !ctx->ev[0]) {
    for (int i = 0; i <= ogx_ctx::kMaxTimed; ++i) {
      cudaError_t e = cudaEventCreate(&ctx->ev[i]);
      if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaEventCreate");
    }
  }
  ctx->timing = on != 0;
  return OGX_OK;
}

extern "C" int ogx_ctx_kernel_times(ogx_ctx* ctx, const char** names, float* ms, int cap) {
  if (!ctx || !ctx->timing || ctx->ev_count == 0) return 0;
  if (cudaEventSynchronize(ctx->ev[ctx->ev_count]) != cudaSuccess) return -1;
  const int n = std::min(cap, ctx->ev_count);
  for (int i = 0; i < n; ++i) {
    if (names) names[i] = ctx->ev_name[i];
    if (ms) cudaEventElapsedTime(&ms[i], ctx->ev[i], ctx->ev[i + 1]);
  }
  return n;
}

extern "C" ogx_status ogx_ctx_set_stage_timeline(ogx_ctx* ctx, int on) {
  if (!ctx) return ogx_fail(OGX_ERR_INVALID, "ctx is NULL");
  cudaSetDevice(ctx->device);
  if (on && !ctx->stage_ev[0]) {
    for (int i = 0; i <= ogx_ctx::kMaxStages; ++i) {
      cudaError_t e = cudaEventCreate(&ctx->stage_ev[i]);
      if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaEventCreate");
    }
  }
  ctx->stages = on != 0;
  ctx->stage_count = 0;
  return OGX_OK;
}

extern "C" int ogx_ctx_stage_timeline(ogx_ctx* ctx, const char** names, float* ms, int cap) {
  if (!ctx || !ctx->stages || ctx->stage_count == 0) return 0;
  if (cudaEventSynchronize(ctx->stage_ev[ctx->stage_count]) != cudaSuccess) return -1;
  const int n = std::min(cap, ctx->stage_count);
  for (int i = 0; i < n; ++i) {
    if (names) names[i] = ctx->stage_name[i];
    if (ms) {
      cudaEventSynchronize(ctx->stage_ev[1 + i]);
      cudaEventElapsedTime(&ms[i], ctx->stage_ev[0], ctx->stage_ev[1 + i]);
    }
  }
  return n;
}

extern "C" int ogx_ctx_work_counts(ogx_ctx* ctx, int32_t* counts, int cap) {
  if (!ctx || !ctx->d_counts || cap < kCntSlots) return 0;
  if (cudaMemcpyAsync(counts, ctx->d_counts, kCntSlots * sizeof(int), cudaMemcpyDeviceToHost,
                      ctx->stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    return -1;
  return kCntSlots;
}

bool ogx_pageable_reads(int dev) {
  static std::atomic<int> known[16];  // 0 unknown, 1 no, 2 yes
  if (dev < 0 || dev >= 16) return false;
  int k = known[dev].load();
  if (k == 0) {
    int a = 0, t = 0;
    const bool ok = cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess &&
                    cudaDeviceGetAttribute(&t, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) ==
                        cudaSuccess;
    if (!ok) cudaGetLastError();
    k = ok && a == 1 && t == 1 ? 2 : 1;
    known[dev].store(k);
  }
  return k == 2;
}

size_t ogx_scratch_bytes_per_pair() {
  return 2 * kBuckets * sizeof(int) + sizeof(PolishRec) + sizeof(RefineRec) + 2 * sizeof(int);
}

ogx_status ogx_ctx::ensure_scratch(int npairs) {
  if ((size_t)npairs <= cap_pairs && d_counts) return OGX_OK;
  cudaStreamSynchronize(stream);
  free_scratch();
  size_t cap = std::max<size_t>(1024, (size_t)npairs + npairs / 4);
  cudaError_t e;
  if ((e = cudaMalloc(&d_lists, kBuckets * cap * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&d_elists, kBuckets * cap * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&d_polish, cap * sizeof(PolishRec))) != cudaSuccess ||
      (e = cudaMalloc(&d_refine, cap * sizeof(RefineRec))) != cudaSuccess ||
      (e = cudaMalloc(&d_refine_full, cap * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&d_spill, cap * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&d_resume, kResumeCap * sizeof(EpaResume))) != cudaSuccess ||
      (e = cudaMalloc(&d_counts, 64 * sizeof(int))) != cudaSuccess) {
    free_scratch();
    return ogx_cuda_fail(e, "scratch allocation");
  }
  cap_pairs = cap;
  return OGX_OK;
}

ogx_status ogx_ctx::ensure_aux() {
  if (fork_ev) return OGX_OK;
  cudaError_t e;
  for (int b = 0; b < fork_width; ++b) {
    if ((e = cudaStreamCreateWithFlags(&aux[b], cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&join_ev[b], cudaEventDisableTiming)) != cudaSuccess)
      return ogx_cuda_fail(e, "bucket streams");
  }
  if ((e = cudaStreamCreateWithFlags(&aux_r, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&route_ev, cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&rjoin_ev, cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming)) != cudaSuccess)
    return ogx_cuda_fail(e, "bucket streams");
  return OGX_OK;
}

ogx_status ogx_ctx::ensure_stage(size_t host_bytes, size_t dev_bytes) {
  cudaError_t e;
  if (host_bytes > h_stage_bytes) {
    cudaStreamSynchronize(stream);
    if (h_stage) cudaFreeHost(h_stage);
    h_stage = nullptr;
    h_stage_bytes = 0;
    if ((e = cudaMallocHost(&h_stage, host_bytes)) != cudaSuccess)
      return ogx_cuda_fail(e, "pinned staging allocation");
    h_stage_bytes = host_bytes;
  }
  if (dev_bytes > d_stage_bytes) {
    cudaStreamSynchronize(stream);
    if (d_stage) cudaFree(d_stage);
    d_stage = nullptr;
    d_stage_bytes = 0;
    if ((e = cudaMalloc(&d_stage, dev_bytes)) != cudaSuccess)
      return ogx_cuda_fail(e, "device staging allocation");
    d_stage_bytes = dev_bytes;
  }
  return OGX_OK;
}

// ---------------------------------------------------------------------------------
// pool

extern "C" ogx_status ogx_pool_create(ogx_ctx* ctx, int num_bodies, const int32_t* counts,
                                      ogx_pool** out) {
  if (!ctx || !out || (!counts && num_bodies > 0))
    return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (num_bodies < 0) return ogx_fail(OGX_ERR_INVALID, "num_bodies < 0");
  std::vector<BodyRef> refs(num_bodies);
  std::vector<int64_t> voff(num_bodies);
  uint64_t quad = 0;
  int64_t pts = 0;
  for (int b = 0; b < num_bodies; ++b) {
    if (counts[b] < 1) return ogx_fail(OGX_ERR_INVALID, "body %d has %d points", b, counts[b]);
    refs[b].quad = (uint32_t)quad;
    refs[b].n = counts[b];
    voff[b] = pts;
    quad += 3 * (uint64_t)((counts[b] + 3) / 4);
    pts += counts[b];
    if (quad >= (1ull << 32))
      return ogx_fail(OGX_ERR_CAPACITY, "pool exceeds 2^32 float4 blocks (%.1f GB)", quad * 16e-9);
  }
  cudaSetDevice(ctx->device);
  ogx_pool* p = new ogx_pool();
  p->ctx = ctx;
  p->nbodies = num_bodies;
  p->npoints = pts;
  p->nfloats = 4 * quad;
  cudaError_t e;
  if ((e = cudaMalloc(&p->d_points, std::max<size_t>(16, p->nfloats * sizeof(float)))) != cudaSuccess ||
      (e = cudaMalloc(&p->d_bodies, std::max<size_t>(8, num_bodies * sizeof(BodyRef)))) != cudaSuccess ||
      (e = cudaMalloc(&p->d_voff, std::max<size_t>(8, num_bodies * sizeof(int64_t)))) != cudaSuccess) {
    ogx_pool_destroy(p);
    return ogx_cuda_fail(e, "pool allocation");
  }
  p->h_voff = voff;
  if (num_bodies > 0) {
    if ((e = cudaMemcpy(p->d_bodies, refs.data(), num_bodies * sizeof(BodyRef),
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(p->d_voff, voff.data(), num_bodies * sizeof(int64_t),
                        cudaMemcpyHostToDevice)) != cudaSuccess) {
      ogx_pool_destroy(p);
      return ogx_cuda_fail(e, "pool table upload");
    }
  }
  *out = p;
  return OGX_OK;
}

extern "C" ogx_status ogx_pool_destroy(ogx_pool* p) {
  if (!p) return OGX_OK;
  cudaSetDevice(p->ctx->device);
  cudaStreamSynchronize(p->ctx->stream);
  cudaFree(p->d_points);
  cudaFree(p->d_bodies);
  cudaFree(p->d_voff);
  delete p;
  return OGX_OK;
}

extern "C" int ogx_pool_num_bodies(const ogx_pool* p) { return p ? p->nbodies : 0; }
extern "C" int64_t ogx_pool_num_points(const ogx_pool* p) { return p ? p->npoints : 0; }

extern "C" ogx_status ogx_pool_device_layout(const ogx_pool* p, float** d_points, void** d_bodies) {
  if (!p) return ogx_fail(OGX_ERR_INVALID, "pool is NULL");
  if (d_points) *d_points = p->d_points;
  if (d_bodies) *d_bodies = p->d_bodies;
  return OGX_OK;
}

ogx_status pool_pack(ogx_ctx* ctx, const ogx_pool* p, const float* d_aos) {
  if (p->nbodies == 0) return OGX_OK;
  cudaError_t e = launch_pack(d_aos, p->d_voff, p->d_bodies, p->nbodies, p->d_points, g_grid_pack,
                              ctx->stream);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "k_pack launch");
  return OGX_OK;
}

extern "C" ogx_status ogx_pool_load_device(ogx_ctx* ctx, ogx_pool* p, const float* d_coords) {
  if (!ctx || !p || (!d_coords && p->npoints > 0)) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  ogx_status s = pool_pack(ctx, p, d_coords);
  if (!s) ctx->last_launches = p->nbodies ? 1 : 0;
  return s;
}

extern "C" ogx_status ogx_pool_upload(ogx_ctx* ctx, ogx_pool* p, const float* coords) {
  if (!ctx || !p || (!coords && p->npoints > 0)) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  if (p->npoints == 0) return OGX_OK;
  cudaSetDevice(ctx->device);
  const size_t bytes = (size_t)p->npoints * 3 * sizeof(float);
  cudaPointerAttributes attr;
  const bool pinned = cudaPointerGetAttributes(&attr, coords) == cudaSuccess &&
                      (attr.type == cudaMemoryTypeHost || attr.type == cudaMemoryTypeManaged);
  cudaGetLastError();
  if (pinned && attr.devicePointer) {
    // page-locked host memory is device-addressable: the packing kernel reads the
    // caller's array directly (one pass over the host data, no staging copy)
    ctx->last_launches = 0;
    ogx_status s = pool_pack(ctx, p, static_cast<const float*>(attr.devicePointer));
    if (!s) ctx->last_launches = 1;
    return s;
  }
  const char* force = std::getenv("OGX_UPLOAD_STAGED");
  if (!pinned && ogx_pageable_reads(ctx->device) && !(force && force[0] == '1')) {
    // a device that reads pageable memory through the host's page tables packs straight
    // from the caller's array too; the call then waits for the pack, since a pageable
    // array may be changed or freed as soon as the call returns
    ctx->last_launches = 0;
    ogx_status s = pool_pack(ctx, p, coords);
    if (s) return s;
    ctx->last_launches = 1;
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "pool pack from host memory");
    return OGX_OK;
  }
  ogx_status s = ctx->ensure_stage(pinned ? 0 : bytes, bytes);
  if (s) return s;
  const void* src = coords;
  if (!pinned) {
    // stage pageable memory through the pinned buffer (parallel host copy)
    cudaStreamSynchronize(ctx->stream);  // the pinned buffer may still be in use
    const int nt = (int)std::min<size_t>(16, std::max<size_t>(1, bytes >> 24));
    std::vector<std::thread> th;
    for (int k = 0; k < nt; ++k)
      th.emplace_back([&, k] {
        const size_t lo = bytes * k / nt, hi = bytes * (k + 1) / nt;
        memcpy((char*)ctx->h_stage + lo, (const char*)coords + lo, hi - lo);
      });
    for (auto& x : th) x.join();
    src = ctx->h_stage;
  }
  cudaError_t e = cudaMemcpyAsync(ctx->d_stage, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "pool upload copy");
  ctx->last_launches = 0;
  s = pool_pack(ctx, p, static_cast<const float*>(ctx->d_stage));
  if (!s) ctx->last_launches = 1;
  return s;
}

// ---------------------------------------------------------------------------------
// batched queries

ogx_status ogx_run(ogx_ctx* ctx, const float* d_pool, const BodyRef* d_bodies, int nbodies,
                   int npairs, const gkCollisionPair* d_pairs, gkSimplex* d_smp, float* d_dist,
                   float* d_nrm, int32_t* d_status, int mode, const int2* d_warm, const float* d_xf) {
  if (npairs < 0) return ogx_fail(OGX_ERR_INVALID, "npairs < 0");
  if (npairs == 0) {
    ctx->last_launches = 0;
    return OGX_OK;
  }
  if (!d_pairs || !d_smp || !d_dist || (mode != kModeGjk && !d_nrm))
    return ogx_fail(OGX_ERR_INVALID, "NULL output or pair buffer");
  cudaSetDevice(ctx->device);
  ogx_status s = ctx->ensure_scratch(npairs);
  if (s) return s;
  DevBatch B;
  B.pool = d_pool;
  B.bodies = d_bodies;
  B.nbodies = nbodies;
  B.pairs = reinterpret_cast<const int2*>(d_pairs);
  B.npairs = npairs;
  B.smp = d_smp;
  B.dist = d_dist;
  B.nrm = d_nrm;
  B.status = d_status;
  B.lists = ctx->d_lists;
  B.elists = ctx->d_elists;
  B.counts = ctx->d_counts;
  B.polish = ctx->d_polish;
  B.refine = ctx->d_refine;
  B.refine_full = ctx->d_refine_full;
  B.spill = ctx->d_spill;
  B.resume = ctx->d_resume;
  B.resume_cap = ogx_ctx::kResumeCap;
  B.warm = d_warm;
  B.subtab = g_subtab;
  B.xf = d_xf;
  B.cfg = ctx->cfg;
  B.mode = mode;
  if (d_xf && mode != kModeGjkEpa) return ogx_fail(OGX_ERR_INVALID, "posed bodies: GJK + EPA calls only");
  cudaStream_t st = ctx->stream;
  int launches = 0;
  ctx->ev_count = 0;
  static const char* kGjkName[kBuckets] = {"gjk<=16", "gjk<=32", "gjk<=64", "gjk<=128",
                                           "gjk<=256", "gjk<=512", "gjk>512"};
  static const char* kEpaName[kBuckets] = {"epa<=16", "epa<=32", "epa<=64", "epa<=128",
                                           "epa<=256", "epa<=512", "epa>512"};
  cudaError_t e = cudaMemsetAsync(ctx->d_counts, 0, kCntSlots * sizeof(int), st);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "counter reset");
  const int bin_grid = std::min(g_grid_bin, (npairs + 255) / 256);
  ctx->mark("bin");
  e = launch_bin(B, bin_grid, st);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "k_bin launch");
  ++launches;
  // The seven bucket kernels of a stage run concurrently (one stream each, forked from
  // and joined back into the context's stream) so that the tail of one bucket overlaps
  // the others' work; with per-kernel timing on they run in sequence.
  const bool fork = !ctx->timing && ctx->fork_ok && ctx->ensure_aux() == OGX_OK;
  const int W = ctx->fork_width;  // bucket b runs on aux[b mod W]
  // optional stage timeline of a forked call (not while a graph is being captured)
  bool staged = false;
  if (fork && ctx->stages && ctx->stage_ev[0]) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cs);
    staged = cs == cudaStreamCaptureStatusNone && cudaEventRecord(ctx->stage_ev[0], st) == cudaSuccess;
    ctx->stage_count = 0;
  }
  auto stage = [&](const char* name, cudaStream_t s2) {
    if (!staged || ctx->stage_count >= ogx_ctx::kMaxStages) return;
    if (cudaEventRecord(ctx->stage_ev[1 + ctx->stage_count], s2) == cudaSuccess)
      ctx->stage_name[ctx->stage_count++] = name;
  };
  auto bucket_stream = [&](int b) -> cudaStream_t { return fork ? ctx->aux[b % W] : st; };
  auto fork_out = [&]() -> cudaError_t {
    if (!fork) return cudaSuccess;
    cudaError_t r = cudaEventRecord(ctx->fork_ev, st);
    for (int b = 0; b < W && r == cudaSuccess; ++b) r = cudaStreamWaitEvent(ctx->aux[b], ctx->fork_ev, 0);
    return r;
  };
  auto join_in = [&]() -> cudaError_t {
    if (!fork) return cudaSuccess;
    cudaError_t r = cudaSuccess;
    for (int b = 0; b < W && r == cudaSuccess; ++b) {
      r = cudaEventRecord(ctx->join_ev[b], ctx->aux[b]);
      if (r == cudaSuccess) r = cudaStreamWaitEvent(st, ctx->join_ev[b], 0);
    }
    return r;
  };
  // Every bucket stream starts after the binning.  EPA bucket b takes only the contacts of
  // GJK bucket b, so it follows that kernel on the same stream instead of waiting for every
  // GJK bucket; the context's stream waits for all GJK buckets (the refinement needs them).
  e = fork_out();
  if (e != cudaSuccess) return ogx_cuda_fail(e, "bucket fork");
  if (mode != kModeEpa) {
    for (int b = kBuckets - 1; b >= 0 && e == cudaSuccess; --b) {
      const Launch& k = d_xf ? g_gjkp[b] : g_gjkv[ctx->choice[0][b]];
      ctx->mark(kGjkName[b]);
      k.fn<<<fit_grid(k.grid, npairs, k.L), kBlock, k.smem, bucket_stream(b)>>>(B, b);
      stage(kGjkName[b], bucket_stream(b));
      ++launches;
    }
    if (e == cudaSuccess) e = join_in();
    if (e != cudaSuccess) return ogx_cuda_fail(e, "GJK launches");
  }
  // The FP64 refinement (separated pairs) and the EPA buckets (contacts) touch disjoint
  // pairs: forked, the refinement runs on the context's stream (and aux_r) beside the EPA
  // buckets, followed there by the full-capacity pass over the few contacts it finds; the
  // spill and polish passes of the buckets' contacts wait for the buckets only, and
  // everything joins back into the context's stream.
  const bool refine = mode != kModeEpa && (ctx->cfg.flags & OGX_F_FP64_POLISH);
  if (mode != kModeGjk) {
    for (int b = kBuckets - 1; b >= 0 && e == cudaSuccess; --b) {
      const Launch& k = d_xf ? g_epap[b] : g_epav[ctx->choice[1][b]];
      ctx->mark(kEpaName[b]);
      k.fn<<<fit_grid(k.grid, npairs, k.L), kBlock, k.smem, bucket_stream(b)>>>(B, b);
      stage(kEpaName[b], bucket_stream(b));
      ++launches;
    }
    if (e != cudaSuccess) return ogx_cuda_fail(e, "EPA launches");
  }
  const cudaStream_t rst = st;
  if (refine) {
    ctx->mark("refine");
    e = launch_refine(B, fit_grid(g_grid_refine, npairs, 1), fit_grid(g_grid_pack, npairs, 1), rst,
                      fork ? ctx->aux_r : rst, fork ? ctx->route_ev : nullptr);
    if (e == cudaSuccess && fork) {
      e = cudaEventRecord(ctx->rjoin_ev, ctx->aux_r);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(rst, ctx->rjoin_ev, 0);
    }
    if (e != cudaSuccess) return ogx_cuda_fail(e, "k_refine launch");
    stage("refine", rst);
    launches += 3;
    if (mode != kModeGjk) {
      // the contacts the refinement found (usually none), after it on the same stream
      ctx->mark("epa_late");
      e = launch_epa_spill(B, fit_grid(g_grid_spill, std::max(1, npairs / 256), 32), rst, true);
      if (e != cudaSuccess) return ogx_cuda_fail(e, "k_epa_spill launch");
      stage("epa_late", rst);
      ++launches;
    }
  }
  if (mode != kModeGjk) {
    // contacts that outgrew the bucket kernels' working set or need the certified re-run,
    // at full capacity (polished in the same kernel), beside the polish of the others
    cudaStream_t sst = st, pst = st;
    if (fork) {
      sst = ctx->aux[0];
      pst = ctx->aux[1];
      for (int b = 0; b < W && e == cudaSuccess; ++b) e = cudaEventRecord(ctx->join_ev[b], ctx->aux[b]);
      for (int b = 0; b < W && e == cudaSuccess; ++b) {
        if (sst != ctx->aux[b]) e = cudaStreamWaitEvent(sst, ctx->join_ev[b], 0);
        if (e == cudaSuccess && b != 1) e = cudaStreamWaitEvent(pst, ctx->join_ev[b], 0);
      }
      if (e != cudaSuccess) return ogx_cuda_fail(e, "EPA join");
    }
    ctx->mark("epa_spill");
    e = launch_epa_spill(B, fit_grid(g_grid_spill, npairs, 32), sst);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "k_epa_spill launch");
    stage("epa_spill", sst);
    ++launches;
    if (ctx->cfg.flags & OGX_F_FP64_POLISH) {
      ctx->mark("polish");
      e = launch_polish(B, fit_grid(g_grid_polish, npairs, 1), pst);
      if (e != cudaSuccess) return ogx_cuda_fail(e, "k_polish launch");
      stage("polish", pst);
      ++launches;
    }
    if (fork) {
      e = cudaEventRecord(ctx->join_ev[0], sst);
      if (e == cudaSuccess) e = cudaEventRecord(ctx->join_ev[1], pst);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ctx->join_ev[0], 0);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ctx->join_ev[1], 0);
      if (e != cudaSuccess) return ogx_cuda_fail(e, "spill join");
    }
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return ogx_cuda_fail(e, "pipeline launch");
  stage("end", st);
  if (ctx->timing) cudaEventRecord(ctx->ev[ctx->ev_count], st);
  ctx->last_launches = launches;
  return OGX_OK;
}

extern "C" ogx_status ogx_gjk(ogx_ctx* ctx, const ogx_pool* pool, int npairs,
                              const gkCollisionPair* d_pairs, gkSimplex* d_simplices,
                              float* d_distances, int32_t* d_status) {
  if (!ctx || !pool) return ogx_fail(OGX_ERR_INVALID, "NULL context or pool");
  return ogx_run(ctx, pool->d_points, pool->d_bodies, pool->nbodies, npairs, d_pairs, d_simplices,
                 d_distances, nullptr, d_status, kModeGjk);
}

extern "C" ogx_status ogx_gjk_epa(ogx_ctx* ctx, const ogx_pool* pool, int npairs,
                                  const gkCollisionPair* d_pairs, gkSimplex* d_simplices,
                                  float* d_distances, float* d_normals, int32_t* d_status) {
  if (!ctx || !pool) return ogx_fail(OGX_ERR_INVALID, "NULL context or pool");
  return ogx_run(ctx, pool->d_points, pool->d_bodies, pool->nbodies, npairs, d_pairs, d_simplices,
                 d_distances, d_normals, d_status, kModeGjkEpa);
}

extern "C" ogx_status ogx_epa(ogx_ctx* ctx, const ogx_pool* pool, int npairs,
                              const gkCollisionPair* d_pairs, gkSimplex* d_simplices,
                              float* d_distances, float* d_normals, int32_t* d_status) {
  if (!ctx || !pool) return ogx_fail(OGX_ERR_INVALID, "NULL context or pool");
  return ogx_run(ctx, pool->d_points, pool->d_bodies, pool->nbodies, npairs, d_pairs, d_simplices,
                 d_distances, d_normals, d_status, kModeEpa);
}

// ---------------------------------------------------------------------------------
// kernel choice and autotuning

extern "C" ogx_status ogx_ctx_get_kernel_choice(const ogx_ctx* ctx, int kind, int bucket, int* lanes,
                                                int* blocks) {
  if (!ctx || kind < 0 || kind > 1 || bucket < 0 || bucket >= kBuckets)
    return ogx_fail(OGX_ERR_INVALID, "bad kind/bucket");
  const Launch& k = (kind == 0 ? g_gjkv : g_epav)[ctx->choice[kind][bucket]];
  if (lanes) *lanes = k.L;
  if (blocks) *blocks = k.K;
  return OGX_OK;
}

extern "C" ogx_status ogx_ctx_set_kernel_choice(ogx_ctx* ctx, int kind, int bucket, int lanes, int blocks) {
  if (!ctx || kind < 0 || kind > 1 || bucket < 0 || bucket >= kBuckets)
    return ogx_fail(OGX_ERR_INVALID, "bad kind/bucket");
  const std::vector<Launch>& vs = kind == 0 ? g_gjkv : g_epav;
  for (int i = 0; i < (int)vs.size(); ++i)
    if (vs[i].L == lanes && vs[i].K == blocks && serves(vs[i], bucket)) {
      ctx->choice[kind][bucket] = i;
      return OGX_OK;
    }
  return ogx_fail(OGX_ERR_INVALID, "no variant (%d lanes, %d blocks) for bucket %d", lanes, blocks, bucket);
}

// ---------------------------------------------------------------------------------
// CUDA graphs: the launch sequence of a call is fixed (persistent kernels, work counts on
// the device), so one call can be captured once and replayed with one launch.

struct ogx_graph {
  ogx_ctx* ctx = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int launches = 0;
};

extern "C" ogx_status ogx_graph_create(ogx_ctx* ctx, const ogx_pool* pool, int npairs,
                                       const gkCollisionPair* d_pairs, gkSimplex* d_simplices,
                                       float* d_distances, float* d_normals, int32_t* d_status, int mode,
                                       ogx_graph** out) {
  if (!ctx || !pool || !out) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  if (mode < kModeGjk || mode > kModeEpa) return ogx_fail(OGX_ERR_INVALID, "mode %d", mode);
  if (!ctx->stream) return ogx_fail(OGX_ERR_INVALID, "graphs need a context with its own stream");
  *out = nullptr;
  cudaSetDevice(ctx->device);
  // everything the call allocates is allocated before the capture
  ogx_status s = ctx->ensure_scratch(npairs);
  if (s) return s;
  const bool timing = ctx->timing;
  ctx->timing = false;
  cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    ctx->timing = timing;
    return ogx_cuda_fail(e, "cudaStreamBeginCapture");
  }
  s = ogx_run(ctx, pool->d_points, pool->d_bodies, pool->nbodies, npairs, d_pairs, d_simplices, d_distances,
              d_normals, d_status, mode);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &graph);
  ctx->timing = timing;
  if (s) {
    if (graph) cudaGraphDestroy(graph);
    return s;
  }
  if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaStreamEndCapture");
  ogx_graph* G = new ogx_graph();
  G->ctx = ctx;
  G->graph = graph;
  G->launches = ctx->last_launches;
  e = cudaGraphInstantiate(&G->exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    delete G;
    return ogx_cuda_fail(e, "cudaGraphInstantiate");
  }
  *out = G;
  return OGX_OK;
}

extern "C" ogx_status ogx_graph_launch(ogx_graph* G) {
  if (!G) return ogx_fail(OGX_ERR_INVALID, "NULL graph");
  cudaSetDevice(G->ctx->device);
  const cudaError_t e = cudaGraphLaunch(G->exec, G->ctx->stream);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaGraphLaunch");
  G->ctx->last_launches = G->launches;
  return OGX_OK;
}

extern "C" int ogx_graph_kernel_launches(const ogx_graph* G) { return G ? G->launches : 0; }

extern "C" ogx_status ogx_graph_destroy(ogx_graph* G) {
  if (!G) return OGX_OK;
  cudaSetDevice(G->ctx->device);
  if (G->exec) cudaGraphExecDestroy(G->exec);
  if (G->graph) cudaGraphDestroy(G->graph);
  delete G;
  return OGX_OK;
}

// Times every compiled variant that can serve each bucket on the caller's batch (round r
// runs candidate r of every bucket at once, `reps` times, keeping the best time) and keeps
// the fastest per bucket for this context and for contexts created later on the device.
extern "C" ogx_status ogx_autotune(ogx_ctx* ctx, const ogx_pool* pool, int npairs, const gkCollisionPair* d_pairs,
                                   int reps) {
  if (!ctx || !pool || !d_pairs || npairs <= 0) return ogx_fail(OGX_ERR_INVALID, "bad autotune arguments");
  cudaSetDevice(ctx->device);
  gkSimplex* smp = nullptr;
  float *dist = nullptr, *nrm = nullptr;
  cudaError_t e = cudaMalloc(&smp, npairs * sizeof(gkSimplex));
  if (e == cudaSuccess) e = cudaMalloc(&dist, npairs * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&nrm, 3 * (size_t)npairs * sizeof(float));
  if (e != cudaSuccess) {
    cudaFree(smp);
    cudaFree(dist);
    return ogx_cuda_fail(e, "autotune buffers");
  }
  std::vector<int> cands[2][kBuckets];
  int rounds = 0;
  for (int kind = 0; kind < 2; ++kind)
    for (int b = 0; b < kBuckets; ++b) {
      const std::vector<Launch>& vs = kind == 0 ? g_gjkv : g_epav;
      for (int i = 0; i < (int)vs.size(); ++i)
        if (serves(vs[i], b)) cands[kind][b].push_back(i);
      rounds = std::max(rounds, (int)cands[kind][b].size());
    }
  float best[2][kBuckets];
  int pick[2][kBuckets], pick_prior[2][kBuckets];
  for (int kind = 0; kind < 2; ++kind)
    for (int b = 0; b < kBuckets; ++b) {
      best[kind][b] = INFINITY;
      pick[kind][b] = pick_prior[kind][b] = ctx->choice[kind][b];
    }
  const bool was_timing = ctx->timing;
  ogx_status s = ogx_ctx_set_timing(ctx, 1);
  for (int r = 0; r < rounds && !s; ++r) {
    for (int kind = 0; kind < 2; ++kind)
      for (int b = 0; b < kBuckets; ++b) {
        const auto& c = cands[kind][b];
        if (!c.empty()) ctx->choice[kind][b] = c[r % c.size()];
      }
    for (int k = 0; k < std::max(1, reps) && !s; ++k) {
      s = ogx_run(ctx, pool->d_points, pool->d_bodies, pool->nbodies, npairs, d_pairs, smp, dist, nrm, nullptr,
                  kModeGjkEpa);
      if (s) break;
      const char* names[ogx_ctx::kMaxTimed];
      float ms[ogx_ctx::kMaxTimed];
      const int n = ogx_ctx_kernel_times(ctx, names, ms, ogx_ctx::kMaxTimed);
      for (int i = 0; i < n; ++i) {
        int kind = -1, b = -1;
        if (!strncmp(names[i], "gjk", 3)) kind = 0;
        if (!strncmp(names[i], "epa", 3)) kind = 1;
        if (kind < 0) continue;
        const char* bn = names[i] + 3;
        static const char* kB[kBuckets] = {"<=16", "<=32", "<=64", "<=128", "<=256", "<=512", ">512"};
        for (int q = 0; q < kBuckets; ++q)
          if (!strcmp(bn, kB[q])) b = q;
        if (b < 0 || r >= (int)cands[kind][b].size()) continue;  // this round repeats a candidate
        if (ms[i] < best[kind][b]) {
          best[kind][b] = ms[i];
          pick[kind][b] = ctx->choice[kind][b];
        }
      }
    }
  }
  // The candidates were timed one after another, but a call runs the buckets
  // concurrently: keep the picked set only if a whole concurrent call with it is not
  // slower than with the set the context started from (best of three each).
  ogx_ctx_set_timing(ctx, 0);
  auto whole_call = [&](int (*ch)[kBuckets], float* best_ms) -> ogx_status {
    for (int kind = 0; kind < 2; ++kind)
      for (int b = 0; b < kBuckets; ++b) ctx->choice[kind][b] = ch[kind][b];
    *best_ms = INFINITY;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    ogx_status r = ce == cudaSuccess ? OGX_OK : ogx_cuda_fail(ce, "autotune events");
    for (int k = 0; k < 4 && !r; ++k) {
      cudaEventRecord(e0, ctx->stream);
      r = ogx_run(ctx, pool->d_points, pool->d_bodies, pool->nbodies, npairs, d_pairs, smp, dist, nrm, nullptr,
                  kModeGjkEpa);
      cudaEventRecord(e1, ctx->stream);
      float ms = 0.0f;
      if (!r && cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
          k > 0)  // the first run warms up
        *best_ms = std::min(*best_ms, ms);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return r;
  };
  if (!s) {
    int prior[2][kBuckets];
    for (int kind = 0; kind < 2; ++kind)
      for (int b = 0; b < kBuckets; ++b) prior[kind][b] = pick_prior[kind][b];
    float t_pick = INFINITY, t_prior = INFINITY;
    s = whole_call(pick, &t_pick);
    if (!s) s = whole_call(prior, &t_prior);
    if (!s && t_prior < t_pick)
      for (int kind = 0; kind < 2; ++kind)
        for (int b = 0; b < kBuckets; ++b) pick[kind][b] = prior[kind][b];
  }
  ogx_ctx_set_timing(ctx, was_timing);
  cudaFree(smp);
  cudaFree(dist);
  cudaFree(nrm);
  if (s) {
    set_defaults(ctx);
    return s;
  }
  for (int kind = 0; kind < 2; ++kind)
    for (int b = 0; b < kBuckets; ++b) ctx->choice[kind][b] = pick[kind][b];
  if (ctx->device < 16) {
    std::lock_guard<std::mutex> lk(g_init_mu);
    for (int kind = 0; kind < 2; ++kind)
      for (int b = 0; b < kBuckets; ++b) g_tuned[ctx->device][kind][b] = pick[kind][b];
    g_tuned_valid[ctx->device] = true;
  }
  return OGX_OK;
}
