// ogx_server.cu -- serving loop: resident rigid bodies, per-tick transforms, continuous
// batching of pair requests over a fixed set of device slots.
//
// The reference's per-frame path (visualization/integrate_final_gjk.cu:1028-1037) moves
// every body on the host, uploads the pairs of the frame and runs the indexed GJK/EPA
// functions synchronously.  Here:
//  * the bodies live on the device in their own frame (the local pool); a transform
//    update writes a world-space copy of the pool into one of `world_slots` ring
//    buffers with one kernel (version = tick number), so requests of older ticks still
//    in flight keep reading their own copy; with `fused_transform` it uploads the poses
//    only and the GJK/EPA kernels apply them as they read the points (posed kernels);
//  * requests (a pair list of one tick) are queued; a scheduler thread admits the oldest
//    queued request as soon as a slot (stream + device buffers for `slot_pairs` pairs) is
//    free and the pairs in flight stay within `max_pairs_in_flight` and their device
//    working memory within `max_bytes_in_flight`; admitted requests run concurrently on
//    their slots' streams;
//  * each slot's pipeline: pairs host->device, warm-start lookup, GJK + EPA (the engine's
//    kernels), warm-start store, results device->host, one event; the scheduler copies the
//    results out when the event completes and frees the slot;
//  * warm starts: a device hash table maps (body i, body j) to the first vertex pair of
//    the last simplex found for it; GJK starts there instead of at vertex 0.  The table is
//    a lossy cache (bounded probing, a full window overwrites the home slot) shared by
//    all slots; a stale or torn entry only changes the starting point, and out-of-range
//    indices are ignored by the GJK kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ogx_engine.h"

using namespace ogx;

namespace {

constexpr uint64_t kEmptyKey = ~0ull;
constexpr int kWarmProbe = 16;

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

// world = R p + t per point (R row-major in xf[0..9), t in xf[9..12)), evaluated in FP64
// and rounded once, so that the host can reproduce every world coordinate exactly
__global__ void k_transform(const float* __restrict__ local, const BodyRef* __restrict__ bodies,
                            int nbodies, const float* __restrict__ xf, float* __restrict__ world) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int b = warp; b < nbodies; b += nwarps) {
    const BodyRef r = bodies[b];
    const int n4 = round4(body_points(r));
    const size_t base = 4 * (size_t)r.quad;
    const float* m = xf + 12 * (size_t)b;
    const double r00 = m[0], r01 = m[1], r02 = m[2], r10 = m[3], r11 = m[4], r12 = m[5];
    const double r20 = m[6], r21 = m[7], r22 = m[8], tx = m[9], ty = m[10], tz = m[11];
    for (int i = lane; i < n4; i += 32) {
      const double x = local[base + i], y = local[base + n4 + i], z = local[base + 2 * n4 + i];
      world[base + i] = (float)(r00 * x + r01 * y + r02 * z + tx);
      world[base + n4 + i] = (float)(r10 * x + r11 * y + r12 * z + ty);
      world[base + 2 * n4 + i] = (float)(r20 * x + r21 * y + r22 * z + tz);
    }
  }
}

__global__ void k_warm_lookup(const int2* __restrict__ pairs, int n, const unsigned long long* __restrict__ keys,
                              const int2* __restrict__ vals, uint64_t mask, int2* __restrict__ warm) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int2 pr = pairs[p];
    const uint64_t key = ((uint64_t)(uint32_t)pr.x << 32) | (uint32_t)pr.y;
    const uint64_t h = mix64(key);
    int2 w = make_int2(-1, -1);
    for (int k = 0; k < kWarmProbe; ++k) {
      const uint64_t s = (h + k) & mask;
      const uint64_t kk = keys[s];
      if (kk == key) {
        w = vals[s];
        break;
      }
      if (kk == kEmptyKey) break;
    }
    warm[p] = w;
  }
}

__global__ void k_warm_store(const int2* __restrict__ pairs, int n, const gkSimplex* __restrict__ smp,
                             unsigned long long* __restrict__ keys, int2* __restrict__ vals, uint64_t mask) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int2 pr = pairs[p];
    if (pr.x < 0 || pr.y < 0) continue;
    const uint64_t key = ((uint64_t)(uint32_t)pr.x << 32) | (uint32_t)pr.y;
    const uint64_t h = mix64(key);
    const int2 v = make_int2(smp[p].vrtx_idx[0][0], smp[p].vrtx_idx[0][1]);
    uint64_t slot = h & mask;
    for (int k = 0; k < kWarmProbe; ++k) {
      const uint64_t s = (h + k) & mask;
      const unsigned long long kk = keys[s];
      if (kk == key) {
        slot = s;
        break;
      }
      if (kk == kEmptyKey) {
        const unsigned long long prev = atomicCAS(&keys[s], kEmptyKey, (unsigned long long)key);
        if (prev == kEmptyKey || prev == key) {
          slot = s;
          break;
        }
      }
    }
    keys[slot] = key;
    vals[slot] = v;
  }
}

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  int64_t version = 0;
  int npairs = 0;
  std::vector<gkCollisionPair> pairs;  // copied at submit
  gkSimplex* out_smp = nullptr;
  float* out_dist = nullptr;
  float* out_nrm = nullptr;
  int32_t* out_status = nullptr;
  Clock::time_point t_submit, t_done;
  Clock::time_point t_admit, t_staged;  // admitted to a slot; host staging done, first copy queued
  float device_ms = -1.0f;             // first device operation to results in host memory
  int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
  ogx_status err = OGX_OK;
  // broad-phase request: the pairs come from the device grid of the version's world copy
  bool broad = false;
  float cell = 0.0f, margin = 0.0f;
  int max_pairs = 0;
  gkCollisionPair* out_pairs = nullptr;
  int32_t* out_count = nullptr;  // [0] overlapping pairs found, [1] error flags
};

// true when p is page-locked host memory the device can copy into directly
bool is_pinned(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

struct Slot {
  ogx_ctx* ctx = nullptr;
  gkCollisionPair* d_pairs = nullptr;
  gkSimplex* d_smp = nullptr;
  float* d_dist = nullptr;
  float* d_nrm = nullptr;
  int32_t* d_status = nullptr;
  int2* d_warm = nullptr;
  gkCollisionPair* h_pairs = nullptr;  // pinned staging
  gkSimplex* h_smp = nullptr;
  float* h_dist = nullptr;
  float* h_nrm = nullptr;
  int32_t* h_status = nullptr;
  cudaEvent_t done = nullptr;
  cudaEvent_t start = nullptr;  // the request's first device operation (timing)
  Request* req = nullptr;
  int world = -1;
  bool direct[5] = {};  // results copied straight into the caller's (pinned) arrays
  // broad-phase requests: grid scratch, the count read back between the two stages
  ogx_broad* broad = nullptr;
  int* d_bres = nullptr;
  int* h_bres = nullptr;
  cudaEvent_t counted = nullptr;
  int stage = 0;  // 0 idle, 1 broad phase running, 2 narrow phase running
  int reserved = 0;  // pairs counted against the in-flight budget
};

}  // namespace

struct ogx_server {
  int device = 0;
  ogx_server_config sc{};
  ogx_config cfg{};
  ogx_ctx* pctx = nullptr;  // owns the local pool and the transform stream
  ogx_pool* local = nullptr;
  std::vector<float*> d_world;
  std::vector<float*> d_xf;
  std::vector<float*> h_xf;
  std::vector<int64_t> world_version;
  std::vector<int> world_refs;
  std::vector<char> world_writing;  // a transform upload into the slot is under way
  std::vector<cudaEvent_t> world_ready;
  int64_t next_version = 0;
  std::vector<Slot> slots;
  unsigned long long* d_keys = nullptr;
  int2* d_vals = nullptr;
  uint64_t warm_mask = 0;
  int grid_aux = 0;

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::unordered_map<int64_t, Request*> reqs;
  int64_t next_id = 1;
  int64_t pairs_in_flight = 0;
  int64_t bytes_per_pair = 0;  // device working memory of one pair of a request
  int64_t max_bytes = 0;       // admission budget in device bytes
  int64_t peak_bytes = 0;
  bool stop = false;
  std::thread sched;

  void loop();
  bool admit(Request* r, Slot& s, int w);
  bool launch_narrow(Request* r, Slot& s, int w);
  void finish(Slot& s);
  void release();
};

ogx_status broad_run(ogx_broad* B, cudaStream_t st, const float* d_points, const ogx::BodyRef* d_bodies,
                     int nbodies, float cell, float margin, int max_pairs, gkCollisionPair* d_pairs,
                     int* d_result);

namespace {

template <class T>
cudaError_t dalloc(T** p, size_t n) {
  return cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(16, n * sizeof(T)));
}
template <class T>
cudaError_t halloc(T** p, size_t n) {
  return cudaMallocHost(reinterpret_cast<void**>(p), std::max<size_t>(16, n * sizeof(T)));
}

}  // namespace

bool ogx_server::admit(Request* r, Slot& s, int w) {
  cudaStream_t st = s.ctx->stream;
  cudaError_t e = cudaStreamWaitEvent(st, world_ready[w], 0);
  if (e != cudaSuccess) {
    r->err = ogx_cuda_fail(e, "server request launch");
    return false;
  }
  s.req = r;
  s.world = w;
  r->t_admit = Clock::now();
  if (!r->broad) {
    std::memcpy(s.h_pairs, r->pairs.data(), r->npairs * sizeof(gkCollisionPair));
    r->t_staged = Clock::now();
    e = cudaEventRecord(s.start, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s.d_pairs, s.h_pairs, r->npairs * sizeof(gkCollisionPair), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
      r->err = ogx_cuda_fail(e, "server request launch");
      return false;
    }
    return launch_narrow(r, s, w);
  }
  // stage 1: pairs from the grid, count back to the host
  const int cap = std::min(r->max_pairs, sc.slot_pairs);
  r->t_staged = r->t_admit;
  e = cudaEventRecord(s.start, st);
  if (e != cudaSuccess) {
    r->err = ogx_cuda_fail(e, "server broad phase");
    return false;
  }
  ogx_status os = broad_run(s.broad, st, d_world[w], local->d_bodies, local->nbodies, r->cell, r->margin, cap,
                            s.d_pairs, s.d_bres);
  if (os) {
    r->err = os;
    return false;
  }
  e = cudaMemcpyAsync(s.h_bres, s.d_bres, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaEventRecord(s.counted, st);
  if (e != cudaSuccess) {
    r->err = ogx_cuda_fail(e, "server broad phase");
    return false;
  }
  s.stage = 1;
  return true;
}

bool ogx_server::launch_narrow(Request* r, Slot& s, int w) {
  const int n = r->npairs;
  cudaStream_t st = s.ctx->stream;
  cudaError_t e = cudaSuccess;
  s.stage = 2;
  const int grid = std::max(1, std::min(grid_aux, (n + 255) / 256));
  if (n > 0 && sc.warm_start) {
    k_warm_lookup<<<grid, 256, 0, st>>>(reinterpret_cast<const int2*>(s.d_pairs), n, d_keys, d_vals,
                                        warm_mask, s.d_warm);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    r->err = ogx_cuda_fail(e, "server request launch");
    return false;
  }
  // fused transform: the bodies as stored, with the version's poses
  const float* pts = sc.fused_transform ? local->d_points : d_world[w];
  const float* xf = sc.fused_transform ? d_xf[w] : nullptr;
  ogx_status os = n > 0 ? ogx_run(s.ctx, pts, local->d_bodies, local->nbodies, n, s.d_pairs, s.d_smp, s.d_dist,
                                  s.d_nrm, s.d_status, kModeGjkEpa, sc.warm_start ? s.d_warm : nullptr, xf)
                        : OGX_OK;
  if (os) {
    r->err = os;
    return false;
  }
  if (n > 0 && sc.warm_start) {
    k_warm_store<<<grid, 256, 0, st>>>(reinterpret_cast<const int2*>(s.d_pairs), n, s.d_smp, d_keys, d_vals,
                                       warm_mask);
    e = cudaGetLastError();
  }
  // results go straight to the caller's arrays when those are page-locked, else through
  // the slot's pinned staging (copied out when the request completes)
  void* dst[5] = {r->out_smp, r->out_dist, r->out_nrm, r->out_status, r->broad ? r->out_pairs : nullptr};
  void* stage[5] = {s.h_smp, s.h_dist, s.h_nrm, s.h_status, s.h_pairs};
  const void* src[5] = {s.d_smp, s.d_dist, s.d_nrm, s.d_status, s.d_pairs};
  const size_t bytes[5] = {n * sizeof(gkSimplex), n * sizeof(float), 3 * n * sizeof(float), n * sizeof(int32_t),
                           n * sizeof(gkCollisionPair)};
  for (int k = 0; k < 5 && e == cudaSuccess; ++k) {
    s.direct[k] = is_pinned(dst[k]);
    if (!dst[k] || n == 0) continue;
    e = cudaMemcpyAsync(s.direct[k] ? dst[k] : stage[k], src[k], bytes[k], cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaEventRecord(s.done, st);
  if (e != cudaSuccess) {
    r->err = ogx_cuda_fail(e, "server request launch");
    return false;
  }
  return true;
}

void ogx_server::finish(Slot& s) {
  Request* r = s.req;
  const int n = r->npairs;
  if (r->out_smp && !s.direct[0]) std::memcpy(r->out_smp, s.h_smp, n * sizeof(gkSimplex));
  if (r->out_dist && !s.direct[1]) std::memcpy(r->out_dist, s.h_dist, n * sizeof(float));
  if (r->out_nrm && !s.direct[2]) std::memcpy(r->out_nrm, s.h_nrm, 3 * n * sizeof(float));
  if (r->out_status && !s.direct[3]) std::memcpy(r->out_status, s.h_status, n * sizeof(int32_t));
  if (r->broad && r->out_pairs && !s.direct[4]) std::memcpy(r->out_pairs, s.h_pairs, n * sizeof(gkCollisionPair));
}

void ogx_server::loop() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  while (!stop) {
    bool progress = false;
    // completions
    for (Slot& s : slots) {
      if (!s.req) continue;
      Request* r = s.req;
      bool failed = false;
      if (s.stage == 1) {
        // broad phase done: size the narrow phase by the pairs found
        const cudaError_t q = cudaEventQuery(s.counted);
        if (q == cudaErrorNotReady) continue;
        if (q == cudaSuccess) {
          const int found = s.h_bres[0];
          if (r->out_count) {
            r->out_count[0] = found;
            r->out_count[1] = s.h_bres[1];
          }
          r->npairs = std::min(found, std::min(r->max_pairs, sc.slot_pairs));
          // the narrow phase holds only the pairs found: release the rest of the budget
          pairs_in_flight -= s.reserved - r->npairs;
          s.reserved = r->npairs;
          failed = !launch_narrow(r, s, s.world);
        } else {
          r->err = ogx_cuda_fail(q, "server broad phase");
          failed = true;
        }
        progress = true;
        if (!failed) continue;
      } else {
        const cudaError_t q = cudaEventQuery(s.done);
        if (q == cudaErrorNotReady) continue;
        if (q == cudaSuccess) {
          finish(s);
          float ms = -1.0f;
          if (cudaEventElapsedTime(&ms, s.start, s.done) == cudaSuccess) r->device_ms = ms;
          r->state = 2;
        } else {
          r->err = ogx_cuda_fail(q, "server request");
          failed = true;
        }
      }
      if (failed) r->state = 3;
      r->t_done = Clock::now();
      pairs_in_flight -= s.reserved;
      world_refs[s.world] -= 1;
      s.req = nullptr;
      s.world = -1;
      s.stage = 0;
      progress = true;
    }
    if (progress) cv_done.notify_all();
    // admissions, oldest first
    while (!queue.empty()) {
      Request* r = queue.front();
      const int want = r->broad ? std::min(r->max_pairs, sc.slot_pairs) : r->npairs;
      // admission by the pairs and the device memory in flight (a request that exceeds a
      // budget alone still runs once nothing else does)
      if (pairs_in_flight > 0 && (pairs_in_flight + want > sc.max_pairs_in_flight ||
                                  (pairs_in_flight + want) * bytes_per_pair > max_bytes))
        break;
      Slot* free_slot = nullptr;
      for (Slot& s : slots)
        if (!s.req) {
          free_slot = &s;
          break;
        }
      if (!free_slot) break;
      queue.pop_front();
      const int w = (int)(r->version % sc.world_slots);
      if (world_version[w] != r->version) {
        r->err = ogx_fail(OGX_ERR_INVALID, "transform version %lld was overwritten", (long long)r->version);
        r->state = 3;
        r->t_done = Clock::now();
        cv_done.notify_all();
        continue;
      }
      r->state = 1;
      if (!admit(r, *free_slot, w)) {
        r->state = 3;
        r->t_done = Clock::now();
        free_slot->req = nullptr;
        free_slot->world = -1;
        free_slot->stage = 0;
        cv_done.notify_all();
        continue;
      }
      free_slot->reserved = want;
      pairs_in_flight += want;
      peak_bytes = std::max(peak_bytes, pairs_in_flight * bytes_per_pair);
      world_refs[w] += 1;
      progress = true;
    }
    bool busy = false;
    for (Slot& s : slots) busy |= s.req != nullptr;
    if (!progress) {
      if (busy)
        cv_work.wait_for(lk, std::chrono::microseconds(20));
      else
        cv_work.wait_for(lk, std::chrono::milliseconds(5));
    }
  }
}

void ogx_server::release() {
  for (Slot& s : slots) {
    // the broad-phase scratch refers to the slot's context: release it first
    if (s.broad) ogx_broad_destroy(s.broad);
    s.broad = nullptr;
    if (s.ctx) ogx_ctx_destroy(s.ctx);
    cudaFree(s.d_pairs);
    cudaFree(s.d_smp);
    cudaFree(s.d_dist);
    cudaFree(s.d_nrm);
    cudaFree(s.d_status);
    cudaFree(s.d_warm);
    cudaFreeHost(s.h_pairs);
    cudaFreeHost(s.h_smp);
    cudaFreeHost(s.h_dist);
    cudaFreeHost(s.h_nrm);
    cudaFreeHost(s.h_status);
    if (s.done) cudaEventDestroy(s.done);
    if (s.start) cudaEventDestroy(s.start);
    cudaFree(s.d_bres);
    cudaFreeHost(s.h_bres);
    if (s.counted) cudaEventDestroy(s.counted);
  }
  slots.clear();
  for (float* p : d_world) cudaFree(p);
  for (float* p : d_xf) cudaFree(p);
  for (float* p : h_xf) cudaFreeHost(p);
  for (cudaEvent_t e : world_ready)
    if (e) cudaEventDestroy(e);
  d_world.clear();
  d_xf.clear();
  h_xf.clear();
  world_ready.clear();
  cudaFree(d_keys);
  cudaFree(d_vals);
  d_keys = nullptr;
  d_vals = nullptr;
  if (local) ogx_pool_destroy(local);
  local = nullptr;
  if (pctx) ogx_ctx_destroy(pctx);
  pctx = nullptr;
  for (auto& kv : reqs) delete kv.second;
  reqs.clear();
}

extern "C" void ogx_server_config_default(ogx_server_config* sc) {
  if (!sc) return;
  sc->slots = 4;
  sc->slot_pairs = 262144;
  sc->max_pairs_in_flight = 1 << 20;
  sc->world_slots = 4;
  sc->warm_start = 1;
  sc->warm_capacity_log2 = 22;
  sc->max_bytes_in_flight = 0;
  sc->fused_transform = 0;
}

extern "C" ogx_status ogx_server_create(int device, const ogx_config* cfg, const ogx_server_config* scfg,
                                        int num_bodies, const int32_t* counts, const float* local_xyz,
                                        ogx_server** out) {
  if (!out || !counts || !local_xyz || num_bodies <= 0) return ogx_fail(OGX_ERR_INVALID, "bad server arguments");
  *out = nullptr;
  ogx_server_config sc;
  ogx_server_config_default(&sc);
  if (scfg) sc = *scfg;
  if (sc.slots < 1 || sc.slots > 64 || sc.slot_pairs < 1 || sc.world_slots < 2 || sc.world_slots > 64 ||
      sc.max_pairs_in_flight < sc.slot_pairs || sc.warm_capacity_log2 < 10 || sc.warm_capacity_log2 > 30 ||
      sc.fused_transform < 0 || sc.fused_transform > 1 || sc.max_bytes_in_flight < 0)
    return ogx_fail(OGX_ERR_INVALID, "server config out of range");
  ogx_server* S = new ogx_server();
  S->sc = sc;
  ogx_status st = ogx_ctx_create(device, cfg, nullptr, &S->pctx);
  if (st) {
    delete S;
    return st;
  }
  S->device = S->pctx->device;
  S->cfg = S->pctx->cfg;
  st = ogx_pool_create(S->pctx, num_bodies, counts, &S->local);
  if (!st) st = ogx_pool_upload(S->pctx, S->local, local_xyz);
  cudaError_t e = cudaSuccess;
  const size_t nf = S->local ? S->local->nfloats : 0;
  for (int w = 0; !st && w < sc.world_slots; ++w) {
    float *dw = nullptr, *dx = nullptr, *hx = nullptr;
    cudaEvent_t ev = nullptr;
    if ((e = dalloc(&dw, nf)) != cudaSuccess || (e = dalloc(&dx, 12 * (size_t)num_bodies)) != cudaSuccess ||
        (e = halloc(&hx, 12 * (size_t)num_bodies)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
      st = ogx_cuda_fail(e, "server world buffers");
    S->d_world.push_back(dw);
    S->d_xf.push_back(dx);
    S->h_xf.push_back(hx);
    S->world_ready.push_back(ev);
    S->world_version.push_back(-1);
    S->world_refs.push_back(0);
    S->world_writing.push_back(0);
  }
  // Slots spread their size buckets over streams of their own only as far as the
  // process's hardware work queues go (CUDA_DEVICE_MAX_CONNECTIONS, 8 by default): a
  // slot needs its own stream, the refinement's and the bucket streams, and streams
  // beyond the queue count share queues and serialise behind unrelated work.
  const char* conn_env = std::getenv("CUDA_DEVICE_MAX_CONNECTIONS");
  const int conn = conn_env ? std::max(1, std::atoi(conn_env)) : 8;
  const int per_slot = (conn - 2) / sc.slots;  // two queues kept for the server's own streams
  for (int i = 0; !st && i < sc.slots; ++i) {
    S->slots.emplace_back();
    Slot& s = S->slots.back();
    st = ogx_ctx_create(S->device, &S->cfg, nullptr, &s.ctx);
    if (st) break;
    s.ctx->fork_ok = per_slot >= 4;
    s.ctx->fork_width = std::min(kBuckets, std::max(2, per_slot - 2));
    for (int k = 0; k < 2; ++k)
      for (int b = 0; b < kBuckets; ++b) s.ctx->choice[k][b] = S->pctx->choice[k][b];
    const size_t n = sc.slot_pairs;
    if ((e = dalloc(&s.d_pairs, n)) != cudaSuccess || (e = dalloc(&s.d_smp, n)) != cudaSuccess ||
        (e = dalloc(&s.d_dist, n)) != cudaSuccess || (e = dalloc(&s.d_nrm, 3 * n)) != cudaSuccess ||
        (e = dalloc(&s.d_status, n)) != cudaSuccess || (e = dalloc(&s.d_warm, n)) != cudaSuccess ||
        (e = halloc(&s.h_pairs, n)) != cudaSuccess || (e = halloc(&s.h_smp, n)) != cudaSuccess ||
        (e = halloc(&s.h_dist, n)) != cudaSuccess || (e = halloc(&s.h_nrm, 3 * n)) != cudaSuccess ||
        (e = halloc(&s.h_status, n)) != cudaSuccess ||
        (e = cudaEventCreate(&s.done)) != cudaSuccess || (e = cudaEventCreate(&s.start)) != cudaSuccess) {
      st = ogx_cuda_fail(e, "server slot buffers");
      break;
    }
    st = s.ctx->ensure_scratch(sc.slot_pairs);
    if (!st) st = ogx_broad_create(s.ctx, num_bodies, &s.broad);
    if (!st && ((e = dalloc(&s.d_bres, 2)) != cudaSuccess || (e = halloc(&s.h_bres, 2)) != cudaSuccess ||
                (e = cudaEventCreateWithFlags(&s.counted, cudaEventDisableTiming)) != cudaSuccess))
      st = ogx_cuda_fail(e, "server broad-phase buffers");
  }
  if (!st && sc.warm_start) {
    const size_t cap = (size_t)1 << sc.warm_capacity_log2;
    S->warm_mask = cap - 1;
    if ((e = dalloc(&S->d_keys, cap)) != cudaSuccess || (e = dalloc(&S->d_vals, cap)) != cudaSuccess ||
        (e = cudaMemset(S->d_keys, 0xff, cap * sizeof(unsigned long long))) != cudaSuccess)
      st = ogx_cuda_fail(e, "server warm-start table");
  }
  if (!st) {
    S->grid_aux = 4 * S->pctx->sm_count;
    if ((e = cudaStreamSynchronize(S->pctx->stream)) != cudaSuccess) st = ogx_cuda_fail(e, "server setup");
  }
  if (!st) {
    // a request's device working memory per pair: its pairs, results and warm-start
    // entries, and the pipeline's work lists (sized 1.25 x the pairs)
    S->bytes_per_pair = (int64_t)(sizeof(gkCollisionPair) + sizeof(gkSimplex) + 4 * sizeof(float) +
                                  sizeof(int32_t) + sizeof(int2)) +
                        (int64_t)(5 * ogx_scratch_bytes_per_pair()) / 4;
    S->max_bytes = sc.max_bytes_in_flight;
    if (S->max_bytes == 0) {
      size_t free_b = 0, total_b = 0;
      if ((e = cudaMemGetInfo(&free_b, &total_b)) != cudaSuccess) st = ogx_cuda_fail(e, "server memory info");
      S->max_bytes = (int64_t)(free_b / 2);
    }
  }
  if (st) {
    S->release();
    delete S;
    return st;
  }
  S->sched = std::thread([S] { S->loop(); });
  *out = S;
  return OGX_OK;
}

extern "C" ogx_status ogx_server_destroy(ogx_server* S) {
  if (!S) return OGX_OK;
  {
    std::unique_lock<std::mutex> lk(S->mu);
    S->stop = true;
    // a transform upload copies into a ring slot's staging and launches into its device
    // buffer without the lock: wait until none is under way before anything is freed
    auto writing = [&] {
      for (char c : S->world_writing)
        if (c) return true;
      return false;
    };
    const auto deadline = Clock::now() + std::chrono::seconds(10);
    while (writing())
      if (S->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && writing())
        return ogx_fail(OGX_ERR_BUSY, "a transform upload is still running after 10 s; server stopped, not freed");
  }
  S->cv_work.notify_all();
  if (S->sched.joinable()) S->sched.join();
  cudaSetDevice(S->device);
  for (Slot& s : S->slots)
    if (s.ctx) cudaStreamSynchronize(s.ctx->stream);
  S->release();
  delete S;
  return OGX_OK;
}

extern "C" ogx_status ogx_server_set_transforms(ogx_server* S, const float* xf, int64_t* version) {
  if (!S || !xf || !version) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  // a pose with a NaN or an infinity would put non-finite points into the world copy
  // that every request of the version reads: refuse the update
  {
    const size_t nf = 12 * (size_t)S->local->nbodies;
    for (size_t i = 0; i < nf; ++i)
      if (!ogx::is_finite(xf[i]))
        return ogx_fail(OGX_ERR_INVALID, "pose of body %zu has a NaN or infinite entry", i / 12);
  }
  std::unique_lock<std::mutex> lk(S->mu);
  if (S->stop) return ogx_fail(OGX_ERR_INVALID, "server is being destroyed");
  // the next version's ring slot must not be read by a request in flight or queued, nor
  // be written by another upload (another caller may take that version meanwhile)
  auto in_use = [&](int w) {
    if (S->world_refs[w] > 0 || S->world_writing[w]) return true;
    for (Request* r : S->queue)
      if (r->version % S->sc.world_slots == w && r->version == S->world_version[w]) return true;
    return false;
  };
  const auto deadline = Clock::now() + std::chrono::seconds(10);
  int64_t v_mine = S->next_version;
  int w = (int)(v_mine % S->sc.world_slots);
  while (in_use(w)) {
    if (S->cv_done.wait_until(lk, deadline) == std::cv_status::timeout) {
      v_mine = S->next_version;
      w = (int)(v_mine % S->sc.world_slots);
      if (in_use(w)) return ogx_fail(OGX_ERR_BUSY, "transform ring slot %d still in use after 10 s", w);
      break;
    }
    v_mine = S->next_version;
    w = (int)(v_mine % S->sc.world_slots);
  }
  // reserve the version and the slot, then stage and upload without the lock: the
  // scheduler keeps admitting and completing requests meanwhile (the copy into the pinned
  // staging alone takes ~0.3 ms for 20k bodies)
  S->next_version = v_mine + 1;
  S->world_version[w] = -1;
  S->world_writing[w] = 1;
  lk.unlock();
  cudaSetDevice(S->device);
  const size_t bytes = 12 * (size_t)S->local->nbodies * sizeof(float);
  // the pinned staging of this ring slot was last read by its previous transform upload
  cudaError_t e = cudaEventSynchronize(S->world_ready[w]);
  if (e == cudaSuccess) {
    std::memcpy(S->h_xf[w], xf, bytes);
    e = cudaMemcpyAsync(S->d_xf[w], S->h_xf[w], bytes, cudaMemcpyHostToDevice, S->pctx->stream);
  }
  if (e == cudaSuccess && !S->sc.fused_transform) {
    k_transform<<<8 * S->pctx->sm_count, 256, 0, S->pctx->stream>>>(S->local->d_points, S->local->d_bodies,
                                                                     S->local->nbodies, S->d_xf[w], S->d_world[w]);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(S->world_ready[w], S->pctx->stream);
  lk.lock();
  S->world_writing[w] = 0;
  if (e == cudaSuccess) S->world_version[w] = v_mine;
  lk.unlock();
  S->cv_done.notify_all();
  if (e != cudaSuccess) return ogx_cuda_fail(e, "server transform");
  *version = v_mine;
  return OGX_OK;
}

extern "C" ogx_status ogx_server_submit(ogx_server* S, int64_t version, int npairs, const gkCollisionPair* pairs,
                                        gkSimplex* simplices, float* distances, float* normals, int32_t* status,
                                        int64_t* ticket) {
  if (!S || !ticket || (!pairs && npairs > 0)) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  if (npairs < 0 || npairs > S->sc.slot_pairs)
    return ogx_fail(OGX_ERR_CAPACITY, "a request holds at most %d pairs (got %d)", S->sc.slot_pairs, npairs);
  Request* r = new Request();
  r->npairs = npairs;
  r->pairs.assign(pairs, pairs + npairs);
  r->out_smp = simplices;
  r->out_dist = distances;
  r->out_nrm = normals;
  r->out_status = status;
  r->version = version;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (version < 0 || version >= S->next_version ||
        S->world_version[version % S->sc.world_slots] != version) {
      delete r;
      return ogx_fail(OGX_ERR_INVALID, "transform version %lld is not resident", (long long)version);
    }
    r->id = S->next_id++;
    S->reqs[r->id] = r;
    if (npairs == 0) {
      r->state = 2;
      r->t_done = r->t_submit;
    } else {
      S->queue.push_back(r);
    }
    *ticket = r->id;
  }
  S->cv_work.notify_all();
  return OGX_OK;
}

extern "C" ogx_status ogx_server_wait(ogx_server* S, int64_t ticket, double timeout_s, double* latency_ms) {
  return ogx_server_wait_phases(S, ticket, timeout_s, latency_ms, nullptr);
}

extern "C" ogx_status ogx_server_wait_phases(ogx_server* S, int64_t ticket, double timeout_s, double* latency_ms,
                                             double* phases_ms) {
  if (!S) return ogx_fail(OGX_ERR_INVALID, "NULL server");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return ogx_fail(OGX_ERR_INVALID, "unknown ticket %lld", (long long)ticket);
  Request* r = it->second;
  const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                          std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9));
  while (r->state < 2) {
    if (S->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && r->state < 2)
      return ogx_fail(OGX_ERR_BUSY, "request %lld not done", (long long)ticket);
  }
  const ogx_status err = r->state == 3 ? r->err : OGX_OK;
  auto ms = [](Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
  };
  const double lat = ms(r->t_submit, r->t_done);
  if (latency_ms) *latency_ms = lat;
  if (phases_ms) {
    const bool ran = r->state == 2 && r->npairs > 0;
    phases_ms[0] = ran ? ms(r->t_submit, r->t_admit) : 0.0;
    phases_ms[1] = ran ? ms(r->t_admit, r->t_staged) : 0.0;
    phases_ms[2] = ran ? (double)r->device_ms : 0.0;
    phases_ms[3] = ran ? lat - phases_ms[0] - phases_ms[1] - phases_ms[2] : 0.0;
  }
  S->reqs.erase(it);
  delete r;
  return err;
}

extern "C" ogx_status ogx_server_submit_broadphase(ogx_server* S, int64_t version, float cell, float margin,
                                                    int max_pairs, gkCollisionPair* pairs, int32_t* count,
                                                    gkSimplex* simplices, float* distances, float* normals,
                                                    int32_t* status, int64_t* ticket) {
  if (!S || !ticket) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  if (!(cell > 0.0f) || !(margin >= 0.0f) || max_pairs < 1)
    return ogx_fail(OGX_ERR_INVALID, "bad broad-phase arguments");
  if (S->sc.fused_transform)
    return ogx_fail(OGX_ERR_INVALID, "broad-phase requests read the world copy, which a fused-transform server does not keep");
  Request* r = new Request();
  r->broad = true;
  r->cell = cell;
  r->margin = margin;
  r->max_pairs = std::min(max_pairs, S->sc.slot_pairs);
  r->out_pairs = pairs;
  r->out_count = count;
  r->out_smp = simplices;
  r->out_dist = distances;
  r->out_nrm = normals;
  r->out_status = status;
  r->version = version;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (version < 0 || version >= S->next_version ||
        S->world_version[version % S->sc.world_slots] != version) {
      delete r;
      return ogx_fail(OGX_ERR_INVALID, "transform version %lld is not resident", (long long)version);
    }
    r->id = S->next_id++;
    S->reqs[r->id] = r;
    S->queue.push_back(r);
    *ticket = r->id;
  }
  S->cv_work.notify_all();
  return OGX_OK;
}

extern "C" ogx_status ogx_server_poll(ogx_server* S, int64_t ticket, int* done) {
  if (!S || !done) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return ogx_fail(OGX_ERR_INVALID, "unknown ticket %lld", (long long)ticket);
  *done = it->second->state >= 2;
  return OGX_OK;
}

extern "C" ogx_status ogx_server_admission(ogx_server* S, int64_t* max_pairs, int64_t* max_bytes,
                                           int64_t* bytes_per_pair, int64_t* peak_bytes) {
  if (!S) return ogx_fail(OGX_ERR_INVALID, "NULL server");
  std::lock_guard<std::mutex> lk(S->mu);
  if (max_pairs) *max_pairs = S->sc.max_pairs_in_flight;
  if (max_bytes) *max_bytes = S->max_bytes;
  if (bytes_per_pair) *bytes_per_pair = S->bytes_per_pair;
  if (peak_bytes) *peak_bytes = S->peak_bytes;
  return OGX_OK;
}

extern "C" ogx_status ogx_server_world_layout(ogx_server* S, int64_t version, float** d_points, void** d_bodies) {
  if (!S || !d_points || !d_bodies) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(S->mu);
  const int w = (int)(version % S->sc.world_slots);
  if (version < 0 || S->world_version[w] != version)
    return ogx_fail(OGX_ERR_INVALID, "transform version %lld is not resident", (long long)version);
  if (S->sc.fused_transform)
    return ogx_fail(OGX_ERR_INVALID, "a fused-transform server keeps no world copy");
  *d_points = S->d_world[w];
  *d_bodies = S->local->d_bodies;
  return OGX_OK;
}
