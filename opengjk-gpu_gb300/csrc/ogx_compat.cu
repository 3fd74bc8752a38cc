// ogx_compat.cu -- the reference-compatible half of the C ABI: OpenGJK-GPU's host API
// (GJK/gpu/openGJK.h, examples/gpu/example.h) re-implemented on the engine.
//
// The reference functions take gkPolytope descriptors (point count + pointer to xyz
// interleaved coordinates), either in host memory (high-level calls) or in device memory
// (mid-level *_device and indexed calls, whose coordinates a caller may rewrite with its
// own kernels between calls).  Every call here copies the referenced bodies into the
// engine's padded SoA pool (on the device: a count -> prefix-sum -> pack sequence), runs
// the engine pipeline and, like the reference, returns when the results are complete.
// Each call leases an engine context of its own (stream, pool and result buffers) from a
// per-device free list, created on first need: calls from several host threads run side
// by side, and a thread's calls reuse warm contexts.
//
// Deliberate differences from the reference (documented bugs not reproduced):
//  * computeCollisionInformation uploads the input distances (the reference does not,
//    GJK/gpu/openGJK.cu:2838-2845, so its EPA reads uninitialised memory);
//  * contact_normals may be NULL where the reference documents it as nullable
//    (examples/gpu/example.h:39) -- the reference writes through it regardless.
#include <cuda_runtime.h>

#include <atomic>
#include <string.h>

#include <algorithm>
#include <cstdlib>
#include <condition_variable>
#include <deque>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "ogx_engine.h"

using namespace ogx;

namespace {

// ---------------------------------------------------------------------------------
// device kernels: descriptor arrays -> pool

// source descriptor of pool body i: body 2k / 2k+1 of pair k, taken from two arrays
// (bd1[k], bd2[k]) or from one array through a device pair list (a[pairs[k].idx1],
// a[pairs[k].idx2]).  Negative indices give an empty descriptor (rejected).
struct DescSrc {
  const gkPolytope* a;
  const gkPolytope* b;              // second array, or null
  const gkCollisionPair* pairs;     // pair list into a, or null
  __device__ gkPolytope get(int i) const {
    if (pairs) {
      const gkCollisionPair p = pairs[i >> 1];
      const int idx = (i & 1) ? p.idx2 : p.idx1;
      if (idx < 0) {
        gkPolytope z;
        z.numpoints = 0;
        z.coord = nullptr;
        return z;
      }
      return a[idx];
    }
    return (i & 1) ? b[i >> 1] : a[i >> 1];
  }
};

constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;
constexpr int kScanChunk = kScanBlock * kScanItems;

__device__ __forceinline__ uint32_t quads_of(int n) { return n < 1 ? 0u : 3u * (uint32_t)((n + 3) / 4); }

// block-wide exclusive scan of one value per thread (1024 threads)
__device__ uint32_t block_excl_scan(uint32_t x, uint32_t* total) {
  __shared__ uint32_t warp_sums[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t inc = x;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_sums[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    uint32_t s = warp_sums[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    warp_sums[lane] = s;
  }
  __syncthreads();
  const uint32_t base = wid ? warp_sums[wid - 1] : 0u;
  if (total) *total = warp_sums[31];
  __syncthreads();
  return base + inc - x;
}

__global__ void __launch_bounds__(kScanBlock) k_desc_sums(DescSrc src, int nb, uint32_t* block_sums) {
  const int base = blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
  uint32_t s = 0;
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < nb) s += quads_of(src.get(base + k).numpoints);
  uint32_t tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

// one block: exclusive scan of the block sums in place; grand total and validity flag
__global__ void __launch_bounds__(kScanBlock) k_scan_sums(uint32_t* sums, int nblocks, uint32_t* total) {
  uint32_t carry = 0;
  for (int start = 0; start < nblocks; start += kScanBlock) {
    const int i = start + threadIdx.x;
    const uint32_t x = i < nblocks ? sums[i] : 0u;
    uint32_t t;
    const uint32_t e = block_excl_scan(x, &t);
    if (i < nblocks) sums[i] = carry + e;
    carry += t;
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kScanBlock) k_desc_offsets(DescSrc src, int nb, const uint32_t* block_base,
                                                             BodyRef* bodies, int* bad) {
  const int base = blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
  int nn[kScanItems];
  uint32_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    nn[k] = base + k < nb ? src.get(base + k).numpoints : 0;
    s += quads_of(nn[k]);
  }
  uint32_t off = block_excl_scan(s, nullptr) + block_base[blockIdx.x];
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k >= nb) break;
    BodyRef r;
    r.quad = off;
    r.n = nn[k];
    bodies[base + k] = r;
    if (nn[k] < 1) atomicExch(bad, 1);
    off += quads_of(nn[k]);
  }
}

// bodies with a NaN or infinite coordinate are marked as k_pack does (negated count)
__global__ void k_desc_pack(DescSrc src, int nb, BodyRef* __restrict__ bodies, float* __restrict__ pool) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int b = warp; b < nb; b += nwarps) {
    const BodyRef r = bodies[b];
    if (r.n < 1) continue;
    const float* c = src.get(b).coord;
    const int n4 = round4(r.n);
    float* dst = pool + 4 * (size_t)r.quad;
    bool finite = true;
    for (int i = lane; i < n4; i += 32) {
      const int s = i < r.n ? i : 0;
      const float x = c[3 * s], y = c[3 * s + 1], z = c[3 * s + 2];
      finite = finite && is_finite(x) && is_finite(y) && is_finite(z);
      dst[i] = x;
      dst[n4 + i] = y;
      dst[2 * n4 + i] = z;
    }
    finite = __all_sync(0xffffffffu, finite);
    if (lane == 0 && !finite) bodies[b].n = -r.n;
  }
}

// Bodies given in double (the *_f64 calls): every separated pair continues GJK in FP64 on
// the caller's double points from the FP32 pass's final simplex -- exact supports and
// exact Minkowski points, one thread per pair -- so its distance carries no rounding of
// the inputs; its simplex, witnesses and normal are replaced with the continuation's.
// Contacts keep the FP32 pass's result (their depth is within the inputs' rounding of
// the FP64 one, far inside the 1e-4 depth tolerance); a pair the continuation finds
// enclosed lies within rounding of touching and keeps it too.
__global__ void __launch_bounds__(128) k_refine64(const float* __restrict__ pool, const BodyRef* __restrict__ bodies,
                                                  const double* __restrict__ c64, const int64_t* __restrict__ voff,
                                                  const int2* __restrict__ pairs, int npairs, gkSimplex* smp,
                                                  float* dist, float* nrm) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += gridDim.x * blockDim.x) {
    const float dp = dist[p];
    if (!(dp > FLT_EPSILON)) continue;  // contacts, and bad input (NaN)
    const int2 pr = pairs[p];
    const BodyRef ra = bodies[pr.x], rb = bodies[pr.y];
    if (ra.n < 1 || rb.n < 1) continue;
    D64Bodies B;
    B.bind64(pool, ra, rb, c64 + 3 * voff[pr.x], c64 + 3 * voff[pr.y]);
    GjkState g;
    load_simplex(smp + p, dp, g);
    if (smp[p].nvrtx < 1 || smp[p].nvrtx > 3) continue;
    g.certain = false;
    g.status = 0;
    SerialTeam t;
    gjk_refine(t, B, g, kRefineIters);
    if (gjk_contact(g)) continue;
    store_simplex(smp + p, g);
    dist[p] = g.dist;
    if (nrm) store3(nrm + 3 * (size_t)p, sep_normal(g));
  }
}

__global__ void k_pairs_iota(gkCollisionPair* pairs, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    pairs[i].idx1 = 2 * i;
    pairs[i].idx2 = 2 * i + 1;
  }
}

// ---------------------------------------------------------------------------------
// shared state of the compatible API

struct Compat {
  ogx_ctx* ctx = nullptr;
  // device pool built per call
  float* d_points = nullptr;
  size_t points_cap = 0;  // floats
  BodyRef* d_bodies = nullptr;
  size_t bodies_cap = 0;
  int64_t* d_voff = nullptr;
  size_t voff_cap = 0;
  uint32_t* d_scan = nullptr;  // block sums + total + flag
  size_t scan_cap = 0;
  // pairs and results for host-buffer calls
  gkCollisionPair* d_pairs = nullptr;
  size_t pairs_cap = 0;
  gkSimplex* d_smp = nullptr;
  size_t smp_cap = 0;
  float* d_dist = nullptr;
  size_t dist_cap = 0;
  float* d_nrm = nullptr;
  size_t nrm_cap = 0;
  double* d_c64 = nullptr;  // the *_f64 calls: the bodies' double coordinates, pool order
  size_t c64_cap = 0;
  const float** d_src = nullptr;  // per body: the caller's coordinate pointer (k_pack_ptrs)
  size_t src_cap = 0;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  float last_ms = 0.0f;
  // page-locked staging of the results of host-buffer calls into pageable caller arrays
  char* h_res = nullptr;
  size_t h_res_bytes = 0;
};

constexpr int kMaxDevices = 16;
std::mutex g_compat_mu;  // guards the free lists
std::vector<Compat*> g_free[kMaxDevices];
thread_local float t_last_ms = 0.0f;  // GPU time of this thread's last call

template <class T>
ogx_status grow(T** p, size_t* cap, size_t need, const char* what) {
  if (need <= *cap && *p) return OGX_OK;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const size_t n = std::max<size_t>(need + need / 4, 256);
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
  if (e != cudaSuccess) return ogx_cuda_fail(e, what);
  *cap = n;
  return OGX_OK;
}

// Host worker threads for the calls' parallel host loops, started on first use and kept
// for the process (a call used to start up to 16 threads for each of its loops, ~100
// thread starts a call).  run(n, fn) runs fn(k) for k = 1..n-1 on the workers and fn(0)
// on the caller, and returns when all have run; calls from several host threads share
// the workers (their pieces queue in order).
class HostWorkers {
 public:
  static HostWorkers& get() {
    static HostWorkers w;
    return w;
  }
  int size() const { return (int)threads_.size(); }
  void run(int n, const std::function<void(int)>& fn) {
    if (n <= 1 || threads_.empty()) {
      for (int k = 0; k < std::max(n, 1); ++k) fn(k);
      return;
    }
    Group g{&fn, 0};
    {
      std::lock_guard<std::mutex> lk(mu_);
      for (int k = 1; k < n; ++k) queue_.push_back(Task{&g, k});
    }
    cv_.notify_all();
    fn(0);
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return g.done == n - 1; });
  }
  ~HostWorkers() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : threads_) t.join();
  }

 private:
  struct Group {
    const std::function<void(int)>* fn;
    int done;
  };
  struct Task {
    Group* g;
    int k;
  };
  HostWorkers() {
    const int hw = (int)std::thread::hardware_concurrency();
    const int n = std::max(0, std::min(15, hw - 1));
    for (int i = 0; i < n; ++i) threads_.emplace_back([this] { loop(); });
  }
  void loop() {
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      cv_.wait(lk, [&] { return stop_ || !queue_.empty(); });
      if (queue_.empty()) return;  // stopping
      const Task t = queue_.front();
      queue_.pop_front();
      lk.unlock();
      (*t.g->fn)(t.k);
      lk.lock();
      ++t.g->done;
      done_cv_.notify_all();
    }
  }
  std::vector<std::thread> threads_;
  std::deque<Task> queue_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  bool stop_ = false;
};

// Host copy of `bytes` bytes on up to 16 threads (one for small copies).
void parallel_copy(void* dst, const void* src, size_t bytes) {
  const int nt = (int)std::min<size_t>(16, std::max<size_t>(1, bytes >> 22));
  if (nt == 1) {
    memcpy(dst, src, bytes);
    return;
  }
  HostWorkers::get().run(nt, [=](int k) {
    const size_t a = bytes * k / nt, b = bytes * (k + 1) / nt;
    memcpy(static_cast<char*>(dst) + a, static_cast<const char*>(src) + a, b - a);
  });
}

// fn(lo, hi, k) over [0, n) in nt contiguous pieces, piece k on a worker (the caller's
// thread takes piece 0)
template <class F>
void parallel_for(int n, int nt, F fn) {
  HostWorkers::get().run(nt, [&](int k) { fn((int)((int64_t)n * k / nt), (int)((int64_t)n * (k + 1) / nt), k); });
}

// Host-buffer calls pack the caller's points on the device (k_pack_ptrs) where it reads
// pageable host memory directly (ogx_pageable_reads); OGX_COMPAT_GATHER=1 in the
// environment forces the host gather instead.
bool pageable_reads(int dev) {
  const char* force = std::getenv("OGX_COMPAT_GATHER");
  if (force && force[0] == '1') return false;
  return ogx_pageable_reads(dev);
}

bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// A context leased for the duration of one call; back on its device's free list after.
struct Lease {
  Compat* c = nullptr;
  int dev = 0;
  Lease() = default;
  Lease(const Lease&) = delete;
  Lease& operator=(const Lease&) = delete;
  ~Lease() {
    if (!c) return;
    std::lock_guard<std::mutex> lk(g_compat_mu);
    g_free[dev].push_back(c);
  }
};

ogx_status lease(Lease& L) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return ogx_fail(OGX_ERR_NO_DEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
  }
  if (dev < 0 || dev >= kMaxDevices) return ogx_fail(OGX_ERR_INVALID, "device index %d", dev);
  L.dev = dev;
  {
    std::lock_guard<std::mutex> lk(g_compat_mu);
    if (!g_free[dev].empty()) {
      L.c = g_free[dev].back();
      g_free[dev].pop_back();
      return OGX_OK;
    }
  }
  Compat* c = new Compat();
  ogx_status s = ogx_ctx_create(dev, nullptr, nullptr, &c->ctx);
  if (s) {
    delete c;
    return s;
  }
  cudaEventCreate(&c->t0);
  cudaEventCreate(&c->t1);
  L.c = c;
  return OGX_OK;
}

// Build the pool from descriptors that live in DEVICE memory (nb bodies).
ogx_status pool_from_device_desc(Compat& c, DescSrc src, int nb) {
  cudaStream_t st = c.ctx->stream;
  const int nblocks = (nb + kScanChunk - 1) / kScanChunk;
  ogx_status s = grow(&c.d_bodies, &c.bodies_cap, (size_t)nb, "compat body table");
  if (!s) s = grow(&c.d_scan, &c.scan_cap, (size_t)nblocks + 2, "compat scan buffer");
  if (s) return s;
  cudaMemsetAsync(c.d_scan + nblocks + 1, 0, sizeof(uint32_t), st);
  k_desc_sums<<<nblocks, kScanBlock, 0, st>>>(src, nb, c.d_scan);
  k_scan_sums<<<1, kScanBlock, 0, st>>>(c.d_scan, nblocks, c.d_scan + nblocks);
  k_desc_offsets<<<nblocks, kScanBlock, 0, st>>>(src, nb, c.d_scan, c.d_bodies,
                                                 reinterpret_cast<int*>(c.d_scan + nblocks + 1));
  uint32_t tot[2];
  cudaError_t e = cudaMemcpyAsync(tot, c.d_scan + nblocks, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "descriptor scan");
  if (tot[1]) return ogx_fail(OGX_ERR_INVALID, "a polytope has numpoints < 1");
  s = grow(&c.d_points, &c.points_cap, 4 * (size_t)tot[0] + 4, "compat pool");
  if (s) return s;
  const int grid = std::min(8 * c.ctx->sm_count, (nb + 7) / 8);
  k_desc_pack<<<std::max(grid, 1), 256, 0, st>>>(src, nb, c.d_bodies, c.d_points);
  e = cudaGetLastError();
  if (e != cudaSuccess) return ogx_cuda_fail(e, "descriptor pack");
  return OGX_OK;
}

// The pool's body table from host descriptors (pairs (a[i], b[i]) when b is given, else
// the bodies of a), in two parallel passes over pieces of the descriptors: per piece the
// point and float4-block totals (and the first invalid descriptor), then, after a prefix
// over the pieces, every body's offsets.
struct HostTables {
  std::vector<int32_t> counts;
  std::vector<const float*> src;
  std::vector<int64_t> voff;
  std::vector<BodyRef> refs;
  int64_t pts = 0;
  uint64_t quad = 0;
};

ogx_status host_tables(const gkPolytope* a, const gkPolytope* b, int nb, HostTables& T) {
  T.counts.resize(nb);
  T.src.resize(nb);
  T.voff.resize(nb);
  T.refs.resize(nb);
  std::vector<int32_t>& counts = T.counts;
  std::vector<const float*>& src = T.src;
  std::vector<int64_t>& voff = T.voff;
  std::vector<BodyRef>& refs = T.refs;
  const int nt = (int)std::min<int64_t>(16, std::max<int64_t>(1, nb >> 15));
  std::vector<int64_t> piece_pts(nt + 1, 0), piece_quad(nt + 1, 0);
  std::vector<int> bad(nt, -1);
  parallel_for(nb, nt, [&](int lo, int hi, int k) {
    int64_t np = 0, nq = 0;
    for (int i = lo; i < hi; ++i) {
      const gkPolytope& p = b ? ((i & 1) ? b[i >> 1] : a[i >> 1]) : a[i];
      if (p.numpoints < 1 || !p.coord) {
        bad[k] = i;
        return;
      }
      counts[i] = p.numpoints;
      src[i] = p.coord;
      np += p.numpoints;
      nq += 3 * (int64_t)((p.numpoints + 3) / 4);
    }
    piece_pts[k + 1] = np;
    piece_quad[k + 1] = nq;
  });
  for (int k = 0; k < nt; ++k)
    if (bad[k] >= 0) {
      const gkPolytope& p = b ? ((bad[k] & 1) ? b[bad[k] >> 1] : a[bad[k] >> 1]) : a[bad[k]];
      return ogx_fail(OGX_ERR_INVALID, "polytope %d: numpoints %d, coord %p", bad[k], p.numpoints, (void*)p.coord);
    }
  for (int k = 0; k < nt; ++k) {
    piece_pts[k + 1] += piece_pts[k];
    piece_quad[k + 1] += piece_quad[k];
  }
  T.pts = piece_pts[nt];
  T.quad = (uint64_t)piece_quad[nt];
  if (T.quad >= (1ull << 32)) return ogx_fail(OGX_ERR_CAPACITY, "pool exceeds 2^32 float4 blocks");
  parallel_for(nb, nt, [&](int lo, int hi, int k) {
    int64_t np = piece_pts[k], nq = piece_quad[k];
    for (int i = lo; i < hi; ++i) {
      voff[i] = np;
      refs[i].quad = (uint32_t)nq;
      refs[i].n = counts[i];
      np += counts[i];
      nq += 3 * (int64_t)((counts[i] + 3) / 4);
    }
  });
  return OGX_OK;
}

// The body table, the coordinate pointers and the offsets up (a device that reads
// pageable memory packs the points from the caller's arrays itself), the pool grown.
ogx_status upload_tables(Compat& c, const HostTables& T, int nb) {
  ogx_ctx* ctx = c.ctx;
  cudaStream_t st = ctx->stream;
  const size_t tb = nb * sizeof(BodyRef), pb = nb * sizeof(const float*), ob = nb * sizeof(int64_t);
  ogx_status s = ctx->ensure_stage(tb + pb + ob, 0);
  if (!s) s = grow(&c.d_bodies, &c.bodies_cap, (size_t)nb, "compat body table");
  if (!s) s = grow(&c.d_src, &c.src_cap, (size_t)nb, "compat coordinate pointers");
  if (!s) s = grow(&c.d_voff, &c.voff_cap, (size_t)nb, "compat offsets");
  if (!s) s = grow(&c.d_points, &c.points_cap, 4 * (size_t)T.quad + 4, "compat pool");
  if (s) return s;
  cudaStreamSynchronize(st);  // staging buffers may still be read by a previous call
  char* h = static_cast<char*>(ctx->h_stage);
  parallel_copy(h, T.refs.data(), tb);
  parallel_copy(h + tb, T.src.data(), pb);
  parallel_copy(h + tb + pb, T.voff.data(), ob);
  cudaError_t e = cudaMemcpyAsync(c.d_bodies, h, tb, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c.d_src, h + tb, pb, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c.d_voff, h + tb + pb, ob, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "body table upload");
  return OGX_OK;
}

// Build the pool from descriptors in HOST memory with host coordinates.
ogx_status pool_from_host_desc(Compat& c, const gkPolytope* a, const gkPolytope* b, int nb) {
  HostTables T;
  ogx_status s0 = host_tables(a, b, nb, T);
  if (s0) return s0;
  const std::vector<int32_t>& counts = T.counts;
  const std::vector<const float*>& src = T.src;
  const std::vector<int64_t>& voff = T.voff;
  const std::vector<BodyRef>& refs = T.refs;
  const int64_t pts = T.pts;
  const uint64_t quad = T.quad;
  ogx_ctx* ctx = c.ctx;
  cudaStream_t st = ctx->stream;
  const size_t bytes = (size_t)pts * 3 * sizeof(float);
  if (pageable_reads(ctx->device)) {
    // the body table and the coordinate pointers up, the points packed from where the
    // caller keeps them
    ogx_status s = upload_tables(c, T, nb);
    if (s) return s;
    const cudaError_t e = launch_pack_ptrs(c.d_src, nb, c.d_bodies, c.d_points, 8 * ctx->sm_count, st);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "polytope pack from host memory");
    return OGX_OK;
  }
  ogx_status s = ctx->ensure_stage(bytes + nb * (sizeof(BodyRef) + sizeof(int64_t)), bytes);
  if (!s) s = grow(&c.d_bodies, &c.bodies_cap, (size_t)nb, "compat body table");
  if (!s) s = grow(&c.d_voff, &c.voff_cap, (size_t)nb, "compat offsets");
  if (!s) s = grow(&c.d_points, &c.points_cap, 4 * (size_t)quad + 4, "compat pool");
  if (s) return s;
  cudaStreamSynchronize(st);  // staging buffers may still be read by a previous call
  char* h = static_cast<char*>(ctx->h_stage);
  // Gather the coordinates into the pinned staging in pieces of bodies, on up to 16
  // threads, and upload each piece as soon as it is gathered: the copy engine moves piece
  // k while the threads gather piece k + 1.
  // (no more shares than workers + this thread: share 0 waits for the others' pieces)
  const int gt = (int)std::min<int64_t>(std::min(16, HostWorkers::get().size() + 1), std::max<int64_t>(1, pts >> 18));
  const int pieces = bytes >= ((size_t)64 << 20) ? 8 : 1;
  std::vector<std::atomic<int>> gathered(pieces);
  for (auto& g : gathered) g.store(0);
  auto piece_begin = [&](int pc) { return (int)((int64_t)nb * pc / pieces); };
  // shares 1..gt-1 of every piece on the workers, share 0 and the uploads on this thread
  cudaError_t e = cudaSuccess;
  HostWorkers::get().run(gt, [&](int k) {
    for (int pc = 0; pc < pieces; ++pc) {
      const int i0 = piece_begin(pc), i1 = piece_begin(pc + 1);
      for (int i = (int)(i0 + (int64_t)(i1 - i0) * k / gt); i < (int)(i0 + (int64_t)(i1 - i0) * (k + 1) / gt); ++i)
        memcpy(h + voff[i] * 12, src[i], (size_t)counts[i] * 12);
      if (k > 0) {
        gathered[pc].fetch_add(1);
        continue;
      }
      while (gathered[pc].load() < gt - 1) std::this_thread::yield();
      const size_t b0 = (size_t)voff[i0] * 12, b1 = i1 < nb ? (size_t)voff[i1] * 12 : bytes;
      if (e == cudaSuccess && b1 > b0)
        e = cudaMemcpyAsync(static_cast<char*>(ctx->d_stage) + b0, h + b0, b1 - b0, cudaMemcpyHostToDevice, st);
    }
  });
  memcpy(h + bytes, refs.data(), nb * sizeof(BodyRef));
  memcpy(h + bytes + nb * sizeof(BodyRef), voff.data(), nb * sizeof(int64_t));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c.d_bodies, h + bytes, nb * sizeof(BodyRef), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c.d_voff, h + bytes + nb * sizeof(BodyRef), nb * sizeof(int64_t),
                        cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "polytope upload");
  ogx_pool tmp;
  tmp.ctx = ctx;
  tmp.nbodies = nb;
  tmp.npoints = pts;
  tmp.d_points = c.d_points;
  tmp.d_bodies = c.d_bodies;
  tmp.d_voff = c.d_voff;
  return pool_pack(ctx, &tmp, static_cast<const float*>(ctx->d_stage));
}

ogx_status ensure_results(Compat& c, int n) {
  ogx_status s = grow(&c.d_pairs, &c.pairs_cap, (size_t)n, "compat pairs");
  if (!s) s = grow(&c.d_smp, &c.smp_cap, (size_t)n, "compat simplices");
  if (!s) s = grow(&c.d_dist, &c.dist_cap, (size_t)n, "compat distances");
  if (!s) s = grow(&c.d_nrm, &c.nrm_cap, 3 * (size_t)n, "compat normals");
  return s;
}

ogx_status run_timed(Compat& c, int nbodies, int npairs, const gkCollisionPair* d_pairs, gkSimplex* d_smp,
                     float* d_dist, float* d_nrm, int mode, bool exact64 = false) {
  cudaEventRecord(c.t0, c.ctx->stream);
  ogx_status s = ogx_run(c.ctx, c.d_points, c.d_bodies, nbodies, npairs, d_pairs, d_smp, d_dist, d_nrm,
                         nullptr, mode);
  if (!s && exact64 && mode != kModeEpa) {
    const int grid = std::min(8 * c.ctx->sm_count, (npairs + 127) / 128);
    k_refine64<<<std::max(grid, 1), 128, 0, c.ctx->stream>>>(c.d_points, c.d_bodies, c.d_c64, c.d_voff,
                                                            reinterpret_cast<const int2*>(d_pairs), npairs,
                                                            d_smp, d_dist, mode == kModeGjk ? nullptr : d_nrm);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) s = ogx_cuda_fail(e, "k_refine64 launch");
  }
  cudaEventRecord(c.t1, c.ctx->stream);
  if (s) return s;
  cudaError_t e = cudaStreamSynchronize(c.ctx->stream);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "engine pipeline");
  cudaEventElapsedTime(&c.last_ms, c.t0, c.t1);
  t_last_ms = c.last_ms;
  return OGX_OK;
}

ogx_status finish(Compat& c) {
  cudaError_t e = cudaStreamSynchronize(c.ctx->stream);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "copy back");
  return OGX_OK;
}

// host-buffer query over pairs (2i, 2i+1) or explicit pairs; results to host arrays
ogx_status host_query(const gkPolytope* a, const gkPolytope* b, int nbodies, int npairs,
                      const gkCollisionPair* host_pairs, gkSimplex* smp, float* dist, float* nrm,
                      float* w1, float* w2, int mode, bool upload_in, const ogx_polytope_f64* a64 = nullptr,
                      const ogx_polytope_f64* b64 = nullptr) {
  if (npairs <= 0) return OGX_OK;  // the reference returns early for n <= 0
  if (!a || !smp || !dist) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  Lease L;
  ogx_status s = lease(L);
  if (s) return s;
  Compat* c = L.c;
  cudaStream_t st = c->ctx->stream;
  s = pool_from_host_desc(*c, a, b, nbodies);
  if (!s) s = ensure_results(*c, npairs);
  if (s) return s;
  std::vector<double> c64;
  if (a64) {
    // the double coordinates in the pool's body order (body i as pool_from_host_desc)
    for (int i = 0; i < nbodies; ++i) {
      const ogx_polytope_f64& p = b64 ? ((i & 1) ? b64[i >> 1] : a64[i >> 1]) : a64[i];
      c64.insert(c64.end(), p.coord, p.coord + 3 * (size_t)p.numpoints);
    }
    s = grow(&c->d_c64, &c->c64_cap, std::max<size_t>(c64.size(), 1), "compat double coordinates");
    if (s) return s;
  }
  cudaError_t e = cudaSuccess;
  if (a64) e = cudaMemcpyAsync(c->d_c64, c64.data(), c64.size() * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "double coordinate upload");
  if (host_pairs) {
    const int nt = (int)std::min<int64_t>(16, std::max<int64_t>(1, npairs >> 16));
    std::vector<int> bad(nt, -1);
    parallel_for(npairs, nt, [&](int lo, int hi, int k) {
      for (int i = lo; i < hi; ++i)
        if (host_pairs[i].idx1 < 0 || host_pairs[i].idx1 >= nbodies || host_pairs[i].idx2 < 0 ||
            host_pairs[i].idx2 >= nbodies) {
          bad[k] = i;
          return;
        }
    });
    for (int k = 0; k < nt; ++k)
      if (bad[k] >= 0) return ogx_fail(OGX_ERR_INVALID, "pair %d: index out of range", bad[k]);
    e = cudaMemcpyAsync(c->d_pairs, host_pairs, npairs * sizeof(gkCollisionPair), cudaMemcpyHostToDevice, st);
  } else {
    k_pairs_iota<<<std::min(1024, (npairs + 255) / 256), 256, 0, st>>>(c->d_pairs, npairs);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && upload_in) {
    e = cudaMemcpyAsync(c->d_smp, smp, npairs * sizeof(gkSimplex), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_dist, dist, npairs * sizeof(float), cudaMemcpyHostToDevice, st);
  }
  if (e != cudaSuccess) return ogx_cuda_fail(e, "input upload");
  s = run_timed(*c, nbodies, npairs, c->d_pairs, c->d_smp, c->d_dist, c->d_nrm, mode, a64 != nullptr);
  if (s) return s;
  // Results: straight into page-locked caller arrays; pageable ones through the pinned
  // staging (a full-rate copy) and a parallel host copy.  (Writing pageable arrays from
  // a copy kernel, where the device can, measured slower: a caller's fresh result arrays
  // are first touched by the device, and the page faults are taken on its side.)
  const bool want_nrm = nrm && mode != kModeGjk;
  const size_t sb = npairs * sizeof(gkSimplex), db = npairs * sizeof(float), nbytes = 3 * db;
  const bool direct = is_pinned(smp) && is_pinned(dist) && (!want_nrm || is_pinned(nrm));
  char* hs = nullptr;
  if (!direct) {
    const size_t need = sb + db + (want_nrm ? nbytes : 0);
    if (need > c->h_res_bytes) {
      if (c->h_res) cudaFreeHost(c->h_res);
      c->h_res = nullptr;
      c->h_res_bytes = 0;
      if ((e = cudaMallocHost(&c->h_res, need)) != cudaSuccess) return ogx_cuda_fail(e, "pinned result staging");
      c->h_res_bytes = need;
    }
    hs = c->h_res;
  }
  e = cudaMemcpyAsync(direct ? (void*)smp : hs, c->d_smp, sb, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(direct ? (void*)dist : hs + sb, c->d_dist, db, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && want_nrm)
    e = cudaMemcpyAsync(direct ? (void*)nrm : hs + sb + db, c->d_nrm, nbytes, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "result copy");
  s = finish(*c);
  if (s) return s;
  if (!direct) {
    parallel_copy(smp, hs, sb);
    parallel_copy(dist, hs + sb, db);
    if (want_nrm) parallel_copy(nrm, hs + sb + db, nbytes);
  }
  if (w1 || w2) {
    for (int i = 0; i < npairs; ++i)
      for (int k = 0; k < 3; ++k) {
        if (w1) w1[3 * i + k] = smp[i].witnesses[0][k];
        if (w2) w2[3 * i + k] = smp[i].witnesses[1][k];
      }
  }
  return OGX_OK;
}

// device-buffer query from device descriptors
ogx_status device_query(DescSrc src, int nbodies, int npairs, gkSimplex* d_smp, float* d_dist, float* d_nrm,
                        int mode) {
  if (npairs <= 0) return OGX_OK;
  if (!src.a || !d_smp || !d_dist) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  Lease L;
  ogx_status s = lease(L);
  if (s) return s;
  Compat* c = L.c;
  s = pool_from_device_desc(*c, src, nbodies);
  if (s) return s;
  s = ensure_results(*c, npairs);
  if (s) return s;
  k_pairs_iota<<<std::min(1024, (npairs + 255) / 256), 256, 0, c->ctx->stream>>>(c->d_pairs, npairs);
  const gkCollisionPair* d_pairs = c->d_pairs;
  float* nrm = d_nrm;
  if (!nrm && mode != kModeGjk) {  // nullable normals: write into scratch
    s = ensure_results(*c, npairs);
    if (s) return s;
    nrm = c->d_nrm;
  }
  return run_timed(*c, nbodies, npairs, d_pairs, d_smp, d_dist, nrm, mode);
}

ogx_status copy_to_device_desc(int n, const gkPolytope* host, gkPolytope** d_desc, float** d_coord) {
  int64_t pts = 0;
  for (int i = 0; i < n; ++i) {
    if (host[i].numpoints < 1 || !host[i].coord)
      return ogx_fail(OGX_ERR_INVALID, "polytope %d: numpoints %d", i, host[i].numpoints);
    pts += host[i].numpoints;
  }
  cudaError_t e = cudaMalloc(d_coord, std::max<int64_t>(1, pts) * 3 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(d_desc, std::max(1, n) * sizeof(gkPolytope));
  if (e != cudaSuccess) return ogx_cuda_fail(e, "device polytope arrays");
  std::vector<float> staging((size_t)pts * 3);
  std::vector<gkPolytope> desc(host, host + n);
  int64_t off = 0;
  for (int i = 0; i < n; ++i) {
    memcpy(staging.data() + 3 * off, host[i].coord, host[i].numpoints * 12);
    desc[i].coord = *d_coord + 3 * off;
    off += host[i].numpoints;
  }
  e = cudaMemcpy(*d_coord, staging.data(), staging.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(*d_desc, desc.data(), n * sizeof(gkPolytope), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "device polytope upload");
  return OGX_OK;
}

}  // namespace

// =================================================================================
// high-level API (host buffers)

// compute_minimum_distance (GJK/gpu/openGJK.h:91); GJK::GPU::computeDistances
// (examples/gpu/example.h:21-25)
extern "C" ogx_status ogx_compute_minimum_distance(int n, const gkPolytope* bd1, const gkPolytope* bd2,
                                                   gkSimplex* simplices, float* distances) {
  if (n > 0 && !bd2) return ogx_fail(OGX_ERR_INVALID, "bd2 is NULL");
  return host_query(bd1, bd2, 2 * n, n, nullptr, simplices, distances, nullptr, nullptr, nullptr,
                    kModeGjk, false);
}

// computeCollisionInformation(n, ...) (GJK/gpu/openGJK.h:112); GJK::GPU::computeEPA
// (examples/gpu/example.h:41-46): simplices and distances are inputs (from GJK) and
// outputs; contact_normals may be NULL.
extern "C" ogx_status ogx_compute_collision_information(int n, const gkPolytope* bd1, const gkPolytope* bd2,
                                                        gkSimplex* simplices, float* distances,
                                                        float* contact_normals) {
  if (n > 0 && !bd2) return ogx_fail(OGX_ERR_INVALID, "bd2 is NULL");
  return host_query(bd1, bd2, 2 * n, n, nullptr, simplices, distances, contact_normals, nullptr, nullptr,
                    kModeEpa, true);
}

// compute_gjk_epa (GJK/gpu/openGJK.h:134); GJK::GPU::computeGJKAndEPA
// (examples/gpu/example.h:62-67)
extern "C" ogx_status ogx_compute_gjk_epa(int n, const gkPolytope* bd1, const gkPolytope* bd2,
                                          gkSimplex* simplices, float* distances, float* contact_normals) {
  if (n > 0 && !bd2) return ogx_fail(OGX_ERR_INVALID, "bd2 is NULL");
  return host_query(bd1, bd2, 2 * n, n, nullptr, simplices, distances, contact_normals, nullptr, nullptr,
                    kModeGjkEpa, false);
}

// GJK::GPU::computeCollisionInformation as documented in README.md:39-46 (the reference
// code has no such function): EPA from given GJK simplices/distances, witnesses also
// returned as n x 3 arrays, contact_normals nullable.
extern "C" ogx_status ogx_compute_collision_information_witnesses(int n, const gkPolytope* bd1,
                                                                  const gkPolytope* bd2, gkSimplex* simplices,
                                                                  float* distances, float* witness1,
                                                                  float* witness2, float* contact_normals) {
  if (n > 0 && !bd2) return ogx_fail(OGX_ERR_INVALID, "bd2 is NULL");
  return host_query(bd1, bd2, 2 * n, n, nullptr, simplices, distances, contact_normals, witness1, witness2,
                    kModeEpa, true);
}

// =================================================================================
// mid-level API (explicit device memory)

// allocate_and_copy_device_arrays (GJK/gpu/openGJK.h:212)
extern "C" ogx_status ogx_allocate_and_copy_device_arrays(int n, const gkPolytope* bd1, const gkPolytope* bd2,
                                                          gkPolytope** d_bd1, gkPolytope** d_bd2,
                                                          float** d_coord1, float** d_coord2,
                                                          gkSimplex** d_simplices, float** d_distances) {
  if (n < 0 || !bd1 || !bd2 || !d_bd1 || !d_bd2 || !d_coord1 || !d_coord2 || !d_simplices || !d_distances)
    return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  ogx_status s = copy_to_device_desc(n, bd1, d_bd1, d_coord1);
  if (!s) s = copy_to_device_desc(n, bd2, d_bd2, d_coord2);
  if (s) return s;
  cudaError_t e = cudaMalloc(d_simplices, std::max(1, n) * sizeof(gkSimplex));
  if (e == cudaSuccess) e = cudaMalloc(d_distances, std::max(1, n) * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(*d_simplices, 0, std::max(1, n) * sizeof(gkSimplex));
  if (e != cudaSuccess) return ogx_cuda_fail(e, "result arrays");
  return OGX_OK;
}

// compute_minimum_distance_device (GJK/gpu/openGJK.h:237)
extern "C" ogx_status ogx_compute_minimum_distance_device(int n, const gkPolytope* d_bd1,
                                                          const gkPolytope* d_bd2, gkSimplex* d_simplices,
                                                          float* d_distances) {
  DescSrc src{d_bd1, d_bd2, nullptr};
  if (n > 0 && !d_bd2) return ogx_fail(OGX_ERR_INVALID, "d_bd2 is NULL");
  return device_query(src, 2 * n, n, d_simplices, d_distances, nullptr, kModeGjk);
}

// compute_epa_device (GJK/gpu/openGJK.h:255)
extern "C" ogx_status ogx_compute_epa_device(int n, const gkPolytope* d_bd1, const gkPolytope* d_bd2,
                                             gkSimplex* d_simplices, float* d_distances,
                                             float* d_contact_normals) {
  DescSrc src{d_bd1, d_bd2, nullptr};
  if (n > 0 && !d_bd2) return ogx_fail(OGX_ERR_INVALID, "d_bd2 is NULL");
  return device_query(src, 2 * n, n, d_simplices, d_distances, d_contact_normals, kModeEpa);
}

// copy_results_from_device (GJK/gpu/openGJK.h:273)
extern "C" ogx_status ogx_copy_results_from_device(int n, const gkSimplex* d_simplices,
                                                   const float* d_distances, gkSimplex* simplices,
                                                   float* distances) {
  if (n <= 0) return OGX_OK;
  cudaError_t e = cudaMemcpy(simplices, d_simplices, n * sizeof(gkSimplex), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(distances, d_distances, n * sizeof(float), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "copy_results_from_device");
  return OGX_OK;
}

// free_device_arrays (GJK/gpu/openGJK.h:292)
extern "C" ogx_status ogx_free_device_arrays(gkPolytope* d_bd1, gkPolytope* d_bd2, float* d_coord1,
                                             float* d_coord2, gkSimplex* d_simplices, float* d_distances) {
  cudaFree(d_bd1);
  cudaFree(d_bd2);
  cudaFree(d_coord1);
  cudaFree(d_coord2);
  cudaFree(d_simplices);
  cudaFree(d_distances);
  return OGX_OK;
}

// allocate_epa_device_arrays (GJK/gpu/openGJK.h:155); d_contact_normals nullable
extern "C" ogx_status ogx_allocate_epa_device_arrays(int n, float** d_witness1, float** d_witness2,
                                                     float** d_contact_normals) {
  if (n < 0 || !d_witness1 || !d_witness2) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  const size_t b = std::max(1, n) * 3 * sizeof(float);
  cudaError_t e = cudaMalloc(d_witness1, b);
  if (e == cudaSuccess) e = cudaMalloc(d_witness2, b);
  if (e == cudaSuccess && d_contact_normals) e = cudaMalloc(d_contact_normals, b);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "EPA arrays");
  return OGX_OK;
}

// copy_epa_results_from_device (GJK/gpu/openGJK.h:173)
extern "C" ogx_status ogx_copy_epa_results_from_device(int n, const float* d_witness1, const float* d_witness2,
                                                       const float* d_contact_normals, float* witness1,
                                                       float* witness2, float* contact_normals) {
  if (n <= 0) return OGX_OK;
  const size_t b = (size_t)n * 3 * sizeof(float);
  cudaError_t e = cudaMemcpy(witness1, d_witness1, b, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(witness2, d_witness2, b, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && d_contact_normals && contact_normals)
    e = cudaMemcpy(contact_normals, d_contact_normals, b, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "copy_epa_results_from_device");
  return OGX_OK;
}

// free_epa_device_arrays (GJK/gpu/openGJK.h:194)
extern "C" ogx_status ogx_free_epa_device_arrays(float* d_witness1, float* d_witness2, float* d_contact_normals) {
  cudaFree(d_witness1);
  cudaFree(d_witness2);
  cudaFree(d_contact_normals);
  return OGX_OK;
}

// =================================================================================
// indexed API

// allocate_indexed_device (GJK/gpu/openGJK.h:330): pool of polytopes with device
// coordinates, pair buffer for max_pairs, result buffers; d_contact_normals nullable
extern "C" ogx_status ogx_allocate_indexed_device(int num_polytopes, int max_pairs, const gkPolytope* polytopes,
                                                  gkPolytope** d_polytopes, float** d_coords,
                                                  gkCollisionPair** d_pairs, gkSimplex** d_simplices,
                                                  float** d_distances, float** d_contact_normals) {
  if (num_polytopes < 0 || max_pairs < 0 || !polytopes || !d_polytopes || !d_coords || !d_pairs ||
      !d_simplices || !d_distances)
    return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  ogx_status s = copy_to_device_desc(num_polytopes, polytopes, d_polytopes, d_coords);
  if (s) return s;
  const size_t m = std::max(1, max_pairs);
  cudaError_t e = cudaMalloc(d_pairs, m * sizeof(gkCollisionPair));
  if (e == cudaSuccess) e = cudaMalloc(d_simplices, m * sizeof(gkSimplex));
  if (e == cudaSuccess) e = cudaMalloc(d_distances, m * sizeof(float));
  if (e == cudaSuccess && d_contact_normals) e = cudaMalloc(d_contact_normals, 3 * m * sizeof(float));
  if (e != cudaSuccess) return ogx_cuda_fail(e, "indexed arrays");
  return OGX_OK;
}

// free_indexed_device (GJK/gpu/openGJK.h:352)
extern "C" ogx_status ogx_free_indexed_device(gkPolytope* d_polytopes, float* d_coords, gkCollisionPair* d_pairs,
                                              gkSimplex* d_simplices, float* d_distances,
                                              float* d_contact_normals) {
  cudaFree(d_polytopes);
  cudaFree(d_coords);
  cudaFree(d_pairs);
  cudaFree(d_simplices);
  cudaFree(d_distances);
  cudaFree(d_contact_normals);
  return OGX_OK;
}

// upload_pairs_device (GJK/gpu/openGJK.h:368)
extern "C" ogx_status ogx_upload_pairs_device(int num_pairs, const gkCollisionPair* pairs,
                                              gkCollisionPair* d_pairs) {
  if (num_pairs <= 0) return OGX_OK;
  cudaError_t e = cudaMemcpy(d_pairs, pairs, num_pairs * sizeof(gkCollisionPair), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "upload_pairs_device");
  return OGX_OK;
}

// compute_minimum_distance_indexed (GJK/gpu/openGJK.h:398)
extern "C" ogx_status ogx_compute_minimum_distance_indexed(int num_polytopes, int num_pairs,
                                                           const gkPolytope* polytopes,
                                                           const gkCollisionPair* pairs, gkSimplex* simplices,
                                                           float* distances) {
  if (num_polytopes <= 0 || num_pairs <= 0) return OGX_OK;
  if (!pairs) return ogx_fail(OGX_ERR_INVALID, "pairs is NULL");
  return host_query(polytopes, nullptr, num_polytopes, num_pairs, pairs, simplices, distances, nullptr,
                    nullptr, nullptr, kModeGjk, false);
}

// compute_minimum_distance_indexed_device (GJK/gpu/openGJK.h:419)
extern "C" ogx_status ogx_compute_minimum_distance_indexed_device(int num_pairs, const gkPolytope* d_polytopes,
                                                                  const gkCollisionPair* d_pairs,
                                                                  gkSimplex* d_simplices, float* d_distances) {
  if (num_pairs > 0 && !d_pairs) return ogx_fail(OGX_ERR_INVALID, "d_pairs is NULL");
  return device_query(DescSrc{d_polytopes, nullptr, d_pairs}, 2 * num_pairs, num_pairs, d_simplices,
                      d_distances, nullptr, kModeGjk);
}

// compute_epa_indexed (GJK/gpu/openGJK.h:473): simplices/distances in/out
extern "C" ogx_status ogx_compute_epa_indexed(int num_polytopes, int num_pairs, const gkPolytope* polytopes,
                                              const gkCollisionPair* pairs, gkSimplex* simplices,
                                              float* distances, float* contact_normals) {
  if (num_polytopes <= 0 || num_pairs <= 0) return OGX_OK;
  if (!pairs) return ogx_fail(OGX_ERR_INVALID, "pairs is NULL");
  return host_query(polytopes, nullptr, num_polytopes, num_pairs, pairs, simplices, distances,
                    contact_normals, nullptr, nullptr, kModeEpa, true);
}

// compute_epa_indexed_device (GJK/gpu/openGJK.h:450)
extern "C" ogx_status ogx_compute_epa_indexed_device(int num_pairs, const gkPolytope* d_polytopes,
                                                     const gkCollisionPair* d_pairs, gkSimplex* d_simplices,
                                                     float* d_distances, float* d_contact_normals) {
  if (num_pairs > 0 && !d_pairs) return ogx_fail(OGX_ERR_INVALID, "d_pairs is NULL");
  return device_query(DescSrc{d_polytopes, nullptr, d_pairs}, 2 * num_pairs, num_pairs, d_simplices,
                      d_distances, d_contact_normals, kModeEpa);
}

// compute_gjk_epa_indexed (GJK/gpu/openGJK.h:497)
extern "C" ogx_status ogx_compute_gjk_epa_indexed(int num_polytopes, int num_pairs, const gkPolytope* polytopes,
                                                  const gkCollisionPair* pairs, gkSimplex* simplices,
                                                  float* distances, float* contact_normals) {
  if (num_polytopes <= 0 || num_pairs <= 0) return OGX_OK;
  if (!pairs) return ogx_fail(OGX_ERR_INVALID, "pairs is NULL");
  return host_query(polytopes, nullptr, num_polytopes, num_pairs, pairs, simplices, distances,
                    contact_normals, nullptr, nullptr, kModeGjkEpa, false);
}

// GJK::GPU::timer() (examples/gpu/example.h:9): GPU time of the engine pipeline of the
// calling thread's last reference-compatible call, in milliseconds.
extern "C" float ogx_compat_last_gpu_ms(void) { return t_last_ms; }

// =================================================================================
// FP64 layouts (the reference built with USE_32BITS off, GJK/common.h:44-60).  The
// coordinates are rounded once to float, the engine runs on them as on any FP32 input,
// and the results are widened to double: they carry the rounding of the inputs (a
// relative 6e-8 of each coordinate), not that of an FP64 computation.

namespace {

// FP32 copies of FP64 descriptor arrays: one float coordinate buffer, descriptors into it
struct Narrowed {
  std::vector<float> coords;
  std::vector<gkPolytope> a, b;
};

ogx_status narrow_desc(const ogx_polytope_f64* src, int n, std::vector<gkPolytope>& out, std::vector<float>& coords,
                       std::vector<int64_t>& first) {
  out.resize(n);
  for (int i = 0; i < n; ++i) {
    if (src[i].numpoints < 1 || !src[i].coord)
      return ogx_fail(OGX_ERR_INVALID, "polytope %d: numpoints %d, coord %p", i, src[i].numpoints,
                      (void*)src[i].coord);
    first.push_back((int64_t)coords.size());
    for (int k = 0; k < 3 * src[i].numpoints; ++k) coords.push_back((float)src[i].coord[k]);
    out[i].numpoints = src[i].numpoints;
    for (int k = 0; k < 3; ++k) out[i].s[k] = (float)src[i].s[k];
    out[i].s_idx = src[i].s_idx;
    out[i].coord = nullptr;  // set once the buffer stops growing
  }
  return OGX_OK;
}

ogx_status narrow(int na, const ogx_polytope_f64* a, int nb, const ogx_polytope_f64* b, Narrowed& N) {
  std::vector<int64_t> fa, fb;
  ogx_status s = narrow_desc(a, na, N.a, N.coords, fa);
  if (!s && b) s = narrow_desc(b, nb, N.b, N.coords, fb);
  if (s) return s;
  for (int i = 0; i < na; ++i) N.a[i].coord = N.coords.data() + fa[i];
  for (int i = 0; b && i < nb; ++i) N.b[i].coord = N.coords.data() + fb[i];
  return OGX_OK;
}

void narrow_simplex(const ogx_simplex_f64& d, gkSimplex& f) {
  f.nvrtx = d.nvrtx;
  for (int k = 0; k < 4; ++k)
    for (int c = 0; c < 3; ++c) f.vrtx[k][c] = (float)d.vrtx[k][c];
  for (int k = 0; k < 4; ++k) {
    f.vrtx_idx[k][0] = d.vrtx_idx[k][0];
    f.vrtx_idx[k][1] = d.vrtx_idx[k][1];
  }
  for (int w = 0; w < 2; ++w)
    for (int c = 0; c < 3; ++c) f.witnesses[w][c] = (float)d.witnesses[w][c];
}

void widen_simplex(const gkSimplex& f, ogx_simplex_f64& d) {
  d.nvrtx = f.nvrtx;
  for (int k = 0; k < 4; ++k)
    for (int c = 0; c < 3; ++c) d.vrtx[k][c] = f.vrtx[k][c];
  for (int k = 0; k < 4; ++k) {
    d.vrtx_idx[k][0] = f.vrtx_idx[k][0];
    d.vrtx_idx[k][1] = f.vrtx_idx[k][1];
  }
  for (int w = 0; w < 2; ++w)
    for (int c = 0; c < 3; ++c) d.witnesses[w][c] = f.witnesses[w][c];
}

// host_query on FP64 arrays: pairs (a[i], b[i]) when b is given, else pairs into a
ogx_status host_query_f64(const ogx_polytope_f64* a, const ogx_polytope_f64* b, int nbodies, int npairs,
                          const gkCollisionPair* pairs, ogx_simplex_f64* smp, double* dist, double* nrm,
                          double* w1, double* w2, int mode, bool upload_in) {
  if (npairs <= 0) return OGX_OK;
  if (!a || !smp || !dist) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  Narrowed N;
  ogx_status s = b ? narrow(npairs, a, npairs, b, N) : narrow(nbodies, a, 0, nullptr, N);
  if (s) return s;
  std::vector<gkSimplex> s32(npairs);
  std::vector<float> d32(npairs), n32(nrm ? 3 * (size_t)npairs : 0);
  std::vector<float> w32a(w1 ? 3 * (size_t)npairs : 0), w32b(w2 ? 3 * (size_t)npairs : 0);
  if (upload_in)
    for (int i = 0; i < npairs; ++i) {
      narrow_simplex(smp[i], s32[i]);
      d32[i] = (float)dist[i];
    }
  s = host_query(N.a.data(), b ? N.b.data() : nullptr, nbodies, npairs, pairs, s32.data(), d32.data(),
                 nrm ? n32.data() : nullptr, w1 ? w32a.data() : nullptr, w2 ? w32b.data() : nullptr, mode,
                 upload_in, a, b);
  if (s) return s;
  for (int i = 0; i < npairs; ++i) {
    widen_simplex(s32[i], smp[i]);
    dist[i] = d32[i];
  }
  for (size_t k = 0; k < n32.size(); ++k) nrm[k] = n32[k];
  for (size_t k = 0; k < w32a.size(); ++k) w1[k] = w32a[k];
  for (size_t k = 0; k < w32b.size(); ++k) w2[k] = w32b[k];
  return OGX_OK;
}

}  // namespace

// compute_minimum_distance / GJK::GPU::computeDistances with gkFloat = double
extern "C" ogx_status ogx_compute_minimum_distance_f64(int n, const ogx_polytope_f64* bd1,
                                                       const ogx_polytope_f64* bd2, ogx_simplex_f64* simplices,
                                                       double* distances) {
  if (n > 0 && !bd2) return ogx_fail(OGX_ERR_INVALID, "bd2 is NULL");
  return host_query_f64(bd1, bd2, 2 * n, n, nullptr, simplices, distances, nullptr, nullptr, nullptr, kModeGjk,
                        false);
}

// computeCollisionInformation(n, ...) / GJK::GPU::computeEPA with gkFloat = double
extern "C" ogx_status ogx_compute_collision_information_f64(int n, const ogx_polytope_f64* bd1,
                                                            const ogx_polytope_f64* bd2,
                                                            ogx_simplex_f64* simplices, double* distances,
                                                            double* contact_normals) {
  if (n > 0 && !bd2) return ogx_fail(OGX_ERR_INVALID, "bd2 is NULL");
  return host_query_f64(bd1, bd2, 2 * n, n, nullptr, simplices, distances, contact_normals, nullptr, nullptr,
                        kModeEpa, true);
}

// compute_gjk_epa / GJK::GPU::computeGJKAndEPA with gkFloat = double
extern "C" ogx_status ogx_compute_gjk_epa_f64(int n, const ogx_polytope_f64* bd1, const ogx_polytope_f64* bd2,
                                              ogx_simplex_f64* simplices, double* distances,
                                              double* contact_normals) {
  if (n > 0 && !bd2) return ogx_fail(OGX_ERR_INVALID, "bd2 is NULL");
  return host_query_f64(bd1, bd2, 2 * n, n, nullptr, simplices, distances, contact_normals, nullptr, nullptr,
                        kModeGjkEpa, false);
}

// GJK::GPU::computeCollisionInformation (README.md:39-46 form) with gkFloat = double
extern "C" ogx_status ogx_compute_collision_information_witnesses_f64(
    int n, const ogx_polytope_f64* bd1, const ogx_polytope_f64* bd2, ogx_simplex_f64* simplices,
    double* distances, double* witness1, double* witness2, double* contact_normals) {
  if (n > 0 && !bd2) return ogx_fail(OGX_ERR_INVALID, "bd2 is NULL");
  return host_query_f64(bd1, bd2, 2 * n, n, nullptr, simplices, distances, contact_normals, witness1, witness2,
                        kModeEpa, true);
}

// compute_minimum_distance_indexed with gkFloat = double
extern "C" ogx_status ogx_compute_minimum_distance_indexed_f64(int num_polytopes, int num_pairs,
                                                               const ogx_polytope_f64* polytopes,
                                                               const gkCollisionPair* pairs,
                                                               ogx_simplex_f64* simplices, double* distances) {
  if (num_polytopes <= 0 || num_pairs <= 0) return OGX_OK;
  if (!pairs) return ogx_fail(OGX_ERR_INVALID, "pairs is NULL");
  return host_query_f64(polytopes, nullptr, num_polytopes, num_pairs, pairs, simplices, distances, nullptr,
                        nullptr, nullptr, kModeGjk, false);
}

// compute_epa_indexed with gkFloat = double: simplices/distances in/out
extern "C" ogx_status ogx_compute_epa_indexed_f64(int num_polytopes, int num_pairs,
                                                  const ogx_polytope_f64* polytopes, const gkCollisionPair* pairs,
                                                  ogx_simplex_f64* simplices, double* distances,
                                                  double* contact_normals) {
  if (num_polytopes <= 0 || num_pairs <= 0) return OGX_OK;
  if (!pairs) return ogx_fail(OGX_ERR_INVALID, "pairs is NULL");
  return host_query_f64(polytopes, nullptr, num_polytopes, num_pairs, pairs, simplices, distances,
                        contact_normals, nullptr, nullptr, kModeEpa, true);
}

// compute_gjk_epa_indexed with gkFloat = double
extern "C" ogx_status ogx_compute_gjk_epa_indexed_f64(int num_polytopes, int num_pairs,
                                                      const ogx_polytope_f64* polytopes,
                                                      const gkCollisionPair* pairs, ogx_simplex_f64* simplices,
                                                      double* distances, double* contact_normals) {
  if (num_polytopes <= 0 || num_pairs <= 0) return OGX_OK;
  if (!pairs) return ogx_fail(OGX_ERR_INVALID, "pairs is NULL");
  return host_query_f64(polytopes, nullptr, num_polytopes, num_pairs, pairs, simplices, distances,
                        contact_normals, nullptr, nullptr, kModeGjkEpa, false);
}
