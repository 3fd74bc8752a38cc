// ogx_compat.cu -- the reference-compatible half of the C ABI: OpenGJK-GPU's host API
// (GJK/gpu/openGJK.h, examples/gpu/example.h) re-implemented on the engine.
//
// The reference functions take gkPolytope descriptors (point count + pointer to xyz
// interleaved coordinates), either in host memory (high-level calls) or in device memory
// (mid-level *_device and indexed calls, whose coordinates a caller may rewrite with its
// own kernels between calls).  Every call here copies the referenced bodies into the
// engine's padded SoA pool (on the device: a count -> prefix-sum -> pack sequence), runs
// the engine pipeline and, like the reference, returns when the results are complete.
// The calls share one engine context per device (created on first use).
//
// Deliberate differences from the reference (documented bugs not reproduced):
//  * computeCollisionInformation uploads the input distances (the reference does not,
//    GJK/gpu/openGJK.cu:2838-2845, so its EPA reads uninitialised memory);
//  * contact_normals may be NULL where the reference documents it as nullable
//    (examples/gpu/example.h:39) -- the reference writes through it regardless.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
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

__global__ void k_desc_pack(DescSrc src, int nb, const BodyRef* __restrict__ bodies, float* __restrict__ pool) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int b = warp; b < nb; b += nwarps) {
    const BodyRef r = bodies[b];
    if (r.n < 1) continue;
    const float* c = src.get(b).coord;
    const int n4 = round4(r.n);
    float* dst = pool + 4 * (size_t)r.quad;
    for (int i = lane; i < n4; i += 32) {
      const int s = i < r.n ? i : 0;
      dst[i] = c[3 * s];
      dst[n4 + i] = c[3 * s + 1];
      dst[2 * n4 + i] = c[3 * s + 2];
    }
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
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  float last_ms = 0.0f;
};

std::mutex g_compat_mu;
Compat g_compat[16];

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

ogx_status compat(Compat** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return ogx_fail(OGX_ERR_NO_DEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
  }
  if (dev >= 16) return ogx_fail(OGX_ERR_INVALID, "device index %d", dev);
  Compat& c = g_compat[dev];
  if (!c.ctx) {
    ogx_status s = ogx_ctx_create(dev, nullptr, nullptr, &c.ctx);
    if (s) return s;
    cudaEventCreate(&c.t0);
    cudaEventCreate(&c.t1);
  }
  *out = &c;
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

// Build the pool from descriptors in HOST memory with host coordinates.
ogx_status pool_from_host_desc(Compat& c, const gkPolytope* a, const gkPolytope* b, int nb) {
  std::vector<int32_t> counts(nb);
  std::vector<const float*> src(nb);
  std::vector<int64_t> voff(nb);
  std::vector<BodyRef> refs(nb);
  int64_t pts = 0;
  uint64_t quad = 0;
  for (int i = 0; i < nb; ++i) {
    const gkPolytope& p = b ? ((i & 1) ? b[i >> 1] : a[i >> 1]) : a[i];
    if (p.numpoints < 1 || !p.coord)
      return ogx_fail(OGX_ERR_INVALID, "polytope %d: numpoints %d, coord %p", i, p.numpoints, (void*)p.coord);
    counts[i] = p.numpoints;
    src[i] = p.coord;
    voff[i] = pts;
    refs[i].quad = (uint32_t)quad;
    refs[i].n = p.numpoints;
    pts += p.numpoints;
    quad += 3 * (uint64_t)((p.numpoints + 3) / 4);
    if (quad >= (1ull << 32)) return ogx_fail(OGX_ERR_CAPACITY, "pool exceeds 2^32 float4 blocks");
  }
  ogx_ctx* ctx = c.ctx;
  cudaStream_t st = ctx->stream;
  const size_t bytes = (size_t)pts * 3 * sizeof(float);
  ogx_status s = ctx->ensure_stage(bytes + nb * (sizeof(BodyRef) + sizeof(int64_t)), bytes);
  if (!s) s = grow(&c.d_bodies, &c.bodies_cap, (size_t)nb, "compat body table");
  if (!s) s = grow(&c.d_voff, &c.voff_cap, (size_t)nb, "compat offsets");
  if (!s) s = grow(&c.d_points, &c.points_cap, 4 * (size_t)quad + 4, "compat pool");
  if (s) return s;
  cudaStreamSynchronize(st);  // staging buffers may still be read by a previous call
  char* h = static_cast<char*>(ctx->h_stage);
  // gather all coordinates (parallel for large batches)
  const int nt = (int)std::min<int64_t>(16, std::max<int64_t>(1, pts >> 18));
  std::vector<std::thread> th;
  for (int k = 0; k < nt; ++k)
    th.emplace_back([&, k] {
      for (int i = (int)((int64_t)nb * k / nt); i < (int)((int64_t)nb * (k + 1) / nt); ++i)
        memcpy(h + voff[i] * 12, src[i], (size_t)counts[i] * 12);
    });
  for (auto& t : th) t.join();
  memcpy(h + bytes, refs.data(), nb * sizeof(BodyRef));
  memcpy(h + bytes + nb * sizeof(BodyRef), voff.data(), nb * sizeof(int64_t));
  cudaError_t e = cudaMemcpyAsync(ctx->d_stage, h, bytes, cudaMemcpyHostToDevice, st);
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
                     float* d_dist, float* d_nrm, int mode) {
  cudaEventRecord(c.t0, c.ctx->stream);
  ogx_status s = ogx_run(c.ctx, c.d_points, c.d_bodies, nbodies, npairs, d_pairs, d_smp, d_dist, d_nrm,
                         nullptr, mode);
  cudaEventRecord(c.t1, c.ctx->stream);
  if (s) return s;
  cudaError_t e = cudaStreamSynchronize(c.ctx->stream);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "engine pipeline");
  cudaEventElapsedTime(&c.last_ms, c.t0, c.t1);
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
                      float* w1, float* w2, int mode, bool upload_in) {
  if (npairs <= 0) return OGX_OK;  // the reference returns early for n <= 0
  if (!a || !smp || !dist) return ogx_fail(OGX_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(g_compat_mu);
  Compat* c;
  ogx_status s = compat(&c);
  if (s) return s;
  cudaStream_t st = c->ctx->stream;
  s = pool_from_host_desc(*c, a, b, nbodies);
  if (!s) s = ensure_results(*c, npairs);
  if (s) return s;
  cudaError_t e;
  if (host_pairs) {
    for (int i = 0; i < npairs; ++i)
      if (host_pairs[i].idx1 < 0 || host_pairs[i].idx1 >= nbodies || host_pairs[i].idx2 < 0 ||
          host_pairs[i].idx2 >= nbodies)
        return ogx_fail(OGX_ERR_INVALID, "pair %d: index out of range", i);
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
  s = run_timed(*c, nbodies, npairs, c->d_pairs, c->d_smp, c->d_dist, c->d_nrm, mode);
  if (s) return s;
  e = cudaMemcpyAsync(smp, c->d_smp, npairs * sizeof(gkSimplex), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dist, c->d_dist, npairs * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && nrm && mode != kModeGjk)
    e = cudaMemcpyAsync(nrm, c->d_nrm, 3 * (size_t)npairs * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "result copy");
  s = finish(*c);
  if (s) return s;
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
  std::lock_guard<std::mutex> lk(g_compat_mu);
  Compat* c;
  ogx_status s = compat(&c);
  if (s) return s;
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
// last reference-compatible call on the current device, in milliseconds.
extern "C" float ogx_compat_last_gpu_ms(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev >= 16) return 0.0f;
  return g_compat[dev].last_ms;
}
