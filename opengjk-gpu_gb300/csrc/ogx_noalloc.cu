// ogx_noalloc.cu -- GJK + EPA without any device allocation.
//
// Some callers must not allocate device memory at query time: physics or rendering
// loops whose device memory is owned by their own arena and must not grow behind their
// back, real-time tick loops that cannot afford the allocator's latency spikes, and
// plugins whose host application forbids them to allocate GPU memory.  ogx_gjk_epa_noalloc
// serves them: the caller passes the pool (engine layout), the pairs and the outputs,
// and the pipeline's work lists live in one file-scope device array instead of memory
// from cudaMalloc.
//
// Limits and behaviour (also in include/ogx.h):
//  * at most kNoAllocMaxPairs pairs per call; larger batches are rejected with
//    OGX_ERR_CAPACITY;
//  * the array (kNoAllocScratchBytes, 1,835,264 bytes) exists on every GPU that loads the
//    library, from load until the process exits;
//  * every call uses the same array and the array keeps the last call's contents; the
//    work-list counters must start at zero and each call clears them itself (a memset on
//    the caller's stream) before its first kernel; the lists are only read below their
//    counters, so nothing else needs clearing.  Calls that overlap on the GPU (different
//    streams, or different host threads) race on the array -- serialise them;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) and the launch sizes; make that first call before any
//    stream capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "ogx_engine.h"

using namespace ogx;

namespace {

constexpr int kNoAllocMaxPairs = 16384;
constexpr int kNoAllocBlock = 128;

// scratch layout inside the static array (byte offsets, all 256-aligned)
constexpr size_t kOffCounts = 0;
constexpr size_t kOffLists = 256;
constexpr size_t kOffElists = kOffLists + (size_t)kBuckets * kNoAllocMaxPairs * sizeof(int);
constexpr size_t kOffRefine = kOffElists + (size_t)kBuckets * kNoAllocMaxPairs * sizeof(int);
constexpr size_t kOffRefineFull = kOffRefine + (size_t)kNoAllocMaxPairs * sizeof(RefineRec);
constexpr size_t kOffPolish = kOffRefineFull + (size_t)kNoAllocMaxPairs * sizeof(int);
constexpr size_t kOffSpill = kOffPolish + (size_t)kNoAllocMaxPairs * sizeof(PolishRec);
constexpr size_t kNoAllocScratchBytes = kOffSpill + (size_t)kNoAllocMaxPairs * sizeof(int);

static_assert(kNoAllocScratchBytes == 1835264, "the size is documented in include/ogx.h");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct Setup {
  bool ready = false;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
  KernelInfo gjk[kBuckets], epa[kBuckets];
  int grid_gjk[kBuckets], grid_epa[kBuckets];
  size_t smem_epa[kBuckets];
  int grid_bin = 0, grid_refine = 0, grid_polish = 0, grid_spill = 0;
};

std::mutex g_mu;
Setup g_setup[16];

// one pair per warp (32 lanes), the fewest registers that fit the bucket
const KernelInfo* pick(const KernelInfo* a, int na, const KernelInfo* b, int nb, int bucket) {
  static const int cap[kBuckets] = {16, 32, 64, 128, 256, 512, 0};
  const KernelInfo* best = nullptr;
  for (int k = 0; k < na + nb; ++k) {
    const KernelInfo* v = k < na ? &a[k] : &b[k - na];
    if (v->L != 32) continue;
    if (bucket == kBuckets - 1) {
      if (v->K == 0) return v;
      continue;
    }
    if (v->K == 0 || 4 * v->L * v->K < cap[bucket]) continue;
    if (!best || v->K < best->K) best = v;
  }
  return best;
}

ogx_status setup(int dev, Setup** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  Setup& s = g_setup[dev];
  if (s.ready) {
    *out = &s;
    return OGX_OK;
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
  s.scratch = static_cast<unsigned char*>(p);
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "cudaDeviceGetAttribute");
  const KernelInfo *ga, *gb, *ea, *eb;
  const int nga = gjk_variants_a(&ga), ngb = gjk_variants_b(&gb);
  const int nea = epa_variants_a(&ea), neb = epa_variants_b(&eb);
  for (int b = 0; b < kBuckets; ++b) {
    const KernelInfo* g = pick(ga, nga, gb, ngb, b);
    const KernelInfo* q = pick(ea, nea, eb, neb, b);
    if (!g || !q) return ogx_fail(OGX_ERR_CUDA, "no kernel variant for bucket %d", b);
    s.gjk[b] = *g;
    s.epa[b] = *q;
    s.smem_epa[b] = (size_t)(kNoAllocBlock / q->L) * epa_team_stride(q->L);
    // launches here take no dynamic shared memory beyond the default 48 KB per block
    if (s.smem_epa[b] > 48 * 1024)
      return ogx_fail(OGX_ERR_CUDA, "EPA variant for bucket %d needs %zu B of shared memory (> 48 KB)", b,
                      s.smem_epa[b]);
    int per = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, g->fn, kNoAllocBlock, 0);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "occupancy");
    s.grid_gjk[b] = std::max(1, per) * sms;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, q->fn, kNoAllocBlock, s.smem_epa[b]);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "occupancy");
    s.grid_epa[b] = std::max(1, per) * sms;
  }
  int per = 0;
  e = refine_occupancy(kNoAllocBlock, &per);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "occupancy");
  s.grid_refine = std::max(1, per) * sms;
  e = epa_spill_occupancy(kNoAllocBlock, &per);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "occupancy");
  s.grid_spill = std::max(1, per) * sms;
  e = polish_occupancy(kNoAllocBlock, &per);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "occupancy");
  s.grid_polish = std::max(1, per) * sms;
  s.grid_bin = 4 * sms;
  s.ready = true;
  *out = &s;
  return OGX_OK;
}

}  // namespace

// GJK then EPA over npairs <= 16384 pairs of a pool in the engine layout, allocating
// nothing.  No counterpart in the reference.  See the file comment for who needs it and
// the limits.
extern "C" ogx_status ogx_gjk_epa_noalloc(const float* d_points, const void* d_bodies, int num_bodies,
                                          int npairs, const gkCollisionPair* d_pairs, gkSimplex* d_simplices,
                                          float* d_distances, float* d_normals, int32_t* d_status,
                                          const ogx_config* cfg, void* stream) {
  if (npairs < 0 || num_bodies < 0) return ogx_fail(OGX_ERR_INVALID, "negative size");
  if (npairs > kNoAllocMaxPairs)
    return ogx_fail(OGX_ERR_CAPACITY, "ogx_gjk_epa_noalloc takes at most %d pairs per call (got %d)",
                    kNoAllocMaxPairs, npairs);
  if (npairs == 0) return OGX_OK;
  if (!d_points || !d_bodies || !d_pairs || !d_simplices || !d_distances || !d_normals)
    return ogx_fail(OGX_ERR_INVALID, "NULL pool, pair or output pointer");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 16) {
    cudaGetLastError();
    return ogx_fail(OGX_ERR_NO_DEVICE, "no usable CUDA device");
  }
  Setup* S = nullptr;
  ogx_status st = setup(dev, &S);
  if (st) return st;
  const ogx_config c = cfg ? *cfg : default_config();
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  DevBatch B;
  B.pool = d_points;
  B.bodies = static_cast<const BodyRef*>(d_bodies);
  B.nbodies = num_bodies;
  B.pairs = reinterpret_cast<const int2*>(d_pairs);
  B.npairs = npairs;
  B.smp = d_simplices;
  B.dist = d_distances;
  B.nrm = d_normals;
  B.status = d_status;
  B.counts = reinterpret_cast<int*>(S->scratch + kOffCounts);
  B.lists = reinterpret_cast<int*>(S->scratch + kOffLists);
  B.elists = reinterpret_cast<int*>(S->scratch + kOffElists);
  B.refine = reinterpret_cast<RefineRec*>(S->scratch + kOffRefine);
  B.refine_full = reinterpret_cast<int*>(S->scratch + kOffRefineFull);
  B.polish = reinterpret_cast<PolishRec*>(S->scratch + kOffPolish);
  B.spill = reinterpret_cast<int*>(S->scratch + kOffSpill);
  B.resume = nullptr;  // capacity spills restart at full capacity
  B.resume_cap = 0;
  B.warm = nullptr;
  B.subtab = nullptr;  // the decision tree (same outcomes as the engine's table)
  B.xf = nullptr;
  B.cfg = c;
  B.mode = kModeGjkEpa;

  // the counters must start at zero; the lists are only read below their counters
  e = cudaMemsetAsync(B.counts, 0, kCntSlots * sizeof(int), s);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "counter reset");
  e = launch_bin(B, std::min(S->grid_bin, (npairs + 255) / 256), s);
  for (int b = kBuckets - 1; b >= 0 && e == cudaSuccess; --b) {
    S->gjk[b].fn<<<S->grid_gjk[b], kNoAllocBlock, 0, s>>>(B, b);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && (c.flags & OGX_F_FP64_POLISH)) e = launch_refine(B, S->grid_refine, S->grid_bin, s, s, nullptr);
  for (int b = kBuckets - 1; b >= 0 && e == cudaSuccess; --b) {
    S->epa[b].fn<<<S->grid_epa[b], kNoAllocBlock, S->smem_epa[b], s>>>(B, b);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = launch_epa_spill(B, S->grid_spill, s);
  if (e == cudaSuccess) e = launch_epa_spill(B, S->grid_spill, s, true);
  if (e == cudaSuccess && (c.flags & OGX_F_FP64_POLISH)) e = launch_polish(B, S->grid_polish, s);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "no-allocation pipeline launch");
  return OGX_OK;
}
