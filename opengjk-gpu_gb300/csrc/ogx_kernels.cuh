// ogx_kernels.cuh -- device kernels of the batched pipeline.
//
//   k_pack    AoS points (bodies concatenated) -> padded SoA pool, one warp per body
//   k_bin     validate each pair and append it to the work list of its size bucket
//             (bucket = larger point count: <=16, 32, 64, 128, 256, 512, more)
//   k_gjk     persistent GJK over one bucket: a team of L lanes per pair, both bodies
//             in registers (K float4 blocks of x, y, z per lane and body); contacts are
//             appended to the bucket's EPA list, pairs whose FP32 distance is not
//             certain to polish_rel to the FP64 polish list
//   k_epa     persistent EPA over one bucket's contacts, polytope in shared memory
//   k_polish  FP64 re-solve of the listed pairs, one thread per pair (full warps of
//             FP64 work instead of one lane per team)
// All work lists are filled with warp-aggregated atomics; kernels stride over them, so
// the grid size is independent of the batch (persistent launch, graph-capturable).
#pragma once

#include "ogx_bodies.cuh"
#include "ogx_epa.cuh"
#include "ogx_gjk.cuh"

namespace ogx {

constexpr int kBuckets = 7;
constexpr int kBucketMax[kBuckets] = {16, 32, 64, 128, 256, 512, 0x7fffffff};

OGX_HD int bucket_of(int m) {
  return m <= 16 ? 0 : m <= 32 ? 1 : m <= 64 ? 2 : m <= 128 ? 3 : m <= 256 ? 4 : m <= 512 ? 5 : 6;
}

// FP64 refinement request of a separated pair: the support pair along the final
// direction and whether the FP32 pass proved it exact
struct RefineRec {
  int pair;
  int wa, wb;
  int certain;
};

// FP64 re-solve request: GJK simplex (kind 0) or the final EPA face (kind 1)
struct PolishRec {
  int pair;
  int kind;
  int face[3][2];
};

enum { kModeGjk = 1, kModeGjkEpa = 2, kModeEpa = 3 };

// counter slots in DevBatch::counts
constexpr int kCntGjk = 0;                  // [0, kBuckets)
constexpr int kCntEpa = kBuckets;           // [kBuckets, 2 kBuckets)
constexpr int kCntPolish = 2 * kBuckets;    // EPA faces to re-solve in FP64
constexpr int kCntRefine = 2 * kBuckets + 1;  // separated pairs to refine in FP64
constexpr int kCntRefineFull = 2 * kBuckets + 2;  // of those, the ones to continue in FP64
constexpr int kCntSpill = 2 * kBuckets + 3;  // contacts that outgrew the small EPA capacity
constexpr int kCntRefineBig = 2 * kBuckets + 4;  // of the FP64 continuations, bodies > 128 points
constexpr int kCntSpillLate = 2 * kBuckets + 5;  // contacts found by the FP64 refinement
constexpr int kCntResume = 2 * kBuckets + 6;  // capacity spills saved for the full pass to resume
constexpr int kCntSlots = 2 * kBuckets + 7;
// FP64 continuations of pairs whose bodies have at most this many points run one thread
// per pair (FP64 instructions then serve 32 pairs); larger ones one warp per pair
constexpr int kRefineLaneMax = 128;
constexpr int kRefineIters = 16;

struct DevBatch {
  const float* pool;
  const BodyRef* bodies;
  int nbodies;
  const int2* pairs;  // gkCollisionPair
  int npairs;
  gkSimplex* smp;
  float* dist;
  float* nrm;       // may be null in GJK mode
  int32_t* status;  // may be null
  int* lists;       // kBuckets regions of npairs entries
  int* elists;      // kBuckets regions of npairs entries
  int* counts;      // kCntSlots
  PolishRec* polish;
  RefineRec* refine;  // npairs entries
  int* refine_full;   // npairs entries: pair ids whose FP32 support was not certain
                      // (small bodies from the front, large ones from the back)
  int* spill;         // npairs entries: contacts to re-run at full EPA capacity
  EpaResume* resume;  // resume_cap saved small-capacity expansions (null: none)
  int resume_cap;
  const int2* warm;   // optional: GJK start vertex indices per pair (out of range: ignored)
  const uint32_t* subtab;  // sub-distance decision table (fill_subtab); null: the tree
  ogx_config cfg;
  int mode;
};

// Append `want` lanes' items to a list guarded by counter *ctr; returns the slot of this
// lane (valid where want).  One atomic per converged group of lanes.
__device__ __forceinline__ int warp_append(int* ctr, bool want) {
  const unsigned act = __activemask();
  const unsigned m = __ballot_sync(act, want);
  if (m == 0u) return -1;
  const int wl = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (wl == leader) base = atomicAdd(ctr, __popc(m));
  base = __shfl_sync(act, base, leader);
  return base + __popc(m & ((1u << wl) - 1u));
}

__device__ __forceinline__ void store_simplex(gkSimplex* s, const GjkState& g) {
  s->nvrtx = g.n;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const bool live = k < g.n;
    s->vrtx[k][0] = live ? g.P[k].x : 0.f;
    s->vrtx[k][1] = live ? g.P[k].y : 0.f;
    s->vrtx[k][2] = live ? g.P[k].z : 0.f;
    s->vrtx_idx[k][0] = live ? g.ia[k] : 0;
    s->vrtx_idx[k][1] = live ? g.ib[k] : 0;
  }
  s->witnesses[0][0] = g.w0.x;
  s->witnesses[0][1] = g.w0.y;
  s->witnesses[0][2] = g.w0.z;
  s->witnesses[1][0] = g.w1.x;
  s->witnesses[1][1] = g.w1.y;
  s->witnesses[1][2] = g.w1.z;
}

__device__ __forceinline__ void load_simplex(const gkSimplex* s, float dist, GjkState& g) {
  g.n = s->nvrtx;
  if (g.n < 1 || g.n > 4) g.n = 1;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    g.P[k] = v3<float>(s->vrtx[k][0], s->vrtx[k][1], s->vrtx[k][2]);
    g.ia[k] = s->vrtx_idx[k][0];
    g.ib[k] = s->vrtx_idx[k][1];
  }
  g.w0 = v3<float>(s->witnesses[0][0], s->witnesses[0][1], s->witnesses[0][2]);
  g.w1 = v3<float>(s->witnesses[1][0], s->witnesses[1][1], s->witnesses[1][2]);
  g.dist = dist;
  g.status = 0;
  g.polish = false;
}

__device__ __forceinline__ void store3(float* p, fv3 v) {
  p[0] = v.x;
  p[1] = v.y;
  p[2] = v.z;
}

// ---------------------------------------------------------------------------------
// source of body points for bucket kernels: registers (K > 0) or memory (K == 0)
template <int L, int K>
struct SrcOf {
  typedef RegBodies<L, K> type;
};
template <int L>
struct SrcOf<L, 0> {
  typedef MemBodies type;
};

template <int L, int K>
__device__ __forceinline__ void bind_src(RegBodies<L, K>& s, const float* pool, BodyRef a,
                                         BodyRef b, int lane) {
  s.bind(pool, a, b, lane);
}
template <int L>
__device__ __forceinline__ void bind_src(MemBodies& s, const float* pool, BodyRef a, BodyRef b,
                                         int) {
  s.bind(pool, a, b);
}

// Store one finished pair's GJK result and route it (EPA list, FP64 refinement list).
__device__ __forceinline__ void gjk_store(const DevBatch& B, int bucket, int p, const GjkState& g, bool lead) {
  const bool contact = gjk_contact(g);
  if (lead) {
    store_simplex(B.smp + p, g);
    B.dist[p] = g.dist;
    if (B.status) B.status[p] = g.status;
    if (B.mode == kModeGjkEpa && !contact && !g.polish) store3(B.nrm + 3 * (size_t)p, sep_normal(g));
    // pairs sent to the FP64 refinement get their normal there
  }
  const bool to_epa = lead && B.mode == kModeGjkEpa && contact;
  const int e = warp_append(B.counts + kCntEpa + bucket, to_epa);
  if (to_epa) B.elists[(size_t)bucket * B.npairs + e] = p;
  const int q = warp_append(B.counts + kCntRefine, lead && g.polish);
  if (lead && g.polish) {
    RefineRec r;
    r.pair = p;
    r.wa = g.wa;
    r.wb = g.wb;
    r.certain = g.certain ? 1 : 0;
    B.refine[q] = r;
  }
}

template <int L, int K, int OCC = 1>
__global__ void __launch_bounds__(128, OCC) k_gjk(DevBatch B, int bucket) {
  const WarpTeam<L> t;
  const int team = (blockIdx.x * blockDim.x + threadIdx.x) / L;
  const int nteams = (gridDim.x * blockDim.x) / L;
  const int cnt = B.counts[kCntGjk + bucket];
  const int* list = B.lists + (size_t)bucket * B.npairs;
  for (int j = team; j < cnt; j += nteams) {
    const int p = list[j];
    const int2 pr = B.pairs[p];
    const BodyRef ra = B.bodies[pr.x], rb = B.bodies[pr.y];
    typename SrcOf<L, K>::type src;
    bind_src<L>(src, B.pool, ra, rb, t.lane());
    int2 ws = make_int2(0, 0);
    if (B.warm) {
      ws = B.warm[p];
      if (ws.x < 0 || ws.x >= ra.n || ws.y < 0 || ws.y >= rb.n) ws = make_int2(0, 0);
    }
    GjkState g;
    gjk_pair(t, src, B.cfg, g, ws.x, ws.y, B.subtab);
    gjk_store(B, bucket, p, g, t.lane() == 0);
  }
}


// kFull: the full-capacity pass over the spill list -- certified re-runs where the entry
// asks for FP64 planes, and the FP64 polish of the result done here by lane 0 instead of
// through the polish list, so that the polish pass need not wait for this one
// spill list entry codes: a pair index, or a saved expansion to resume
constexpr int kSpill64 = 1 << 30;      // the re-run solves every face plane in FP64
constexpr int kSpillResume = 1 << 29;  // low bits: the EpaResume record to continue

template <int L, int K, bool kFull = false, class Mem>
__device__ __forceinline__ bool epa_item(const WarpTeam<L>& t, const DevBatch& B, const Config& cfg, int p,
                                         Mem& M, bool can_spill, int* spill_code = nullptr,
                                         const EpaResume* rs = nullptr) {
  const int2 pr = B.pairs[p];
  typename SrcOf<L, K>::type src;
  bind_src<L>(src, B.pool, B.bodies[pr.x], B.bodies[pr.y], t.lane());
  GjkState g;
  load_simplex(B.smp + p, B.dist[p], g);
  EpaOut o;
  const EpaResumeSink sink{can_spill ? B.resume : nullptr, B.counts + kCntResume, B.resume_cap};
  epa_pair<kFull>(t, src, cfg, g, M, o, can_spill, sink, rs);
  if (o.spill) {
    if (o.resume >= 0 && t.lane() == 0) B.resume[o.resume].pair = p;
    if (spill_code) *spill_code = o.resume >= 0 ? (kSpillResume | o.resume) : (p | (o.spill64 ? kSpill64 : 0));
    return false;
  }
  const bool lead = t.lane() == 0;
  if (kFull && lead && o.polish) {
    epa_polish(src, o);
    o.polish = false;
  }
  if (lead) {
    B.dist[p] = o.dist;
    gkSimplex* s = B.smp + p;
    s->witnesses[0][0] = o.w0.x;
    s->witnesses[0][1] = o.w0.y;
    s->witnesses[0][2] = o.w0.z;
    s->witnesses[1][0] = o.w1.x;
    s->witnesses[1][1] = o.w1.y;
    s->witnesses[1][2] = o.w1.z;
    store3(B.nrm + 3 * (size_t)p, o.nrm);
    if (B.status) B.status[p] = (B.mode == kModeEpa ? 0 : B.status[p]) | o.status;
  }
  const int q = warp_append(B.counts + kCntPolish, lead && o.polish);
  if (lead && o.polish) {
    PolishRec r;
    r.pair = p;
    r.kind = 1;
    for (int k = 0; k < 3; ++k) {
      r.face[k][0] = o.face[k][0];
      r.face[k][1] = o.face[k][1];
    }
    B.polish[q] = r;
  }
  return true;
}

// EPA over one bucket's contacts with the small working set (EpaMemSmall per team in
// shared memory); contacts that need more than kEpaSmallIters expansions, or whose FP32
// expansion met an inconsistent horizon, go to the spill list
template <int L, int K, int OCC = 1>
__global__ void __launch_bounds__(128, OCC) k_epa(DevBatch B, int bucket) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  EpaMemSmall* mem = reinterpret_cast<EpaMemSmall*>(smem_raw);
  const WarpTeam<L> t;
  EpaMemSmall& M = mem[threadIdx.x / L];
  const int team = (blockIdx.x * blockDim.x + threadIdx.x) / L;
  const int nteams = (gridDim.x * blockDim.x) / L;
  const int cnt = B.counts[kCntEpa + bucket];
  const int* list = B.elists + (size_t)bucket * B.npairs;
  for (int j = team; j < cnt; j += nteams) {
    const int p = list[j];
    int code = 0;
    const bool ok = epa_item<L, K>(t, B, B.cfg, p, M, true, &code);
    const bool lead = t.lane() == 0;
    const int q = warp_append(B.counts + kCntSpill, lead && !ok);
    if (lead && !ok) B.spill[q] = code;
    t.sync();  // the next pair reuses M
  }
}

// ---------------------------------------------------------------------------------
// launch table (one translation unit per kernel family, see ogx_k_*.cu)

typedef void (*BucketKernel)(DevBatch, int);

struct KernelInfo {
  BucketKernel fn;
  int L;  // lanes per pair
  int K;  // float4 blocks per lane and body kept in registers (0: read from memory);
          // + 256 * m for a variant compiled for at least m resident blocks per SM
          // (fewer registers per thread, more warps)
};
constexpr int kOccShift = 8;
OGX_HD int variant_blocks(int K) { return K & ((1 << kOccShift) - 1); }

// Compiled variants of the bucket kernels (ogx_k_gjk_*.cu / ogx_k_epa_*.cu).  A variant
// (L, K) can serve a bucket whose bodies have at most 4 L K points (K = 0: any size, the
// points are re-read from memory).  The engine picks one per bucket (autotuned).
int gjk_variants(const KernelInfo** out);
int epa_variants(const KernelInfo** out);
int gjk_variants_a(const KernelInfo** out);
int gjk_variants_b(const KernelInfo** out);
int gjk_variants_c(const KernelInfo** out);
int gjk_variants_d(const KernelInfo** out);
int epa_variants_a(const KernelInfo** out);
int epa_variants_b(const KernelInfo** out);
int epa_variants_c(const KernelInfo** out);

// non-template kernels (ogx_k_misc.cu)
cudaError_t launch_refine(const DevBatch& B, int grid, int grid_full, cudaStream_t st, cudaStream_t st2,
                          cudaEvent_t routed);
cudaError_t launch_epa_spill(const DevBatch& B, int grid, cudaStream_t st, bool late = false);
cudaError_t epa_spill_occupancy(int block, int* per_sm);
cudaError_t refine_occupancy(int block, int* per_sm);
cudaError_t launch_pack(const float* aos, const int64_t* voff, BodyRef* bodies, int nbodies,
                        float* pool, int grid, cudaStream_t st);
cudaError_t launch_bin(const DevBatch& B, int grid, cudaStream_t st);
cudaError_t launch_polish(const DevBatch& B, int grid, cudaStream_t st);
cudaError_t polish_occupancy(int block, int* per_sm);

}  // namespace ogx
