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
  const float* xf;    // posed kernels only: 12 floats per body (R row-major, t), the pool
                      // then holds the bodies in their own frame
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
// source of body points for bucket kernels: registers (K > 0), memory (K == 0), or
// memory staged through D shared-memory slots per lane (K == 0, D > 0)
template <int L, int K, int D = 0>
struct SrcOf {
  typedef RegBodies<L, K> type;
};
template <int L>
struct SrcOf<L, 0, 0> {
  typedef MemBodies type;
};
template <int L, int D>
struct SrcOf<L, 0, D> {
  typedef StagedBodies<L, D> type;
};

// the GJK kernels' memory scans keep four blocks per lane in flight
template <int L, int K, int D = 0>
struct GjkSrcOf {
  typedef typename SrcOf<L, K, D>::type type;
};
template <int L>
struct GjkSrcOf<L, 0, 0> {
  typedef WideMemBodies type;
};
// posed kernel variants (memory scans only): the source of the plain variant with the
// poses applied on the fly
template <bool kPosed, class Src>
struct PoseOf {
  typedef Src type;
};
template <class Src>
struct PoseOf<true, Src> {
  typedef Posed<Src> type;
};

// shared memory of the staging slots of a block of kStageStride threads
OGX_HD constexpr size_t staging_bytes(int D) { return D > 0 ? (size_t)(D + 1) * 3 * sizeof(float4) * kStageStride : 0; }

// xa, xb: the poses of the pair's bodies (read by posed sources only)
template <int L, int K>
__device__ __forceinline__ void bind_src(RegBodies<L, K>& s, const float* pool, BodyRef a,
                                         BodyRef b, int lane, float4*, const float*, const float*) {
  s.bind(pool, a, b, lane);
}
template <int L>
__device__ __forceinline__ void bind_src(MemBodies& s, const float* pool, BodyRef a, BodyRef b,
                                         int, float4*, const float*, const float*) {
  s.bind(pool, a, b);
}
template <int L, int D>
__device__ __forceinline__ void bind_src(StagedBodies<L, D>& s, const float* pool, BodyRef a,
                                         BodyRef b, int lane, float4* slots, const float*, const float*) {
  s.bind(pool, a, b, lane, slots);
}
template <int L, class Base>
__device__ __forceinline__ void bind_src(Posed<Base>& s, const float* pool, BodyRef a, BodyRef b,
                                         int, float4*, const float* xa, const float* xb) {
  s.bind_posed(pool, a, b, xa, xb);
}
// the pose of body i (posed kernels), or null
template <bool kPosed>
__device__ __forceinline__ const float* pose_of(const DevBatch& B, int i) {
  return kPosed ? B.xf + 12 * (size_t)i : nullptr;
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

template <int L, int K, int OCC = 1, int D = 0, bool kPosed = false>
__global__ void __launch_bounds__(kStageStride, OCC) k_gjk(DevBatch B, int bucket) {
  extern __shared__ __align__(16) unsigned char smem_raw[];  // staging slots (D > 0)
  float4* slots = reinterpret_cast<float4*>(smem_raw) + threadIdx.x;
  const WarpTeam<L> t;
  const int team = (blockIdx.x * blockDim.x + threadIdx.x) / L;
  const int nteams = (gridDim.x * blockDim.x) / L;
  const int cnt = B.counts[kCntGjk + bucket];
  const int* list = B.lists + (size_t)bucket * B.npairs;
  for (int j = team; j < cnt; j += nteams) {
    const int p = list[j];
    const int2 pr = B.pairs[p];
    const BodyRef ra = B.bodies[pr.x], rb = B.bodies[pr.y];
    typename PoseOf<kPosed, typename GjkSrcOf<L, K, D>::type>::type src;
    bind_src<L>(src, B.pool, ra, rb, t.lane(), slots, pose_of<kPosed>(B, pr.x), pose_of<kPosed>(B, pr.y));
    int2 ws = make_int2(0, 0);
    if (B.warm) {
      ws = B.warm[p];
      if (ws.x < 0 || ws.x >= ra.n || ws.y < 0 || ws.y >= rb.n) ws = make_int2(0, 0);
    }
    GjkState g;
    gjk_pair(t, src, B.cfg, g, ws.x, ws.y, B.subtab);
    gjk_store(B, bucket, p, g, t.lane() == 0);
  }
  if constexpr (D > 0) cp_async_wait<0>();  // no copy outlives the block
}


// kFull: the full-capacity pass over the spill list -- certified re-runs where the entry
// asks for FP64 planes, and the FP64 polish of the result done here by lane 0 instead of
// through the polish list, so that the polish pass need not wait for this one
// spill list entry codes: a pair index, or a saved expansion to resume
constexpr int kSpill64 = 1 << 30;      // the re-run solves every face plane in FP64
constexpr int kSpillResume = 1 << 29;  // low bits: the EpaResume record to continue

template <int L, int K, bool kFull = false, int D = 0, bool kPosed = false, class Mem>
__device__ __forceinline__ bool epa_item(const WarpTeam<L>& t, const DevBatch& B, const Config& cfg, int p,
                                         Mem& M, bool can_spill, int* spill_code = nullptr,
                                         const EpaResume* rs = nullptr, float4* slots = nullptr) {
  const int2 pr = B.pairs[p];
  typename PoseOf<kPosed, typename SrcOf<L, K, D>::type>::type src;
  bind_src<L>(src, B.pool, B.bodies[pr.x], B.bodies[pr.y], t.lane(), slots, pose_of<kPosed>(B, pr.x),
              pose_of<kPosed>(B, pr.y));
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
// Byte stride between the teams' working sets in shared memory: whole 128-byte lines
// plus 4 L bytes, so that the teams of a warp start L banks apart and their lanes' 4-byte
// and 1-byte accesses to the same field of their own working sets fall in different banks
// (the unpadded 2288-byte sets started 28 banks apart, and lanes of neighbouring teams
// met in the same banks: 466k conflicts in one 16-point EPA launch).
OGX_HD constexpr size_t epa_team_stride(int L) {
  return (sizeof(EpaMemSmall) + 127) / 128 * 128 + (L >= 4 ? (4 * (size_t)L) % 128 : 16);
}

// shared memory of k_epa: the teams' working sets, then the staging slots (D > 0)
template <int L>
OGX_HD constexpr size_t epa_mem_bytes() { return (kStageStride / L) * epa_team_stride(L); }

template <int L, int K, int OCC = 1, int D = 0, bool kPosed = false>
__global__ void __launch_bounds__(kStageStride, OCC) k_epa(DevBatch B, int bucket) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4* slots = reinterpret_cast<float4*>(smem_raw + epa_mem_bytes<L>()) + threadIdx.x;
  const WarpTeam<L> t;
  EpaMemSmall& M = *reinterpret_cast<EpaMemSmall*>(smem_raw + (threadIdx.x / L) * epa_team_stride(L));
  const int team = (blockIdx.x * blockDim.x + threadIdx.x) / L;
  const int nteams = (gridDim.x * blockDim.x) / L;
  const int cnt = B.counts[kCntEpa + bucket];
  const int* list = B.elists + (size_t)bucket * B.npairs;
  for (int j = team; j < cnt; j += nteams) {
    const int p = list[j];
    int code = 0;
    const bool ok = epa_item<L, K, false, D, kPosed>(t, B, B.cfg, p, M, true, &code, nullptr, slots);
    const bool lead = t.lane() == 0;
    const int q = warp_append(B.counts + kCntSpill, lead && !ok);
    if (lead && !ok) B.spill[q] = code;
    t.sync();  // the next pair reuses M
  }
  if constexpr (D > 0) cp_async_wait<0>();  // no copy outlives the block
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
          // + 65536 * D for a memory variant that stages D blocks per lane through
          // shared memory
};
constexpr int kOccShift = 8;
constexpr int kStageShift = 16;
OGX_HD int variant_blocks(int K) { return K & ((1 << kOccShift) - 1); }
OGX_HD int variant_stages(int K) { return (K >> kStageShift) & 0xff; }

// Compiled variants of the bucket kernels (ogx_k_gjk_*.cu / ogx_k_epa_*.cu).  A variant
// (L, K) can serve a bucket whose bodies have at most 4 L K points (K = 0: any size, the
// points are re-read from memory).  The engine picks one per bucket (autotuned).
int gjk_variants(const KernelInfo** out);
int epa_variants(const KernelInfo** out);
int gjk_variants_a(const KernelInfo** out);
int gjk_variants_b(const KernelInfo** out);
int gjk_variants_c(const KernelInfo** out);
int gjk_variants_d(const KernelInfo** out);
int gjk_variants_e(const KernelInfo** out);
int epa_variants_a(const KernelInfo** out);
int epa_variants_b(const KernelInfo** out);
int epa_variants_c(const KernelInfo** out);
int epa_variants_d(const KernelInfo** out);
// the posed kernels (ogx_k_posed.cu): one GJK and one EPA variant per bucket
void posed_variants(const KernelInfo** gjk, const KernelInfo** epa);

// non-template kernels (ogx_k_misc.cu)
cudaError_t launch_refine(const DevBatch& B, int grid, int grid_full, cudaStream_t st, cudaStream_t st2,
                          cudaEvent_t routed);
cudaError_t launch_epa_spill(const DevBatch& B, int grid, cudaStream_t st, bool late = false);
cudaError_t epa_spill_occupancy(int block, int* per_sm);
cudaError_t refine_occupancy(int block, int* per_sm);
cudaError_t launch_pack(const float* aos, const int64_t* voff, BodyRef* bodies, int nbodies,
                        float* pool, int grid, cudaStream_t st);
// packs bodies whose points the device reads where the caller keeps them (src[b]: xyz of
// body b, host memory of a device that reads pageable memory); bodies[] already holds
// each body's count and pool offset
cudaError_t launch_pack_ptrs(const float* const* src, int nbodies, BodyRef* bodies, float* pool, int grid,
                             cudaStream_t st);
cudaError_t launch_bin(const DevBatch& B, int grid, cudaStream_t st);
cudaError_t launch_polish(const DevBatch& B, int grid, cudaStream_t st);
cudaError_t polish_occupancy(int block, int* per_sm);

}  // namespace ogx
