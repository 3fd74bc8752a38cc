// ogx_k_misc.cu -- pool packing, pair binning and the FP64 polish pass.
#include "ogx_kernels.cuh"

namespace ogx {

// ---------------------------------------------------------------------------------
// Packs every body and marks the ones with a NaN or infinite coordinate in the body
// table (point count stored negated, see body_points), which the binning turns into
// OGX_PAIR_BAD_INPUT for their pairs; a later upload of finite points clears the mark.
__global__ void k_pack(const float* __restrict__ aos, const int64_t* __restrict__ voff,
                       BodyRef* __restrict__ bodies, int nbodies, float* __restrict__ pool) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int b = warp; b < nbodies; b += nwarps) {
    const BodyRef r = bodies[b];
    const int n = body_points(r);
    const int n4 = round4(n);
    const float* src = aos + 3 * voff[b];
    float* dst = pool + 4 * (size_t)r.quad;
    bool finite = true;
    for (int i = lane; i < n4; i += 32) {
      const int s = i < n ? i : 0;
      const float x = src[3 * s], y = src[3 * s + 1], z = src[3 * s + 2];
      finite = finite && is_finite(x) && is_finite(y) && is_finite(z);
      dst[i] = x;
      dst[n4 + i] = y;
      dst[2 * n4 + i] = z;
    }
    finite = __all_sync(0xffffffffu, finite);
    if (lane == 0) bodies[b].n = finite ? n : -n;
  }
}

// ---------------------------------------------------------------------------------
__device__ __forceinline__ bool pair_ok(const DevBatch& B, int2 pr) {
  return pr.x >= 0 && pr.x < B.nbodies && pr.y >= 0 && pr.y < B.nbodies;
}

__device__ __forceinline__ void mark_bad(const DevBatch& B, int p) {
  B.dist[p] = __int_as_float(0x7fc00000);
  if (B.status) B.status[p] = OGX_S_BAD_INPUT;
  if (B.nrm) store3(B.nrm + 3 * (size_t)p, v3<float>(1.f, 0.f, 0.f));
  if (B.mode != kModeEpa) B.smp[p].nvrtx = 0;
}

__global__ void k_bin(DevBatch B) {
  const int stride = gridDim.x * blockDim.x;
  const int n32 = (B.npairs + 31) & ~31;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n32; p += stride) {
    const bool in = p < B.npairs;
    int b = -1;
    bool bad = false;
    bool work = false;
    if (in) {
      const int2 pr = B.pairs[p];
      bad = !pair_ok(B, pr);
      if (!bad) {
        const int na = B.bodies[pr.x].n, nb = B.bodies[pr.y].n;
        bad = na < 1 || nb < 1;
        b = bucket_of(na > nb ? na : nb);
      }
      if (bad) {
        mark_bad(B, p);
      } else if (B.mode == kModeEpa) {
        // EPA only: contacts go to the EPA lists, separated pairs only get a normal
        const gkSimplex& s = B.smp[p];
        work = s.nvrtx == 4 || !(B.dist[p] > FLT_EPSILON);
        if (!work) {
          MemBodies mb;
          mb.bind(B.pool, B.bodies[pr.x], B.bodies[pr.y]);
          store3(B.nrm + 3 * (size_t)p, simplex_sep_normal(mb, s));
          if (B.status) B.status[p] = 0;
        }
      } else {
        work = true;
      }
    }
    // warp-aggregated append per bucket
    const int key = work ? b : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int wl = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    if (key >= 0) {
      int* ctr = B.counts + (B.mode == kModeEpa ? kCntEpa : kCntGjk) + key;
      int* list = (B.mode == kModeEpa ? B.elists : B.lists) + (size_t)key * B.npairs;
      int base = 0;
      if (wl == leader) base = atomicAdd(ctr, __popc(peers));
      base = __shfl_sync(peers, base, leader);
      list[base + __popc(peers & ((1u << wl) - 1u))] = p;
    }
  }
}

// After FP64 refinement: contacts join their bucket's EPA list, separated pairs get their
// normal from the refined witnesses.
__device__ void refine_store(const DevBatch& B, int p, const BodyRef& ra, const BodyRef& rb, const GjkState& g) {
  store_simplex(B.smp + p, g);
  B.dist[p] = g.dist;
  if (B.status) B.status[p] |= g.status;
  if (B.mode == kModeGjkEpa) {
    if (gjk_contact(g)) {
      // the FP32 pass called it separated: a contact within rounding of the boundary,
      // for the certified full-capacity pass over the late list (filled from the end of
      // the spill array: these pairs are not contacts of the FP32 pass, so both lists
      // together hold at most npairs entries)
      const int q = atomicAdd(B.counts + kCntSpillLate, 1);
      B.spill[B.npairs - 1 - q] = p | kSpill64;
    } else {
      store3(B.nrm + 3 * (size_t)p, sep_normal(g));
    }
  }
}

// The pair's bodies for the FP64 passes: as stored, or posed (the posed pipeline)
__device__ __forceinline__ void bind_mem(MemBodies& mb, const DevBatch& B, int2, BodyRef ra, BodyRef rb) {
  mb.bind(B.pool, ra, rb);
}
__device__ __forceinline__ void bind_mem(Posed<MemBodies>& mb, const DevBatch& B, int2 pr, BodyRef ra,
                                         BodyRef rb) {
  mb.bind_posed(B.pool, ra, rb, B.xf + 12 * (size_t)pr.x, B.xf + 12 * (size_t)pr.y);
}
// lane j's bodies, for a scan by the whole warp
__device__ __forceinline__ void shfl_bodies(MemBodies& to, const MemBodies& from, int j) {
  for (int w = 0; w < 2; ++w) {
    to.base[w] = reinterpret_cast<const float*>(
        __shfl_sync(0xffffffffu, reinterpret_cast<long long>(from.base[w]), j));
    to.n[w] = __shfl_sync(0xffffffffu, from.n[w], j);
    to.n4[w] = __shfl_sync(0xffffffffu, from.n4[w], j);
  }
}
__device__ __forceinline__ void shfl_bodies(Posed<MemBodies>& to, const Posed<MemBodies>& from, int j) {
  shfl_bodies(static_cast<MemBodies&>(to), static_cast<const MemBodies&>(from), j);
  for (int w = 0; w < 2; ++w)
    to.xf[w] = reinterpret_cast<const float*>(
        __shfl_sync(0xffffffffu, reinterpret_cast<long long>(from.xf[w]), j));
}

// Re-solve of separated pairs (one thread per pair).  Pairs whose final support the GJK
// kernel proved exact only need the exact closest point of their simplex, computed in
// double-float arithmetic; the others are passed to k_refine_lane / k_refine_full.
template <bool kPosed>
__global__ void __launch_bounds__(128) k_refine(DevBatch B) {
  const int cnt = B.counts[kCntRefine];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
    const RefineRec rr = B.refine[k];
    const int p = rr.pair;
    const int2 pr = B.pairs[p];
    const BodyRef ra = B.bodies[pr.x], rb = B.bodies[pr.y];
    if (!rr.certain) {
      if ((ra.n > rb.n ? ra.n : rb.n) <= kRefineLaneMax) {
        const int q = atomicAdd(B.counts + kCntRefineFull, 1);
        B.refine_full[q] = p;
      } else {
        const int q = atomicAdd(B.counts + kCntRefineBig, 1);
        B.refine_full[B.npairs - 1 - q] = p;
      }
      continue;
    }
    typename PoseOf<kPosed, MemBodies>::type mb;
    bind_mem(mb, B, pr, ra, rb);
    GjkState g;
    load_simplex(B.smp + p, B.dist[p], g);
    g.certain = true;
    SerialTeam one;
    gjk_refine(one, mb, g, kRefineIters);
    refine_store(B, p, ra, rb, g);
  }
}

// FP64 continuation of GJK for the pairs with an uncertain FP32 support and bodies of
// at most kRefineLaneMax points: one thread per pair, so that each FP64 instruction
// serves 32 pairs (FP64 issues at 1/64 of the FP32 rate here).
template <bool kPosed>
__global__ void __launch_bounds__(128) k_refine_lane(DevBatch B) {
  const int cnt = B.counts[kCntRefineFull];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
    const int p = B.refine_full[k];
    const int2 pr = B.pairs[p];
    const BodyRef ra = B.bodies[pr.x], rb = B.bodies[pr.y];
    typename PoseOf<kPosed, MemBodies>::type mb;
    bind_mem(mb, B, pr, ra, rb);
    GjkState g;
    load_simplex(B.smp + p, B.dist[p], g);
    g.certain = false;
    SerialTeam one;
    gjk_refine(one, mb, g, kRefineIters);
    refine_store(B, p, ra, rb, g);
  }
}

// The same for larger bodies: a warp takes 32 pairs, one per lane; each FP64 iteration
// runs the exact-support scans of every unfinished pair with all 32 lanes (pair j's
// bodies and direction broadcast from lane j), then each lane takes its own pair's FP64
// sub-distance step, so the scalar FP64 work serves 32 pairs per instruction.
template <bool kPosed>
__global__ void __launch_bounds__(128) k_refine_full(DevBatch B) {
  const WarpTeam<32> t;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int cnt = B.counts[kCntRefineBig];
  for (int base = 32 * warp; base < cnt; base += 32 * nwarps) {
    const int k = base + lane;
    const bool valid = k < cnt;
    int p = -1;
    BodyRef ra{0u, 1}, rb{0u, 1};
    typename PoseOf<kPosed, MemBodies>::type mb;
    bind_mem(mb, B, make_int2(0, 0), ra, rb);  // never scanned: this lane's r.done stays set
    GjkState g;
    RefineState r;
    r.done = true;
    if (valid) {
      p = B.refine_full[B.npairs - 1 - k];
      const int2 pr = B.pairs[p];
      ra = B.bodies[pr.x];
      rb = B.bodies[pr.y];
      bind_mem(mb, B, pr, ra, rb);
      load_simplex(B.smp + p, B.dist[p], g);
      g.certain = false;
      refine_begin(mb, g, kRefineIters, r);
    }
    for (;;) {
      const unsigned m = __ballot_sync(full, !r.done);
      if (m == 0u) break;
      int my_xa = 0, my_xb = 0;
      for (unsigned mm = m; mm != 0u; mm &= mm - 1u) {
        const int j = __ffs(mm) - 1;
        typename PoseOf<kPosed, MemBodies>::type bj;
        shfl_bodies(bj, mb, j);
        const dv3 vj = v3<double>(__shfl_sync(full, r.v.x, j), __shfl_sync(full, r.v.y, j),
                                  __shfl_sync(full, r.v.z, j));
        double va, vb;
        const int xa = exact_support(t, bj, 0, -vj, va);
        const int xb = exact_support(t, bj, 1, vj, vb);
        if (lane == j) {
          my_xa = xa;
          my_xb = xb;
        }
      }
      if (!r.done) refine_step(mb, r, my_xa, my_xb);
    }
    if (valid) {
      refine_end(mb, r, g);
      refine_store(B, p, ra, rb, g);
    }
  }
}

template <bool kPosed>
__global__ void __launch_bounds__(128) k_polish(DevBatch B) {
  const int cnt = B.counts[kCntPolish];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
    const PolishRec r = B.polish[k];
    const int p = r.pair;
    const int2 pr = B.pairs[p];
    typename PoseOf<kPosed, MemBodies>::type mb;
    bind_mem(mb, B, pr, B.bodies[pr.x], B.bodies[pr.y]);
    gkSimplex* s = B.smp + p;
    {
      EpaOut o;
      for (int m = 0; m < 3; ++m) {
        o.face[m][0] = r.face[m][0];
        o.face[m][1] = r.face[m][1];
      }
      const float* n = B.nrm + 3 * (size_t)p;
      o.nrm = v3<float>(n[0], n[1], n[2]);
      o.dist = B.dist[p];
      o.status = 0;
      epa_polish(mb, o);
      if (!(o.status & OGX_S_POLISHED)) continue;
      B.dist[p] = o.dist;
      s->witnesses[0][0] = o.w0.x;
      s->witnesses[0][1] = o.w0.y;
      s->witnesses[0][2] = o.w0.z;
      s->witnesses[1][0] = o.w1.x;
      s->witnesses[1][1] = o.w1.y;
      s->witnesses[1][2] = o.w1.z;
      store3(B.nrm + 3 * (size_t)p, o.nrm);
    }
    if (B.status) B.status[p] |= OGX_S_POLISHED;
  }
}


// Pack from a table of coordinate pointers (one per body, xyz interleaved) that address
// the caller's host arrays: on a device that reads pageable host memory through the host's
// page tables (cudaDevAttrPageableMemoryAccess, the GPU of a Grace system over NVLink-C2C)
// the kernel loads the points where the caller keeps them, so the host gathers nothing.
// Bodies with a NaN or infinite coordinate are marked as k_pack does.
__global__ void k_pack_ptrs(const float* const* __restrict__ src, int nb, BodyRef* __restrict__ bodies,
                            float* __restrict__ pool) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int b = warp; b < nb; b += nwarps) {
    const BodyRef r = bodies[b];
    const float* c = src[b];
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

cudaError_t launch_pack_ptrs(const float* const* src, int nbodies, BodyRef* bodies, float* pool, int grid,
                             cudaStream_t st) {
  if (nbodies <= 0) return cudaSuccess;
  k_pack_ptrs<<<grid, 256, 0, st>>>(src, nbodies, bodies, pool);
  return cudaGetLastError();
}

cudaError_t launch_pack(const float* aos, const int64_t* voff, BodyRef* bodies, int nbodies,
                        float* pool, int grid, cudaStream_t st) {
  k_pack<<<grid, 256, 0, st>>>(aos, voff, bodies, nbodies, pool);
  return cudaGetLastError();
}

cudaError_t launch_bin(const DevBatch& B, int grid, cudaStream_t st) {
  k_bin<<<grid, 256, 0, st>>>(B);
  return cudaGetLastError();
}

// EPA at full capacity over the spill list: contacts that ran out of the small working
// set, and -- certified, every face plane from FP64, exact supports -- contacts whose FP32
// expansion met an inconsistent horizon or stopped short of the FP32 rounding level; or
// (late != 0) over the contacts the FP64 refinement found, all certified.  One warp per
// contact, points read from memory (any body size).
template <bool kPosed>
__global__ void __launch_bounds__(128) k_epa_spill(DevBatch B, int late) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  EpaMemCert* mem = reinterpret_cast<EpaMemCert*>(smem_raw);
  const WarpTeam<32> t;
  EpaMemCert& M = mem[threadIdx.x / 32];
  const int team = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int nteams = (gridDim.x * blockDim.x) / 32;
  const int cnt = B.counts[late ? kCntSpillLate : kCntSpill];
  Config cfg64 = B.cfg;
  cfg64.flags |= OGX_F_EPA_FP64_PLANES;
  for (int j = team; j < cnt; j += nteams) {
    const int e = late ? B.spill[B.npairs - 1 - j] : B.spill[j];
    if (e & kSpillResume) {  // continue the small pass's saved expansion
      const EpaResume* rs = B.resume + (e & (kSpillResume - 1));
      epa_item<32, 0, true, 0, kPosed>(t, B, B.cfg, rs->pair, M, false, nullptr, rs);
    } else {
      epa_item<32, 0, true, 0, kPosed>(t, B, (e & kSpill64) ? cfg64 : B.cfg, e & ~kSpill64, M, false);
    }
    t.sync();
  }
}

// the launchers run the posed kernels when the batch carries poses (B.xf)
cudaError_t launch_epa_spill(const DevBatch& B, int grid, cudaStream_t st, bool late) {
  if (B.xf)
    k_epa_spill<true><<<grid, 128, 4 * sizeof(EpaMemCert), st>>>(B, late ? 1 : 0);
  else
    k_epa_spill<false><<<grid, 128, 4 * sizeof(EpaMemCert), st>>>(B, late ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t epa_spill_occupancy(int block, int* per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_epa_spill<false>, block,
                                                       (block / 32) * sizeof(EpaMemCert));
}

cudaError_t launch_polish(const DevBatch& B, int grid, cudaStream_t st) {
  if (B.xf)
    k_polish<true><<<grid, 128, 0, st>>>(B);
  else
    k_polish<false><<<grid, 128, 0, st>>>(B);
  return cudaGetLastError();
}

// k_refine routes the continuations; the two continuation kernels are independent and
// run on st and st2 (the same stream when st2 == st; the caller joins st2 back)
cudaError_t launch_refine(const DevBatch& B, int grid, int grid_full, cudaStream_t st, cudaStream_t st2,
                          cudaEvent_t routed) {
  if (B.xf)
    k_refine<true><<<grid, 128, 0, st>>>(B);
  else
    k_refine<false><<<grid, 128, 0, st>>>(B);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && st2 != st) {
    e = cudaEventRecord(routed, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st2, routed, 0);
  }
  if (e != cudaSuccess) return e;
  if (B.xf) {
    k_refine_lane<true><<<grid, 128, 0, st>>>(B);
    k_refine_full<true><<<grid_full, 128, 0, st2>>>(B);
  } else {
    k_refine_lane<false><<<grid, 128, 0, st>>>(B);
    k_refine_full<false><<<grid_full, 128, 0, st2>>>(B);
  }
  return cudaGetLastError();
}

cudaError_t refine_occupancy(int block, int* per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_refine<false>, block, 0);
}

cudaError_t polish_occupancy(int block, int* per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_polish<false>, block, 0);
}

}  // namespace ogx
