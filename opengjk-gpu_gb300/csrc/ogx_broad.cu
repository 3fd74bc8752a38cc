// ogx_broad.cu -- device broad phase: candidate pairs from the bodies' boxes on a uniform
// grid, the producer of the narrow phase's pair lists.
//
// The reference's visualiser builds its per-frame pairs with a uniform grid (count / scan
// / generate, visualization/integrate_final_gjk.cu:467-570 and 916-1002, with the scan of
// visualization/utils/scan_kernels.cuh:194) and copies counts to the host between steps.
// Here everything stays on the device and the output is deterministic:
//   1. k_box       axis-aligned box of every body (min / max over its points), grown by a
//                  margin, and the number of grid cells it touches;
//   2. scan        cell entries per body -> entry offsets;
//   3. k_entries   one entry (cell key, body) per touched cell, counted per hash bucket;
//   4. scan        bucket counts -> bucket offsets; k_scatter groups entries by bucket;
//   5. k_pairs     per body i: every body j > i sharing one of i's cells whose box
//                  overlaps i's box, emitted only in the cell holding the low corner of
//                  the two boxes' intersection (so once); pass 1 counts, a scan gives
//                  each body its output range, pass 2 writes and sorts the range by j.
// The result is every overlapping pair (i < j) exactly once, sorted by (i, j),
// whatever the grid resolution; the cell size only changes the work.
#include <cuda_runtime.h>

#include <algorithm>

#include "ogx_engine.h"

using namespace ogx;

namespace {

constexpr int kMaxCellsPerBody = 64;
constexpr int kAxisBits = 21;                  // cell coordinates in (-2^20, 2^20)
constexpr int kAxisBias = 1 << (kAxisBits - 1);

__device__ __forceinline__ uint64_t cell_key(int x, int y, int z) {
  const uint64_t m = (1ull << kAxisBits) - 1ull;
  return ((uint64_t)(x + kAxisBias) & m) | (((uint64_t)(y + kAxisBias) & m) << kAxisBits) |
         (((uint64_t)(z + kAxisBias) & m) << (2 * kAxisBits));
}

__device__ __forceinline__ uint32_t key_hash(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  return (uint32_t)k;
}

__device__ __forceinline__ int cell_of(float x, float inv) { return (int)floorf(x * inv); }

// flags in the error word
enum { kErrCellRange = 1, kErrCellsPerBody = 2 };

__global__ void k_box(const float* __restrict__ pool, const BodyRef* __restrict__ bodies, int n, float margin,
                      float inv_cell, float4* __restrict__ lo, float4* __restrict__ hi, int* __restrict__ ncells,
                      int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int b = warp; b < n; b += nwarps) {
    const BodyRef r = bodies[b];
    if (r.n < 1) {  // no points, or a NaN / infinite coordinate: the body takes no cell
      if (lane == 0) {
        lo[b] = make_float4(INFINITY, INFINITY, INFINITY, 0.0f);
        hi[b] = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
        ncells[b] = 0;
      }
      continue;
    }
    const int n4 = round4(r.n);
    const float* X = pool + 4 * (size_t)r.quad;
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = lane; i < r.n; i += 32)
      for (int c = 0; c < 3; ++c) {
        const float v = X[c * n4 + i];
        mn[c] = fminf(mn[c], v);
        mx[c] = fmaxf(mx[c], v);
      }
    for (int o = 16; o > 0; o >>= 1)
      for (int c = 0; c < 3; ++c) {
        mn[c] = fminf(mn[c], __shfl_xor_sync(0xffffffffu, mn[c], o));
        mx[c] = fmaxf(mx[c], __shfl_xor_sync(0xffffffffu, mx[c], o));
      }
    if (lane == 0) {
      const float4 l = make_float4(mn[0] - margin, mn[1] - margin, mn[2] - margin, 0.0f);
      const float4 h = make_float4(mx[0] + margin, mx[1] + margin, mx[2] + margin, 0.0f);
      lo[b] = l;
      hi[b] = h;
      long long cnt = 1;
      bool bad = false;
      const float ll[3] = {l.x, l.y, l.z}, hh[3] = {h.x, h.y, h.z};
      for (int c = 0; c < 3; ++c) {
        const int a = cell_of(ll[c], inv_cell), z = cell_of(hh[c], inv_cell);
        bad |= !(a > -kAxisBias && z < kAxisBias);
        cnt *= (long long)(z - a + 1);
      }
      if (bad) atomicOr(err, kErrCellRange);
      if (cnt > kMaxCellsPerBody) atomicOr(err, kErrCellsPerBody);
      ncells[b] = (bad || cnt > kMaxCellsPerBody) ? 0 : (int)cnt;
    }
  }
}

// exclusive scan of n ints in place: tiles of 1024 (one block each) are reduced, the
// tile sums scanned by one block, then every tile scanned with its offset
constexpr int kTile = 1024;

__device__ __forceinline__ int block_incl_scan(int x, int* warp_sums) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = warp_sums[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_sums[lane] = t;
  }
  __syncthreads();
  return x + (w > 0 ? warp_sums[w - 1] : 0);
}

__global__ void __launch_bounds__(kTile) k_tile_sums(const int* __restrict__ a, int n, int* __restrict__ sums) {
  __shared__ int ws[32];
  const int i = blockIdx.x * kTile + threadIdx.x;
  const int inc = block_incl_scan(i < n ? a[i] : 0, ws);
  if (threadIdx.x == kTile - 1) sums[blockIdx.x] = inc;
}

// one block: exclusive scan of the tile sums (at most kTile * kTile elements overall)
__global__ void __launch_bounds__(kTile) k_scan_sums(int* __restrict__ sums, int ntiles, int* __restrict__ total) {
  __shared__ int ws[32];
  const int x = threadIdx.x < ntiles ? sums[threadIdx.x] : 0;
  const int inc = block_incl_scan(x, ws);
  if (threadIdx.x < ntiles) sums[threadIdx.x] = inc - x;
  if (threadIdx.x == kTile - 1 && total) *total = inc;
}

__global__ void __launch_bounds__(kTile) k_tile_scan(int* __restrict__ a, int n, const int* __restrict__ sums) {
  __shared__ int ws[32];
  const int i = blockIdx.x * kTile + threadIdx.x;
  const int x = i < n ? a[i] : 0;
  const int inc = block_incl_scan(x, ws);
  if (i < n) a[i] = sums[blockIdx.x] + inc - x;
}

__global__ void k_entries(const float4* __restrict__ lo, const float4* __restrict__ hi, int n, float inv_cell,
                          const int* __restrict__ eoff, unsigned long long* __restrict__ ekey,
                          int* __restrict__ ebody, uint32_t bmask, int* __restrict__ bcount) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
    const int e0 = eoff[b], e1 = eoff[b + 1];
    if (e1 == e0) continue;
    const float4 l = lo[b], h = hi[b];
    const int x0 = cell_of(l.x, inv_cell), x1 = cell_of(h.x, inv_cell);
    const int y0 = cell_of(l.y, inv_cell), y1 = cell_of(h.y, inv_cell);
    const int z0 = cell_of(l.z, inv_cell), z1 = cell_of(h.z, inv_cell);
    int e = e0;
    for (int x = x0; x <= x1; ++x)
      for (int y = y0; y <= y1; ++y)
        for (int z = z0; z <= z1; ++z) {
          const uint64_t k = cell_key(x, y, z);
          ekey[e] = k;
          ebody[e] = b;
          atomicAdd(bcount + (key_hash(k) & bmask), 1);
          ++e;
        }
  }
}

__global__ void k_scatter(const unsigned long long* __restrict__ ekey, const int* __restrict__ ebody,
                          const int* __restrict__ ne_dev, uint32_t bmask, int* __restrict__ bcursor,
                          unsigned long long* __restrict__ skey, int* __restrict__ sbody) {
  const int ne = *ne_dev;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
    const uint64_t k = ekey[e];
    const int s = atomicAdd(bcursor + (key_hash(k) & bmask), 1);
    skey[s] = k;
    sbody[s] = ebody[e];
  }
}

// pass 0 counts the pairs of every body, pass 1 writes them at off[i] and sorts by j
template <int PASS>
__global__ void k_pairs(const float4* __restrict__ lo, const float4* __restrict__ hi, int n, float inv_cell,
                        const int* __restrict__ eoff, const unsigned long long* __restrict__ ekey,
                        uint32_t bmask, const int* __restrict__ boff, const int* __restrict__ bend,
                        const unsigned long long* __restrict__ skey, const int* __restrict__ sbody,
                        int* __restrict__ pcount, int2* __restrict__ out, int cap) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 li = lo[i], hi_ = hi[i];
    int cnt = 0;
    const int base = PASS == 1 ? pcount[i] : 0;
    for (int e = eoff[i]; e < eoff[i + 1]; ++e) {
      const uint64_t k = ekey[e];
      const uint32_t h = key_hash(k) & bmask;
      for (int s = boff[h]; s < bend[h]; ++s) {
        if (skey[s] != k) continue;
        const int j = sbody[s];
        if (j <= i) continue;
        const float4 lj = lo[j], hj = hi[j];
        const float mx = fmaxf(li.x, lj.x), my = fmaxf(li.y, lj.y), mz = fmaxf(li.z, lj.z);
        if (mx > fminf(hi_.x, hj.x) || my > fminf(hi_.y, hj.y) || mz > fminf(hi_.z, hj.z)) continue;
        if (cell_key(cell_of(mx, inv_cell), cell_of(my, inv_cell), cell_of(mz, inv_cell)) != k) continue;
        if (PASS == 1 && base + cnt < cap) out[base + cnt] = make_int2(i, j);
        ++cnt;
      }
    }
    if (PASS == 0) {
      pcount[i] = cnt;
    } else {
      // sort this body's range by j (insertion sort: ranges are short)
      const int m = min(cnt, cap - base);
      for (int a = 1; a < m; ++a) {
        const int2 v = out[base + a];
        int b = a - 1;
        while (b >= 0 && out[base + b].y > v.y) {
          out[base + b + 1] = out[base + b];
          --b;
        }
        out[base + b + 1] = v;
      }
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------------
// bodies made of several convex parts (sub-meshes): pair expansion and reduction

static __global__ void k_sub_count(const int2* __restrict__ bp, int n, const int* __restrict__ cnt, int nb,
                            int* __restrict__ out) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int2 q = bp[p];
    const bool ok = q.x >= 0 && q.x < nb && q.y >= 0 && q.y < nb;
    out[p] = ok ? cnt[q.x] * cnt[q.y] : 0;
  }
}

static __global__ void k_sub_expand(const int2* __restrict__ bp, int n, const int* __restrict__ first,
                             const int* __restrict__ cnt, int nb, const int* __restrict__ off, int cap,
                             int2* __restrict__ sub, int* __restrict__ owner) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int2 q = bp[p];
    if (!(q.x >= 0 && q.x < nb && q.y >= 0 && q.y < nb)) continue;
    const int fa = first[q.x], ca = cnt[q.x], fb = first[q.y], cb = cnt[q.y];
    int w = off[p];
    for (int a = 0; a < ca; ++a)
      for (int b = 0; b < cb; ++b, ++w)
        if (w < cap) {
          sub[w] = make_int2(fa + a, fb + b);
          if (owner) owner[w] = p;
        }
  }
}

// smallest distance (most penetrating) over each body pair's parts; -1 / +inf when none
static __global__ void k_sub_reduce(const int* __restrict__ off, int n, int cap, const float* __restrict__ dist,
                             float* __restrict__ best, int* __restrict__ arg) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int e = min(off[p + 1], cap);
    float b = INFINITY;
    int k = -1;
    for (int i = off[p]; i < e; ++i)
      if (dist[i] < b) {
        b = dist[i];
        k = i;
      }
    best[p] = b;
    if (arg) arg[p] = k;
  }
}

// ---------------------------------------------------------------------------------
// Bounding-sphere mode: the reference's own pair semantics (visualization/
// integrate_final_gjk.cu:467-570).  Body b is a sphere (x, y, z, r); it lives in the one
// grid cell of its centre, floor((p + boundary) / cell) per axis clamped to
// [0, grid_size), and pairs (i, j > i) are the bodies in i's 27 neighbouring cells whose
// spheres overlap: fx*fx + fy*fy + fz*fz < (r_i + r_j)^2, evaluated in FP32 in that order
// (no fused multiply-add, as the reference builds its CUDA).  Pairs whose centres lie
// more than one cell apart are not found even when the spheres overlap -- the
// reference's behaviour, kept.  The reference stores at most a fixed number of bodies
// per cell and drops the rest in an order set by atomics; the cells here have no such
// capacity, so the pair sets agree whenever no reference cell overflows.

__device__ __forceinline__ void sphere_cell(float4 s, float cell, float boundary, int grid, int& cx, int& cy,
                                            int& cz) {
  cx = min(max((int)floorf(__fdiv_rn(__fadd_rn(s.x, boundary), cell)), 0), grid - 1);
  cy = min(max((int)floorf(__fdiv_rn(__fadd_rn(s.y, boundary), cell)), 0), grid - 1);
  cz = min(max((int)floorf(__fdiv_rn(__fadd_rn(s.z, boundary), cell)), 0), grid - 1);
}

__device__ __forceinline__ bool spheres_overlap(float4 a, float4 b) {
  const float fx = __fsub_rn(a.x, b.x), fy = __fsub_rn(a.y, b.y), fz = __fsub_rn(a.z, b.z);
  const float r = __fadd_rn(a.w, b.w);
  const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)), __fmul_rn(fz, fz));
  return d2 < __fmul_rn(r, r);
}

__global__ void k_sph_entries(const float4* __restrict__ sph, int n, float cell, float boundary, int grid,
                              unsigned long long* __restrict__ ekey, int* __restrict__ ebody, uint32_t bmask,
                              int* __restrict__ bcount, int* __restrict__ nentries) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *nentries = n;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
    int cx, cy, cz;
    sphere_cell(sph[b], cell, boundary, grid, cx, cy, cz);
    const uint64_t k = cell_key(cx, cy, cz);
    ekey[b] = k;
    ebody[b] = b;
    atomicAdd(bcount + (key_hash(k) & bmask), 1);
  }
}

// pass 0 counts the pairs of every body, pass 1 writes them at off[i] and sorts by j
template <int PASS>
__global__ void k_sph_pairs(const float4* __restrict__ sph, int n, float cell, float boundary, int grid,
                            uint32_t bmask, const int* __restrict__ boff, const int* __restrict__ bend,
                            const unsigned long long* __restrict__ skey, const int* __restrict__ sbody,
                            int* __restrict__ pcount, int2* __restrict__ out, int cap) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 si = sph[i];
    int cx, cy, cz;
    sphere_cell(si, cell, boundary, grid, cx, cy, cz);
    int cnt = 0;
    const int base = PASS == 1 ? pcount[i] : 0;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int x = cx + dx, y = cy + dy, z = cz + dz;
          if (x < 0 || x >= grid || y < 0 || y >= grid || z < 0 || z >= grid) continue;
          const uint64_t k = cell_key(x, y, z);
          const uint32_t h = key_hash(k) & bmask;
          for (int s = boff[h]; s < bend[h]; ++s) {
            if (skey[s] != k) continue;
            const int j = sbody[s];
            if (j <= i || !spheres_overlap(si, sph[j])) continue;
            if (PASS == 1 && base + cnt < cap) out[base + cnt] = make_int2(i, j);
            ++cnt;
          }
        }
    if (PASS == 0) {
      pcount[i] = cnt;
    } else {
      const int m = min(cnt, cap - base);
      for (int a = 1; a < m; ++a) {
        const int2 v = out[base + a];
        int c = a - 1;
        while (c >= 0 && out[base + c].y > v.y) {
          out[base + c + 1] = out[base + c];
          --c;
        }
        out[base + c + 1] = v;
      }
    }
  }
}

struct ogx_broad {
  ogx_ctx* ctx = nullptr;
  int max_bodies = 0;
  uint32_t nbuckets = 0;
  float4 *lo = nullptr, *hi = nullptr;
  int* eoff = nullptr;        // max_bodies + 1
  unsigned long long* ekey = nullptr;
  int* ebody = nullptr;       // max_bodies * kMaxCellsPerBody entries
  unsigned long long* skey = nullptr;
  int* sbody = nullptr;
  int* boff = nullptr;        // nbuckets
  int* bend = nullptr;        // nbuckets
  int* pcount = nullptr;      // max_bodies + 1
  int* scal = nullptr;        // [0] entries, [1] pairs, [2] error flags
  int* tiles = nullptr;       // tile sums of the scans
};

// exclusive scan of a[0..n) on the stream; *total = the sum (may be null)
cudaError_t scan(ogx_broad* B, int* a, int n, int* total, cudaStream_t st) {
  const int ntiles = (n + kTile - 1) / kTile;
  if (ntiles > kTile) return cudaErrorInvalidValue;
  k_tile_sums<<<ntiles, kTile, 0, st>>>(a, n, B->tiles);
  k_scan_sums<<<1, kTile, 0, st>>>(B->tiles, ntiles, total);
  k_tile_scan<<<ntiles, kTile, 0, st>>>(a, n, B->tiles);
  return cudaGetLastError();
}

// exclusive scan of a[0..n) (n <= kTile * kTile) on a stream, with a caller's buffer of
// kTile ints for the tile sums (also used by the collision response)
ogx_status broad_scan(int* a, int n, int* total, cudaStream_t st, int* tiles) {
  const int ntiles = (n + kTile - 1) / kTile;
  if (ntiles > kTile) return ogx_fail(OGX_ERR_CAPACITY, "scan of %d elements", n);
  k_tile_sums<<<ntiles, kTile, 0, st>>>(a, n, tiles);
  k_scan_sums<<<1, kTile, 0, st>>>(tiles, ntiles, total);
  k_tile_scan<<<ntiles, kTile, 0, st>>>(a, n, tiles);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? OGX_OK : ogx_cuda_fail(e, "scan launch");
}

extern "C" ogx_status ogx_broad_create(ogx_ctx* ctx, int max_bodies, ogx_broad** out) {
  if (!ctx || !out || max_bodies < 1) return ogx_fail(OGX_ERR_INVALID, "bad broad-phase arguments");
  *out = nullptr;
  cudaSetDevice(ctx->device);
  ogx_broad* B = new ogx_broad();
  B->ctx = ctx;
  B->max_bodies = max_bodies;
  // about two buckets per expected entry (a body touches ~4-8 cells at a sensible cell
  // size); the scans take at most kTile * kTile elements
  uint32_t nb = 1024;
  while (nb < 8u * (uint32_t)max_bodies && nb < (uint32_t)(kTile * kTile)) nb <<= 1;
  if ((size_t)max_bodies + 1 > (size_t)kTile * kTile)
    return ogx_fail(OGX_ERR_CAPACITY, "broad phase takes at most %d bodies", kTile * kTile - 1);
  B->nbuckets = nb;
  const size_t ne = (size_t)max_bodies * kMaxCellsPerBody;
  cudaError_t e;
  if ((e = cudaMalloc(&B->lo, max_bodies * sizeof(float4))) != cudaSuccess ||
      (e = cudaMalloc(&B->hi, max_bodies * sizeof(float4))) != cudaSuccess ||
      (e = cudaMalloc(&B->eoff, (max_bodies + 1) * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&B->ekey, ne * sizeof(unsigned long long))) != cudaSuccess ||
      (e = cudaMalloc(&B->ebody, ne * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&B->skey, ne * sizeof(unsigned long long))) != cudaSuccess ||
      (e = cudaMalloc(&B->sbody, ne * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&B->boff, nb * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&B->bend, nb * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&B->pcount, (max_bodies + 1) * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&B->scal, 4 * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&B->tiles, kTile * sizeof(int))) != cudaSuccess) {
    ogx_broad_destroy(B);
    return ogx_cuda_fail(e, "broad-phase allocation");
  }
  *out = B;
  return OGX_OK;
}

extern "C" ogx_status ogx_broad_destroy(ogx_broad* B) {
  if (!B) return OGX_OK;
  cudaSetDevice(B->ctx->device);
  cudaFree(B->lo);
  cudaFree(B->hi);
  cudaFree(B->eoff);
  cudaFree(B->ekey);
  cudaFree(B->ebody);
  cudaFree(B->skey);
  cudaFree(B->sbody);
  cudaFree(B->boff);
  cudaFree(B->bend);
  cudaFree(B->pcount);
  cudaFree(B->scal);
  cudaFree(B->tiles);
  delete B;
  return OGX_OK;
}

ogx_status broad_run(ogx_broad* B, cudaStream_t st, const float* d_points, const BodyRef* d_bodies, int nbodies,
                     float cell, float margin, int max_pairs, gkCollisionPair* d_pairs, int* d_result) {
  if (nbodies > B->max_bodies) return ogx_fail(OGX_ERR_CAPACITY, "%d bodies > broad-phase capacity %d", nbodies,
                                               B->max_bodies);
  if (!(cell > 0.0f) || !(margin >= 0.0f) || max_pairs < 0 || !d_result)
    return ogx_fail(OGX_ERR_INVALID, "bad broad-phase arguments");
  const int sms = B->ctx->sm_count;
  const float inv = 1.0f / cell;
  const uint32_t bmask = B->nbuckets - 1u;
  cudaError_t e = cudaMemsetAsync(B->scal, 0, 4 * sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(B->boff, 0, B->nbuckets * sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(B->eoff + nbodies, 0, sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(B->pcount + nbodies, 0, sizeof(int), st);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "broad-phase reset");
  const int gw = std::max(1, std::min(8 * sms, (nbodies + 3) / 4));
  k_box<<<gw, 128, 0, st>>>(d_points, d_bodies, nbodies, margin, inv, B->lo, B->hi, B->eoff, B->scal + 2);
  e = scan(B, B->eoff, nbodies + 1, B->scal + 0, st);
  const int gb = std::max(1, std::min(8 * sms, (nbodies + 127) / 128));
  if (e == cudaSuccess) {
    k_entries<<<gb, 128, 0, st>>>(B->lo, B->hi, nbodies, inv, B->eoff, B->ekey, B->ebody, bmask, B->boff);
    e = scan(B, B->boff, (int)B->nbuckets, nullptr, st);
  }
  // the scatter advances a copy of the bucket offsets, leaving it at the buckets' ends
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(B->bend, B->boff, B->nbuckets * sizeof(int), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) {
    k_scatter<<<8 * sms, 256, 0, st>>>(B->ekey, B->ebody, B->scal + 0, bmask, B->bend, B->skey, B->sbody);
    k_pairs<0><<<gb, 128, 0, st>>>(B->lo, B->hi, nbodies, inv, B->eoff, B->ekey, bmask, B->boff, B->bend,
                                   B->skey, B->sbody, B->pcount, nullptr, 0);
    e = scan(B, B->pcount, nbodies + 1, B->scal + 1, st);
  }
  if (e == cudaSuccess)
    k_pairs<1><<<gb, 128, 0, st>>>(B->lo, B->hi, nbodies, inv, B->eoff, B->ekey, bmask, B->boff, B->bend,
                                   B->skey, B->sbody, B->pcount, reinterpret_cast<int2*>(d_pairs), max_pairs);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "broad-phase launch");
  e = cudaMemcpyAsync(d_result, B->scal + 1, 2 * sizeof(int), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return ogx_cuda_fail(e, "broad-phase launch");
  return OGX_OK;
}

extern "C" ogx_status ogx_broadphase(ogx_broad* B, const ogx_pool* pool, float cell, float margin, int max_pairs,
                                     gkCollisionPair* d_pairs, int* d_result) {
  if (!B || !pool) return ogx_fail(OGX_ERR_INVALID, "NULL broad phase or pool");
  cudaSetDevice(B->ctx->device);
  return broad_run(B, B->ctx->stream, pool->d_points, pool->d_bodies, pool->nbodies, cell, margin, max_pairs,
                   d_pairs, d_result);
}

// Candidate pairs from bounding spheres with the reference's semantics (see k_sph_pairs).
extern "C" ogx_status ogx_broadphase_spheres(ogx_broad* B, const float* d_spheres, int num_bodies, float cell,
                                             float boundary, int grid_size, int max_pairs, gkCollisionPair* d_pairs,
                                             int* d_result) {
  if (!B || !d_spheres || !d_result) return ogx_fail(OGX_ERR_INVALID, "NULL broad phase, spheres or result");
  if (num_bodies < 0 || num_bodies > B->max_bodies)
    return ogx_fail(OGX_ERR_CAPACITY, "%d bodies for a broad phase of %d", num_bodies, B->max_bodies);
  if (!(cell > 0.0f) || !(boundary >= 0.0f) || grid_size < 1 || grid_size >= kAxisBias || max_pairs < 0)
    return ogx_fail(OGX_ERR_INVALID, "bad broad-phase arguments");
  cudaSetDevice(B->ctx->device);
  cudaStream_t st = B->ctx->stream;
  const int sms = B->ctx->sm_count;
  const uint32_t bmask = B->nbuckets - 1u;
  const float4* sph = reinterpret_cast<const float4*>(d_spheres);
  cudaError_t e = cudaMemsetAsync(B->scal, 0, 4 * sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(B->boff, 0, B->nbuckets * sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(B->pcount + num_bodies, 0, sizeof(int), st);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "broad-phase reset");
  const int gb = std::max(1, std::min(8 * sms, (num_bodies + 127) / 128));
  k_sph_entries<<<gb, 128, 0, st>>>(sph, num_bodies, cell, boundary, grid_size, B->ekey, B->ebody, bmask, B->boff,
                                    B->scal + 0);
  e = scan(B, B->boff, (int)B->nbuckets, nullptr, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(B->bend, B->boff, B->nbuckets * sizeof(int), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) {
    k_scatter<<<8 * sms, 256, 0, st>>>(B->ekey, B->ebody, B->scal + 0, bmask, B->bend, B->skey, B->sbody);
    k_sph_pairs<0><<<gb, 128, 0, st>>>(sph, num_bodies, cell, boundary, grid_size, bmask, B->boff, B->bend, B->skey,
                                       B->sbody, B->pcount, nullptr, 0);
    e = scan(B, B->pcount, num_bodies + 1, B->scal + 1, st);
  }
  if (e == cudaSuccess)
    k_sph_pairs<1><<<gb, 128, 0, st>>>(sph, num_bodies, cell, boundary, grid_size, bmask, B->boff, B->bend, B->skey,
                                       B->sbody, B->pcount, reinterpret_cast<int2*>(d_pairs), max_pairs);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_result, B->scal + 1, 2 * sizeof(int), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return ogx_cuda_fail(e, "broad-phase launch");
  return OGX_OK;
}

// Sub-mesh pair expansion (visualization/integrate_final_gjk.cu:265-302): body pair p of
// bodies A, B becomes parts (first[A] + a, first[B] + b) for a < count[A], b < count[B],
// a-major, body pairs in order.  d_offsets[num_body_pairs + 1] receives each body pair's
// first expanded pair (the last entry = the total, which may exceed max_sub_pairs: then
// only the first max_sub_pairs are written).  d_owner (optional) gets the body pair of
// each expanded pair.
extern "C" ogx_status ogx_expand_submesh_pairs(ogx_ctx* ctx, int num_body_pairs, const gkCollisionPair* d_body_pairs,
                                               int num_bodies, const int32_t* d_first_part,
                                               const int32_t* d_part_count, int max_sub_pairs,
                                               gkCollisionPair* d_sub_pairs, int32_t* d_owner, int32_t* d_offsets) {
  if (!ctx || num_body_pairs < 0 || num_bodies < 0 || max_sub_pairs < 0 || !d_offsets ||
      (num_body_pairs > 0 && (!d_body_pairs || !d_first_part || !d_part_count || !d_sub_pairs)))
    return ogx_fail(OGX_ERR_INVALID, "bad expansion arguments");
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  int* tiles = nullptr;
  cudaError_t e = cudaMallocAsync(&tiles, kTile * sizeof(int), st);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "expansion scratch");
  const int g = std::max(1, std::min(8 * ctx->sm_count, (num_body_pairs + 255) / 256));
  e = cudaMemsetAsync(d_offsets + num_body_pairs, 0, sizeof(int), st);
  if (e == cudaSuccess && num_body_pairs > 0)
    k_sub_count<<<g, 256, 0, st>>>(reinterpret_cast<const int2*>(d_body_pairs), num_body_pairs, d_part_count,
                                   num_bodies, d_offsets);
  ogx_status s = e == cudaSuccess ? broad_scan(d_offsets, num_body_pairs + 1, nullptr, st, tiles)
                                  : ogx_cuda_fail(e, "expansion");
  if (!s && num_body_pairs > 0) {
    k_sub_expand<<<g, 256, 0, st>>>(reinterpret_cast<const int2*>(d_body_pairs), num_body_pairs, d_first_part,
                                    d_part_count, num_bodies, d_offsets, max_sub_pairs,
                                    reinterpret_cast<int2*>(d_sub_pairs), d_owner);
    if ((e = cudaGetLastError()) != cudaSuccess) s = ogx_cuda_fail(e, "expansion launch");
  }
  cudaFreeAsync(tiles, st);
  return s;
}

// Per body pair, the smallest distance over its expanded pairs (the closest or most
// penetrating part pair) and its index (-1 and +inf for a body pair with no parts).
extern "C" ogx_status ogx_reduce_submesh_pairs(ogx_ctx* ctx, int num_body_pairs, const int32_t* d_offsets,
                                               int max_sub_pairs, const float* d_sub_distances,
                                               float* d_best_distance, int32_t* d_best_index) {
  if (!ctx || num_body_pairs < 0 || (num_body_pairs > 0 && (!d_offsets || !d_sub_distances || !d_best_distance)))
    return ogx_fail(OGX_ERR_INVALID, "bad reduction arguments");
  if (num_body_pairs == 0) return OGX_OK;
  cudaSetDevice(ctx->device);
  const int g = std::max(1, std::min(8 * ctx->sm_count, (num_body_pairs + 255) / 256));
  k_sub_reduce<<<g, 256, 0, ctx->stream>>>(d_offsets, num_body_pairs, max_sub_pairs, d_sub_distances,
                                           d_best_distance, d_best_index);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? OGX_OK : ogx_cuda_fail(e, "reduction launch");
}
