// ogx_stream.cu -- one GJK + EPA call from host memory to host memory with the transfers
// overlapped with the kernels.
//
// The pairs go up in C ranges of equal size and the points in C body ranges cut so that
// range k holds the bodies pair range k references first (copy engine, stream `up`).
// Each body range is packed into the pool layout on the context's stream as it lands;
// chunk j of the pairs then runs on one of up to four lane contexts (own stream and work
// lists), so that chunks overlap one another as well as the copies, and its results come
// back (stream `down`) while later chunks compute.  The
// reference's high-level functions copy everything, compute, and copy back in sequence
// (GJK/gpu/openGJK.cu:2791-2819); here only the first chunk's upload and the last chunk's
// download are exposed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <vector>

#include "ogx_engine.h"

using namespace ogx;

namespace {

ogx_status ensure_io(ogx_ctx* c, size_t n) {
  if (n <= c->io_cap && c->d_io_pairs) return OGX_OK;
  cudaStreamSynchronize(c->stream);
  cudaFree(c->d_io_pairs);
  cudaFree(c->d_io_smp);
  cudaFree(c->d_io_dist);
  cudaFree(c->d_io_nrm);
  cudaFree(c->d_io_status);
  c->d_io_pairs = nullptr;
  c->d_io_smp = nullptr;
  c->d_io_dist = nullptr;
  c->d_io_nrm = nullptr;
  c->d_io_status = nullptr;
  c->io_cap = 0;
  const size_t cap = std::max<size_t>(1024, n);
  cudaError_t e;
  if ((e = cudaMalloc(&c->d_io_pairs, cap * sizeof(gkCollisionPair))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_io_smp, cap * sizeof(gkSimplex))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_io_dist, cap * sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_io_nrm, 3 * cap * sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_io_status, cap * sizeof(int32_t))) != cudaSuccess)
    return ogx_cuda_fail(e, "streamed call buffers");
  c->io_cap = cap;
  return OGX_OK;
}

// packs bodies [b0, b1) of the uploaded xyz into the pool layout
cudaError_t pack_range(const ogx_ctx* ctx, ogx_pool* pool, const float* d_aos, int b0, int b1, cudaStream_t st) {
  const int n = b1 - b0;
  if (n <= 0) return cudaSuccess;
  return launch_pack(d_aos, pool->d_voff + b0, pool->d_bodies + b0, n, pool->d_points,
                     std::max(1, std::min(8 * ctx->sm_count, (n + 7) / 8)), st);
}

constexpr int kStreamMaxRanges = 64;
constexpr int kStreamMaxLanes = 8;
constexpr int kStreamLanes = 4;
constexpr int kLaneForkConnections = 16;
constexpr int kLaneForkWidth = 2;

ogx_status ensure_streams(ogx_ctx* c, int nev) {
  cudaError_t e;
  if (!c->up && (e = cudaStreamCreateWithFlags(&c->up, cudaStreamNonBlocking)) != cudaSuccess)
    return ogx_cuda_fail(e, "copy stream");
  if (!c->down && (e = cudaStreamCreateWithFlags(&c->down, cudaStreamNonBlocking)) != cudaSuccess)
    return ogx_cuda_fail(e, "copy stream");
  while ((int)c->sev.size() < nev) {
    cudaEvent_t ev;
    if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
      return ogx_cuda_fail(e, "event");
    c->sev.push_back(ev);
  }
  return OGX_OK;
}

ogx_status streamed(ogx_ctx* ctx, ogx_pool* pool, const float* xyz, int npairs, const gkCollisionPair* pairs,
                    gkSimplex* simplices, float* distances, float* normals, int32_t* status,
                    const std::vector<int>& pb, int lanes) {
  cudaSetDevice(ctx->device);
  const int C = (int)pb.size() - 1;
  const int nb = pool->nbodies;
  int widest = 0;
  for (int j = 0; j < C; ++j) widest = std::max(widest, pb[j + 1] - pb[j]);
  ogx_status s = ensure_io(ctx, npairs);
  if (!s) s = ensure_streams(ctx, 4 * C);
  // chunks run side by side on `lanes` contexts (own stream and work lists each), so that
  // one chunk's kernels overlap the next chunk's as well as the copies
  const int S = std::min(C, lanes);
  while (!s && (int)ctx->sub.size() < S) {
    ogx_ctx* c = nullptr;
    s = ogx_ctx_create(ctx->device, &ctx->cfg, nullptr, &c);
    if (!s) {
      c->fork_width = kLaneForkWidth;
      ctx->sub.push_back(c);
    }
  }
  // a lane also spreads its size buckets over two streams of its own (plus one for the
  // FP64 refinement), when the process has enough hardware work queues for them: with
  // the runtime's default of 8, or with more streams than queues, the copy streams would
  // share a queue with a lane's kernels and wait behind them behind one another
  const char* conn_env = std::getenv("CUDA_DEVICE_MAX_CONNECTIONS");
  const bool lane_fork = conn_env && std::atoi(conn_env) >= kLaneForkConnections;
  for (int i = 0; !s && i < S; ++i) {
    ogx_ctx* c = ctx->sub[i];
    c->cfg = ctx->cfg;
    c->timing = false;
    c->fork_ok = lane_fork;
    for (int k = 0; k < 2; ++k)
      for (int b = 0; b < kBuckets; ++b) c->choice[k][b] = ctx->choice[k][b];
    s = c->ensure_scratch(widest);
  }
  if (!s) s = ctx->ensure_stage(0, (size_t)pool->npoints * 3 * sizeof(float));
  // the last range runs on this context, with every size bucket on a stream of its own:
  // nothing else is left to overlap it with, so its latency is the tail of the call
  if (!s && C > 1) s = ctx->ensure_scratch(widest);
  if (s) return s;

  // optional timeline (context timing on): per chunk, the end of its body upload, the end
  // of its pair upload, its compute start and end, the end of its download
  const bool tl = ctx->timing;
  std::vector<cudaEvent_t> tev;
  if (tl) {
    tev.resize(1 + 5 * C);
    for (auto& x : tev) cudaEventCreate(&x);
    cudaEventRecord(tev[0], ctx->up);
    cudaStreamWaitEvent(ctx->stream, tev[0], 0);
    cudaStreamWaitEvent(ctx->down, tev[0], 0);
  }
  auto mark = [&](int j, int k, cudaStream_t s2) {
    if (tl) cudaEventRecord(tev[1 + 5 * j + k], s2);
  };
  cudaEvent_t* ev_body = ctx->sev.data();
  cudaEvent_t* ev_pair = ev_body + C;
  cudaEvent_t* ev_done = ev_pair + C;
  cudaEvent_t* ev_packed = ev_done + C;
  const float* d_aos = static_cast<const float*>(ctx->d_stage);
  cudaError_t e = cudaSuccess;
  // Body range k holds the bodies that pair range k references first: chunk k then waits
  // only for body ranges 0..k (indices out of range need no body; the kernels flag them).
  // Each range is cut, uploaded and launched before the next one's pairs are scanned, so
  // that the scan of later ranges overlaps the copies already in flight.
  std::vector<int> bb(C + 1, nb);
  bb[0] = 0;
  int launches = 0;
  int need = -1;  // highest body referenced by pair ranges 0..k
  for (int k = 0; k < C && e == cudaSuccess; ++k) {
    for (int i = pb[k]; i < pb[k + 1]; ++i) need = std::max(need, std::max(pairs[i].idx1, pairs[i].idx2));
    if (k + 1 < C) bb[k + 1] = std::max(bb[k], std::min(nb, need + 1));
    const int64_t v0 = bb[k] < nb ? pool->h_voff[bb[k]] : pool->npoints;
    const int64_t v1 = bb[k + 1] < nb ? pool->h_voff[bb[k + 1]] : pool->npoints;
    if (v1 > v0)
      e = cudaMemcpyAsync(const_cast<float*>(d_aos) + 3 * v0, xyz + 3 * v0, (v1 - v0) * 3 * sizeof(float),
                          cudaMemcpyHostToDevice, ctx->up);
    if (e == cudaSuccess) e = cudaEventRecord(ev_body[k], ctx->up);
    mark(k, 0, ctx->up);
    if (e == cudaSuccess && pb[k + 1] > pb[k])
      e = cudaMemcpyAsync(ctx->d_io_pairs + pb[k], pairs + pb[k], (pb[k + 1] - pb[k]) * sizeof(gkCollisionPair),
                          cudaMemcpyHostToDevice, ctx->up);
    if (e == cudaSuccess) e = cudaEventRecord(ev_pair[k], ctx->up);
    mark(k, 1, ctx->up);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "streamed upload");
    // chunk k of the pairs runs on lane k % S once the bodies it needs are packed and its
    // pairs are up
    const int j = k;
    // body range j, packed in order on the context's stream: ranges 0..j then hold every
    // body that pair range j references
    e = cudaStreamWaitEvent(ctx->stream, ev_body[j], 0);
    if (e == cudaSuccess) e = pack_range(ctx, pool, d_aos, bb[j], bb[j + 1], ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev_packed[j], ctx->stream);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "streamed pack");
    launches += bb[j + 1] > bb[j];
    ogx_ctx* c = (j == C - 1 && C > 1) ? ctx : ctx->sub[j % S];
    cudaStream_t cs = c->stream;
    e = cudaStreamWaitEvent(cs, ev_packed[j], 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ev_pair[j], 0);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "streamed wait");
    mark(j, 2, cs);
    const int p0 = pb[j], n = pb[j + 1] - pb[j];
    if (n > 0) {
      s = ogx_run(c, pool->d_points, pool->d_bodies, nb, n, ctx->d_io_pairs + p0, ctx->d_io_smp + p0,
                  ctx->d_io_dist + p0, ctx->d_io_nrm + 3 * (size_t)p0, ctx->d_io_status + p0, kModeGjkEpa);
      if (s) return s;
      launches += c->last_launches;
    }
    mark(j, 3, cs);
    e = cudaEventRecord(ev_done[j], cs);
    // results of range j
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->down, ev_done[j], 0);
    if (e == cudaSuccess && n > 0)
      e = cudaMemcpyAsync(simplices + p0, ctx->d_io_smp + p0, n * sizeof(gkSimplex), cudaMemcpyDeviceToHost,
                          ctx->down);
    if (e == cudaSuccess && n > 0)
      e = cudaMemcpyAsync(distances + p0, ctx->d_io_dist + p0, n * sizeof(float), cudaMemcpyDeviceToHost,
                          ctx->down);
    if (e == cudaSuccess && n > 0)
      e = cudaMemcpyAsync(normals + 3 * (size_t)p0, ctx->d_io_nrm + 3 * (size_t)p0, 3 * n * sizeof(float),
                          cudaMemcpyDeviceToHost, ctx->down);
    if (e == cudaSuccess && n > 0 && status)
      e = cudaMemcpyAsync(status + p0, ctx->d_io_status + p0, n * sizeof(int32_t), cudaMemcpyDeviceToHost,
                          ctx->down);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "streamed download");
    mark(j, 4, ctx->down);
  }
  e = cudaStreamSynchronize(ctx->down);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  for (int i = 0; i < S && e == cudaSuccess; ++i) e = cudaStreamSynchronize(ctx->sub[i]->stream);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "streamed call");
  if (tl) {
    ctx->stream_timeline.assign(5 * C, 0.0f);
    for (int i = 0; i < 5 * C; ++i) cudaEventElapsedTime(&ctx->stream_timeline[i], tev[0], tev[1 + i]);
    for (auto& x : tev) cudaEventDestroy(x);
  }
  ctx->last_launches = launches;
  return OGX_OK;
}

ogx_status check_args(ogx_ctx* ctx, ogx_pool* pool, const float* xyz, int npairs, const gkCollisionPair* pairs,
                      gkSimplex* simplices, float* distances, float* normals) {
  if (!ctx || !pool || (!xyz && pool->npoints > 0) || (!pairs && npairs > 0) || npairs < 0)
    return ogx_fail(OGX_ERR_INVALID, "bad streamed-call arguments");
  if (npairs > 0 && (!simplices || !distances || !normals)) return ogx_fail(OGX_ERR_INVALID, "NULL output array");
  return OGX_OK;
}

}  // namespace

extern "C" ogx_status ogx_gjk_epa_streamed(ogx_ctx* ctx, ogx_pool* pool, const float* xyz, int npairs,
                                           const gkCollisionPair* pairs, gkSimplex* simplices, float* distances,
                                           float* normals, int32_t* status, int chunks) {
  ogx_status s = check_args(ctx, pool, xyz, npairs, pairs, simplices, distances, normals);
  if (s || npairs == 0) return s;
  const int C = std::max(1, std::min(chunks, kStreamMaxRanges));
  std::vector<int> pb(C + 1);
  for (int j = 0; j <= C; ++j) pb[j] = (int)((int64_t)npairs * j / C);
  return streamed(ctx, pool, xyz, npairs, pairs, simplices, distances, normals, status, pb, kStreamLanes);
}

extern "C" ogx_status ogx_gjk_epa_streamed_ranges(ogx_ctx* ctx, ogx_pool* pool, const float* xyz, int npairs,
                                                  const gkCollisionPair* pairs, gkSimplex* simplices,
                                                  float* distances, float* normals, int32_t* status,
                                                  const int* pair_bounds, int nranges, int lanes) {
  ogx_status s = check_args(ctx, pool, xyz, npairs, pairs, simplices, distances, normals);
  if (s) return s;
  if (!pair_bounds || nranges < 1 || nranges > kStreamMaxRanges || lanes < 0 || lanes > kStreamMaxLanes)
    return ogx_fail(OGX_ERR_INVALID, "bad pair ranges or lane count");
  std::vector<int> pb(pair_bounds, pair_bounds + nranges + 1);
  if (pb[0] != 0 || pb[nranges] != npairs) return ogx_fail(OGX_ERR_INVALID, "pair ranges must cover [0, npairs)");
  for (int j = 0; j < nranges; ++j)
    if (pb[j + 1] < pb[j]) return ogx_fail(OGX_ERR_INVALID, "pair range bounds must not decrease");
  if (npairs == 0) return OGX_OK;
  return streamed(ctx, pool, xyz, npairs, pairs, simplices, distances, normals, status, pb,
                  lanes ? lanes : kStreamLanes);
}

extern "C" int ogx_ctx_stream_timeline(const ogx_ctx* ctx, float* ms, int cap) {
  if (!ctx) return 0;
  const int n = (int)ctx->stream_timeline.size();
  if (ms) for (int i = 0; i < n && i < cap; ++i) ms[i] = ctx->stream_timeline[i];
  return n;
}
