// ogx_stream.cu -- one GJK + EPA call from host memory to host memory with the transfers
// overlapped with the kernels.
//
// The points of the pool go up in body ranges (copy engine, stream `up`), the pairs in
// ranges of pairs; chunk j of the pairs starts (context stream) as soon as every body it
// references and its pairs are on the device, after packing the new body ranges into the
// pool layout; its results come back (stream `down`) while later chunks compute.  The
// reference's high-level functions copy everything, compute, and copy back in sequence
// (GJK/gpu/openGJK.cu:2791-2819); here only the first chunk's upload and the last chunk's
// download are exposed.
#include <cuda_runtime.h>

#include <algorithm>
#include <thread>
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

}  // namespace

extern "C" ogx_status ogx_gjk_epa_streamed(ogx_ctx* ctx, ogx_pool* pool, const float* xyz, int npairs,
                                           const gkCollisionPair* pairs, gkSimplex* simplices, float* distances,
                                           float* normals, int32_t* status, int chunks) {
  if (!ctx || !pool || (!xyz && pool->npoints > 0) || (!pairs && npairs > 0) || npairs < 0)
    return ogx_fail(OGX_ERR_INVALID, "bad streamed-call arguments");
  if (npairs == 0) return OGX_OK;
  if (!simplices || !distances || !normals) return ogx_fail(OGX_ERR_INVALID, "NULL output array");
  cudaSetDevice(ctx->device);
  const int C = std::max(1, std::min(chunks, 64));
  const int nb = pool->nbodies;
  ogx_status s = ensure_io(ctx, npairs);
  if (!s) s = ensure_streams(ctx, 3 * C);
  if (!s) s = ctx->ensure_stage(0, (size_t)pool->npoints * 3 * sizeof(float));
  if (!s) s = ctx->ensure_scratch(npairs);
  if (s) return s;

  // body ranges of about equal point counts
  std::vector<int> bb(C + 1, nb);
  bb[0] = 0;
  for (int k = 1; k < C; ++k) {
    const int64_t target = pool->npoints * k / C;
    bb[k] = (int)(std::lower_bound(pool->h_voff.begin(), pool->h_voff.end(), target) - pool->h_voff.begin());
    bb[k] = std::max(bb[k], bb[k - 1]);
  }
  // pair ranges of equal size and the highest body each references (host threads)
  std::vector<int> pb(C + 1);
  for (int j = 0; j <= C; ++j) pb[j] = (int)((int64_t)npairs * j / C);
  std::vector<int> need(C, -1);
  {
    std::vector<std::thread> th;
    for (int j = 0; j < C; ++j)
      th.emplace_back([&, j] {
        int m = -1;
        for (int i = pb[j]; i < pb[j + 1]; ++i) m = std::max(m, std::max(pairs[i].idx1, pairs[i].idx2));
        need[j] = m;
      });
    for (auto& t : th) t.join();
  }
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
  const float* d_aos = static_cast<const float*>(ctx->d_stage);
  cudaError_t e = cudaSuccess;
  // uploads, interleaved so that pair range j follows the bodies it most likely needs
  for (int k = 0; k < C && e == cudaSuccess; ++k) {
    const int64_t p0 = bb[k] < nb ? pool->h_voff[bb[k]] : pool->npoints;
    const int64_t p1 = bb[k + 1] < nb ? pool->h_voff[bb[k + 1]] : pool->npoints;
    if (p1 > p0)
      e = cudaMemcpyAsync(const_cast<float*>(d_aos) + 3 * p0, xyz + 3 * p0, (p1 - p0) * 3 * sizeof(float),
                          cudaMemcpyHostToDevice, ctx->up);
    if (e == cudaSuccess) e = cudaEventRecord(ev_body[k], ctx->up);
    mark(k, 0, ctx->up);
    if (e == cudaSuccess && pb[k + 1] > pb[k])
      e = cudaMemcpyAsync(ctx->d_io_pairs + pb[k], pairs + pb[k], (pb[k + 1] - pb[k]) * sizeof(gkCollisionPair),
                          cudaMemcpyHostToDevice, ctx->up);
    if (e == cudaSuccess) e = cudaEventRecord(ev_pair[k], ctx->up);
    mark(k, 1, ctx->up);
  }
  if (e != cudaSuccess) return ogx_cuda_fail(e, "streamed upload");
  // compute: pack body ranges on first use, then the pair range
  int packed = 0;  // body ranges [0, packed) are in the pool
  int launches = 0;
  for (int j = 0; j < C; ++j) {
    // body range holding the highest body this pair range references (invalid indices
    // are flagged by the kernels; they need no body)
    int kneed = 0;
    if (need[j] >= nb) kneed = C - 1;
    else if (need[j] >= 0) kneed = (int)(std::upper_bound(bb.begin(), bb.end(), need[j]) - bb.begin()) - 1;
    kneed = std::min(std::max(kneed, 0), C - 1);
    while (packed <= kneed) {
      e = cudaStreamWaitEvent(ctx->stream, ev_body[packed], 0);
      const int n = bb[packed + 1] - bb[packed];
      if (e == cudaSuccess && n > 0)
        e = launch_pack(d_aos, pool->d_voff + bb[packed], pool->d_bodies + bb[packed], n, pool->d_points,
                        std::max(1, std::min(8 * ctx->sm_count, (n + 7) / 8)), ctx->stream);
      if (e != cudaSuccess) return ogx_cuda_fail(e, "streamed pack");
      ++launches;
      ++packed;
    }
    e = cudaStreamWaitEvent(ctx->stream, ev_pair[j], 0);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "streamed wait");
    mark(j, 2, ctx->stream);
    const int p0 = pb[j], n = pb[j + 1] - pb[j];
    if (n > 0) {
      s = ogx_run(ctx, pool->d_points, pool->d_bodies, nb, n, ctx->d_io_pairs + p0, ctx->d_io_smp + p0,
                  ctx->d_io_dist + p0, ctx->d_io_nrm + 3 * (size_t)p0, ctx->d_io_status + p0, kModeGjkEpa);
      if (s) return s;
      launches += ctx->last_launches;
    }
    mark(j, 3, ctx->stream);
    e = cudaEventRecord(ev_done[j], ctx->stream);
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
  // bodies never referenced are still packed, so the pool holds the whole upload
  while (packed < C) {
    e = cudaStreamWaitEvent(ctx->stream, ev_body[packed], 0);
    const int n = bb[packed + 1] - bb[packed];
    if (e == cudaSuccess && n > 0)
      e = launch_pack(d_aos, pool->d_voff + bb[packed], pool->d_bodies + bb[packed], n, pool->d_points,
                      std::max(1, std::min(8 * ctx->sm_count, (n + 7) / 8)), ctx->stream);
    if (e != cudaSuccess) return ogx_cuda_fail(e, "streamed pack");
    ++launches;
    ++packed;
  }
  e = cudaStreamSynchronize(ctx->down);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return ogx_cuda_fail(e, "streamed call");
  if (tl) {
    ctx->stream_timeline.assign(5 * C, 0.0f);
    for (int i = 0; i < 5 * C; ++i) cudaEventElapsedTime(&ctx->stream_timeline[i], tev[0], tev[1 + i]);
    for (auto& x : tev) cudaEventDestroy(x);
  }
  ctx->last_launches = launches;
  return OGX_OK;
}

extern "C" int ogx_ctx_stream_timeline(const ogx_ctx* ctx, float* ms, int cap) {
  if (!ctx) return 0;
  const int n = (int)ctx->stream_timeline.size();
  if (ms) for (int i = 0; i < n && i < cap; ++i) ms[i] = ctx->stream_timeline[i];
  return n;
}
