// ogx_response.cu -- collision response from the GJK/EPA results: one normal impulse per
// contact (with restitution and the angular terms of both bodies) and a Baumgarte position
// correction for penetrating pairs, summed per body.
//
// The reference's visualiser applies the same model (visualization/integrate_final_gjk.cu:
// 572-689) with float atomics, so its sums depend on the order the GPU happens to run
// the contacts in.  Here the contributions of each contact are written once (k_impulse),
// the contacts of every body are listed with a count / scan / fill (k_count, k_fill), and
// each body adds its own contributions in contact order (k_gather): the result is
// deterministic.  Every impulse of one call is computed from the input velocities
// (a Jacobi step, as in the reference).
#include <cuda_runtime.h>

#include <algorithm>

#include "ogx_engine.h"

using namespace ogx;

namespace {

struct Contrib {
  float dv[2][3];  // linear velocity change of body 1, body 2
  float dw[2][3];  // angular velocity change (world frame)
  float dp[2][3];  // position correction
  int active;
};

__device__ __forceinline__ float3 qrot(float4 q, float3 v) {
  // v + 2 w (u x v) + 2 u x (u x v), q = (x, y, z, w) unit
  const float3 u = make_float3(q.x, q.y, q.z);
  const float3 t = make_float3(2.f * (u.y * v.z - u.z * v.y), 2.f * (u.z * v.x - u.x * v.z),
                               2.f * (u.x * v.y - u.y * v.x));
  return make_float3(v.x + q.w * t.x + (u.y * t.z - u.z * t.y), v.y + q.w * t.y + (u.z * t.x - u.x * t.z),
                     v.z + q.w * t.z + (u.x * t.y - u.y * t.x));
}
__device__ __forceinline__ float3 qrot_inv(float4 q, float3 v) { return qrot(make_float4(-q.x, -q.y, -q.z, q.w), v); }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__global__ void k_impulse(const ogx_body_state S, int nbodies, const int2* __restrict__ pairs, int npairs,
                          const float* __restrict__ dist, const float* __restrict__ nrm,
                          const gkSimplex* __restrict__ smp, ogx_response_params P, Contrib* __restrict__ out) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += gridDim.x * blockDim.x) {
    Contrib c = {};
    const int2 pr = pairs[p];
    const float d = dist[p];
    bool ok = pr.x >= 0 && pr.x < nbodies && pr.y >= 0 && pr.y < nbodies && pr.x != pr.y && d <= P.contact_eps;
    float3 n = make_float3(nrm[3 * p], nrm[3 * p + 1], nrm[3 * p + 2]);
    const float nl = sqrtf(dot3(n, n));
    ok = ok && nl >= 1e-4f;
    if (ok) {
      n = make_float3(n.x / nl, n.y / nl, n.z / nl);
      const int a = pr.x, b = pr.y;
      const float ima = S.inv_mass[a], imb = S.inv_mass[b];
      const float3 pa = make_float3(S.pos[3 * a], S.pos[3 * a + 1], S.pos[3 * a + 2]);
      const float3 pb = make_float3(S.pos[3 * b], S.pos[3 * b + 1], S.pos[3 * b + 2]);
      const float4 qa = make_float4(S.quat[4 * a], S.quat[4 * a + 1], S.quat[4 * a + 2], S.quat[4 * a + 3]);
      const float4 qb = make_float4(S.quat[4 * b], S.quat[4 * b + 1], S.quat[4 * b + 2], S.quat[4 * b + 3]);
      const float3 va = make_float3(S.vel[3 * a], S.vel[3 * a + 1], S.vel[3 * a + 2]);
      const float3 vb = make_float3(S.vel[3 * b], S.vel[3 * b + 1], S.vel[3 * b + 2]);
      const float3 wa = make_float3(S.ang[3 * a], S.ang[3 * a + 1], S.ang[3 * a + 2]);
      const float3 wb = make_float3(S.ang[3 * b], S.ang[3 * b + 1], S.ang[3 * b + 2]);
      const float3 ia = make_float3(S.inv_inertia[3 * a], S.inv_inertia[3 * a + 1], S.inv_inertia[3 * a + 2]);
      const float3 ib = make_float3(S.inv_inertia[3 * b], S.inv_inertia[3 * b + 1], S.inv_inertia[3 * b + 2]);
      const gkSimplex& s = smp[p];
      const float3 ra = make_float3(s.witnesses[0][0] - pa.x, s.witnesses[0][1] - pa.y, s.witnesses[0][2] - pa.z);
      const float3 rb = make_float3(s.witnesses[1][0] - pb.x, s.witnesses[1][1] - pb.y, s.witnesses[1][2] - pb.z);
      // position correction along n for penetrating pairs (distance = -depth)
      if (d < 0.0f && ima + imb > 0.0f) {
        const float corr = P.baumgarte * (-d) / (ima + imb);
        for (int k = 0; k < 3; ++k) {
          const float nk = k == 0 ? n.x : (k == 1 ? n.y : n.z);
          c.dp[0][k] = -corr * ima * nk;
          c.dp[1][k] = corr * imb * nk;
        }
        c.active = 1;
      }
      // relative normal velocity at the contact point (body 2 relative to body 1)
      const float3 ua = cross3(wa, ra), ub = cross3(wb, rb);
      const float3 rv = make_float3((vb.x + ub.x) - (va.x + ua.x), (vb.y + ub.y) - (va.y + ua.y),
                                    (vb.z + ub.z) - (va.z + ua.z));
      const float vn = dot3(rv, n);
      if (vn <= 0.0f) {
        const float3 ta = qrot_inv(qa, cross3(ra, n)), tb = qrot_inv(qb, cross3(rb, n));
        const float3 Ita = make_float3(ia.x * ta.x, ia.y * ta.y, ia.z * ta.z);
        const float3 Itb = make_float3(ib.x * tb.x, ib.y * tb.y, ib.z * tb.z);
        const float den = ima + imb + dot3(ta, Ita) + dot3(tb, Itb);
        if (den > 0.0f) {
          const float e = (-vn > P.restitution_threshold) ? P.restitution : 0.0f;
          const float j = -(1.0f + e) * vn / den;
          const float3 dwa = qrot(qa, make_float3(-j * Ita.x, -j * Ita.y, -j * Ita.z));
          const float3 dwb = qrot(qb, make_float3(j * Itb.x, j * Itb.y, j * Itb.z));
          const float nk[3] = {n.x, n.y, n.z};
          const float wak[3] = {dwa.x, dwa.y, dwa.z}, wbk[3] = {dwb.x, dwb.y, dwb.z};
          for (int k = 0; k < 3; ++k) {
            c.dv[0][k] = -j * nk[k] * ima;
            c.dv[1][k] = j * nk[k] * imb;
            c.dw[0][k] = wak[k];
            c.dw[1][k] = wbk[k];
          }
          c.active = 1;
        }
      }
    }
    out[p] = c;
  }
}

__global__ void k_count(const int2* __restrict__ pairs, int npairs, int nbodies, const Contrib* __restrict__ c,
                        int* __restrict__ cnt) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += gridDim.x * blockDim.x) {
    if (!c[p].active) continue;
    atomicAdd(cnt + pairs[p].x, 1);
    atomicAdd(cnt + pairs[p].y, 1);
  }
}

// entries: 2 * contact + side (0 = body 1, 1 = body 2), placed per body in any order;
// k_gather sorts each body's short list before summing
__global__ void k_fill(const int2* __restrict__ pairs, int npairs, const Contrib* __restrict__ c,
                       int* __restrict__ cursor, int* __restrict__ entries) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += gridDim.x * blockDim.x) {
    if (!c[p].active) continue;
    entries[atomicAdd(cursor + pairs[p].x, 1)] = 2 * p;
    entries[atomicAdd(cursor + pairs[p].y, 1)] = 2 * p + 1;
  }
}

__global__ void k_gather(ogx_body_state S, int nbodies, const int* __restrict__ off, int* __restrict__ entries,
                         const Contrib* __restrict__ c, float* __restrict__ vel_out, float* __restrict__ ang_out,
                         float* __restrict__ pos_out) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbodies; b += gridDim.x * blockDim.x) {
    const int e0 = off[b], e1 = off[b + 1];
    // contact order: insertion sort of this body's entries
    for (int i = e0 + 1; i < e1; ++i) {
      const int v = entries[i];
      int k = i - 1;
      while (k >= e0 && entries[k] > v) {
        entries[k + 1] = entries[k];
        --k;
      }
      entries[k + 1] = v;
    }
    float dv[3] = {0.f, 0.f, 0.f}, dw[3] = {0.f, 0.f, 0.f}, dp[3] = {0.f, 0.f, 0.f};
    for (int i = e0; i < e1; ++i) {
      const int e = entries[i];
      const Contrib& x = c[e >> 1];
      const int side = e & 1;
      for (int k = 0; k < 3; ++k) {
        dv[k] += x.dv[side][k];
        dw[k] += x.dw[side][k];
        dp[k] += x.dp[side][k];
      }
    }
    for (int k = 0; k < 3; ++k) {
      vel_out[3 * b + k] = S.vel[3 * b + k] + dv[k];
      ang_out[3 * b + k] = S.ang[3 * b + k] + dw[k];
      pos_out[3 * b + k] = S.pos[3 * b + k] + dp[k];
    }
  }
}

}  // namespace

ogx_status broad_scan(int* a, int n, int* total, cudaStream_t st, int* tiles);

extern "C" void ogx_response_params_default(ogx_response_params* p) {
  if (!p) return;
  p->contact_eps = FLT_EPSILON;
  p->baumgarte = 0.2f;
  p->restitution = 0.5f;
  p->restitution_threshold = 1.0f;
}

extern "C" ogx_status ogx_contact_response(ogx_ctx* ctx, int nbodies, const ogx_body_state* state, int npairs,
                                           const gkCollisionPair* d_pairs, const float* d_distances,
                                           const float* d_normals, const gkSimplex* d_simplices,
                                           const ogx_response_params* params, float* d_vel_out,
                                           float* d_ang_out, float* d_pos_out) {
  if (!ctx || !state || nbodies < 0 || npairs < 0) return ogx_fail(OGX_ERR_INVALID, "bad response arguments");
  if (nbodies == 0) return OGX_OK;
  if (!state->pos || !state->quat || !state->vel || !state->ang || !state->inv_mass || !state->inv_inertia ||
      !d_vel_out || !d_ang_out || !d_pos_out || (npairs > 0 && (!d_pairs || !d_distances || !d_normals ||
                                                                !d_simplices)))
    return ogx_fail(OGX_ERR_INVALID, "NULL response array");
  if (nbodies + 1 > 1024 * 1024) return ogx_fail(OGX_ERR_CAPACITY, "response takes at most %d bodies", 1024 * 1024 - 1);
  cudaSetDevice(ctx->device);
  ogx_response_params P;
  ogx_response_params_default(&P);
  if (params) P = *params;
  cudaStream_t st = ctx->stream;
  // scratch: contributions, per-body counts / offsets / cursors, entries, scan tiles
  Contrib* c = nullptr;
  int *cnt = nullptr, *cur = nullptr, *ent = nullptr, *tiles = nullptr;
  const size_t np = std::max(1, npairs);
  cudaError_t e;
  if ((e = cudaMallocAsync(&c, np * sizeof(Contrib), st)) != cudaSuccess ||
      (e = cudaMallocAsync(&cnt, (nbodies + 1) * sizeof(int), st)) != cudaSuccess ||
      (e = cudaMallocAsync(&cur, (nbodies + 1) * sizeof(int), st)) != cudaSuccess ||
      (e = cudaMallocAsync(&ent, 2 * np * sizeof(int), st)) != cudaSuccess ||
      (e = cudaMallocAsync(&tiles, 1024 * sizeof(int), st)) != cudaSuccess) {
    cudaFreeAsync(c, st);
    cudaFreeAsync(cnt, st);
    cudaFreeAsync(cur, st);
    cudaFreeAsync(ent, st);
    cudaFreeAsync(tiles, st);
    return ogx_cuda_fail(e, "response scratch");
  }
  const int g = std::max(1, std::min(8 * ctx->sm_count, (std::max(npairs, nbodies) + 255) / 256));
  e = cudaMemsetAsync(cnt, 0, (nbodies + 1) * sizeof(int), st);
  if (e == cudaSuccess && npairs > 0) {
    k_impulse<<<g, 256, 0, st>>>(*state, nbodies, reinterpret_cast<const int2*>(d_pairs), npairs, d_distances,
                                 d_normals, d_simplices, P, c);
    k_count<<<g, 256, 0, st>>>(reinterpret_cast<const int2*>(d_pairs), npairs, nbodies, c, cnt);
  }
  ogx_status s = e == cudaSuccess ? broad_scan(cnt, nbodies + 1, nullptr, st, tiles) : ogx_cuda_fail(e, "response");
  if (!s && (e = cudaMemcpyAsync(cur, cnt, (nbodies + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
    s = ogx_cuda_fail(e, "response copy");
  if (!s) {
    if (npairs > 0)
      k_fill<<<g, 256, 0, st>>>(reinterpret_cast<const int2*>(d_pairs), npairs, c, cur, ent);
    k_gather<<<g, 256, 0, st>>>(*state, nbodies, cnt, ent, c, d_vel_out, d_ang_out, d_pos_out);
    if ((e = cudaGetLastError()) != cudaSuccess) s = ogx_cuda_fail(e, "response launch");
  }
  cudaFreeAsync(c, st);
  cudaFreeAsync(cnt, st);
  cudaFreeAsync(cur, st);
  cudaFreeAsync(ent, st);
  cudaFreeAsync(tiles, st);
  return s;
}
