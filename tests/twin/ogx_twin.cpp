// ogx_twin.cpp -- TEST BUILD ONLY.  Runs the engine's per-pair GJK/EPA code (the same
// __host__ __device__ source the CUDA kernels instantiate) on the CPU with a one-lane
// team, so the algorithm can be checked against the oracle on a machine without a GPU
// and GPU results can be compared with the identical arithmetic on the host.  The
// product library never contains this file.
#include <pthread.h>
#include <string.h>

#include <vector>

#include "ogx_bodies.cuh"
#include "ogx_epa.cuh"
#include "ogx_gjk.cuh"

using namespace ogx;

namespace {

struct Job {
  int lo, hi, mode;
  const float* pool;
  const uint32_t* quad;
  const int32_t* counts;
  const int32_t* pairs;
  const ogx_config* cfg;
  float* dist;
  gkSimplex* smp;
  float* nrm;
  int32_t* status;
  int32_t* iters;
  const float* xf;  // poses (12 floats per body) for the posed pipeline, or null
};

struct Work {
  EpaMemSmall small;
  EpaMemCert full;
};

void bind(MemBodies& B, const Job& J, int b1, int b2, BodyRef A, BodyRef Bb) { B.bind(J.pool, A, Bb); }
void bind(Posed<MemBodies>& B, const Job& J, int b1, int b2, BodyRef A, BodyRef Bb) {
  B.bind_posed(J.pool, A, Bb, J.xf + 12 * (size_t)b1, J.xf + 12 * (size_t)b2);
}

template <class Bodies>
void one(const Job& J, int i, Work& M) {
  const int b1 = J.pairs[2 * i], b2 = J.pairs[2 * i + 1];
  BodyRef A{J.quad[b1], J.counts[b1]}, Bb{J.quad[b2], J.counts[b2]};
  Bodies B;
  bind(B, J, b1, b2, A, Bb);
  SerialTeam t;
  GjkState g;
  gjk_pair(t, B, *J.cfg, g);
  // same order as the device pipeline: the contact decision is taken on the FP32 GJK
  // result, separated pairs are then re-solved in FP64, contacts go through EPA
  bool contact = gjk_contact(g);
  bool late = false;  // a contact only the FP64 refinement found
  if (g.polish) {
    gjk_refine(t, B, g, 16);
    contact = gjk_contact(g);
    late = contact;
  }
  gkSimplex& s = J.smp[i];
  s.nvrtx = g.n;
  for (int k = 0; k < 4; ++k) {
    const bool live = k < g.n;
    s.vrtx[k][0] = live ? g.P[k].x : 0.f;
    s.vrtx[k][1] = live ? g.P[k].y : 0.f;
    s.vrtx[k][2] = live ? g.P[k].z : 0.f;
    s.vrtx_idx[k][0] = live ? g.ia[k] : 0;
    s.vrtx_idx[k][1] = live ? g.ib[k] : 0;
  }
  float d = g.dist;
  fv3 w0 = g.w0, w1 = g.w1, n = v3<float>(0.f, 0.f, 0.f);
  int st = g.status, ei = 0;
  if (J.mode == 2) {
    if (contact) {
      // as on the device: the small working set first, full capacity when it runs out;
      // contacts found by the refinement go straight to the certified full pass
      EpaOut o;
      if (late) {
        o.spill = true;
        o.spill64 = true;
      } else {
        epa_pair(t, B, *J.cfg, g, M.small, o, true);
      }
      if (o.spill) {
        ogx_config c = *J.cfg;
        if (o.spill64) c.flags |= OGX_F_EPA_FP64_PLANES;
        epa_pair<true>(t, B, c, g, M.full, o, false);
      }
      if (o.polish) epa_polish(B, o);
      d = o.dist;
      w0 = o.w0;
      w1 = o.w1;
      n = o.nrm;
      st |= o.status;
      ei = o.iters;
    } else {
      n = sep_normal(g);
    }
  }
  J.dist[i] = d;
  s.witnesses[0][0] = w0.x;
  s.witnesses[0][1] = w0.y;
  s.witnesses[0][2] = w0.z;
  s.witnesses[1][0] = w1.x;
  s.witnesses[1][1] = w1.y;
  s.witnesses[1][2] = w1.z;
  if (J.nrm) {
    J.nrm[3 * i] = n.x;
    J.nrm[3 * i + 1] = n.y;
    J.nrm[3 * i + 2] = n.z;
  }
  if (J.status) J.status[i] = st;
  if (J.iters) {
    J.iters[2 * i] = g.iters;
    J.iters[2 * i + 1] = ei;
  }
}

void* worker(void* arg) {
  const Job& J = *static_cast<const Job*>(arg);
  Work* M = new Work;
  for (int i = J.lo; i < J.hi; ++i) {
    if (J.xf)
      one<Posed<MemBodies>>(J, i, *M);
    else
      one<MemBodies>(J, i, *M);
  }
  delete M;
  return nullptr;
}

}  // namespace

extern "C" {

int twin_config(int reference, ogx_config* out) {
  *out = reference ? reference_config() : default_config();
  return 0;
}

// posed points of every body (the fused-transform pipeline's world points): out and
// local are xyz of all bodies concatenated, xf 12 floats per body
int twin_pose_points(int nbodies, const int32_t* counts, const float* local, const float* xf, float* out) {
  size_t k = 0;
  for (int b = 0; b < nbodies; ++b)
    for (int i = 0; i < counts[b]; ++i, ++k) {
      const fv3 p = pose_point(xf + 12 * (size_t)b, v3<float>(local[3 * k], local[3 * k + 1], local[3 * k + 2]));
      out[3 * k] = p.x;
      out[3 * k + 1] = p.y;
      out[3 * k + 2] = p.z;
    }
  return 0;
}

// xf: null, or poses (12 floats per body) to run the posed pipeline on the pool's bodies
int twin_run_posed(int npairs, const float* pool, const uint32_t* quad, const int32_t* counts,
                   const int32_t* pairs, int mode, const ogx_config* cfg, float* dist, gkSimplex* smp,
                   float* nrm, int32_t* status, int32_t* iters, int nthreads, const float* xf) {
  if (npairs < 0 || (mode != 1 && mode != 2)) return -1;
  Job base{0, npairs, mode, pool, quad, counts, pairs, cfg, dist, smp, nrm, status, iters, xf};
  if (nthreads <= 1 || npairs < 64) {
    worker(&base);
    return 0;
  }
  if (nthreads > 64) nthreads = 64;
  std::vector<pthread_t> th(nthreads);
  std::vector<Job> jobs(nthreads, base);
  for (int k = 0; k < nthreads; ++k) {
    jobs[k].lo = (int)((int64_t)npairs * k / nthreads);
    jobs[k].hi = (int)((int64_t)npairs * (k + 1) / nthreads);
    pthread_create(&th[k], nullptr, worker, &jobs[k]);
  }
  for (int k = 0; k < nthreads; ++k) pthread_join(th[k], nullptr);
  return 0;
}

int twin_run(int npairs, const float* pool, const uint32_t* quad, const int32_t* counts,
             const int32_t* pairs, int mode, const ogx_config* cfg, float* dist, gkSimplex* smp,
             float* nrm, int32_t* status, int32_t* iters, int nthreads) {
  return twin_run_posed(npairs, pool, quad, counts, pairs, mode, cfg, dist, smp, nrm, status, iters, nthreads,
                        nullptr);
}
}
