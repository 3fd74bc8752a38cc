// ogx_k_gjk_e.cu -- GJK bucket kernel variants for bodies read from memory with the
// blocks staged through shared memory (4 blocks per lane in flight with cp.async), with
// 4 and 8 lanes per pair, capped at 128 registers (4 blocks of 4 warps per SM).  On the
// GB300 the autotuner keeps the register-loaded scans instead: the per-lane 16-byte
// copies and shared-memory reads take about twice the instructions of the loads they
// replace (bodies above 512 points, 200k-pair power-law batch: 104.6 M against 55.9 M
// warp instructions, 347 us against 220 us), more than the load latency they hide.
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_gjk<4, 0, 4, 4>, 4, (4 << kOccShift) + (4 << kStageShift)},
    {k_gjk<8, 0, 4, 4>, 8, (4 << kOccShift) + (4 << kStageShift)},
};

int gjk_variants_e(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
