// ogx_k_gjk_e.cu -- GJK bucket kernel variants that run each team's pairs as a queue
// (k_gjk_q: a team that finishes a pair starts its next one while the other teams of
// the warp keep iterating), memory-read scans, 2-8 lanes per pair, capped at 128
// registers (4 blocks of 4 warps per SM).
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_gjk_q<2, 0, 4>, 2, (4 << kOccShift) + (1 << kQueueShift)},
    {k_gjk_q<4, 0, 4>, 4, (4 << kOccShift) + (1 << kQueueShift)},
    {k_gjk_q<8, 0, 4>, 8, (4 << kOccShift) + (1 << kQueueShift)},
};

int gjk_variants_e(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
