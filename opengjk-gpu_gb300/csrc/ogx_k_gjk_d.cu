// ogx_k_gjk_d.cu -- GJK bucket kernel variants that read the bodies from memory on every
// support scan (no register copy), with 1-16 lanes per pair: many pairs per warp share
// each instruction of the per-pair step, and the scans hit L1/L2.
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_gjk<1, 0>, 1, 0}, {k_gjk<2, 0>, 2, 0}, {k_gjk<4, 0>, 4, 0},
    {k_gjk<8, 0>, 8, 0}, {k_gjk<16, 0>, 16, 0},
    // the same capped at 128 registers (4 blocks of 4 warps per SM)
    {k_gjk<1, 0, 4>, 1, 4 << kOccShift}, {k_gjk<2, 0, 4>, 2, 4 << kOccShift},
    {k_gjk<4, 0, 4>, 4, 4 << kOccShift}, {k_gjk<8, 0, 4>, 8, 4 << kOccShift},
    // capped at 96 registers (5 blocks per SM; a few spills)
    {k_gjk<1, 0, 5>, 1, 5 << kOccShift}, {k_gjk<4, 0, 5>, 4, 5 << kOccShift},
};

int gjk_variants_d(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
