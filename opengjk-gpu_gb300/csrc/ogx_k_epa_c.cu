// ogx_k_epa_c.cu -- EPA bucket kernel variants that read the bodies from memory on every
// support scan, with 4-16 lanes per pair, and register-capped variants.
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_epa<4, 0>, 4, 0}, {k_epa<8, 0>, 8, 0}, {k_epa<16, 0>, 16, 0},
    // capped at 96 registers (5 blocks of 4 warps per SM)
    {k_epa<4, 1, 5>, 4, 1 + (5 << kOccShift)}, {k_epa<8, 1, 5>, 8, 1 + (5 << kOccShift)},
    {k_epa<8, 2, 5>, 8, 2 + (5 << kOccShift)}, {k_epa<8, 0, 5>, 8, 5 << kOccShift},
    {k_epa<16, 0, 5>, 16, 5 << kOccShift},
    // two register blocks at 128 registers (4 blocks per SM; the 96-register build spills)
    {k_epa<8, 2, 4>, 8, 2 + (4 << kOccShift)},
};

int epa_variants_c(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
