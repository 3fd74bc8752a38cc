// ogx_k_epa_c.cu -- EPA bucket kernel variants that read the bodies from memory on every
// support scan, with 4-16 lanes per pair.
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_epa<4, 0>, 4, 0}, {k_epa<8, 0>, 8, 0}, {k_epa<16, 0>, 16, 0},
};

int epa_variants_c(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
