// ogx_k_epa_b.cu -- EPA bucket kernel variants with 32 lanes per pair and the
// memory-streamed variant for bodies above 512 points.
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_epa<32, 1>, 32, 1}, {k_epa<32, 2>, 32, 2}, {k_epa<32, 4>, 32, 4}, {k_epa<32, 0>, 32, 0},
};

int epa_variants_b(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
