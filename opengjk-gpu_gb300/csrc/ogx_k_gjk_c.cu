// ogx_k_gjk_c.cu -- GJK bucket kernel variants with 1 and 2 lanes per pair for the
// smallest bodies (16 or 32 pairs per warp, no cross-lane reduction in the supports).
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_gjk<1, 4>, 1, 4},
    {k_gjk<2, 2>, 2, 2}, {k_gjk<2, 4>, 2, 4},
};

int gjk_variants_c(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
