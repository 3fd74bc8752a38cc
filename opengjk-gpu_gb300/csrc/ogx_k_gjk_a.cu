// ogx_k_gjk_a.cu -- GJK bucket kernel variants with 4 and 8 lanes per pair.
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_gjk<4, 1>, 4, 1}, {k_gjk<4, 2>, 4, 2}, {k_gjk<4, 4>, 4, 4},
    {k_gjk<8, 1>, 8, 1}, {k_gjk<8, 2>, 8, 2}, {k_gjk<8, 4>, 8, 4},
};

int gjk_variants_a(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
