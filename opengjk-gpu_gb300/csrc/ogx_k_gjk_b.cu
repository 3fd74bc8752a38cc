// ogx_k_gjk_b.cu -- GJK bucket kernel variants with 16 and 32 lanes per pair, and the
// memory-streamed variant for bodies above 512 points.
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_gjk<16, 1>, 16, 1}, {k_gjk<16, 2>, 16, 2}, {k_gjk<16, 4>, 16, 4},
    {k_gjk<32, 1>, 32, 1}, {k_gjk<32, 2>, 32, 2}, {k_gjk<32, 4>, 32, 4},
    {k_gjk<32, 0>, 32, 0},
};

int gjk_variants_b(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
