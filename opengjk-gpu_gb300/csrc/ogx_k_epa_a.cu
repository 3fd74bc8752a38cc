// ogx_k_epa_a.cu -- EPA bucket kernel variants with 4, 8 and 16 lanes per pair (the
// polytope lives in shared memory, 2.3 KB per pair).
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_epa<4, 1>, 4, 1},   {k_epa<4, 2>, 4, 2},   {k_epa<4, 4>, 4, 4},
    {k_epa<8, 1>, 8, 1},   {k_epa<8, 2>, 8, 2},   {k_epa<8, 4>, 8, 4},
    {k_epa<16, 1>, 16, 1}, {k_epa<16, 2>, 16, 2}, {k_epa<16, 4>, 16, 4},
};

int epa_variants_a(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
