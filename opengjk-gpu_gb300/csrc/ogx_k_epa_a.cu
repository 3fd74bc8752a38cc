// ogx_k_epa_a.cu -- EPA bucket kernel variants with 8 and 16 lanes per pair (the polytope
// lives in shared memory, 5.7 KB per pair, so teams are at least 8 lanes wide).
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_epa<8, 1>, 8, 1},   {k_epa<8, 2>, 8, 2},   {k_epa<8, 4>, 8, 4},
    {k_epa<16, 1>, 16, 1}, {k_epa<16, 2>, 16, 2}, {k_epa<16, 4>, 16, 4},
};

int epa_variants_a(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
