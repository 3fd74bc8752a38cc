// ogx_k_epa.cu -- EPA bucket kernels (teams of >= 8 lanes: the polytope lives in
// shared memory, 5.7 KB per pair, so fewer, wider teams per block).
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kEpa[kBuckets] = {
    {k_epa<8, 1>, 8, 1},   {k_epa<8, 1>, 8, 1},   {k_epa<8, 2>, 8, 2},   {k_epa<16, 2>, 16, 2},
    {k_epa<32, 2>, 32, 2}, {k_epa<32, 4>, 32, 4}, {k_epa<32, 0>, 32, 0},
};

const KernelInfo* epa_kernels() { return kEpa; }

}  // namespace ogx
