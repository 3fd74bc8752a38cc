// ogx_k_gjk.cu -- GJK bucket kernels: (lanes per pair, register blocks per lane).
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kGjk[kBuckets] = {
    {k_gjk<4, 1>, 4, 1},   {k_gjk<8, 1>, 8, 1},   {k_gjk<8, 2>, 8, 2},   {k_gjk<16, 2>, 16, 2},
    {k_gjk<32, 2>, 32, 2}, {k_gjk<32, 4>, 32, 4}, {k_gjk<32, 0>, 32, 0},
};

const KernelInfo* gjk_kernels() { return kGjk; }

}  // namespace ogx
