// ogx_k_posed.cu -- GJK and EPA bucket kernels for bodies kept in their own frame with a
// pose each (the transform fused into the point reads, DevBatch::xf), one variant per
// size bucket: memory scans at the lane counts the autotuner picks for the world-frame
// kernels on power-law batches, 4 (GJK) or 5 (EPA) resident blocks per SM.
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kGjk[kBuckets] = {
    {k_gjk<1, 0, 4, 0, true>, 1, 4 << kOccShift}, {k_gjk<1, 0, 4, 0, true>, 1, 4 << kOccShift},
    {k_gjk<1, 0, 4, 0, true>, 1, 4 << kOccShift}, {k_gjk<2, 0, 4, 0, true>, 2, 4 << kOccShift},
    {k_gjk<4, 0, 4, 0, true>, 4, 4 << kOccShift}, {k_gjk<8, 0, 4, 0, true>, 8, 4 << kOccShift},
    {k_gjk<8, 0, 4, 0, true>, 8, 4 << kOccShift},
};
static const KernelInfo kEpa[kBuckets] = {
    {k_epa<8, 0, 5, 0, true>, 8, 5 << kOccShift},   {k_epa<8, 0, 5, 0, true>, 8, 5 << kOccShift},
    {k_epa<8, 0, 5, 0, true>, 8, 5 << kOccShift},   {k_epa<8, 0, 5, 0, true>, 8, 5 << kOccShift},
    {k_epa<8, 0, 5, 0, true>, 8, 5 << kOccShift},   {k_epa<8, 0, 5, 0, true>, 8, 5 << kOccShift},
    {k_epa<16, 0, 5, 0, true>, 16, 5 << kOccShift},
};

void posed_variants(const KernelInfo** gjk, const KernelInfo** epa) {
  *gjk = kGjk;
  *epa = kEpa;
}

}  // namespace ogx
