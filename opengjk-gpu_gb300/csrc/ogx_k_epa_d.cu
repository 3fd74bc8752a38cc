// ogx_k_epa_d.cu -- EPA bucket kernel variants for bodies read from memory with the
// blocks staged through shared memory (2 blocks per lane in flight with cp.async), 8
// lanes per pair, capped at 128 registers (4 blocks of 4 warps per SM, which the working
// sets and the slots together still fit).  Measured slower than the register-loaded
// scans on the GB300 (the autotuner keeps those); compiled so that it can pick these
// where the balance between load latency and instruction count differs.  (EPA variants
// with the GJK kernels' four-blocks-in-flight scan at 128 registers were never picked by
// the autotuner on the 1M-pair power-law step and are not compiled.)
#include "ogx_kernels.cuh"

namespace ogx {

static const KernelInfo kVar[] = {
    {k_epa<8, 0, 4, 2>, 8, (4 << kOccShift) + (2 << kStageShift)},
};

int epa_variants_d(const KernelInfo** out) {
  *out = kVar;
  return (int)(sizeof(kVar) / sizeof(kVar[0]));
}

}  // namespace ogx
